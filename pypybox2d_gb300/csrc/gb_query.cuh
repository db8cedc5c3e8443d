// gb_query.cuh -- world queries on the device: the closest hit of a ray
// (World.ray_cast, pypybox2d/world.py:387-440) and the fixtures whose
// broad-phase box overlaps a query box (World.query_aabb, world.py:371-385).
//
// One warp per query; the lanes walk the world's fixtures (coalesced reads of
// the fixture arrays) and the warp reduces.  The reference walks its
// DynamicTree (dynamictree.py:190-273); the tree only prunes, so the set of
// fixtures a query reports is the set of fixtures whose fat AABB passes the
// same tests, which is what the lanes evaluate for every fixture.  All
// arithmetic is float64 in the reference's operation order; in the float64
// unit (no FMA contraction) the results are the reference's doubles.
#pragma once
#include "gb_world.cuh"

namespace gbq {

template <class R> __device__ __forceinline__ vec2<double> vtx(const Batch<R> &B, int f, int k) {
    return cvt<double>(B.f_v[(size_t)f * GB_MAX_POLY_VERTS + k]);
}
template <class R> __device__ __forceinline__ vec2<double> nrm(const Batch<R> &B, int f, int k) {
    return cvt<double>(B.f_n[(size_t)f * GB_MAX_POLY_VERTS + k]);
}

// Circle.ray_cast (shapes.py:147-171): Gino van den Bergen's quadratic
template <class R> __device__ bool ray_circle(const Batch<R> &B, int f, const xform2<double> &xf, vec2<double> p1,
                                              vec2<double> p2, vec2<double> *normal, double *fraction) {
    const vec2<double> position = xf.p + rmul(xf.q, vtx(B, f, 0));
    const double radius = (double)B.f_radius[f];
    const vec2<double> s = p1 - position;
    const double b = dot(s, s) - radius * radius;
    const vec2<double> r = p2 - p1;
    const double c = dot(s, r);
    const double rr = dot(r, r);
    const double sigma = c * c - rr * b;
    if (sigma < 0.0 || rr < 2.220446049250313e-16) return false;
    double a = -(c + sqrt(sigma));
    if (0.0 <= a && a <= 1.0 * rr) {
        a /= rr;
        *fraction = a;
        *normal = normalized(s + a * r);
        return true;
    }
    return false;
}

// Polygon.ray_cast (shapes.py:265-314): clip the ray against each edge's
// half-plane in the polygon's frame
template <class R> __device__ bool ray_polygon(const Batch<R> &B, int f, const xform2<double> &xf, vec2<double> p1,
                                               vec2<double> p2, vec2<double> *normal, double *fraction) {
    const vec2<double> q1 = rmul_t(xf.q, p1 - xf.p);
    const vec2<double> q2 = rmul_t(xf.q, p2 - xf.p);
    const vec2<double> d = q2 - q1;
    double lower = 0.0, upper = 1.0;
    int tagged = -1;
    const int n = B.f_count[f];
    for (int k = 0; k < n; ++k) {
        const vec2<double> nk = nrm(B, f, k);
        const double numerator = dot(nk, vtx(B, f, k) - q1);
        const double denominator = dot(nk, d);
        if (denominator == 0.0) {
            if (numerator < 0.0) return false;
        } else if (denominator < 0.0 && numerator < lower * denominator) {
            lower = numerator / denominator;
            tagged = k;
        } else if (denominator > 0.0 && numerator < upper * denominator) {
            upper = numerator / denominator;
        }
        if (upper < lower) return false;
    }
    if (tagged < 0) return false;
    *normal = rmul(xf.q, nrm(B, f, tagged));
    *fraction = lower;
    return true;
}

// Edge.ray_cast (shapes.py:655-702).  The normal it returns stays in the
// edge's own frame (the reference does not rotate it).
template <class R> __device__ bool ray_edge(const Batch<R> &B, int f, const xform2<double> &xf, vec2<double> p1,
                                            vec2<double> p2, vec2<double> *normal, double *fraction) {
    const vec2<double> q1 = rmul_t(xf.q, p1 - xf.p);
    const vec2<double> q2 = rmul_t(xf.q, p2 - xf.p);
    const vec2<double> d = q2 - q1;
    const vec2<double> v1 = vtx(B, f, 0), v2 = vtx(B, f, 1);
    const vec2<double> e = v2 - v1;
    vec2<double> nn = normalized(mk<double>(e.y, -e.x));
    const double numerator = dot(nn, v1 - q1);
    const double denominator = dot(nn, d);
    if (denominator == 0.0) return false;
    const double t = numerator / denominator;
    if (t < 0.0 || 1.0 < t) return false;
    const vec2<double> q = q1 + t * d;
    const vec2<double> r = v2 - v1;
    const double rr = dot(r, r);
    if (rr == 0.0) return false;
    const double s = dot(q - v1, r) / rr;
    if (s < 0.0 || 1.0 < s) return false;
    *fraction = t;
    *normal = numerator > 0.0 ? -nn : nn;
    return true;
}

// AABB.test_overlap (aabbmodule.c AABB_test_overlap): a against b
__device__ __forceinline__ bool box_overlap(const dbox &a, double blx, double bly, double bhx, double bhy) {
    return !((blx - a.z) > 0.0 || (bly - a.w) > 0.0 || (a.x - bhx) > 0.0 || (a.y - bhy) > 0.0);
}

}  // namespace gbq

namespace gbq {
// A ray with the segment tests of DynamicTree.ray_cast (dynamictree.py:
// 222-250) at max_fraction 1 (World.ray_cast passes 1.0)
struct RaySeg {
    vec2<double> p1, p2, v, abs_v;
    double slx, sly, shx, shy;
};
__device__ __forceinline__ RaySeg ray_seg(const gb_ray &ray) {
    RaySeg s;
    s.p1 = mk<double>(ray.p1x, ray.p1y);
    s.p2 = mk<double>(ray.p2x, ray.p2y);
    const vec2<double> r = normalized(s.p2 - s.p1);
    s.v = cross(1.0, r);
    s.abs_v = mk<double>(fabs(s.v.x), fabs(s.v.y));
    const vec2<double> t = s.p1 + 1.0 * (s.p2 - s.p1);
    s.slx = pymin(s.p1.x, t.x); s.sly = pymin(s.p1.y, t.y);
    s.shx = pymax(s.p1.x, t.x); s.shy = pymax(s.p1.y, t.y);
    return s;
}
// world-local fixture k: reported by the tree and hit by its shape?
template <class R> __device__ bool ray_fixture(const Batch<R> &B, const WorldHdr &H, int k, const RaySeg &s,
                                               vec2<double> *nrm, double *fr) {
    const int f = H.fbase + k;
    if (!(B.b_flags[H.bbase + B.f_body[f]] & GB_BODY_ACTIVE)) return false;   // an inactive body's fixtures have no proxy
    const dbox a = B.f_aabb[f];
    if (!box_overlap(a, s.slx, s.sly, s.shx, s.shy)) return false;
    const vec2<double> c = mk<double>(0.5 * (a.z + a.x), 0.5 * (a.w + a.y));
    const vec2<double> h = mk<double>(0.5 * (a.z - a.x), 0.5 * (a.w - a.y));
    const double separation = fabs(dot(s.v, s.p1 - c)) - dot(s.abs_v, h);
    if (separation > 0.0) return false;
    const int b = H.bbase + B.f_body[f];
    xform2<double> xf;
    xf.p = B.b_xp[b];
    xf.q = B.b_xq[b];
    const int type = B.f_type[f];
    if (type == GB_SHAPE_CIRCLE) return ray_circle(B, f, xf, s.p1, s.p2, nrm, fr);
    if (type == GB_SHAPE_POLYGON) return ray_polygon(B, f, xf, s.p1, s.p2, nrm, fr);
    if (type == GB_SHAPE_EDGE) return ray_edge(B, f, xf, s.p1, s.p2, nrm, fr);
    return false;
}
// world.py:431: (1 - fraction) * point1 + fraction * point2
__device__ __forceinline__ gb_ray_hit make_hit(const RaySeg &s, int k, vec2<double> n, double fr) {
    gb_ray_hit o;
    o.fixture = k;
    o._pad0 = 0;
    const vec2<double> pt = (1.0 - fr) * s.p1 + fr * s.p2;
    o.px = pt.x; o.py = pt.y; o.nx = n.x; o.ny = n.y; o.fraction = fr;
    return o;
}
}  // namespace gbq

// One warp per ray: the closest hit over the ray's world (ties: the lower
// fixture index).
template <class R> __global__ void k_ray_cast(Batch<R> B, const gb_ray *rays, int n, gb_ray_hit *hits) {
    const int lane = threadIdx.x & 31;
    const int q = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (q >= n) return;
    const gb_ray ray = rays[q];
    const WorldHdr &H = B.hdr[ray.world];
    const gbq::RaySeg seg = gbq::ray_seg(ray);
    const vec2<double> p1 = seg.p1, p2 = seg.p2;
    double best = 2.0;
    int best_f = -1;
    vec2<double> best_n = mk<double>(0.0, 0.0);
    for (int k = lane; k < H.nf; k += 32) {
        vec2<double> nrm;
        double fr = 0.0;
        if (gbq::ray_fixture(B, H, k, seg, &nrm, &fr) && fr < best) { best = fr; best_f = k; best_n = nrm; }
    }
    // lexicographic (fraction, fixture) minimum over the warp
    for (int off = 16; off > 0; off >>= 1) {
        const double ob = __shfl_down_sync(0xffffffffu, best, off);
        const int of = __shfl_down_sync(0xffffffffu, best_f, off);
        const double onx = __shfl_down_sync(0xffffffffu, best_n.x, off);
        const double ony = __shfl_down_sync(0xffffffffu, best_n.y, off);
        if (of >= 0 && (best_f < 0 || ob < best || (ob == best && of < best_f))) {
            best = ob; best_f = of; best_n = mk<double>(onx, ony);
        }
    }
    if (lane == 0) {
        gb_ray_hit o;
        o.fixture = best_f;
        o._pad0 = 0;
        if (best_f >= 0) {
            const vec2<double> pt = (1.0 - best) * p1 + best * p2;
            o.px = pt.x; o.py = pt.y; o.nx = best_n.x; o.ny = best_n.y; o.fraction = best;
        } else {
            o.px = o.py = o.nx = o.ny = 0.0;
            o.fraction = 1.0;
        }
        hits[q] = o;
    }
}

// One warp per ray: every hit (the generator form of World.ray_cast with
// each fraction left at 1), in fixture order; the first `cap` go to
// hits[q * cap ...], counts[q] is the full number.
template <class R> __global__ void k_ray_cast_all(Batch<R> B, const gb_ray *rays, int n, gb_ray_hit *hits, int cap,
                                                  int *counts) {
    const int lane = threadIdx.x & 31;
    const int q = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (q >= n) return;
    const gb_ray ray = rays[q];
    const WorldHdr &H = B.hdr[ray.world];
    const gbq::RaySeg seg = gbq::ray_seg(ray);
    int found = 0;
    for (int k0 = 0; k0 < H.nf; k0 += 32) {
        const int k = k0 + lane;
        vec2<double> nrm = mk<double>(0.0, 0.0);
        double fr = 0.0;
        const bool hit = k < H.nf && gbq::ray_fixture(B, H, k, seg, &nrm, &fr);
        const unsigned m = __ballot_sync(0xffffffffu, hit);
        const int pos = found + __popc(m & ((1u << lane) - 1u));
        if (hit && pos < cap) hits[(size_t)q * cap + pos] = gbq::make_hit(seg, k, nrm, fr);
        found += __popc(m);
    }
    if (lane == 0) counts[q] = found;
}

// One warp per query box: the fixtures whose fat AABB overlaps it
// (DynamicTree.query, dynamictree.py:190-207), in fixture order; the first
// `cap` go to out[q * cap ...], counts[q] is the full number.
template <class R> __global__ void k_query_aabb(Batch<R> B, const gb_aabb_query *qs, int n, int *out, int cap, int *counts) {
    const int lane = threadIdx.x & 31;
    const int q = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (q >= n) return;
    const gb_aabb_query box = qs[q];
    const WorldHdr &H = B.hdr[box.world];
    int found = 0;
    for (int k0 = 0; k0 < H.nf; k0 += 32) {
        const int k = k0 + lane;
        bool hit = false;
        if (k < H.nf)
            hit = (B.b_flags[H.bbase + B.f_body[H.fbase + k]] & GB_BODY_ACTIVE) &&
                  gbq::box_overlap(B.f_aabb[H.fbase + k], box.lx, box.ly, box.ux, box.uy);
        const unsigned m = __ballot_sync(0xffffffffu, hit);
        const int pos = found + __popc(m & ((1u << lane) - 1u));
        if (hit && pos < cap) out[(size_t)q * cap + pos] = k;
        found += __popc(m);
    }
    if (lane == 0) counts[q] = found;
}

// gb_collide.cuh -- narrow phase, GJK distance and time of impact, one pair
// per thread.  Each function follows the reference function it names
// (pypybox2d/collision.py, collision_util.py, distance.py, toi.py); feature
// ids are packed as index_a | index_b << 8 | type_a << 16 | type_b << 24,
// the 4-tuple of contact_util.py:50-99, so warm-start matching compares the
// same keys as the reference.  GJK and TOI always run in float64.
#pragma once
#include "gb_math.cuh"
#include "../../include/gb2d.h"

#define GB_LINEAR_SLOP 0.005
#define GB_POLYGON_RADIUS (2.0 * 0.005)
#define GB_ANGULAR_SLOP 0.03490658503988659
#define GB_MAX_FLOAT 1.7976931348623157e+308
#define GB_EPSILON 2.220446049250313e-16
#define GB_EPSILON_SQR 4.930380657631324e-32
#define GB_RELATIVE_TOL 0.98
#define GB_ABSOLUTE_TOL 0.001
#define GB_VERTEX 0
#define GB_FACE 1

template <class R> struct Manifold {
    int type, count;
    vec2<R> ln, lp;
    vec2<R> plp[2];
    R ni[2], ti[2];
    uint32_t id[2];
};

// A shape as the narrow phase sees it: vertices/normals point into the
// fixture's 8 slots (a circle keeps its centre in slot 0, an edge its
// vertices 1, 2, 0, 3 in slots 0, 1, 2, 3).
template <class R> struct Shape {
    int type, count;
    uint32_t flags;
    R radius;
    const vec2<R> *v;
    const vec2<R> *n;
};

static GB_HD uint32_t fid(int ia, int ib, int ta, int tb) {
    return (uint32_t)(ia & 0xff) | ((uint32_t)(ib & 0xff) << 8) | ((uint32_t)(ta & 0xff) << 16) | ((uint32_t)(tb & 0xff) << 24);
}

template <class R> struct ClipV { vec2<R> v; int ia, ib, ta, tb; };

// collision.py:46-66
template <class R> __device__ void collide_circles(Manifold<R> &m, const Shape<R> &a, xform2<R> xa, const Shape<R> &b, xform2<R> xb) {
    m.count = 0;
    vec2<R> pa = xmul(xa, a.v[0]), pb = xmul(xb, b.v[0]);
    vec2<R> d = pb - pa;
    R dist_sqr = len2(d);
    R radius = a.radius + b.radius;
    if (dist_sqr > sq(radius)) return;
    m.type = GB_M_CIRCLES;
    m.lp = a.v[0];
    m.ln = mk<R>(0, 0);
    m.count = 1;
    m.plp[0] = b.v[0];
    m.id[0] = 0;
}

// collision.py:68-141
template <class R> __device__ void collide_polygon_circle(Manifold<R> &m, const Shape<R> &pa, xform2<R> xa, const Shape<R> &cb, xform2<R> xb) {
    m.count = 0;
    vec2<R> c = xmul(xb, cb.v[0]);
    vec2<R> cl = xmul_t(xa, c);
    int normal_index = 0;
    R separation = (R)-GB_MAX_FLOAT;
    if (sizeof(R) == 4) separation = -3.4028234663852886e+38f;
    R radius = pa.radius + cb.radius;
    int n = pa.count;
    for (int i = 0; i < n; ++i) {
        R s = dot(pa.n[i], cl - pa.v[i]);
        if (s > radius) return;
        if (s > separation) { separation = s; normal_index = i; }
    }
    int i1 = normal_index, i2 = (i1 + 1) % n;
    vec2<R> v1 = pa.v[i1], v2 = pa.v[i2];
    if (separation < (R)GB_EPSILON) {
        m.count = 1; m.type = GB_M_FACE_A;
        m.ln = pa.n[normal_index];
        m.lp = (R)0.5 * (v1 + v2);
        m.plp[0] = cb.v[0];
        m.id[0] = 0;
        return;
    }
    R u1 = dot(cl - v1, v2 - v1);
    R u2 = dot(cl - v2, v1 - v2);
    if (u1 < (R)0) {
        vec2<R> dd = cl - v1;
        if (dot(dd, dd) > sq(radius)) return;
        m.ln = normalized(cl - v1);
        m.lp = v1;
    } else if (u2 < (R)0) {
        vec2<R> dd = cl - v2;
        if (dot(dd, dd) > sq(radius)) return;
        m.ln = normalized(cl - v2);
        m.lp = v2;
    } else {
        vec2<R> fc = (R)0.5 * (v1 + v2);
        R sep = dot(cl - fc, pa.n[i1]);
        if (sep > radius) return;
        m.ln = pa.n[i1];
        m.lp = fc;
    }
    m.count = 1; m.type = GB_M_FACE_A;
    m.plp[0] = cb.v[0];
    m.id[0] = 0;
}

// collision_util.py:31-52
template <class R> __device__ R edge_separation(const Shape<R> &p1, xform2<R> x1, int edge1, const Shape<R> &p2, xform2<R> x2) {
    vec2<R> n1w = rmul(x1.q, p1.n[edge1]);
    vec2<R> n1 = rmul_t(x2.q, n1w);
    int index = 0;
    R min_dot = 0;
    for (int i = 0; i < p2.count; ++i) {
        R d = dot(p2.v[i], n1);
        if (i == 0 || d < min_dot) { min_dot = d; index = i; }
    }
    vec2<R> v1 = xmul(x1, p1.v[edge1]);
    vec2<R> v2 = xmul(x2, p2.v[index]);
    return dot(v2 - v1, n1w);
}

// collision_util.py:54-109 (initial direction from the body origins: the
// reference's Polygon._centroid stays (0, 0), shapes.py:244)
template <class R> __device__ R max_separation(const Shape<R> &p1, xform2<R> x1, const Shape<R> &p2, xform2<R> x2, int *edge_out) {
    int count1 = p1.count;
    vec2<R> z = mk<R>(0, 0);
    vec2<R> d = xmul(x2, z) - xmul(x1, z);
    vec2<R> dl = rmul_t(x1.q, d);
    int edge = 0;
    R max_dot = 0;
    for (int i = 0; i < count1; ++i) {
        R dd = dot(p1.n[i], dl);
        if (i == 0 || dd > max_dot) { max_dot = dd; edge = i; }
    }
    R s = edge_separation(p1, x1, edge, p2, x2);
    int prev_edge = (edge - 1 + count1) % count1;
    R s_prev = edge_separation(p1, x1, prev_edge, p2, x2);
    int next_edge = (edge + 1) % count1;
    R s_next = edge_separation(p1, x1, next_edge, p2, x2);
    int inc, best_edge;
    R best;
    if (s_prev > s && s_prev > s_next) { inc = -1; best_edge = prev_edge; best = s_prev; }
    else if (s_next > s) { inc = 1; best_edge = next_edge; best = s_next; }
    else { *edge_out = edge; return s; }
    for (int guard = 0; guard < 64; ++guard) {
        edge = (inc == -1) ? (best_edge - 1 + count1) % count1 : (best_edge + 1) % count1;
        s = edge_separation(p1, x1, edge, p2, x2);
        if (s > best) { best_edge = edge; best = s; }
        else break;
    }
    *edge_out = best_edge;
    return best;
}

// collision_util.py:135-164
template <class R> __device__ int clip_segment(ClipV<R> out[2], const ClipV<R> in[2], vec2<R> normal, R offset, int via) {
    int n = 0;
    R d0 = dot(normal, in[0].v) - offset;
    R d1 = dot(normal, in[1].v) - offset;
    if (d0 <= (R)0) out[n++] = in[0];
    if (d1 <= (R)0) out[n++] = in[1];
    if (d0 * d1 < (R)0) {
        R interp = d0 / (d0 - d1);
        ClipV<R> cv;
        cv.v = in[0].v + interp * (in[1].v - in[0].v);
        cv.ia = via; cv.ib = in[0].ib; cv.ta = GB_VERTEX; cv.tb = GB_FACE;
        if (n < 2) out[n] = cv;
        n++;
    }
    return n;
}

// collision.py:144-241 (+ collision_util.py:111-133 find_incident_edge)
template <class R> __device__ void collide_polygons(Manifold<R> &m, const Shape<R> &pa, xform2<R> xa, const Shape<R> &pb, xform2<R> xb) {
    m.count = 0;
    R total_radius = pa.radius + pb.radius;
    int edge_a, edge_b;
    R sep_a = max_separation(pa, xa, pb, xb, &edge_a);
    if (sep_a > total_radius) return;
    R sep_b = max_separation(pb, xb, pa, xa, &edge_b);
    if (sep_b > total_radius) return;
    const Shape<R> *p1, *p2;
    xform2<R> x1, x2;
    int edge1, flip;
    if (sep_b > ((R)GB_RELATIVE_TOL * sep_a + (R)GB_ABSOLUTE_TOL)) {
        p1 = &pb; p2 = &pa; x1 = xb; x2 = xa; edge1 = edge_b; m.type = GB_M_FACE_B; flip = 1;
    } else {
        p1 = &pa; p2 = &pb; x1 = xa; x2 = xb; edge1 = edge_a; m.type = GB_M_FACE_A; flip = 0;
    }
    ClipV<R> inc[2];
    {
        vec2<R> n1 = rmul_t(x2.q, rmul(x1.q, p1->n[edge1]));
        int index = 0;
        R min_dot = 0;
        for (int i = 0; i < p2->count; ++i) {
            R d = dot(n1, p2->n[i]);
            if (i == 0 || d < min_dot) { min_dot = d; index = i; }
        }
        int i1 = index, i2 = (i1 + 1) % p2->count;
        inc[0].v = xmul(x2, p2->v[i1]); inc[0].ia = edge1; inc[0].ib = i1; inc[0].ta = GB_FACE; inc[0].tb = GB_VERTEX;
        inc[1].v = xmul(x2, p2->v[i2]); inc[1].ia = edge1; inc[1].ib = i2; inc[1].ta = GB_FACE; inc[1].tb = GB_VERTEX;
    }
    int iv1 = edge1, iv2 = (edge1 + 1) % p1->count;
    vec2<R> v11 = p1->v[iv1], v12 = p1->v[iv2];
    vec2<R> ltan = normalized(v12 - v11);
    vec2<R> lnorm = cross(ltan, (R)1);
    vec2<R> plane = (R)0.5 * (v11 + v12);
    vec2<R> tangent = rmul(x1.q, ltan);
    vec2<R> normal = cross(tangent, (R)1);
    v11 = xmul(x1, v11);
    v12 = xmul(x1, v12);
    R front = dot(normal, v11);
    R side1 = -dot(tangent, v11) + total_radius;
    R side2 = dot(tangent, v12) + total_radius;
    ClipV<R> cp1[2], cp2[2];
    if (clip_segment(cp1, inc, -tangent, side1, iv1) < 2) return;
    if (clip_segment(cp2, cp1, tangent, side2, iv2) < 2) return;
    m.ln = lnorm;
    m.lp = plane;
    int pc = 0;
    for (int i = 0; i < 2; ++i) {
        R separation = dot(normal, cp2[i].v) - front;
        if (separation <= total_radius) {
            m.plp[pc] = xmul_t(x2, cp2[i].v);
            m.id[pc] = flip ? fid(cp2[i].ib, cp2[i].ia, cp2[i].tb, cp2[i].ta) : fid(cp2[i].ia, cp2[i].ib, cp2[i].ta, cp2[i].tb);
            pc++;
        }
    }
    m.count = pc;
}

// collision.py:245-353
template <class R> __device__ void collide_edge_circle(Manifold<R> &m, const Shape<R> &ea, xform2<R> xa, const Shape<R> &cb, xform2<R> xb) {
    m.count = 0;
    vec2<R> Q = xmul_t(xa, xmul(xb, cb.v[0]));
    vec2<R> A = ea.v[0], B = ea.v[1];
    vec2<R> e = B - A;
    R u = dot(e, B - Q);
    R v = dot(e, Q - A);
    R radius = ea.radius + cb.radius;
    if (v <= (R)0) {
        vec2<R> d = Q - A;
        if (dot(d, d) > sq(radius)) return;
        if (ea.flags & GB_FIX_EDGE_HAS_V0) {
            vec2<R> e1 = A - ea.v[2];
            if (dot(e1, A - Q) > (R)0) return;
        }
        m.count = 1; m.type = GB_M_CIRCLES; m.ln = mk<R>(0, 0); m.lp = A;
        m.id[0] = fid(0, 0, GB_VERTEX, GB_VERTEX); m.plp[0] = cb.v[0];
        return;
    }
    if (u <= (R)0) {
        vec2<R> d = Q - B;
        if (dot(d, d) > sq(radius)) return;
        if (ea.flags & GB_FIX_EDGE_HAS_V3) {
            vec2<R> e2 = ea.v[3] - B;
            if (dot(e2, Q - B) > (R)0) return;
        }
        m.count = 1; m.type = GB_M_CIRCLES; m.ln = mk<R>(0, 0); m.lp = B;
        m.id[0] = fid(1, 0, GB_VERTEX, GB_VERTEX); m.plp[0] = cb.v[0];
        return;
    }
    R den = dot(e, e);
    vec2<R> P = ((R)1 / den) * (u * A + v * B);
    vec2<R> d = Q - P;
    if (dot(d, d) > sq(radius)) return;
    vec2<R> n = mk<R>(-e.y, e.x);
    if (dot(n, Q - A) < (R)0) n = mk<R>(-n.x, -n.y);
    n = normalized(n);
    m.count = 1; m.type = GB_M_FACE_A; m.ln = n; m.lp = A;
    m.id[0] = fid(0, 0, GB_FACE, GB_VERTEX); m.plp[0] = cb.v[0];
}

// collision.py:385-690 EPCollider
template <class R> struct EPProxy { vec2<R> v[GB_MAX_POLY_VERTS], n[GB_MAX_POLY_VERTS]; int count; vec2<R> centroid; };
template <class R> struct EPAxis { int type, index; R sep; };

template <class R> __device__ bool ep_valid(vec2<R> n, vec2<R> l11, vec2<R> l12, vec2<R> l21, vec2<R> l22) {
    const R as = (R)-GB_ANGULAR_SLOP;
    bool v1 = (cross(n, l11) >= as) && (cross(l12, n) >= as);
    bool v2 = (cross(n, l21) >= as) && (cross(l22, n) >= as);
    return v1 && v2;
}

template <class R> __device__ void collide_edge_polygon(Manifold<R> &m, const Shape<R> &ea, xform2<R> xa, const Shape<R> &pb, xform2<R> xb) {
    // transform.c Transform_mul_t(xa, xb): position pb - pa (not rotated), rotation Ra^T Rb
    xform2<R> xf;
    xf.p = xb.p - xa.p;
    xf.q.c = xa.q.c * xb.q.c + xa.q.s * xb.q.s;
    xf.q.s = (-xa.q.s) * xb.q.c + xa.q.c * xb.q.s;
    bool has_v0 = (ea.flags & GB_FIX_EDGE_HAS_V0) != 0, has_v3 = (ea.flags & GB_FIX_EDGE_HAS_V3) != 0;
    vec2<R> v1 = ea.v[0], v2 = ea.v[1];
    vec2<R> e = v2 - v1;
    vec2<R> en = normalized(mk<R>(e.y, -e.x));
    EPProxy<R> A, B;
    A.count = 2; A.v[0] = v1; A.v[1] = v2; A.n[0] = en; A.n[1] = -en;
    A.centroid = (R)0.5 * (v1 + v2);
    B.centroid = xmul(xf, mk<R>(0, 0));
    B.count = pb.count;
    for (int i = 0; i < pb.count; ++i) { B.v[i] = xmul(xf, pb.v[i]); B.n[i] = rmul(xf.q, pb.n[i]); }
    const R radius = (R)(2.0 * GB_POLYGON_RADIUS);
    vec2<R> z = mk<R>(0, 0), l11 = z, l12 = z, l21 = z, l22 = z;
    m.count = 0;
    vec2<R> cb = B.centroid;
    if (has_v0) {
        vec2<R> v0 = ea.v[2];
        vec2<R> e0 = v1 - v0, e1 = v2 - v1;
        vec2<R> n0 = normalized(mk<R>(e0.y, -e0.x)), n1 = normalized(mk<R>(e1.y, -e1.x));
        bool convex = cross(n0, n1) >= (R)0;
        bool f0 = dot(n0, cb - v0) >= (R)0, f1 = dot(n1, cb - v1) >= (R)0;
        if (convex) { if (f0 || f1) { l11 = n1; l12 = n0; } else { l11 = -n1; l12 = -n0; } }
        else { if (f0 && f1) { l11 = n0; l12 = n1; } else { l11 = -n0; l12 = -n1; } }
    }
    if (has_v3) {
        vec2<R> v3 = ea.v[3];
        vec2<R> e1 = v2 - v1, e2 = v3 - v2;
        vec2<R> n1 = normalized(mk<R>(e1.y, -e1.x)), n2 = normalized(mk<R>(e2.y, -e2.x));
        bool convex = cross(n1, n2) >= (R)0;
        bool f1 = dot(n1, cb - v1) >= (R)0, f2 = dot(n2, cb - v2) >= (R)0;
        if (convex) { if (f1 || f2) { l21 = n2; l22 = n1; } else { l21 = -n2; l22 = -n1; } }
        else { if (f1 && f2) { l21 = n1; l22 = n2; } else { l21 = -n1; l22 = -n2; } }
    }
    const R neg_max = (sizeof(R) == 4) ? (R)-3.4028234663852886e+38 : (R)-GB_MAX_FLOAT;
    EPAxis<R> ea_ax; ea_ax.type = 0; ea_ax.index = -1; ea_ax.sep = neg_max;
    for (int i = 0; i < 2; ++i) {
        vec2<R> n = (i == 0) ? en : -en;
        if (!ep_valid(n, l11, l12, l21, l22)) continue;
        R mn = 0;
        for (int k = 0; k < B.count; ++k) {
            R d = dot(n, B.v[k] - v1);
            if (k == 0 || d < mn) mn = d;
        }
        if (mn > radius) { ea_ax.type = 1; ea_ax.index = i; ea_ax.sep = mn; break; }
        if (mn > ea_ax.sep) { ea_ax.type = 1; ea_ax.index = i; ea_ax.sep = mn; }
    }
    if (ea_ax.type == 0) return;
    if (ea_ax.sep > radius) return;
    EPAxis<R> pa_ax; pa_ax.type = 0; pa_ax.index = -1; pa_ax.sep = neg_max;
    for (int i = 0; i < B.count; ++i) {
        vec2<R> n = -B.n[i];
        if (!ep_valid(n, l11, l12, l21, l22)) continue;
        R s1 = dot(n, B.v[i] - v1);
        R s2 = dot(n, B.v[i] - v2);
        R s = pymin(s1, s2);
        if (s > radius) { pa_ax.type = 2; pa_ax.index = i; pa_ax.sep = s; }
        if (s > pa_ax.sep) { pa_ax.type = 2; pa_ax.index = i; pa_ax.sep = s; }
    }
    if (pa_ax.type != 0 && pa_ax.sep > radius) return;
    EPAxis<R> prim;
    if (pa_ax.type == 0) prim = ea_ax;
    else if (pa_ax.sep > (R)GB_RELATIVE_TOL * ea_ax.sep + (R)GB_ABSOLUTE_TOL) prim = pa_ax;
    else prim = ea_ax;
    const EPProxy<R> *p1, *p2;
    if (prim.type == 1) { p1 = &A; p2 = &B; m.type = GB_M_FACE_A; }
    else { p1 = &B; p2 = &A; m.type = GB_M_FACE_B; }
    int edge1 = prim.index;
    ClipV<R> inc[2];
    {
        vec2<R> n1 = p1->n[edge1];
        int index = 0;
        R min_dot = 0;
        for (int i = 0; i < p2->count; ++i) {
            R d = dot(n1, p2->n[i]);
            if (i == 0 || d < min_dot) { min_dot = d; index = i; }
        }
        int i1 = index, i2 = (i1 + 1) % p2->count;
        inc[0].v = p2->v[i1]; inc[0].ia = edge1; inc[0].ib = i1; inc[0].ta = GB_FACE; inc[0].tb = GB_VERTEX;
        inc[1].v = p2->v[i2]; inc[1].ia = edge1; inc[1].ib = i2; inc[1].ta = GB_FACE; inc[1].tb = GB_VERTEX;
    }
    int iv1 = edge1, iv2 = (edge1 + 1) % p1->count;
    vec2<R> v11 = p1->v[iv1], v12 = p1->v[iv2];
    vec2<R> tangent = normalized(v12 - v11);
    vec2<R> normal = cross(tangent, (R)1);
    vec2<R> plane = (R)0.5 * (v11 + v12);
    R front = dot(normal, v11);
    R side1 = -dot(tangent, v11) + radius;
    R side2 = dot(tangent, v12) + radius;
    ClipV<R> cp1[2], cp2[2];
    if (clip_segment(cp1, inc, -tangent, side1, iv1) < 2) return;
    if (clip_segment(cp2, cp1, tangent, side2, iv2) < 2) return;
    if (prim.type == 1) { m.ln = normal; m.lp = plane; }
    else { m.ln = rmul_t(xf.q, normal); m.lp = xmul_t(xf, plane); }
    int pc = 0;
    for (int i = 0; i < 2; ++i) {
        R separation = dot(normal, cp2[i].v) - front;
        if (separation <= radius) {
            if (prim.type == 1) {
                m.plp[pc] = xmul_t(xf, cp2[i].v);
                m.id[pc] = fid(cp2[i].ia, cp2[i].ib, cp2[i].ta, cp2[i].tb);
            } else {
                // collision.py:532 stores (type_b, type_a, index_b, index_a)
                m.plp[pc] = cp2[i].v;
                m.id[pc] = fid(cp2[i].tb, cp2[i].ta, cp2[i].ib, cp2[i].ia);
            }
            pc++;
        }
    }
    m.count = pc;
}

// contact.py:294-311 dispatch on the (primary A, B) shape types
template <class R> __device__ void evaluate_manifold(Manifold<R> &m, const Shape<R> &a, xform2<R> xa, const Shape<R> &b, xform2<R> xb) {
    int ta = a.type, tb = b.type;
    if (ta == GB_SHAPE_POLYGON && tb == GB_SHAPE_POLYGON) collide_polygons(m, a, xa, b, xb);
    else if (ta == GB_SHAPE_CIRCLE && tb == GB_SHAPE_CIRCLE) collide_circles(m, a, xa, b, xb);
    else if (ta == GB_SHAPE_POLYGON && tb == GB_SHAPE_CIRCLE) collide_polygon_circle(m, a, xa, b, xb);
    else if (ta == GB_SHAPE_EDGE && tb == GB_SHAPE_CIRCLE) collide_edge_circle(m, a, xa, b, xb);
    else if (ta == GB_SHAPE_EDGE && tb == GB_SHAPE_POLYGON) collide_edge_polygon(m, a, xa, b, xb);
    else m.count = 0;
}

// contact.py:294-311: registered pairs and which of the two is primary (A)
static GB_HD bool pair_registered(int t1, int t2, bool *primary) {
    if (t1 == t2) { *primary = true; return t1 == GB_SHAPE_CIRCLE || t1 == GB_SHAPE_POLYGON; }
    if (t1 == GB_SHAPE_POLYGON && t2 == GB_SHAPE_CIRCLE) { *primary = true; return true; }
    if (t1 == GB_SHAPE_CIRCLE && t2 == GB_SHAPE_POLYGON) { *primary = false; return true; }
    if (t1 == GB_SHAPE_EDGE && (t2 == GB_SHAPE_CIRCLE || t2 == GB_SHAPE_POLYGON)) { *primary = true; return true; }
    if (t2 == GB_SHAPE_EDGE && (t1 == GB_SHAPE_CIRCLE || t1 == GB_SHAPE_POLYGON)) { *primary = false; return true; }
    *primary = true;
    return false;
}

// ------------------------------------------------------------------
// distance.py GJK (float64)
struct DProxy { vec2<double> v[GB_MAX_POLY_VERTS]; int count; double radius; };

template <class R> __device__ void dproxy_init(DProxy &p, const Shape<R> &s) {
    int n = (s.type == GB_SHAPE_CIRCLE) ? 1 : (s.type == GB_SHAPE_POLYGON ? s.count : 2);
    for (int i = 0; i < n; ++i) p.v[i] = mk<double>((double)s.v[i].x, (double)s.v[i].y);
    p.count = n;
    p.radius = (double)s.radius;
}
static __device__ __forceinline__ int dsupport(const DProxy &p, vec2<double> d) {
    int best = 0;
    double bd = 0;
    for (int i = 0; i < p.count; ++i) {
        double x = dot(p.v[i], d);
        if (i == 0 || x > bd) { bd = x; best = i; }
    }
    return best;
}

struct SCache { double metric; int count; int ia[3], ib[3]; };
struct SVert { vec2<double> wa, wb, w; double a; int ia, ib; };

// The reference simplex rebinds _v1/_v2 to copies in solve2/solve3 while new
// support points are written into the three objects captured at the start
// of shape_distance (distance.py:469, 524-531); orig[] are those objects,
// r1o/r2o tell whether _v1/_v2 still refer to them.
struct Simplex {
    SVert orig[3];
    SVert d1, d2;
    int r1o, r2o, count;
    __device__ SVert &v1() { return r1o ? orig[0] : d1; }
    __device__ SVert &v2() { return r2o ? orig[1] : d2; }
    __device__ SVert &v3() { return orig[2]; }
    __device__ SVert &vk(int k) { return k == 0 ? v1() : (k == 1 ? v2() : v3()); }
};

static __device__ double simplex_metric(Simplex &s) {
    if (s.count == 1) return 0.0;
    if (s.count == 2) return len(s.v1().w - s.v2().w);
    return cross(s.v2().w - s.v1().w, s.v3().w - s.v1().w);
}

static __device__ void simplex_solve2(Simplex &s) {
    vec2<double> w1 = s.v1().w, w2 = s.v2().w;
    vec2<double> e12 = w2 - w1;
    double d12_2 = -dot(w1, e12);
    if (d12_2 <= 0.0) { s.v1().a = 1.0; s.count = 1; return; }
    double d12_1 = dot(w2, e12);
    if (d12_1 <= 0.0) { s.v2().a = 1.0; s.count = 1; s.d1 = s.v2(); s.r1o = 0; return; }
    double inv = 1.0 / (d12_1 + d12_2);
    s.v1().a = d12_1 * inv;
    s.v2().a = d12_2 * inv;
    s.count = 2;
}

static __device__ void simplex_solve3(Simplex &s) {
    vec2<double> w1 = s.v1().w, w2 = s.v2().w, w3 = s.v3().w;
    vec2<double> e12 = w2 - w1;
    double d12_1 = dot(w2, e12), d12_2 = -dot(w1, e12);
    vec2<double> e13 = w3 - w1;
    double d13_1 = dot(w3, e13), d13_2 = -dot(w1, e13);
    vec2<double> e23 = w3 - w2;
    double d23_1 = dot(w3, e23), d23_2 = -dot(w2, e23);
    double n123 = cross(e12, e13);
    double d123_1 = n123 * cross(w2, w3);
    double d123_2 = n123 * cross(w3, w1);
    double d123_3 = n123 * cross(w1, w2);
    if (d12_2 <= 0.0 && d13_2 <= 0.0) { s.v1().a = 1.0; s.count = 1; return; }
    if (d12_1 > 0.0 && d12_2 > 0.0 && d123_3 <= 0.0) {
        double inv = 1.0 / (d12_1 + d12_2);
        s.v1().a = d12_1 * inv; s.v2().a = d12_2 * inv; s.count = 2; return;
    }
    if (d13_1 > 0.0 && d13_2 > 0.0 && d123_2 <= 0.0) {
        double inv = 1.0 / (d13_1 + d13_2);
        s.v1().a = d13_1 * inv; s.v3().a = d13_2 * inv; s.count = 2;
        s.d2 = s.v3(); s.r2o = 0; return;
    }
    if (d12_1 <= 0.0 && d23_2 <= 0.0) { s.v2().a = 1.0; s.count = 1; s.d1 = s.v2(); s.r1o = 0; return; }
    if (d13_1 <= 0.0 && d23_1 <= 0.0) { s.v3().a = 1.0; s.count = 1; s.d1 = s.v3(); s.r1o = 0; return; }
    if (d23_1 > 0.0 && d23_2 > 0.0 && d123_1 <= 0.0) {
        double inv = 1.0 / (d23_1 + d23_2);
        s.v2().a = d23_1 * inv; s.v3().a = d23_2 * inv; s.count = 2;
        s.d1 = s.v3(); s.r1o = 0; return;
    }
    double inv = 1.0 / (d123_1 + d123_2 + d123_3);
    s.v1().a = d123_1 * inv; s.v2().a = d123_2 * inv; s.v3().a = d123_3 * inv;
    s.count = 3;
}

// distance.py:424-561 shape_distance
static __device__ double shape_distance(const DProxy &A, const DProxy &B, xform2<double> xa, xform2<double> xb, bool use_radii, SCache &cache) {
    Simplex s;
    s.r1o = 1; s.r2o = 1;
    s.count = cache.count;
    for (int i = 0; i < s.count; ++i) {
        SVert &v = s.orig[i];
        v.ia = cache.ia[i]; v.ib = cache.ib[i];
        v.wa = xmul(xa, A.v[v.ia]); v.wb = xmul(xb, B.v[v.ib]);
        v.w = v.wb - v.wa; v.a = 0.0;
    }
    for (int i = s.count; i < 3; ++i) { s.orig[i].a = 0.0; s.orig[i].ia = 0; s.orig[i].ib = 0; }
    if (s.count > 1) {
        double m1 = cache.metric, m2 = simplex_metric(s);
        if (m2 < 0.5 * m1 || 2.0 * m1 < m2 || m2 < GB_EPSILON) s.count = 0;
    }
    if (s.count == 0) {
        SVert &v = s.orig[0];
        v.ia = 0; v.ib = 0;
        v.wa = xmul(xa, A.v[0]); v.wb = xmul(xb, B.v[0]);
        v.w = v.wb - v.wa;
        s.count = 1;
    }
    int save_ia[3], save_ib[3], save_n;
    for (int iter = 0; iter < 20;) {
        save_n = s.count;
        for (int i = 0; i < s.count; ++i) { save_ia[i] = s.vk(i).ia; save_ib[i] = s.vk(i).ib; }
        if (s.count == 2) simplex_solve2(s);
        else if (s.count == 3) { simplex_solve3(s); break; }
        vec2<double> d;
        if (s.count == 1) d = -s.v1().w;
        else {
            vec2<double> e12 = s.v2().w - s.v1().w;
            double sgn = cross(e12, -s.v1().w);
            d = (sgn > 0.0) ? cross(1.0, e12) : cross(e12, 1.0);
        }
        if (len2(d) < GB_EPSILON_SQR) break;
        SVert &vx = s.orig[s.count];
        vx.ia = dsupport(A, rmul_t(xa.q, -d));
        vx.wa = xmul(xa, A.v[vx.ia]);
        vx.ib = dsupport(B, rmul_t(xb.q, d));
        vx.wb = xmul(xb, B.v[vx.ib]);
        vx.w = vx.wb - vx.wa;
        ++iter;
        bool dup = false;
        for (int i = 0; i < save_n; ++i) if (save_ia[i] == vx.ia && save_ib[i] == vx.ib) { dup = true; break; }
        if (dup) break;
        s.count += 1;
    }
    vec2<double> pa, pb;
    if (s.count == 1) { pa = s.v1().wa; pb = s.v1().wb; }
    else if (s.count == 2) {
        pa = s.v1().a * s.v1().wa + s.v2().a * s.v2().wa;
        pb = s.v1().a * s.v1().wb + s.v2().a * s.v2().wb;
    } else {
        pa = (s.v1().a * s.v1().wa + s.v2().a * s.v2().wa) + s.v3().a * s.v3().wa;
        pb = pa;
    }
    double dist = len(pa - pb);
    cache.metric = simplex_metric(s);
    cache.count = s.count;
    for (int i = 0; i < s.count; ++i) { cache.ia[i] = s.vk(i).ia; cache.ib[i] = s.vk(i).ib; }
    if (use_radii) {
        double ra = A.radius, rb = B.radius;
        if (dist > ra + rb && dist > GB_EPSILON) dist -= ra + rb;
        else dist = 0.0;
    }
    return dist;
}

// ------------------------------------------------------------------
// common.py:870-923 Sweep, toi.py:45-391 time_of_impact (float64)
struct Sweep { vec2<double> lc, c0, c; double a0, a, alpha0; };

static __device__ __forceinline__ xform2<double> sweep_xf(const Sweep &sw, double beta) {
    xform2<double> x;
    x.p = (1.0 - beta) * sw.c0 + beta * sw.c;
    x.q = pose_rot((1.0 - beta) * sw.a0 + beta * sw.a);
    x.p = x.p - rmul(x.q, sw.lc);
    return x;
}
static __device__ __forceinline__ void sweep_advance(Sweep &sw, double alpha) {
    double beta = (alpha - sw.alpha0) / (1.0 - sw.alpha0);
    sw.c0 = (1.0 - beta) * sw.c0 + beta * sw.c;
    sw.a0 = (1.0 - beta) * sw.a0 + beta * sw.a;
    sw.alpha0 = alpha;
}
static __device__ __forceinline__ void sweep_normalize(Sweep &sw) {
    const double TWO_PI = 2.0 * 3.141592653589793;
    double d = TWO_PI * floor(sw.a0 / TWO_PI);
    sw.a0 -= d;
    sw.a -= d;
}

#define SF_POINTS 0
#define SF_FACE_A 1
#define SF_FACE_B 2
#define TOI_FAILED 1
#define TOI_OVERLAPPED 2
#define TOI_TOUCHING 3
#define TOI_SEPARATED 4

struct SepFn {
    const DProxy *A, *B;
    Sweep sa, sb;
    int type;
    vec2<double> axis, lp;
    // with `cache`, the two transforms at the last time asked for: the loop
    // asks for the same time up to three times in a row (the distance and
    // the separation set-up at t1, the push-back's first evaluation at t1
    // and at the last root), and each transform is a float64 sine and
    // cosine.  Measured: the batch-wide first pass 8 % faster with it; the
    // one-warp event loop, whose kernel is held to 80 registers, 4 % slower
    // (more spills), so it computes them afresh.
    bool cache;
    double xt;
    xform2<double> xa, xb;
};

static __device__ __forceinline__ void sep_xf(SepFn &f, double t, xform2<double> *xa, xform2<double> *xb) {
    if (!f.cache) {
        *xa = sweep_xf(f.sa, t);
        *xb = sweep_xf(f.sb, t);
        return;
    }
    if (!(t == f.xt)) {
        f.xa = sweep_xf(f.sa, t);
        f.xb = sweep_xf(f.sb, t);
        f.xt = t;
    }
    *xa = f.xa;
    *xb = f.xb;
}

// toi.py:53-123 (the POINTS axis stays unnormalised, as in the reference)
static __device__ void sep_init(SepFn &f, const SCache &c, double t1) {
    xform2<double> xa, xb;
    sep_xf(f, t1, &xa, &xb);
    int ia0 = c.ia[0], ib0 = c.ib[0];
    if (c.count == 1) {
        f.type = SF_POINTS;
        f.axis = xmul(xb, f.B->v[ib0]) - xmul(xa, f.A->v[ia0]);
        return;
    }
    int ia1 = c.ia[1], ib1 = c.ib[1];
    if (ia0 == ia1) {
        f.type = SF_FACE_B;
        vec2<double> lb1 = f.B->v[ib0], lb2 = f.B->v[ib1];
        f.axis = normalized(cross(lb2 - lb1, 1.0));
        vec2<double> normal = rmul(xb.q, f.axis);
        f.lp = 0.5 * (lb1 + lb2);
        vec2<double> pb = xmul(xb, f.lp), pa = xmul(xa, f.A->v[ia0]);
        if (dot(pa - pb, normal) < 0.0) f.axis = -f.axis;
    } else {
        f.type = SF_FACE_A;
        vec2<double> la1 = f.A->v[ia0], la2 = f.A->v[ia1];
        f.axis = normalized(cross(la2 - la1, 1.0));
        vec2<double> normal = rmul(xa.q, f.axis);
        f.lp = 0.5 * (la1 + la2);
        vec2<double> pa = xmul(xa, f.lp), pb = xmul(xb, f.B->v[ib0]);
        if (dot(pb - pa, normal) < 0.0) f.axis = -f.axis;
    }
}

static __device__ double sep_find_min(SepFn &f, double t, int *ia, int *ib) {
    xform2<double> xa, xb;
    sep_xf(f, t, &xa, &xb);
    if (f.type == SF_POINTS) {
        *ia = dsupport(*f.A, rmul_t(xa.q, f.axis));
        *ib = dsupport(*f.B, rmul_t(xb.q, -f.axis));
        return dot(xmul(xb, f.B->v[*ib]) - xmul(xa, f.A->v[*ia]), f.axis);
    } else if (f.type == SF_FACE_A) {
        vec2<double> normal = rmul(xa.q, f.axis);
        vec2<double> pa = xmul(xa, f.lp);
        *ia = -1;
        *ib = dsupport(*f.B, rmul_t(xb.q, -normal));
        return dot(xmul(xb, f.B->v[*ib]) - pa, normal);
    } else {
        vec2<double> normal = rmul(xb.q, f.axis);
        vec2<double> pb = xmul(xb, f.lp);
        *ib = -1;
        *ia = dsupport(*f.A, rmul_t(xa.q, -normal));
        return dot(xmul(xa, f.A->v[*ia]) - pb, normal);
    }
}

static __device__ double sep_eval(SepFn &f, int ia, int ib, double t) {
    xform2<double> xa, xb;
    sep_xf(f, t, &xa, &xb);
    if (f.type == SF_POINTS) return dot(xmul(xb, f.B->v[ib]) - xmul(xa, f.A->v[ia]), f.axis);
    if (f.type == SF_FACE_A) {
        vec2<double> normal = rmul(xa.q, f.axis);
        return dot(xmul(xb, f.B->v[ib]) - xmul(xa, f.lp), normal);
    }
    vec2<double> normal = rmul(xb.q, f.axis);
    return dot(xmul(xa, f.A->v[ia]) - xmul(xb, f.lp), normal);
}

// toi.py:216-391.  The reference's push-back loop is unbounded; here it
// stops after 1000 rounds with FAILED and sets *limit_hit.
template <bool XF_CACHE = false>
static __device__ int time_of_impact(const DProxy &A, const DProxy &B, const Sweep &swa, const Sweep &swb, double t_max,
                                     double *t_out, bool *limit_hit) {
    int state = 0;
    double out_t = t_max;
    SepFn f;
    f.A = &A; f.B = &B; f.sa = swa; f.sb = swb;
    sweep_normalize(f.sa);
    sweep_normalize(f.sb);
    f.cache = XF_CACHE;
    f.xt = -1.0;   // no time asked for yet (times lie in [0, t_max])
    double total_radius = A.radius + B.radius;
    double target = pymax(GB_LINEAR_SLOP, total_radius - 3.0 * GB_LINEAR_SLOP);
    double tol = 0.25 * GB_LINEAR_SLOP;
    double t1 = 0.0;
    int iter = 0;
    SCache cache;
    cache.metric = 0.0; cache.count = 0;
    for (int i = 0; i < 3; ++i) { cache.ia[i] = 0; cache.ib[i] = 0; }
    for (;;) {
        xform2<double> xa, xb;
        sep_xf(f, t1, &xa, &xb);
        double dist = shape_distance(A, B, xa, xb, false, cache);
        if (dist <= 0.0) { state = TOI_OVERLAPPED; out_t = 0.0; break; }
        if (dist < target + tol) { state = TOI_TOUCHING; out_t = t1; break; }
        sep_init(f, cache, t1);
        bool done = false;
        double t2 = t_max;
        int push_back = 0;
        for (;;) {
            int ia, ib;
            double s2 = sep_find_min(f, t2, &ia, &ib);
            if (s2 > target + tol) { state = TOI_SEPARATED; out_t = t_max; done = true; break; }
            if (s2 > target - tol) { t1 = t2; break; }
            double s1 = sep_eval(f, ia, ib, t1);
            if (s1 < target - tol) { state = TOI_FAILED; out_t = t1; done = true; break; }
            if (s1 <= target + tol) { state = TOI_TOUCHING; out_t = t1; done = true; break; }
            int root_iter = 0;
            double a1 = t1, a2 = t2;
            for (;;) {
                double t;
                if (root_iter & 1) t = a1 + (target - s1) * (a2 - a1) / (s2 - s1);
                else t = 0.5 * (a1 + a2);
                double s = sep_eval(f, ia, ib, t);
                if (fabs(s - target) < tol) { t2 = t; break; }
                if (s > target) { a1 = t; s1 = s; } else { a2 = t; s2 = s; }
                ++root_iter;
                if (root_iter == 50) break;
            }
            ++push_back;
            if (push_back == 1000) { state = TOI_FAILED; out_t = t1; done = true; *limit_hit = true; break; }
        }
        ++iter;
        if (done) break;
        if (iter == 20) { state = TOI_FAILED; out_t = t1; break; }
    }
    *t_out = out_t;
    return state;
}

// gb_step.cuh -- World.step (pypybox2d/world.py:307-354) for one world,
// executed by one group of threads (see gb_world.cuh).
//
// Phases and the reference code each one replaces:
//   pair finding ..... broadphase.py:83-109 + contact_manager.py:102-158
//   collide .......... contact_manager.py:174-223 + contact.py:210-268
//   islands .......... world.py:475-573 (union-find; depth-first order only
//                      where the reference's result depends on it)
//   contact solver ... island.py:65-179 + contact.py:375-864, Gauss-Seidel
//                      over graph-coloured constraint batches
//   fixture sync ..... world.py:582-589, body.py:879-885, fixture.py:287-298,
//                      dynamictree.py:152-188
//   continuous ....... world.py:594-821, island.py:181-243, contact.py:866-933
#pragma once
#include <type_traits>
#include "gb_world.cuh"
#include "gb_joints.cuh"
#include "gb_tma.cuh"

#define GB_MAX_TRANSLATION 2.0
#define GB_MAX_TRANSLATION_SQR 4.0
#define GB_MAX_ROTATION (0.5 * 3.141592653589793)
#define GB_MAX_ROTATION_SQR 2.4674011002723395
#define GB_BAUMGARTE 0.2
#define GB_TOI_BAUMGARTE 0.75
#define GB_MAX_LINEAR_CORRECTION 0.2
#define GB_VELOCITY_THRESHOLD 1.0
#define GB_TIME_TO_SLEEP 0.5
#define GB_LINEAR_SLEEP_TOL_SQR 0.0001
#define GB_ANGULAR_SLEEP_TOL_SQR 0.0012184696791468343
#define GB_AABB_EXTENSION 0.1
#define GB_AABB_MULTIPLIER 2.0
#define GB_MAX_SUB_STEPS 8
#define GB_INF_IDX 0x7fffffff

#define R_SIM 1u      // island is simulated this step
#define R_DONE 2u     // position iterations finished (early exit)
#define R_SOLVED 4u   // position_solved
#define R_DFS 8u      // needs the depth-first body order
#define R_STATIC_IN 16u  // (bodies) static body attached to a simulated island
#define R_JBAD 32u    // a joint of the island is not yet within tolerance in this position iteration


// Group-shared scratch scalars of one world.
struct WShared {
    unsigned long long red;
    int nmove;
    int nisland;
    int min_contact;
    double min_alpha;
    int any_dfs;
    int ncons, ncolours;
    int pass;
    int all_allow_sleep;
    int lhcap;            // slots of the TOI loop's pair hash
    // pair-finding grid of the world (find_new_contacts)
    unsigned long long gred[6];
    float gsum;
    int gx, gy, nsmall, nbig;
    float x0, y0, inv_h, cut;
};

// body.py:781-793 awake setter
template <class R> __device__ __forceinline__ void wake_body(const WView<R> &w, int b) {
    uint32_t f = w.B.b_flags[w.bb + b];
    if (!(f & GB_BODY_AWAKE)) { w.B.b_sleep[w.bb + b] = 0.0; w.B.b_flags[w.bb + b] = f | GB_BODY_AWAKE; }
}
template <class R> __device__ __forceinline__ void sleep_body(const WView<R> &w, int b) {
    int g = w.bb + b;
    w.B.b_sleep[g] = 0.0;
    w.B.b_v[g] = mk<R>(0, 0); w.B.b_w[g] = (R)0;
    w.B.b_f[g] = mk<R>(0, 0); w.B.b_torque[g] = (R)0;
    w.B.b_flags[g] &= ~GB_BODY_AWAKE;
}
// body.py:887-889
template <class R> __device__ __forceinline__ void sync_transform(const WView<R> &w, int b) {
    int g = w.bb + b;
    rot2<double> q = pose_rot(w.B.b_a[g]);
    vec2<double> p = w.B.b_c[g] - rmul(q, w.B.b_lc[g]);
    w.B.b_xp[g] = p; w.B.b_xq[g] = q;
}
// body.py:911-918
template <class R> __device__ void body_advance(const WView<R> &w, int b, double alpha) {
    Sweep s = w.sweep(b);
    sweep_advance(s, alpha);
    s.c = s.c0; s.a = s.a0;
    w.put_sweep(b, s);
    rot2<double> q = pose_rot(s.a);
    w.B.b_xq[w.bb + b] = q;
    w.B.b_xp[w.bb + b] = s.c - rmul(q, s.lc);
}

// Order-preserving integer key of a finite double (-0 keyed as +0): for
// finite x, y, (x - y) > 0 holds exactly when x > y, so comparing keys gives
// the reference's float64 tests without float64 arithmetic (a float64
// instruction costs a GB300 warp ~64 cycles).
static __device__ __forceinline__ long long okey(double d) {
    long long b = __double_as_longlong(d);
    if ((b << 1) == 0) b = 0;
    return b < 0 ? (b ^ 0x7fffffffffffffffLL) : b;
}
// aabbmodule.c AABB_test_overlap: !((b.lx - a.ux) > 0 || (b.ly - a.uy) > 0 ||
// (a.lx - b.ux) > 0 || (a.ly - b.uy) > 0)
static __device__ __forceinline__ bool aabb_overlap(dbox a, dbox b) {
    return !(okey(b.x) > okey(a.z) || okey(b.y) > okey(a.w) || okey(a.x) > okey(b.z) || okey(a.y) > okey(b.w));
}

// world.py:958-970
template <class R> __device__ __forceinline__ bool default_filter(const WView<R> &w, int fa, int fb) {
    int ga = w.B.f_group[w.fb + fa], gb = w.B.f_group[w.fb + fb];
    if (ga == gb && ga != 0) return ga > 0;
    return ((w.B.f_mask[w.fb + fa] & w.B.f_cat[w.fb + fb]) != 0) && ((w.B.f_cat[w.fb + fa] & w.B.f_mask[w.fb + fb]) != 0);
}
// contact_manager.py:145,202: the world's contact filter.  A custom filter
// (world.py:123-136) reaches the device as its answers for every ordered
// pair of the world's fixture records; without one the default rule.
template <class R> __device__ __forceinline__ bool pair_filter(const WView<R> &w, int fa, int fb) {
    if (w.B.pf_off) {
        const long long o = w.B.pf_off[w.wi];
        if (o >= 0) return w.B.pf_accept[o + (long long)fa * w.H->nf + fb] != 0;
    }
    return default_filter(w, fa, fb);
}

// body.py:912-927 _should_collide: one body dynamic, and no joint between
// the two that turns collision off (the joint list of body ba)
template <class R> __device__ __forceinline__ bool should_collide(const WView<R> &w, int ba, int bb) {
    if (w.btype(ba) != GB_BODY_DYNAMIC && w.btype(bb) != GB_BODY_DYNAMIC) return false;
    if (w.H->nj == 0) return true;
    const int *off = w.B.b_joff + w.bb + w.wi;
    const int *adj = w.B.b_jadj + 2 * (size_t)w.H->jbase;
    const gb_joint *J = w.B.j + w.H->jbase;
    for (int e = off[ba]; e < off[ba + 1]; ++e) {
        const gb_joint &q = J[adj[e]];
        if (((q.body_a == ba && q.body_b == bb) || (q.body_b == ba && q.body_a == bb)) && !(q.flags & GB_J_COLLIDE_CONNECTED))
            return false;
    }
    return true;
}
template <class R> __device__ __forceinline__ bool fx_sensor(const WView<R> &w, int f) {
    return (w.B.f_flags[w.fb + f] & GB_FIX_SENSOR) != 0;
}

// Append one contact event of a world (index < 0: keyed by its slot, which
// is the order of occurrence when one thread records).  Out of line and
// with scalar arguments, so the kernels that may record keep their
// registers and stack for the common case of no recording.
static __device__ __noinline__ void put_event(gb_event *ev, int *ev_n, int cap, uint32_t *status, int step, int phase, int type,
                                              int fa, int fb, int index, int npts, double n0, double n1, double t0, double t1) {
    int slot = atomicAdd(ev_n, 1);
    if (slot >= cap) { atomicOr(status, GB_ST_EVENT_OVERFLOW); return; }
    gb_event &e = ev[slot];
    e.type = type; e.fixture_a = fa; e.fixture_b = fb; e.point_count = npts;
    e.key = ((long long)step << 48) | ((long long)phase << 40) | (long long)(index >= 0 ? index : slot);
    e.normal_impulse[0] = npts > 0 ? n0 : 0.0; e.normal_impulse[1] = npts > 1 ? n1 : 0.0;
    e.tangent_impulse[0] = npts > 0 ? t0 : 0.0; e.tangent_impulse[1] = npts > 1 ? t1 : 0.0;
}
template <class R> __device__ __forceinline__ void record_event(const WView<R> &w, const EvCtx &ev, int type, int i, int index,
                                                                int npts, const R *ni, const R *ti) {
    const ContactRec<R> &c = w.con(i);
    put_event(w.B.ev + 3 * (size_t)w.cb + 64 * (size_t)w.wi, w.B.ev_n + w.wi, 3 * w.H->ccap + 64, &w.H->status, ev.step, ev.phase,
              type, c.fa, c.fb, index, npts, npts > 0 ? (double)ni[0] : 0.0, npts > 1 ? (double)ni[1] : 0.0,
              npts > 0 ? (double)ti[0] : 0.0, npts > 1 ? (double)ti[1] : 0.0);
}

// contact.py:210-268 Contact.update; returns whether touching changed (the
// wake rule; sensors never wake).  With `ev` on, a change of touching, of a
// sensor too, is recorded as a begin or end event (contact.py:263-266).
template <class R, bool EV = true> __device__ bool contact_update(const WView<R> &w, int i, const EvCtx *ev = nullptr,
                                                                  int ev_index = -1) {
    ContactRec<R> &c = w.con(i);
    Manifold<R> old = c.m;
    c.flags |= GB_C_ENABLED;
    bool was = (c.flags & GB_C_TOUCHING) != 0;
    int ba = w.fbody(c.fa), bb = w.fbody(c.fb);
    Shape<R> sa = w.shape(c.fa), sb = w.shape(c.fb);
    bool touching;
    bool changed = false;
    if (fx_sensor(w, c.fa) || fx_sensor(w, c.fb)) {
        DProxy pa, pb;
        dproxy_init(pa, sa); dproxy_init(pb, sb);
        SCache cache; cache.metric = 0; cache.count = 0;
        for (int k = 0; k < 3; ++k) { cache.ia[k] = 0; cache.ib[k] = 0; }
        double d = shape_distance(pa, pb, w.xfd(ba), w.xfd(bb), true, cache);
        touching = d < 10.0 * GB_EPSILON;
        c.m.count = 0;
    } else {
        evaluate_manifold(c.m, sa, w.xf(ba), sb, w.xf(bb));
        touching = c.m.count > 0;
        for (int k = 0; k < c.m.count; ++k) {
            int found = -1;
            for (int j = old.count - 1; j >= 0; --j)
                if (old.id[j] == c.m.id[k]) { found = j; break; }
            if (found >= 0) { c.m.ni[k] = old.ni[found]; c.m.ti[k] = old.ti[found]; }
            else { c.m.ni[k] = (R)0; c.m.ti[k] = (R)0; }
        }
        changed = touching != was;
    }
    if (touching) c.flags |= GB_C_TOUCHING; else c.flags &= ~GB_C_TOUCHING;
    if (EV && ev && ev->on && touching != was)
        record_event<R>(w, *ev, touching ? GB_EV_BEGIN : GB_EV_END, i, ev_index, 0, nullptr, nullptr);
    return changed;
}

// Contacts that can take part in the TOI loop of this step: neither fixture
// a sensor, a bullet or non-dynamic body on one side, not both bodies
// static (toi_status's conditions that cannot change during the loop; the
// awake, enabled and sub-step conditions are checked on every pass).
template <class R> __device__ __forceinline__ bool toi_candidate(const WView<R> &w, int i) {
    const ContactRec<R> &c = w.con(i);
    if (fx_sensor(w, c.fa) || fx_sensor(w, c.fb)) return false;
    int ba = w.fbody(c.fa), bb = w.fbody(c.fb);
    int ta = w.btype(ba), tb = w.btype(bb);
    if (ta == GB_BODY_STATIC && tb == GB_BODY_STATIC) return false;
    bool col_a = (w.B.b_flags[w.bb + ba] & GB_BODY_BULLET) || ta != GB_BODY_DYNAMIC;
    bool col_b = (w.B.b_flags[w.bb + bb] & GB_BODY_BULLET) || tb != GB_BODY_DYNAMIC;
    return col_a || col_b;
}

// shapes.py compute_aabb (child 0) for the float32 unit: the rotated
// vertices' extent in float32 about the body origin p, widened and added to
// p; equal to shape_aabb to float32 rounding of the extent (~1e-7 m).
template <class R> __device__ dbox shape_aabb_f32(const WView<R> &w, int f, vec2<double> p, rot2<float> q) {
    const Shape<R> s = w.shape(f);
    const float r = (float)s.radius;
    vec2<float> lo, hi;
    if (s.type == GB_SHAPE_CIRCLE) {
        lo = hi = rmul(q, cvt<float>(s.v[0]));
    } else {
        const int n = (s.type == GB_SHAPE_POLYGON) ? s.count : 2;
        lo = hi = rmul(q, cvt<float>(s.v[0]));
        for (int i = 1; i < n; ++i) {
            const vec2<float> v = rmul(q, cvt<float>(s.v[i]));
            lo = mk<float>(fminf(lo.x, v.x), fminf(lo.y, v.y));
            hi = mk<float>(fmaxf(hi.x, v.x), fmaxf(hi.y, v.y));
        }
    }
    if (s.flags & GB_FIX_LOOP_CHILD) return mkbox(p.x + (double)lo.x, p.y + (double)lo.y, p.x + (double)hi.x, p.y + (double)hi.y);
    return mkbox(p.x + (double)(lo.x - r), p.y + (double)(lo.y - r), p.x + (double)(hi.x + r), p.y + (double)(hi.y + r));
}

// shapes.py compute_aabb (child 0), float64; a loop's child edge takes no
// radius margin (shapes.py:822-837)
template <class R> __device__ dbox shape_aabb(const WView<R> &w, int f, xform2<double> x) {
    Shape<R> s = w.shape(f);
    double r = (double)s.radius;
    if (s.type == GB_SHAPE_CIRCLE) {
        vec2<double> p = x.p + rmul(x.q, cvt<double>(s.v[0]));
        return mkbox(p.x - r, p.y - r, p.x + r, p.y + r);
    }
    int n = (s.type == GB_SHAPE_POLYGON) ? s.count : 2;
    vec2<double> lo = xmul(x, cvt<double>(s.v[0])), hi = lo;
    for (int i = (s.type == GB_SHAPE_POLYGON ? 0 : 1); i < n; ++i) {
        vec2<double> v = xmul(x, cvt<double>(s.v[i]));
        lo = mk<double>(cmin(lo.x, v.x), cmin(lo.y, v.y));
        hi = mk<double>(cmax(hi.x, v.x), cmax(hi.y, v.y));
    }
    if (s.flags & GB_FIX_LOOP_CHILD) return mkbox(lo.x, lo.y, hi.x, hi.y);
    return mkbox(lo.x - r, lo.y - r, hi.x + r, hi.y + r);
}

// body.py:879-885 + fixture.py:287-298 + dynamictree.py:152-188 for one
// fixture; returns whether the proxy was re-fattened (enters the move buffer).
template <class R> __device__ bool sync_fixture(const WView<R> &w, int f) {
    int b = w.fbody(f);
    int gbi = w.bb + b;
#if defined(GB_POSE_ROT_F32)
    // float32 unit: the shape's extent about the body origin in float32,
    // added to the float64 origin (shape_aabb_f32)
    const rot2<float> q1 = rot_of_f32(w.B.b_a0[gbi]);
    const vec2<double> p1 = w.B.b_c0[gbi] - cvt<double>(rmul(q1, cvt<float>(w.B.b_lc[gbi])));
    const vec2<double> p2 = w.B.b_xp[gbi];
    const rot2<double> q2d = w.B.b_xq[gbi];
    rot2<float> q2;
    q2.c = (float)q2d.c; q2.s = (float)q2d.s;
    dbox a1 = shape_aabb_f32(w, f, p1, q1), a2 = shape_aabb_f32(w, f, p2, q2);
    vec2<double> disp = p2 - p1;
#else
    xform2<double> x1;
    x1.q = rot_of(w.B.b_a0[gbi]);
    x1.p = w.B.b_c0[gbi] - rmul(x1.q, w.B.b_lc[gbi]);
    xform2<double> x2 = w.xfd(b);
    dbox a1 = shape_aabb(w, f, x1), a2 = shape_aabb(w, f, x2);
    vec2<double> disp = x2.p - x1.p;
#endif
    dbox ab = mkbox(cmin(a1.x, a2.x), cmin(a1.y, a2.y), cmax(a1.z, a2.z), cmax(a1.w, a2.w));
    dbox fat = w.B.f_aabb[w.fb + f];
    if (okey(fat.x) <= okey(ab.x) && okey(fat.y) <= okey(ab.y) && okey(ab.z) <= okey(fat.z) && okey(ab.w) <= okey(fat.w))
        return false;
    dbox nb = mkbox(ab.x - GB_AABB_EXTENSION, ab.y - GB_AABB_EXTENSION, ab.z + GB_AABB_EXTENSION, ab.w + GB_AABB_EXTENSION);
    vec2<double> d = GB_AABB_MULTIPLIER * disp;
    if (d.x < 0.0) { nb.x = nb.x + d.x; nb.y = nb.y + 0.0; } else { nb.z = nb.z + d.x; nb.w = nb.w + 0.0; }
    if (d.y < 0.0) { nb.x = nb.x + 0.0; nb.y = nb.y + d.y; } else { nb.z = nb.z + 0.0; nb.w = nb.w + d.y; }
    w.B.f_aabb[w.fb + f] = nb;
    w.B.f_aabbf[w.fb + f] = boxf_of(nb);
    return true;
}

// ------------------------------------------------------------ pair finding
// broadphase.py:83-109 with the fixed pair order (first move-buffer position
// of the moved proxy, then the other proxy's index) followed by
// contact_manager.py:102-158.  The move buffer is s_move[0..nmove).
template <class R> __device__ __forceinline__ bool pair_candidate(const WView<R> &w, int i, int p, int q, int *first,
                                                                  unsigned long long *hash, int hmask) {
    if (q == p) return false;
    int fq = first[q];
    if (fq < i) return false;  // emitted when q was processed
    if (!aabb_overlap(w.B.f_aabb[w.fb + q], w.B.f_aabb[w.fb + p])) return false;
    int ba = w.fbody(p), bb = w.fbody(q);
    if (ba == bb) return false;
    // an inactive body's fixtures have no proxies (body.py:848-872)
    if (!(w.B.b_flags[w.bb + ba] & w.B.b_flags[w.bb + bb] & GB_BODY_ACTIVE)) return false;
    // does a contact already exist?
    unsigned long long key = ((unsigned long long)(unsigned)min(p, q) << 32) | (unsigned)max(p, q);
    key += 1ull;
    unsigned h = (unsigned)((key * 0x9E3779B97F4A7C15ull) >> 32) & hmask;
    for (int probe = 0; probe <= hmask; ++probe) {
        unsigned long long k = hash[h];
        if (k == key) return false;
        if (k == 0ull) break;
        h = (h + 1) & hmask;
    }
    if (!should_collide(w, bb, ba)) return false;
    if (!pair_filter(w, p, q)) return false;
    bool prim;
    if (!pair_registered(w.B.f_type[w.fb + p], w.B.f_type[w.fb + q], &prim)) return false;
    return true;
}

// Uniform grid over the world's fat AABBs, rebuilt for each pair-finding
// pass: a proxy is listed in every cell its box overlaps (cells twice the
// mean extent, so a box spans at most 3 x 3); proxies larger than four times
// the mean extent (ground boxes, container edges) are "big": they stay out
// of the grid and are tested against every moved proxy.  A moved proxy, big
// or not, scans the cells its box overlaps and takes a listed proxy only in
// the cell holding the lower-left corner of the two boxes' intersection, so
// each overlapping pair is seen once.
// The grid only prunes: every pair is still decided by the exact float64
// overlap test, and the pairs of a moved proxy are sorted by the other
// proxy's index, so the result does not depend on the grid.
#define GB_GRID_MIN_MOVES 8
#define GB_GRID_ITEMS_PER_FIXTURE 9
// The grid works on the float32 copies of the fat boxes: any map from a
// coordinate to a cell that does not decrease with the coordinate lists and
// finds every overlapping pair (the pair's lower-left intersection corner
// lies in both boxes' cell ranges), and the pairs themselves are decided by
// the exact test on the float64 boxes.
static __device__ __forceinline__ int grid_cell(float x, float x0, float inv_h, int n) {
    float t = floorf((x - x0) * inv_h);
    t = fminf(fmaxf(t, 0.0f), (float)(n - 1));
    return (int)t;
}
static __device__ __forceinline__ bool grid_big(const float4 &b, float cut) {
    return (b.z - b.x) > cut || (b.w - b.y) > cut;
}
// order-preserving unsigned key of a float (for shared-memory min/max)
static __device__ __forceinline__ unsigned fkey(float f) {
    unsigned u = __float_as_uint(f);
    return (u >> 31) ? ~u : (u | 0x80000000u);
}
static __device__ __forceinline__ float fkey_inv(unsigned k) {
    return __uint_as_float((k >> 31) ? (k & 0x7fffffffu) : ~k);
}

// Scratch of one world (s_grid): cell ends (2 nf + 2), listed proxies
// (9 nf), big proxies (nf).
template <class R, class G> __device__ void build_pair_grid(const G &g, const WView<R> &w, WShared *sh, int *goff, int *gitem,
                                                            int *gbig) {
    const int nf = w.H->nf;
    const float4 *aabb = w.B.f_aabbf + w.fb;
    if (g.rank() == 0) {
        sh->gsum = 0.0f;
        sh->gred[0] = sh->gred[1] = ~0ull;
        sh->gred[2] = sh->gred[3] = 0ull;
        sh->nbig = 0;
    }
    g.sync();
    // each thread reduces its proxies, then one atomic per warp
    float lsum = 0.0f;
    for (int f = g.rank(); f < nf; f += g.size()) {
        const float4 b = aabb[f];
        lsum += fmaxf(b.z - b.x, b.w - b.y);
    }
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(&sh->gsum, lsum);
    g.sync();
    if (g.rank() == 0) sh->cut = 4.0f * sh->gsum / (float)nf;
    g.sync();
    const float cut = sh->cut;
    unsigned r[4] = {~0u, ~0u, 0u, 0u};
    for (int f = g.rank(); f < nf; f += g.size()) {
        const float4 b = aabb[f];
        if (grid_big(b, cut)) continue;
        const unsigned k[4] = {fkey(b.x), fkey(b.y), fkey(b.z), fkey(b.w)};
        for (int j = 0; j < 2; ++j) r[j] = k[j] < r[j] ? k[j] : r[j];
        for (int j = 2; j < 4; ++j) r[j] = k[j] > r[j] ? k[j] : r[j];
    }
    for (int o = 16; o > 0; o >>= 1)
        for (int j = 0; j < 4; ++j) {
            unsigned x = __shfl_xor_sync(0xffffffffu, r[j], o);
            r[j] = j < 2 ? (x < r[j] ? x : r[j]) : (x > r[j] ? x : r[j]);
        }
    if ((threadIdx.x & 31) == 0 && r[0] != ~0u) {
        atomicMin(&sh->gred[0], (unsigned long long)r[0]); atomicMin(&sh->gred[1], (unsigned long long)r[1]);
        atomicMax(&sh->gred[2], (unsigned long long)r[2]); atomicMax(&sh->gred[3], (unsigned long long)r[3]);
    }
    g.sync();
    if (g.rank() == 0) {
        int gx = 1, gy = 1;
        float x0 = 0.0f, y0 = 0.0f, h = 1.0f;
        if (sh->gred[0] != ~0ull) {
            x0 = fkey_inv((unsigned)sh->gred[0]); y0 = fkey_inv((unsigned)sh->gred[1]);
            const float sx = fkey_inv((unsigned)sh->gred[2]) - x0, sy = fkey_inv((unsigned)sh->gred[3]) - y0;
            h = fmaxf(0.5f * cut, 1e-6f);   // twice the mean extent
            const float cap = 2.0f * (float)nf;
            for (int k = 0; k < 64; ++k) {   // at most 2 nf cells
                const float cx = floorf(sx / h) + 1.0f, cy = floorf(sy / h) + 1.0f;
                if (cx * cy <= cap) { gx = (int)cx; gy = (int)cy; break; }
                h *= 1.5f;
            }
        }
        sh->x0 = x0; sh->y0 = y0; sh->inv_h = 1.0f / h;
        sh->gx = gx; sh->gy = gy;
    }
    g.sync();
    const int ncell = sh->gx * sh->gy;
    const float x0 = sh->x0, y0 = sh->y0, ih = sh->inv_h;
    const int gx = sh->gx, gy = sh->gy;
    for (int c = g.rank(); c < ncell; c += g.size()) goff[c] = 0;
    g.sync();
    for (int f = g.rank(); f < nf; f += g.size()) {
        const float4 b = aabb[f];
        if (grid_big(b, cut)) continue;
        const int cx0 = grid_cell(b.x, x0, ih, gx), cx1 = grid_cell(b.z, x0, ih, gx);
        const int cy0 = grid_cell(b.y, y0, ih, gy), cy1 = grid_cell(b.w, y0, ih, gy);
        for (int cy = cy0; cy <= cy1; ++cy)
            for (int cx = cx0; cx <= cx1; ++cx) atomicAdd(&goff[cy * gx + cx], 1);
    }
    g.sync();
    int nitems = group_scan(g, ncell, [&](int c) { return goff[c]; }, goff);
    g.sync();
    if (nitems > GB_GRID_ITEMS_PER_FIXTURE * nf) {   // cannot happen for boxes below the cut; never past the scratch
        if (g.rank() == 0) sh->gx = 0;
        g.sync();
        return;
    }
    // scatter: afterwards goff[c] is the end of cell c (its start is goff[c - 1])
    for (int f = g.rank(); f < nf; f += g.size()) {
        const float4 b = aabb[f];
        if (grid_big(b, cut)) {
            gbig[atomicAdd(&sh->nbig, 1)] = f;
            continue;
        }
        const int cx0 = grid_cell(b.x, x0, ih, gx), cx1 = grid_cell(b.z, x0, ih, gx);
        const int cy0 = grid_cell(b.y, y0, ih, gy), cy1 = grid_cell(b.w, y0, ih, gy);
        for (int cy = cy0; cy <= cy1; ++cy)
            for (int cx = cx0; cx <= cx1; ++cx) gitem[atomicAdd(&goff[cy * gx + cx], 1)] = f;
    }
    g.sync();
}

template <class R, class G> __device__ void find_new_contacts(const G &g, const WView<R> &w, WShared *sh) {
    int nmove = sh->nmove;
    int nf = w.H->nf;
    int *first = w.B.s_first + w.fb;
    int *mv = w.B.s_move + w.fb;
    int *cnt = w.B.s_cnt + w.fb;
    unsigned long long *hash = w.B.s_hash + 4 * (size_t)w.cb;
    if (nmove == 0) return;
    for (int f = g.rank(); f < nf; f += g.size()) first[f] = GB_INF_IDX;
    g.sync();
    for (int i = g.rank(); i < nmove; i += g.size()) atomicMin(&first[mv[i]], i);
    g.sync();
    int nc = w.H->nc;
    // only contacts of moved proxies can match a candidate pair: size the
    // existence hash for those (after a TOI event a handful, not the world)
    auto involved = [&](int i) {
        const ContactRec<R> &c = w.con(i);
        return (first[c.fa] != GB_INF_IDX || first[c.fb] != GB_INF_IDX) ? 1 : 0;
    };
    int m = group_count(g, nc, involved);
    int hcap = 16;
    while (hcap < 2 * m) hcap <<= 1;
    int hmask = hcap - 1;
    for (int k = g.rank(); k < hcap; k += g.size()) hash[k] = 0ull;
    g.sync();
    for (int i = g.rank(); i < nc; i += g.size()) {
        if (!involved(i)) continue;
        const ContactRec<R> &c = w.con(i);
        unsigned long long key = ((unsigned long long)(unsigned)min(c.fa, c.fb) << 32) | (unsigned)max(c.fa, c.fb);
        key += 1ull;
        unsigned h = (unsigned)((key * 0x9E3779B97F4A7C15ull) >> 32) & hmask;
        for (int probe = 0; probe <= hmask; ++probe) {
            unsigned long long prev = atomicCAS(&hash[h], 0ull, key);
            if (prev == 0ull || prev == key) break;
            h = (h + 1) & hmask;
        }
    }
    g.sync();
    // candidate proxies of a moved proxy: the grid cells its fat AABB can
    // reach plus the big proxies, or every proxy (in index order)
    int *goff = w.B.s_grid + 12 * (size_t)w.fb + 2 * (size_t)w.wi;
    int *gitem = goff + 2 * (size_t)nf + 2;
    int *gbig = gitem + GB_GRID_ITEMS_PER_FIXTURE * (size_t)nf;
    bool use_grid = nmove >= GB_GRID_MIN_MOVES;
    if (use_grid) {
        build_pair_grid(g, w, sh, goff, gitem, gbig);
        use_grid = sh->gx > 0;
    }
    const float4 *aabb = w.B.f_aabbf + w.fb;
    // with a grid every moved proxy, big ones too, scans the cells its box
    // overlaps (the ground box: the bottom row) and the big list
    auto each_candidate = [&](int i, int p, auto &&emit) {
        if (!use_grid) {
            for (int q = 0; q < nf; ++q)
                if (pair_candidate(w, i, p, q, first, hash, hmask)) emit(q);
            return;
        }
        const float4 b = aabb[p];
        const float x0 = sh->x0, y0 = sh->y0, ih = sh->inv_h;
        const int gx = sh->gx, gy = sh->gy;
        const int cx0 = grid_cell(b.x, x0, ih, gx), cx1 = grid_cell(b.z, x0, ih, gx);
        const int cy0 = grid_cell(b.y, y0, ih, gy), cy1 = grid_cell(b.w, y0, ih, gy);
        for (int cy = cy0; cy <= cy1; ++cy)
            for (int cx = cx0; cx <= cx1; ++cx) {
                int c = cy * gx + cx;
                for (int k = c ? goff[c - 1] : 0; k < goff[c]; ++k) {
                    int q = gitem[k];
                    const float4 o = aabb[q];
                    // the cell of the intersection's lower-left corner owns the pair
                    if (grid_cell(fmaxf(b.x, o.x), x0, ih, gx) != cx || grid_cell(fmaxf(b.y, o.y), y0, ih, gy) != cy) continue;
                    if (pair_candidate(w, i, p, q, first, hash, hmask)) emit(q);
                }
            }
        for (int k = 0; k < sh->nbig; ++k) {
            int q = gbig[k];
            if (pair_candidate(w, i, p, q, first, hash, hmask)) emit(q);
        }
    };
    // pass 1: count the new pairs of every move-buffer entry
    for (int i = g.rank(); i < nmove; i += g.size()) {
        int p = mv[i];
        int n = 0;
        if (first[p] == i) each_candidate(i, p, [&](int) { ++n; });
        cnt[i] = n;
    }
    g.sync();
    int total = group_scan(g, nmove, [&](int i) { return cnt[i]; }, cnt);
    g.sync();
    const int ccap = w.H->ccap;
    const int room = ccap - nc;
    // pass 2: the other proxy of each new pair, in index order per entry
    int *pq = w.B.s_colour + w.cb;   // other proxy of new pair t (free outside the island phase)
    int *pp = w.B.s_order + w.cb;    // moved proxy of new pair t
    for (int i = g.rank(); i < nmove; i += g.size()) {
        int p = mv[i];
        if (first[p] != i) continue;
        const int base = cnt[i];
        int k = base;
        each_candidate(i, p, [&](int q) {
            if (k < room) { pq[k] = q; pp[k] = p; }
            ++k;
        });
        if (use_grid) {
            const int end = k < room ? k : room;
            for (int a = base + 1; a < end; ++a) {   // insertion sort by proxy index
                int v = pq[a], b = a - 1;
                while (b >= base && pq[b] > v) { pq[b + 1] = pq[b]; --b; }
                pq[b + 1] = v;
            }
        }
    }
    g.sync();
    // create the contacts in that order (contact.py:313-326 _create)
    const int ncreate = total < room ? total : room;
    for (int t = g.rank(); t < ncreate; t += g.size()) {
        int p = pp[t], q = pq[t];
        int fa = p, fb = q;
        bool prim;
        pair_registered(w.B.f_type[w.fb + p], w.B.f_type[w.fb + q], &prim);
        if (!prim) { fa = q; fb = p; }
        ContactRec<R> &c = w.con(nc + t);
        c.fa = fa; c.fb = fb;
        c.flags = toi_candidate(w, nc + t) ? GB_C_TOI_CAND : 0u;
        c.toi_count = 0; c.toi = 0.0;
        R fra = w.B.f_friction[w.fb + fa], frb = w.B.f_friction[w.fb + fb];
        c.friction = sqrt(fra * frb);
        c.restitution = pymax(w.B.f_restitution[w.fb + fa], w.B.f_restitution[w.fb + fb]);
        Manifold<R> &m = c.m;
        m.type = GB_M_CIRCLES; m.count = 0;
        m.ln = mk<R>(0, 0); m.lp = mk<R>(0, 0);
        for (int k = 0; k < 2; ++k) { m.plp[k] = mk<R>(0, 0); m.ni[k] = (R)0; m.ti[k] = (R)0; m.id[k] = 0; }
    }
    g.sync();
    if (g.rank() == 0) {
        int nn = nc + total;
        if (nn > ccap) { w.H->status |= GB_ST_CONTACT_OVERFLOW; nn = ccap; }
        w.H->nc = nn;
        sh->nmove = 0;
    }
    g.sync();
}

// ------------------------------------------------------------ collide
// One iteration of ContactManager.collide's loop (contact_manager.py:174-223)
// for contact i, where wake[] gives for every body of the world the list
// position from which it counts as awake (-1: awake and non-static when the
// loop starts).  Returns 0 when both bodies are inactive at that point,
// 1 after Contact.update (*woke: touching changed, both bodies woken), 2 when
// the contact is to be destroyed.
template <class R, bool EV = true> __device__ int collide_one(const WView<R> &w, int i, const int *wake, bool *woke,
                                                             const EvCtx *ev = nullptr) {
    ContactRec<R> &c = w.con(i);
    int ba = w.fbody(c.fa), bb = w.fbody(c.fb);
    bool act_a = w.btype(ba) != GB_BODY_STATIC && wake[ba] < i;
    bool act_b = w.btype(bb) != GB_BODY_STATIC && wake[bb] < i;
    *woke = false;
    if (!act_a && !act_b) return 0;
    bool destroy = false;
    if (c.flags & GB_C_FILTER) {
        if (!should_collide(w, bb, ba) || !pair_filter(w, c.fa, c.fb)) destroy = true;
        else c.flags &= ~GB_C_FILTER;
    }
    if (!destroy && !aabb_overlap(w.B.f_aabb[w.fb + c.fa], w.B.f_aabb[w.fb + c.fb])) destroy = true;
    if (destroy) {   // contact_manager.py:160-172: a touching contact ends as it is destroyed
        if (EV && ev && ev->on && (c.flags & GB_C_TOUCHING)) record_event<R>(w, *ev, GB_EV_END, i, i, 0, nullptr, nullptr);
        return 2;
    }
    *woke = contact_update<R, EV>(w, i, ev, i);
    return 1;
}

// contact_manager.py:160-172 destroy of every contact with proc[i] == 2,
// keeping creation order.
template <class R, class G> __device__ void compact_contacts(const G &g, const WView<R> &w, const int *proc) {
    const int nc = w.H->nc;
    int *pref = w.B.s_pref + w.cb;
    int alive = group_scan(g, nc, [&](int i) { return proc[i] == 2 ? 0 : 1; }, pref);
    g.sync();
    if (alive != nc) {
        for (int base = 0; base < nc; base += g.size()) {
            int i = base + g.rank();
            ContactRec<R> rec;
            bool keep = i < nc && proc[i] != 2;
            if (keep) rec = w.con(i);
            g.sync();
            if (keep) w.con(pref[i]) = rec;
            g.sync();
        }
        if (g.rank() == 0) w.H->nc = alive;
    }
    g.sync();
}

template <class R, class G> __device__ void collide(const G &g, const WView<R> &w, const StepParams &sp) {
    const EvCtx ev{sp.events, sp.step_index, GB_EV_PHASE_UPDATE};
    int nb = w.H->nb, nc = w.H->nc;
    int *wake = w.B.s_wake + w.bb;
    int *proc = w.B.s_proc + w.cb;     // 0 = not updated, 1 = updated, 2 = destroy
    for (int b = g.rank(); b < nb; b += g.size())
        wake[b] = (w.awake(b) && w.btype(b) != GB_BODY_STATIC) ? -1 : GB_INF_IDX;
    for (int i = g.rank(); i < nc; i += g.size()) proc[i] = 0;
    g.sync();
    // Least fixed point of the sequential rule "contact i is updated iff one
    // of its bodies is non-static and awake when the loop reaches i"; a body
    // woken by contact j counts as awake for contacts after j.
    for (int round = 0; round <= nc + 1; ++round) {
        bool changed = false;
        for (int i = g.rank(); i < nc; i += g.size()) {
            if (proc[i]) continue;
            bool woke;
            int r = collide_one(w, i, wake, &woke, &ev);
            if (r == 0) continue;
            proc[i] = r;
            if (woke) {
                const ContactRec<R> &c = w.con(i);
                int oa = atomicMin(&wake[w.fbody(c.fa)], i);
                int ob = atomicMin(&wake[w.fbody(c.fb)], i);
                if (oa > i || ob > i) changed = true;
            }
        }
        if (!g.any(changed)) break;
    }
    g.sync();
    for (int b = g.rank(); b < nb; b += g.size())
        if (wake[b] >= 0 && wake[b] != GB_INF_IDX) wake_body(w, b);
    compact_contacts(g, w, proc);
}

// ------------------------------------------------------------ contact solver
// contact.py:375-412 + 414-496
template <class R> __device__ void build_cons(const WView<R> &w, Cons<R> &k, int ci, bool warm, double dt_ratio) {
    const ContactRec<R> &c = w.con(ci);
    int ba = w.fbody(c.fa), bb = w.fbody(c.fb);
    k.cidx = ci; k.ia = ba; k.ib = bb;
    k.ma = w.B.b_inv_mass[w.bb + ba]; k.mb = w.B.b_inv_mass[w.bb + bb];
    k.iA = w.B.b_inv_I[w.bb + ba]; k.iB = w.B.b_inv_I[w.bb + bb];
    k.lca = cvt<R>(w.B.b_lc[w.bb + ba]); k.lcb = cvt<R>(w.B.b_lc[w.bb + bb]);
    k.ra = w.B.f_radius[w.fb + c.fa]; k.rb = w.B.f_radius[w.fb + c.fb];
    k.friction = c.friction; k.restitution = c.restitution;
    k.mcount = c.m.count; k.npts = c.m.count; k.mtype = c.m.type;
    k.ln = c.m.ln; k.lp = c.m.lp;
    for (int j = 0; j < c.m.count; ++j) {
        k.lpts[j] = c.m.plp[j];
        if (warm) { k.ni[j] = (R)dt_ratio * c.m.ni[j]; k.ti[j] = (R)dt_ratio * c.m.ti[j]; }
        else { k.ni[j] = c.m.ni[j]; k.ti[j] = c.m.ti[j]; }
    }
}

template <class R> __device__ __forceinline__ xform2<R> pose_xf(vec2<double> c, double a, vec2<R> lc) {
    xform2<R> x;
    x.q = Rot<R>::of(a);
    x.p = cvt<R>(c) - rmul(x.q, lc);
    return x;
}

// contact.py:414-496 initialize_velocity_constraints + contact_util.py:195-245
// (the transforms and centres of both bodies given; init_velocity below
// derives them from the float64 poses)
template <class R> __device__ void init_velocity_xf(Cons<R> &k, xform2<R> xa, xform2<R> xb, vec2<R> car, vec2<R> cbr,
                                                    vec2<R> va, R wa, vec2<R> vb, R wb) {
    vec2<R> normal, pts[2];
    k.dec = 0;
    if (k.mtype == GB_M_CIRCLES) {
        normal = mk<R>(1, 0);
        vec2<R> pA = xmul(xa, k.lp), pB = xmul(xb, k.lpts[0]);
        vec2<R> dd = pA - pB;
        if (dot(dd, dd) > (R)GB_EPSILON_SQR) normal = normalized(pB - pA);
        vec2<R> cA = pA + k.ra * normal, cB = pB - k.rb * normal;
        pts[0] = (R)0.5 * (cA + cB);
    } else if (k.mtype == GB_M_FACE_A) {
        normal = rmul(xa.q, k.ln);
        vec2<R> plane = xmul(xa, k.lp);
        for (int i = 0; i < k.mcount; ++i) {
            vec2<R> clip = xmul(xb, k.lpts[i]);
            vec2<R> cA = clip + (k.ra - dot(clip - plane, normal)) * normal;
            vec2<R> cB = clip - k.rb * normal;
            pts[i] = (R)0.5 * (cA + cB);
        }
    } else {
        normal = rmul(xb.q, k.ln);
        vec2<R> plane = xmul(xb, k.lp);
        for (int i = 0; i < k.mcount; ++i) {
            vec2<R> clip = xmul(xa, k.lpts[i]);
            vec2<R> cB = clip + (k.rb - dot(clip - plane, normal)) * normal;
            vec2<R> cA = clip - k.ra * normal;
            pts[i] = (R)0.5 * (cA + cB);
        }
        normal = -normal;
    }
    k.normal = normal;
    vec2<R> tangent = cross(normal, (R)1);
    for (int i = 0; i < k.npts; ++i) {
        vec2<R> ra = pts[i] - car, rb = pts[i] - cbr;
        k.rA[i] = ra; k.rB[i] = rb;
        R rna = sq(cross(ra, normal)), rnb = sq(cross(rb, normal));
        R kn = k.ma + k.mb + k.iA * rna + k.iB * rnb;
        k.nm[i] = kn > (R)0 ? (R)1 / kn : (R)0;
        R rta = sq(cross(ra, tangent)), rtb = sq(cross(rb, tangent));
        R kt = k.ma + k.mb + k.iA * rta + k.iB * rtb;
        k.tm[i] = kt > (R)0 ? (R)1 / kt : (R)0;
        k.bias[i] = (R)0;
        R vrel = dot(normal, ((vb + cross(wb, rb)) - va) - cross(wa, ra));
        if (vrel < (R)-GB_VELOCITY_THRESHOLD) { k.bias[i] = -k.restitution * vrel; k.dec |= 1 << i; }
    }
    if (k.npts == 2) {
        R rn1a = cross(k.rA[0], normal), rn1b = cross(k.rB[0], normal);
        R rn2a = cross(k.rA[1], normal), rn2b = cross(k.rB[1], normal);
        R k11 = k.ma + k.mb + k.iA * rn1a * rn1a + k.iB * rn1b * rn1b;
        R k22 = k.ma + k.mb + k.iA * rn2a * rn2a + k.iB * rn2b * rn2b;
        R k12 = k.ma + k.mb + k.iA * rn1a * rn2a + k.iB * rn1b * rn2b;
        if (sq(k11) < (R)1000 * (k11 * k22 - sq(k12))) {
            k.k11 = k11; k.k12 = k12; k.k22 = k22;
            R det = k11 * k22 - k12 * k12;
            if (det != (R)0) det = (R)1 / det;
            k.nm11 = det * k22; k.nm12 = -det * k12; k.nm21 = -det * k12; k.nm22 = det * k11;
        } else {
            k.npts = 1;
            k.dec |= 4;
        }
    }
}

template <class R> __device__ __forceinline__ void init_velocity(Cons<R> &k, vec2<double> ca, double aa, vec2<double> cb, double ab,
                                                                 vec2<R> va, R wa, vec2<R> vb, R wb) {
    init_velocity_xf(k, pose_xf<R>(ca, aa, k.lca), pose_xf<R>(cb, ab, k.lcb), cvt<R>(ca), cvt<R>(cb), va, wa, vb, wb);
}

// contact.py:498-525
template <class R> __device__ __forceinline__ void warm_start(const Cons<R> &k, vec2<R> &va, R &wa, vec2<R> &vb, R &wb) {
    vec2<R> normal = k.normal, tangent = cross(normal, (R)1);
#pragma unroll
    for (int i = 0; i < 2; ++i) {   // i < npts; constant indices keep the constraint in registers
        if (i >= k.npts) break;
        vec2<R> P = k.ni[i] * normal + k.ti[i] * tangent;
        wa = wa - k.iA * cross(k.rA[i], P);
        va = va - k.ma * P;
        wb = wb + k.iB * cross(k.rB[i], P);
        vb = vb + k.mb * P;
    }
}

// contact.py:527-799
template <class R> __device__ __forceinline__ void solve_velocity(Cons<R> &k, vec2<R> &va, R &wa, vec2<R> &vb, R &wb) {
    const R ma = k.ma, mb = k.mb, iA = k.iA, iB = k.iB;
    vec2<R> normal = k.normal, tangent = cross(normal, (R)1);
    R friction = k.friction;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        if (i >= k.npts) break;
        vec2<R> ra = k.rA[i], rb = k.rB[i];
        vec2<R> dv = ((vb + cross(wb, rb)) - va) - cross(wa, ra);
        R vt = dot(dv, tangent);
        R lambda = k.tm[i] * (-vt);
        R maxf = friction * k.ni[i];
        R ni = cclamp(k.ti[i] + lambda, -maxf, maxf);
        lambda = ni - k.ti[i];
        vec2<R> P = lambda * tangent;
        va = va - ma * P;
        wa = wa - iA * cross(ra, P);
        vb = vb + mb * P;
        wb = wb + iB * cross(rb, P);
        k.ti[i] = ni;
    }
    if (k.npts == 1) {
        vec2<R> ra = k.rA[0], rb = k.rB[0];
        vec2<R> dv = ((vb + cross(wb, rb)) - va) - cross(wa, ra);
        R vn = dot(dv, normal);
        R lambda = -k.nm[0] * (vn - k.bias[0]);
        R ni = pymax(k.ni[0] + lambda, (R)0);
        lambda = ni - k.ni[0];
        vec2<R> P = lambda * normal;
        va = va - ma * P;
        wa = wa - iA * cross(ra, P);
        vb = vb + mb * P;
        wb = wb + iB * cross(rb, P);
        k.ni[0] = ni;
    } else {
        vec2<R> a = mk<R>(k.ni[0], k.ni[1]);
        vec2<R> ra1 = k.rA[0], rb1 = k.rB[0], ra2 = k.rA[1], rb2 = k.rB[1];
        vec2<R> dv1 = ((vb + cross(wb, rb1)) - va) - cross(wa, ra1);
        vec2<R> dv2 = ((vb + cross(wb, rb2)) - va) - cross(wa, ra2);
        R vn1 = dot(dv1, normal), vn2 = dot(dv2, normal);
        vec2<R> b = mk<R>(vn1 - k.bias[0], vn2 - k.bias[1]);
        b = b - mk<R>(k.k11 * a.x + k.k12 * a.y, k.k12 * a.x + k.k22 * a.y);
        vec2<R> x;
        bool solved = false;
        x = mk<R>(-(k.nm11 * b.x + k.nm12 * b.y), -(k.nm21 * b.x + k.nm22 * b.y));
        if (x.x >= (R)0 && x.y >= (R)0) solved = true;
        if (!solved) {
            x = mk<R>(-k.nm[0] * b.x, (R)0);
            vn2 = k.k12 * x.x + b.y;
            if (x.x >= (R)0 && vn2 >= (R)0) solved = true;
        }
        if (!solved) {
            x = mk<R>((R)0, -k.nm[1] * b.y);
            vn1 = k.k12 * x.y + b.x;
            if (x.y >= (R)0 && vn1 >= (R)0) solved = true;
        }
        if (!solved) {
            x = mk<R>(0, 0);
            vn1 = b.x; vn2 = b.y;
            if (vn1 >= (R)0 && vn2 >= (R)0) solved = true;
        }
        if (solved) {
            vec2<R> d = x - a;
            vec2<R> p1 = d.x * normal, p2 = d.y * normal;
            va = va - ma * (p1 + p2);
            wa = wa - iA * (cross(ra1, p1) + cross(ra2, p2));
            vb = vb + mb * (p1 + p2);
            wb = wb + iB * (cross(rb1, p1) + cross(rb2, p2));
            k.ni[0] = x.x; k.ni[1] = x.y;
        }
    }
}

// contact_util.py:323-360 + contact.py:809-864 / 866-933 for one
// constraint; returns the constraint's running minimum separation.
template <class R> __device__ double solve_position(const Cons<R> &k, vec2<double> &ca, double &aa, vec2<double> &cb,
                                                   double &ab, double minsep, bool toi, bool toi_a, bool toi_b) {
    R ma = k.ma, mb = k.mb, iA = k.iA, iB = k.iB;
    R baum = (R)GB_BAUMGARTE;
    if (toi) {
        baum = (R)GB_TOI_BAUMGARTE;
        if (!toi_a) { ma = (R)0; iA = (R)0; }
        if (!toi_b) { mb = (R)0; iB = (R)0; }
    }
#pragma unroll
    for (int j = 0; j < 2; ++j) {   // j < point count
        if (j >= k.mcount) break;
        xform2<R> xa = pose_xf<R>(ca, aa, k.lca), xb = pose_xf<R>(cb, ab, k.lcb);
        vec2<R> normal, point;
        R sep;
        if (k.mtype == GB_M_CIRCLES) {
            vec2<R> pA = xmul(xa, k.lp), pB = xmul(xb, k.lpts[0]);
            normal = normalized(pB - pA);
            point = (R)0.5 * (pA + pB);
            sep = dot(pB - pA, normal) - k.ra - k.rb;
        } else if (k.mtype == GB_M_FACE_A) {
            normal = rmul(xa.q, k.ln);
            vec2<R> plane = xmul(xa, k.lp);
            vec2<R> clip = xmul(xb, k.lpts[j]);
            sep = dot(clip - plane, normal) - k.ra - k.rb;
            point = clip;
        } else {
            normal = rmul(xb.q, k.ln);
            vec2<R> plane = xmul(xb, k.lp);
            vec2<R> clip = xmul(xa, k.lpts[j]);
            sep = dot(clip - plane, normal) - k.ra - k.rb;
            point = clip;
            normal = -normal;
        }
        vec2<R> ra = point - cvt<R>(ca), rb = point - cvt<R>(cb);
        minsep = pymin(minsep, (double)sep);
        R C = cclamp(baum * (sep + (R)GB_LINEAR_SLOP), (R)-GB_MAX_LINEAR_CORRECTION, (R)0);
        R rna = sq(cross(ra, normal)), rnb = sq(cross(rb, normal));
        R K = ma + mb + (iA * rna) + (iB * rnb);
        R impulse = K > (R)0 ? -C / K : (R)0;
        vec2<R> P = impulse * normal;
        ca = ca - cvt<double>(ma * P);
        aa = aa - (double)(iA * cross(ra, P));
        cb = cb + cvt<double>(mb * P);
        ab = ab + (double)(iB * cross(rb, P));
    }
    return minsep;
}

// The float32 form of solve_position for the batched solver: each body is
// its step-start position rounded to float32 (cf) and its step-start angle
// reduced to [-pi, pi] (ar), plus the corrections of this step's position
// passes (dc, da), so the passes run without float64 arithmetic; the caller
// adds the corrections to the float64 pose once, after the passes.
static __device__ float solve_position_f32d(const Cons<float> &k, vec2<float> cfa, float ara, vec2<float> &dca, float &daa,
                                            vec2<float> cfb, float arb, vec2<float> &dcb, float &dab, float minsep,
                                            bool toi = false, bool toi_a = false, bool toi_b = false) {
    float ma = k.ma, mb = k.mb, iA = k.iA, iB = k.iB;
    float baum = (float)GB_BAUMGARTE;
    if (toi) {
        baum = (float)GB_TOI_BAUMGARTE;
        if (!toi_a) { ma = 0.0f; iA = 0.0f; }
        if (!toi_b) { mb = 0.0f; iB = 0.0f; }
    }
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        if (j >= k.mcount) break;
        const vec2<float> ca = cfa + dca, cb = cfb + dcb;
        xform2<float> xa, xb;
        xa.q = rot_f32(ara + daa);
        xa.p = ca - rmul(xa.q, k.lca);
        xb.q = rot_f32(arb + dab);
        xb.p = cb - rmul(xb.q, k.lcb);
        vec2<float> normal, point;
        float sep;
        if (k.mtype == GB_M_CIRCLES) {
            vec2<float> pA = xmul(xa, k.lp), pB = xmul(xb, k.lpts[0]);
            normal = normalized(pB - pA);
            point = 0.5f * (pA + pB);
            sep = dot(pB - pA, normal) - k.ra - k.rb;
        } else if (k.mtype == GB_M_FACE_A) {
            normal = rmul(xa.q, k.ln);
            vec2<float> plane = xmul(xa, k.lp);
            vec2<float> clip = xmul(xb, k.lpts[j]);
            sep = dot(clip - plane, normal) - k.ra - k.rb;
            point = clip;
        } else {
            normal = rmul(xb.q, k.ln);
            vec2<float> plane = xmul(xb, k.lp);
            vec2<float> clip = xmul(xa, k.lpts[j]);
            sep = dot(clip - plane, normal) - k.ra - k.rb;
            point = clip;
            normal = -normal;
        }
        vec2<float> ra = point - ca, rb = point - cb;
        minsep = pymin(minsep, sep);
        float C = cclamp(baum * (sep + (float)GB_LINEAR_SLOP), (float)-GB_MAX_LINEAR_CORRECTION, 0.0f);
        float rna = sq(cross(ra, normal)), rnb = sq(cross(rb, normal));
        float K = ma + mb + (iA * rna) + (iB * rnb);
        float impulse = K > 0.0f ? -C / K : 0.0f;
        vec2<float> P = impulse * normal;
        dca = dca - ma * P;
        daa = daa - iA * cross(ra, P);
        dcb = dcb + mb * P;
        dab = dab + iB * cross(rb, P);
    }
    return minsep;
}

// ------------------------------------------------------------ islands + solve
template <class R> __device__ __forceinline__ bool qualifies(const WView<R> &w, const ContactRec<R> &c) {
    return (c.flags & GB_C_ENABLED) && (c.flags & GB_C_TOUCHING) && !fx_sensor(w, c.fa) && !fx_sensor(w, c.fb);
}
static __device__ __forceinline__ int uf_find(int *parent, int x) {
    int p = parent[x];
    while (p != x) { x = p; p = parent[x]; }
    return x;
}
static __device__ __forceinline__ void uf_union(int *parent, int a, int b) {
    for (int guard = 0; guard < 1 << 20; ++guard) {
        a = uf_find(parent, a);
        b = uf_find(parent, b);
        if (a == b) return;
        if (a < b) { int t = a; a = b; b = t; }
        // hook the larger root under the smaller one: the final root of a
        // component is its smallest body index, whatever the schedule.
        if (atomicCAS(&parent[a], a, b) == a) return;
    }
}

// Depth-first island search of world.py:495-573 for one island, used only
// where the reference's result depends on the visit order (island.py:163-179
// reads the last visited body and puts the last non-static one to sleep).
template <class R> __device__ void island_dfs(const WView<R> &w, int seed, int *last, int *last_ns) {
    int *stack = w.B.s_stack + w.bb;
    unsigned char *bvis = w.B.s_bvis + w.bb;
    unsigned char *cvis = w.B.s_cvis + w.cb;
    const int *off = w.B.s_adjoff + w.bb + w.wi;
    const int *adj = w.B.s_adj + 2 * w.cb;
    int sp = 0;
    stack[sp++] = seed;
    bvis[seed] = 1;
    int lb = -1, lns = -1;
    while (sp > 0) {
        int b = stack[--sp];
        lb = b;
        if (w.btype(b) == GB_BODY_STATIC) continue;
        lns = b;
        for (int e = off[b]; e < off[b + 1]; ++e) {
            int ci = adj[e];
            if (cvis[ci]) continue;
            cvis[ci] = 1;
            const ContactRec<R> &c = w.con(ci);
            int fa = w.fbody(c.fa), fbb = w.fbody(c.fb);
            int other = (fa == b) ? fbb : fa;
            if (bvis[other]) continue;
            stack[sp++] = other;
            bvis[other] = 1;
        }
        // the body's joints, in its joint-list order (world.py:547-567)
        if (w.H->nj > 0) {
            const int *joff = w.B.b_joff + w.bb + w.wi;
            const int *jadj = w.B.b_jadj + 2 * (size_t)w.H->jbase;
            unsigned char *jvis = w.B.s_jvis + w.H->jbase;
            const gb_joint *J = w.B.j + w.H->jbase;
            for (int e = joff[b]; e < joff[b + 1]; ++e) {
                const int j = jadj[e];
                if (jvis[j]) continue;
                const int other = J[j].body_a == b ? J[j].body_b : J[j].body_a;
                if (!(w.B.b_flags[w.bb + other] & GB_BODY_ACTIVE)) continue;
                jvis[j] = 1;
                if (bvis[other]) continue;
                stack[sp++] = other;
                bvis[other] = 1;
            }
        }
    }
    *last = lb;
    *last_ns = lns;
}

// A joint of the world takes part in this step's solve: both bodies active
// and a non-static one in a simulated island (world.py:547-567).
template <class R> __device__ __forceinline__ bool joint_simulated(const WView<R> &w, const gb_joint &J, const int *parent,
                                                                   const uint32_t *rootf) {
    const uint32_t fa = w.B.b_flags[w.bb + J.body_a], fb = w.B.b_flags[w.bb + J.body_b];
    if (!(fa & GB_BODY_ACTIVE) || !(fb & GB_BODY_ACTIVE)) return false;
    const bool sa = w.btype(J.body_a) == GB_BODY_STATIC, sb = w.btype(J.body_b) == GB_BODY_STATIC;
    if (sa && sb) return false;
    return (rootf[parent[sa ? J.body_b : J.body_a]] & R_SIM) != 0;
}

// Island search by union-find (world.py:495-573 without the visit order):
// components over qualifying contacts between non-static bodies, the
// simulated flag of each component and its depth-first seed.
#include "gb_controllers.cuh"

template <class R, class G> __device__ void islands_group(const G &g, const WView<R> &w, const StepParams &sp) {
    const int nb = w.H->nb, nc = w.H->nc, nf = w.H->nf;
    int *parent = w.B.s_parent + w.bb;
    uint32_t *rootf = w.B.s_root + w.bb;
    int *seed = w.B.s_seed + w.bb;
    unsigned long long *minsep = w.B.s_minsep + w.bb;
    unsigned long long *minsleep = w.B.s_minsleep + w.bb;
    unsigned long long *claim = w.B.s_claim + w.bb;
    int *cons_of = w.B.s_cons_of + w.cb;
    int *colour = w.B.s_colour + w.cb;
    int *order = w.B.s_order + w.cb;
    int *pref = w.B.s_pref + w.cb;
    Cons<R> *cons = w.B.s_cons + w.cb;
    int *coff = w.B.s_proc + w.cb;
    const double dt = sp.dt;
    const bool warm = (w.H->flags & GB_W_WARM_STARTING) != 0;
    (void)nb; (void)nc; (void)nf; (void)parent; (void)rootf; (void)seed; (void)minsep; (void)minsleep; (void)claim;
    (void)cons_of; (void)colour; (void)order; (void)pref; (void)cons; (void)coff; (void)dt; (void)warm;
    // 1. components of the constraint graph (static bodies do not link)
    for (int b = g.rank(); b < nb; b += g.size()) {
        parent[b] = b; rootf[b] = 0; seed[b] = GB_INF_IDX;
        minsleep[b] = ~0ull;
    }
    g.sync();
    for (int i = g.rank(); i < nc; i += g.size()) {
        const ContactRec<R> &c = w.con(i);
        if (!qualifies(w, c)) continue;
        int ba = w.fbody(c.fa), bb = w.fbody(c.fb);
        if (w.btype(ba) != GB_BODY_STATIC && w.btype(bb) != GB_BODY_STATIC) uf_union(parent, ba, bb);
    }
    // joints link their bodies when both are active and neither is static
    for (int j = g.rank(); j < w.H->nj; j += g.size()) {
        const gb_joint &J = w.B.j[w.H->jbase + j];
        const int ba = J.body_a, bb = J.body_b;
        if (w.btype(ba) == GB_BODY_STATIC || w.btype(bb) == GB_BODY_STATIC) continue;
        if ((w.B.b_flags[w.bb + ba] & GB_BODY_ACTIVE) && (w.B.b_flags[w.bb + bb] & GB_BODY_ACTIVE)) uf_union(parent, ba, bb);
    }
    g.sync();
    for (int b = g.rank(); b < nb; b += g.size()) parent[b] = uf_find(parent, b);
    g.sync();
    bool all_allow = true;
    for (int b = g.rank(); b < nb; b += g.size()) {
        uint32_t f = w.B.b_flags[w.bb + b];
        if (!(f & GB_BODY_ALLOW_SLEEP)) all_allow = false;
        if (w.btype(b) != GB_BODY_STATIC && (f & GB_BODY_AWAKE) && (f & GB_BODY_ACTIVE)) {
            atomicOr(&rootf[parent[b]], R_SIM);
            atomicMin(&seed[parent[b]], b);
        }
    }
    all_allow = !g.any(!all_allow);
    if (g.rank() == 0) w.H->all_allow = all_allow ? 1 : 0;
    g.sync();
}

// Graph colouring of n constraints over their non-static bodies kb[k] (-1:
// static): Jones-Plassmann rounds with fixed hash priorities; a constraint is
// coloured when it holds the highest key on each of its non-static bodies,
// with the lowest colour free on both (per-body masks of the colours taken
// so far; beyond 64 colours, a colour of its own round).  Colour classes
// share no non-static body, so each class is solved in parallel exactly as a
// sequential pass would.  The colours in use are then numbered densely;
// returns their number.  colour[k] must be -1 on entry.  *shared is a
// group-shared int, tmp `cap` ints of scratch; more than cap - 1 colours
// (never, while n < cap) flags GB_ST_ITER_LIMIT and leaves the constraints
// beyond with colours >= the count returned.
template <class R, class G> __device__ int jp_colour(const G &g, const WView<R> &w, int n, const int2 *kb, int *colour,
                                                     int *shared, int *tmp, int cap) {
    const int nb = w.H->nb;
    unsigned long long *claim = w.B.s_claim + w.bb;
    unsigned long long *used = w.B.s_minsep + w.bb;   // free until the position iterations
    for (int b = g.rank(); b < nb; b += g.size()) used[b] = 0ull;
    if (g.rank() == 0) *shared = 0;
    for (int round = 0; round <= n; ++round) {   // >= 1 constraint is coloured per round
        for (int b = g.rank(); b < nb; b += g.size()) claim[b] = 0ull;
        g.sync();
        bool left = false;
        for (int k = g.rank(); k < n; k += g.size()) {
            if (colour[k] >= 0) continue;
            left = true;
            int2 q = kb[k];
            unsigned h = (unsigned)k * 2654435761u;
            h ^= h >> 15; h *= 0x2c1b3c6du; h ^= h >> 12;
            unsigned long long key = ((unsigned long long)h << 32) | (unsigned)(0x7fffffff - k);
            if (q.x >= 0) atomicMax(&claim[q.x], key);
            if (q.y >= 0) atomicMax(&claim[q.y], key);
        }
        if (!g.any(left)) break;
        for (int k = g.rank(); k < n; k += g.size()) {
            if (colour[k] >= 0) continue;
            int2 q = kb[k];
            unsigned h = (unsigned)k * 2654435761u;
            h ^= h >> 15; h *= 0x2c1b3c6du; h ^= h >> 12;
            unsigned long long key = ((unsigned long long)h << 32) | (unsigned)(0x7fffffff - k);
            bool win = (q.x < 0 || claim[q.x] == key) && (q.y < 0 || claim[q.y] == key);
            if (!win) continue;
            // this round's winners share no body: their mask reads and writes do not race
            unsigned long long taken = (q.x >= 0 ? used[q.x] : 0ull) | (q.y >= 0 ? used[q.y] : 0ull);
            int c = __ffsll((long long)~taken) - 1;
            if (c < 0) c = 64 + round;
            else {
                if (q.x >= 0) used[q.x] |= 1ull << c;
                if (q.y >= 0) used[q.y] |= 1ull << c;
            }
            colour[k] = c;
        }
        g.sync();
    }
    // number the colours in use densely (masks leave no gaps below 64; the
    // round colours above it may)
    for (int k = g.rank(); k < n; k += g.size()) atomicMax(shared, colour[k] + 1);
    g.sync();
    int ncol = *shared;
    if (ncol > 64) {
        if (ncol + 1 > cap) {   // never index past the world's slots
            if (g.rank() == 0) w.H->status |= GB_ST_ITER_LIMIT;
            ncol = cap - 1;
        }
        for (int cc = g.rank(); cc < ncol; cc += g.size()) tmp[cc] = 0;
        g.sync();
        for (int k = g.rank(); k < n; k += g.size())
            if (colour[k] >= 0 && colour[k] < ncol) tmp[colour[k]] = 1;
        g.sync();
        if (g.rank() == 0) {
            int d = 0;
            for (int cc = 0; cc < ncol; ++cc) { int u = tmp[cc]; tmp[cc] = d; d += u; }
            *shared = d;
        }
        g.sync();
        for (int k = g.rank(); k < n; k += g.size())
            if (colour[k] >= 0 && colour[k] < ncol) colour[k] = tmp[colour[k]];
        g.sync();
        ncol = *shared;
    }
    return ncol;
}

// Constraint list of the simulated islands in contact-list order, graph
// colouring and the colour-major solver order.
template <class R, class G> __device__ void constraints_group(const G &g, const WView<R> &w, const StepParams &sp) {
    const int nb = w.H->nb, nc = w.H->nc;
    const int *parent = w.B.s_parent + w.bb;
    const uint32_t *rootf = w.B.s_root + w.bb;
    unsigned long long *claim = w.B.s_claim + w.bb;
    int *colour = w.B.s_colour + w.cb;
    int *pref = w.B.s_pref + w.cb;
    Cons<R> *cons = w.B.s_cons + w.cb;
    int *coff = w.B.s_proc + w.cb;
    int *kc = w.B.s_cons_of + w.cb;                 // contact of constraint k
    int2 *kb = w.B.s_kb + w.cb;                     // its non-static bodies (-1: static)
    int *kroot = w.B.s_adj + 2 * (size_t)w.cb;      // its island
    (void)sp;
    // 2. island membership: wake the members of simulated islands (DFS sets
    //    body.awake = True, world.py:520), constraints = qualifying contacts
    //    of simulated islands in contact-list order.
    for (int b = g.rank(); b < nb; b += g.size())
        if (w.btype(b) != GB_BODY_STATIC && (rootf[parent[b]] & R_SIM)) wake_body(w, b);
    int ncons = group_scan(g, nc, [&](int i) {
        const ContactRec<R> &c = w.con(i);
        if (!qualifies(w, c)) return 0;
        int ba = w.fbody(c.fa), bb = w.fbody(c.fb);
        int dyn = (w.btype(ba) != GB_BODY_STATIC) ? ba : bb;
        return (rootf[parent[dyn]] & R_SIM) ? 1 : 0;
    }, pref);
    g.sync();
    for (int i = g.rank(); i < nc; i += g.size()) {
        const ContactRec<R> &c = w.con(i);
        if (!qualifies(w, c)) continue;
        int ba = w.fbody(c.fa), bb = w.fbody(c.fb);
        bool sa = w.btype(ba) == GB_BODY_STATIC, sb = w.btype(bb) == GB_BODY_STATIC;
        int dyn = sa ? bb : ba;
        if (!(rootf[parent[dyn]] & R_SIM)) continue;
        int k = pref[i];
        kc[k] = i;
        kroot[k] = parent[dyn];
        kb[k] = make_int2(sa ? -1 : ba, sb ? -1 : bb);
        colour[k] = -1;
        if (sa) wake_body(w, ba);
        if (sb) wake_body(w, bb);
    }
    g.sync();
    // 3. graph colouring (jp_colour)
    int ncol = jp_colour(g, w, ncons, kb, colour, &w.H->last_ncolours, pref, w.H->ccap);
    // The constraints are stored colour-major: constraint slots [coff[c],
    // coff[c+1]) hold colour c.  Positions inside a colour come from atomics:
    // a colour's constraints share no non-static body, so their order there
    // changes no result.  coff lives in the collide scratch (free during the
    // solve); ncol < ccap because every colour holds a constraint.
    if (ncol + 1 > w.H->ccap) {   // cannot happen while ncons < ccap; never index past the world's slots
        if (g.rank() == 0) w.H->status |= GB_ST_ITER_LIMIT;
        ncol = w.H->ccap - 1;
    }
    for (int cc = g.rank(); cc <= ncol; cc += g.size()) coff[cc] = 0;
    g.sync();
    for (int k = g.rank(); k < ncons; k += g.size())
        if (colour[k] >= 0 && colour[k] < ncol) atomicAdd(&coff[colour[k] + 1], 1);
    g.sync();
    if (g.rank() == 0)
        for (int cc = 1; cc <= ncol; ++cc) coff[cc] += coff[cc - 1];
    g.sync();
    for (int cc = g.rank(); cc < ncol; cc += g.size()) pref[cc] = coff[cc];
    g.sync();
    for (int k = g.rank(); k < ncons; k += g.size()) {
        if (colour[k] < 0 || colour[k] >= ncol) continue;
        int pos = atomicAdd(&pref[colour[k]], 1);
        ConsPos<R> &cp = w.B.s_cp[w.cb + pos];
        cp.cidx = kc[k];
        cp.root = kroot[k];
    }
    if (g.rank() == 0) { w.H->last_ncons = coff[ncol]; w.H->last_ncolours = ncol; }
    g.sync();
    if (sp.record_order) {
        int *out = w.B.order_out + w.cb;
        for (int k = g.rank(); k < w.H->last_ncons; k += g.size()) out[k] = w.B.s_cp[w.cb + k].cidx;
    }
    // 4. joints of the simulated islands (World.joints order), coloured and
    //    laid out colour-major on their own: every velocity iteration solves
    //    all joints before the contacts and every position iteration after
    //    them (island.py:107-148)
    const int nj = w.H->nj;
    if (nj == 0) {
        if (g.rank() == 0) { w.H->last_njcons = 0; w.H->last_njcolours = 0; }
        g.sync();
        return;
    }
    const int jb = w.H->jbase;
    const gb_joint *J = w.B.j + jb;
    int *jkj = w.B.s_jkj + jb;
    int2 *jkb = w.B.s_jkb + jb;
    int *jcol = w.B.s_jcol + jb;
    int *jpref = w.B.s_jpref + jb;
    int *joff = w.B.s_joff + jb + w.wi;   // nj + 1 slots
    const int njc = group_scan(g, nj, [&](int j) { return joint_simulated(w, J[j], parent, rootf) ? 1 : 0; }, jpref);
    g.sync();
    for (int j = g.rank(); j < nj; j += g.size()) {
        if (!joint_simulated(w, J[j], parent, rootf)) continue;
        const int k = jpref[j];
        const int ba = J[j].body_a, bb = J[j].body_b;
        const bool sa = w.btype(ba) == GB_BODY_STATIC, sb = w.btype(bb) == GB_BODY_STATIC;
        jkj[k] = j;
        jkb[k] = make_int2(sa ? -1 : ba, sb ? -1 : bb);
        jcol[k] = -1;
        if (sa) wake_body(w, ba);   // the depth-first search wakes every body it reaches (world.py:520)
        if (sb) wake_body(w, bb);
    }
    g.sync();
    const int njcol = njc > 0 ? jp_colour(g, w, njc, jkb, jcol, &w.H->last_njcolours, joff, nj + 1) : 0;
    for (int cc = g.rank(); cc <= njcol; cc += g.size()) joff[cc] = 0;
    g.sync();
    for (int k = g.rank(); k < njc; k += g.size())
        if (jcol[k] >= 0 && jcol[k] < njcol) atomicAdd(&joff[jcol[k] + 1], 1);
    g.sync();
    if (g.rank() == 0)
        for (int cc = 1; cc <= njcol; ++cc) joff[cc] += joff[cc - 1];
    g.sync();
    for (int cc = g.rank(); cc < njcol; cc += g.size()) jpref[cc] = joff[cc];
    g.sync();
    for (int k = g.rank(); k < njc; k += g.size()) {
        if (jcol[k] < 0 || jcol[k] >= njcol) continue;
        const int pos = atomicAdd(&jpref[jcol[k]], 1);
        const int j = jkj[k];
        JCons &q = w.B.s_jc[jb + pos];
        q.j = j;
        q.ia = J[j].body_a;
        q.ib = J[j].body_b;
        q.root = parent[w.btype(q.ia) == GB_BODY_STATIC ? q.ib : q.ia];
    }
    if (g.rank() == 0) { w.H->last_njcons = joff[njcol]; w.H->last_njcolours = njcol; }
    g.sync();
    if (sp.record_order)
        for (int k = g.rank(); k < w.H->last_njcons; k += g.size()) w.B.jorder_out[jb + k] = w.B.s_jc[jb + k].j;
}

// island.py:71-95 for one body of a simulated island
template <class R> __device__ __forceinline__ void integrate_velocity_body(const WView<R> &w, int b, double dt) {
    const uint32_t *rootf = w.B.s_root + w.bb;
    const int *parent = w.B.s_parent + w.bb;
    if (w.btype(b) == GB_BODY_STATIC || !(rootf[parent[b]] & R_SIM)) return;
    const vec2<R> grav = mk<R>((R)w.H->gx, (R)w.H->gy);
    int gb = w.bb + b;
    w.B.b_c0[gb] = w.B.b_c[gb];
    w.B.b_a0[gb] = w.B.b_a[gb];
    if (w.btype(b) == GB_BODY_DYNAMIC) {
        vec2<R> v = w.B.b_v[gb];
        R om = w.B.b_w[gb];
        const R dtr = (R)dt;
        v = v + dtr * (w.B.b_gscale[gb] * grav + w.B.b_inv_mass[gb] * w.B.b_f[gb]);
        om = om + dtr * w.B.b_inv_I[gb] * w.B.b_torque[gb];
        v = cclamp((R)1 - dtr * w.B.b_ldamp[gb], (R)0, (R)1) * v;
        om = om * cclamp((R)1 - dtr * w.B.b_adamp[gb], (R)0, (R)1);
        w.B.b_v[gb] = v; w.B.b_w[gb] = om;
    }
}

// contact.py:375-496 for constraint k (positions before integration,
// velocities after)
template <class R> __device__ __forceinline__ void init_constraint(const WView<R> &w, int k, const StepParams &sp,
                                                                   bool use_pose = false) {
    ConsPos<R> &cp = w.B.s_cp[w.cb + k];
    Cons<R> q;
    build_cons(w, q, cp.cidx, (w.H->flags & GB_W_WARM_STARTING) != 0, w.H->inv_dt0 * sp.dt);
    int ga = w.bb + q.ia, gbb = w.bb + q.ib;
    if (use_pose) {
        // the float32 centres and rotations k_vinit stored: the same values
        // pose_xf derives from the float64 poses, without float64 arithmetic
        const float4 pa = w.B.s_pose[ga], pb = w.B.s_pose[gbb];
        xform2<R> xa, xb;
        xa.q.c = (R)pa.z; xa.q.s = (R)pa.w;
        xa.p = mk<R>((R)pa.x, (R)pa.y) - rmul(xa.q, q.lca);
        xb.q.c = (R)pb.z; xb.q.s = (R)pb.w;
        xb.p = mk<R>((R)pb.x, (R)pb.y) - rmul(xb.q, q.lcb);
        init_velocity_xf(q, xa, xb, mk<R>((R)pa.x, (R)pa.y), mk<R>((R)pb.x, (R)pb.y), w.B.b_v[ga], w.B.b_w[ga], w.B.b_v[gbb],
                         w.B.b_w[gbb]);
    } else {
        init_velocity(q, w.B.b_c[ga], w.B.b_a[ga], w.B.b_c[gbb], w.B.b_a[gbb], w.B.b_v[ga], w.B.b_w[ga], w.B.b_v[gbb], w.B.b_w[gbb]);
    }
    if (sp.record_order) {   // step record: the set-up decisions of this constraint
        const int bits = rec_setup_bits(q.dec, GB_REC_SETUP_SHIFT);
        if (bits && w.btype(q.ia) != GB_BODY_STATIC) atomicXor(&w.B.rec[ga], bits);
        if (bits && w.btype(q.ib) != GB_BODY_STATIC) atomicXor(&w.B.rec[gbb], bits);
    }
    ConsVel<R> v;
    for (int j = 0; j < 2; ++j) {
        v.ni[j] = j < q.mcount ? q.ni[j] : (R)0;
        v.ti[j] = j < q.mcount ? q.ti[j] : (R)0;
        v.rA[j] = j < q.npts ? q.rA[j] : mk<R>(0, 0);
        v.rB[j] = j < q.npts ? q.rB[j] : mk<R>(0, 0);
        v.nm[j] = j < q.npts ? q.nm[j] : (R)0;
        v.tm[j] = j < q.npts ? q.tm[j] : (R)0;
        v.bias[j] = j < q.npts ? q.bias[j] : (R)0;
    }
    v.ia = q.ia; v.ib = q.ib; v.npts = q.npts; v._pad = 0;
    v.normal = q.normal;
    v.friction = q.friction;
    const bool two = q.npts == 2;
    v.k11 = two ? q.k11 : (R)0; v.k12 = two ? q.k12 : (R)0; v.k22 = two ? q.k22 : (R)0;
    v.nm11 = two ? q.nm11 : (R)0; v.nm12 = two ? q.nm12 : (R)0; v.nm22 = two ? q.nm22 : (R)0;
    w.B.s_cv[w.cb + k] = v;
    cp.ia = q.ia; cp.ib = q.ib;
    cp.mcount = q.mcount; cp.mtype = q.mtype; cp._pad0 = 0; cp._pad1 = 0;
    cp.lca = q.lca; cp.lcb = q.lcb; cp.ln = q.ln; cp.lp = q.lp;
    cp.lpts[0] = q.mcount > 0 ? q.lpts[0] : mk<R>(0, 0);
    cp.lpts[1] = q.mcount > 1 ? q.lpts[1] : mk<R>(0, 0);
    cp.ra = q.ra; cp.rb = q.rb;
}

// The full constraint of the velocity passes from its record and the
// bodies' inverse masses (the fields solve_velocity and warm_start read).
template <class R> __device__ __forceinline__ Cons<R> vel_cons(const ConsVel<R> &v, R ma, R mb, R iA, R iB) {
    Cons<R> q;
    q.ia = v.ia; q.ib = v.ib; q.npts = v.npts;
    q.ma = ma; q.mb = mb; q.iA = iA; q.iB = iB;
    q.normal = v.normal; q.friction = v.friction;
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        q.ni[j] = v.ni[j]; q.ti[j] = v.ti[j];
        q.rA[j] = v.rA[j]; q.rB[j] = v.rB[j];
        q.nm[j] = v.nm[j]; q.tm[j] = v.tm[j]; q.bias[j] = v.bias[j];
    }
    q.k11 = v.k11; q.k12 = v.k12; q.k22 = v.k22;
    q.nm11 = v.nm11; q.nm12 = v.nm12; q.nm21 = v.nm12; q.nm22 = v.nm22;
    return q;
}
// The fields solve_position reads, widened to float64.
template <class R> __device__ __forceinline__ Cons<double> pos_cons_f64(const Cons<R> &k) {
    Cons<double> q;
    q.ia = k.ia; q.ib = k.ib;
    q.ma = (double)k.ma; q.mb = (double)k.mb; q.iA = (double)k.iA; q.iB = (double)k.iB;
    q.mcount = k.mcount; q.mtype = k.mtype;
    q.lca = cvt<double>(k.lca); q.lcb = cvt<double>(k.lcb); q.ln = cvt<double>(k.ln); q.lp = cvt<double>(k.lp);
    q.lpts[0] = cvt<double>(k.lpts[0]); q.lpts[1] = cvt<double>(k.lpts[1]);
    q.ra = (double)k.ra; q.rb = (double)k.rb;
    return q;
}
// The fields solve_position reads.
template <class R> __device__ __forceinline__ Cons<R> pos_cons(const ConsPos<R> &p, R ma, R mb, R iA, R iB) {
    Cons<R> q;
    q.ia = p.ia; q.ib = p.ib;
    q.ma = ma; q.mb = mb; q.iA = iA; q.iB = iB;
    q.mcount = p.mcount; q.mtype = p.mtype;
    q.lca = p.lca; q.lcb = p.lcb; q.ln = p.ln; q.lp = p.lp;
    q.lpts[0] = p.lpts[0]; q.lpts[1] = p.lpts[1];
    q.ra = p.ra; q.rb = p.rb;
    return q;
}

// Warm start, velocity iterations, impulse store, position integration,
// position iterations and transform write-back (island.py:98-159).
//
// With a shared-memory cache (the phased solve kernel) the world's bodies
// live in shared memory during the passes and the constraint records
// stream through `nbuf` shared-memory buffers: the records of each colour
// are cut into chunks of one record per thread, and one thread keeps
// nbuf - 1 chunks of bulk copies (cp.async.bulk, completion on an mbarrier)
// in flight ahead of the chunk being solved.  Without a cache every pass
// reads the records and bodies from global memory.
static __device__ __forceinline__ bool is_neg_zero(float x) { return __float_as_uint(x) == 0x80000000u; }
static __device__ __forceinline__ bool is_neg_zero(double x) {
    return (unsigned long long)__double_as_longlong(x) == 0x8000000000000000ull;
}
struct BodyCache {
    unsigned char *mem;   // nullptr: the passes read and write global memory
    int nbuf;             // constraint chunk buffers after the bodies (0: none)
};
// shared-memory bytes of the body cache and of one chunk buffer
template <class R> __host__ __device__ constexpr int cache_bytes_per_body() {
    return 2 * (int)sizeof(double) + (int)sizeof(double) + 2 * (int)sizeof(R);   // c, a, inverse mass and inertia
}
__host__ __device__ inline size_t align128(size_t x) { return (x + 127) & ~(size_t)127; }
template <class R> __host__ __device__ inline size_t cache_body_bytes(int nb) {
    return align128((size_t)nb * cache_bytes_per_body<R>());
}
template <class R> __host__ __device__ inline size_t chunk_buf_bytes(int threads) {
    size_t a = sizeof(ConsVel<R>), b = sizeof(ConsPos<R>);
    return align128((size_t)threads * (a > b ? a : b));
}
template <class R> __host__ inline size_t solve_smem_bytes(int nb, int threads, int nbuf) {
    return cache_body_bytes<R>(nb) + (size_t)nbuf * chunk_buf_bytes<R>(threads) + 64;
}
#define GB_MAX_PIPE_BUFS 4

// Chunks of the colour-major records: start | count << 22, one per entry.
template <class G> __device__ int chunk_table(const G &g, const int *coff, int ncol, int cap, int *tab, int lim, uint32_t *status) {
    if (g.rank() == 0) {
        int n = 0;
        for (int cc = 0; cc < ncol; ++cc)
            for (int s0 = coff[cc]; s0 < coff[cc + 1]; s0 += cap) {
                int cnt = coff[cc + 1] - s0 < cap ? coff[cc + 1] - s0 : cap;
                if (n < lim) tab[n++] = s0 | (cnt << 22);
                else *status |= GB_ST_ITER_LIMIT;   // more chunks than slots: never past the world's scratch
            }
        tab[-1] = n;
    }
    g.sync();
    int n = tab[-1];
    g.sync();
    return n;
}

// A run of chunk loads through the buffers: chunk q of the run goes to
// buffer q % nbuf; rank 0 issues up to nbuf - 1 chunks ahead.
struct ChunkPipe {
    unsigned char *buf;
    unsigned long long *bar;
    size_t buf_bytes;
    int nbuf;
    unsigned parity;     // bit b: parity of the next completion of buffer b
    int issued;          // chunks issued so far in this run
    int consumed;        // chunks whose completion this thread has seen in this run
};

// After an early exit or a wait that gave up: rank 0 (which issued every
// copy) waits, with the full limit, for each chunk it issued and has not
// seen complete, so no copy lands after the block has left its shared
// memory.  Returns false when one of those waits gives up as well.
template <class G> __device__ bool pipe_drain(const G &g, ChunkPipe &p) {
    bool ok = true;
    if (g.rank() == 0)
        for (; p.consumed < p.issued; ++p.consumed) {
            const int b = p.consumed % p.nbuf;
            if (!mbar_wait(&p.bar[b], (p.parity >> b) & 1u, GB_WAIT_POLLS)) { ok = false; break; }
            p.parity ^= 1u << b;
        }
    return !g.any(!ok);
}

template <class G, class Rec> __device__ __forceinline__ void pipe_issue(const G &g, ChunkPipe &p, int q, const Rec *base,
                                                                        const int *tab, int nch) {
    if (g.rank() == 0) {
        int e = tab[q % nch];
        int s0 = e & ((1 << 22) - 1), cnt = e >> 22;
        int b = q % p.nbuf;
        unsigned bytes = (unsigned)(cnt * sizeof(Rec));
        mbar_arrive_expect_tx(&p.bar[b], bytes);
        bulk_load(p.buf + (size_t)b * p.buf_bytes, base + s0, bytes, &p.bar[b]);
    }
}

template <class R, class G> __device__ void solve_group(const G &g, const WView<R> &w, const StepParams &sp, PhaseClock *pcp = nullptr,
                                                        BodyCache cache = BodyCache{nullptr, 0}) {
    PhaseClock dummy;
    dummy.acc = nullptr;
    PhaseClock &ck = pcp ? *pcp : dummy;
    const int nb = w.H->nb;
    int *parent = w.B.s_parent + w.bb;
    uint32_t *rootf = w.B.s_root + w.bb;
    unsigned long long *minsep = w.B.s_minsep + w.bb;
    int *coff = w.B.s_proc + w.cb;
    ConsVel<R> *cv = w.B.s_cv + w.cb;
    ConsPos<R> *cpos = w.B.s_cp + w.cb;
    const double dt = sp.dt;
    const bool warm = (w.H->flags & GB_W_WARM_STARTING) != 0;
    const int ncol = w.H->last_ncolours;
    const int ncons = w.H->last_ncons;
    const int rank = g.rank();
    // joints: set up after the contacts' warm start, solved before the
    // contacts in each velocity iteration and after them in each position
    // iteration (island.py:107-148); worlds with joints in the solve take the
    // plain passes (no constraint-chunk pipeline, float64 position cache)
    const int njc = w.H->last_njcons, njcol = w.H->last_njcolours;
    JCons *jc = w.B.s_jc + w.H->jbase;
    const int *joff = w.B.s_joff + w.H->jbase + w.wi;
    gb_joint *JJ = w.B.j + w.H->jbase;
    // 6. warm start and velocity iterations, colour by colour
    // body views: shared memory (world-local index) or the batch arrays
    const bool cached = cache.mem != nullptr;
    vec2<R> *vel = w.B.b_v + w.bb;
    R *om = w.B.b_w + w.bb;
    const R *invm = w.B.b_inv_mass + w.bb;
    const R *invi = w.B.b_inv_I + w.bb;
    const R *stat_ii = nullptr;   // cached inverse inertias, -0 marking a static body
    vec2<double> *pc = w.B.b_c + w.bb;
    double *pa = w.B.b_a + w.bb;
    ChunkPipe pipe{nullptr, nullptr, 0, 0, 0u, 0, 0};
    const int polls = w.B.wait_polls;   // limit of the chunk waits (GB_WAIT_POLLS unless a test lowers it)
    int *pipe_fail = nullptr;   // shared flag: some thread's bounded wait gave up
    if (cached) {
        // layout: c[nb] (16) | a[nb] (8) | inverse mass, inertia (R); a static
        // body's inverse inertia is stored as -0 (its zero inertia changes no
        // sum or product the passes form; the sign marks it as static);
        // the velocity passes keep v[nb], w[nb] in the c/a bytes
        unsigned char *m = cache.mem;
        pc = reinterpret_cast<vec2<double> *>(m);
        pa = reinterpret_cast<double *>(m + 16 * (size_t)nb);
        vel = reinterpret_cast<vec2<R> *>(m);
        om = reinterpret_cast<R *>(m + sizeof(vec2<R>) * (size_t)nb);
        R *im = reinterpret_cast<R *>(m + 24 * (size_t)nb);
        R *ii = im + nb;
        stat_ii = ii;
        invm = im; invi = ii;
        for (int b = rank; b < nb; b += g.size()) {
            vel[b] = w.B.b_v[w.bb + b]; om[b] = w.B.b_w[w.bb + b];
            im[b] = w.B.b_inv_mass[w.bb + b];
            ii[b] = w.btype(b) == GB_BODY_STATIC ? -(R)0 : w.B.b_inv_I[w.bb + b];
        }
        if (cache.nbuf > 0) {
            pipe.buf = m + cache_body_bytes<R>(nb);
            pipe.buf_bytes = chunk_buf_bytes<R>(g.size());
            pipe.nbuf = cache.nbuf;
            pipe.bar = reinterpret_cast<unsigned long long *>(pipe.buf + (size_t)cache.nbuf * pipe.buf_bytes);
            pipe_fail = reinterpret_cast<int *>(pipe.bar + pipe.nbuf);
            if (rank == 0) {
                for (int b = 0; b < pipe.nbuf; ++b) mbar_init(&pipe.bar[b], 1);
                *pipe_fail = 0;
                fence_async_shared();
            }
        }
        g.sync();
    }
    auto is_static = [&](int b) { return stat_ii ? is_neg_zero(stat_ii[b]) : w.btype(b) == GB_BODY_STATIC; };
    bool failed = false;
    if (pipe.nbuf > 0 && ncons > 0 && njc == 0) {
        int *tab = w.B.s_pref + w.cb + 1;   // chunk table (entry -1: its length)
        const int nch = chunk_table(g, coff, ncol, g.size(), tab, w.H->ccap - 1, &w.H->status);
        const int runs = sp.vel_iters + (warm ? 1 : 0);
        const int total = runs * nch;
        const int ahead = pipe.nbuf - 1;
        // The bulk copies bring the read-only part of the records; the
        // impulses, the one part the passes write, are loaded and stored by
        // the thread that owns the record (thread r always solves record r
        // of a chunk), one chunk ahead, so the copies never race with them.
        R imp[4] = {(R)0, (R)0, (R)0, (R)0};
        auto load_imp = [&](int q) {
            const int e = tab[q % nch];
            const int s0 = e & ((1 << 22) - 1), cnt = e >> 22;
            if (rank < cnt) {
                const ConsVel<R> &gr = cv[s0 + rank];
                imp[0] = gr.ni[0]; imp[1] = gr.ni[1]; imp[2] = gr.ti[0]; imp[3] = gr.ti[1];
            }
        };
        pipe.issued = pipe.consumed = 0;
        for (int q = 0; q < ahead && q < total; ++q) { pipe_issue(g, pipe, q, cv, tab, nch); ++pipe.issued; }
        if (total > 0) load_imp(0);
        for (int q = 0; q < total; ++q) {
            if (q + ahead < total) { pipe_issue(g, pipe, q + ahead, cv, tab, nch); ++pipe.issued; }
            const int b = q % pipe.nbuf;
            const bool ok = mbar_wait(&pipe.bar[b], (pipe.parity >> b) & 1u, polls);
            if (ok) { pipe.parity ^= 1u << b; ++pipe.consumed; }
            else *pipe_fail = 1;
            const int e = tab[q % nch];
            const int s0 = e & ((1 << 22) - 1), cnt = e >> 22;
            const bool warm_pass = warm && q < nch;
            if (ok && rank < cnt) {
                const ConsVel<R> &rec = reinterpret_cast<const ConsVel<R> *>(pipe.buf + (size_t)b * pipe.buf_bytes)[rank];
                const int ia = rec.ia, ib = rec.ib;
                Cons<R> k = vel_cons(rec, invm[ia], invm[ib], invi[ia], invi[ib]);
                k.ni[0] = imp[0]; k.ni[1] = imp[1]; k.ti[0] = imp[2]; k.ti[1] = imp[3];
                vec2<R> va = vel[ia], vb = vel[ib];
                R wa = om[ia], wb = om[ib];
                if (warm_pass) warm_start(k, va, wa, vb, wb);
                else {
                    solve_velocity(k, va, wa, vb, wb);
                    ConsVel<R> &gr = cv[s0 + rank];
                    gr.ni[0] = k.ni[0]; gr.ni[1] = k.ni[1]; gr.ti[0] = k.ti[0]; gr.ti[1] = k.ti[1];
                }
                // colour classes share no non-static body; static bodies keep v = 0
                if (!is_neg_zero(stat_ii[ia])) { vel[ia] = va; om[ia] = wa; }
                if (!is_neg_zero(stat_ii[ib])) { vel[ib] = vb; om[ib] = wb; }
            }
            if (q + 1 < total) load_imp(q + 1);   // after this thread's own stores
            g.sync();
            if (*pipe_fail) { failed = true; break; }
        }
    } else if (!failed) {
        // one pass over the joints, colour by colour: 0 = set-up with warm
        // start, 1 = velocity iteration
        const double dt_ratio = w.H->inv_dt0 * dt;
        auto joint_pass = [&](int what) {
            for (int cc = 0; cc < njcol; ++cc) {
                for (int k = joff[cc] + rank; k < joff[cc + 1]; k += g.size()) {
                    JCons &q = jc[k];
                    gb_joint &J = JJ[q.j];
                    const int ia = q.ia, ib = q.ib;
                    vec2<double> va = cvt<double>(vel[ia]), vb = cvt<double>(vel[ib]);
                    double wa = (double)om[ia], wb = (double)om[ib];
                    if (what == 0) {
                        const int ga = w.bb + ia, gbb = w.bb + ib;
                        q.lca = w.B.b_lc[ga]; q.lcb = w.B.b_lc[gbb];
                        q.ma = (double)w.B.b_inv_mass[ga]; q.mb = (double)w.B.b_inv_mass[gbb];
                        q.iA = (double)w.B.b_inv_I[ga]; q.iB = (double)w.B.b_inv_I[gbb];
                        joint_init(J, q, w.B.b_c[ga], w.B.b_a[ga], w.B.b_c[gbb], w.B.b_a[gbb], va, wa, vb, wb, dt, dt_ratio,
                                   w.B.b_mass[gbb], warm);
                    } else {
                        joint_velocity(J, q, va, wa, vb, wb, dt);
                    }
                    if (!is_static(ia)) { vel[ia] = cvt<R>(va); om[ia] = (R)wa; }
                    if (!is_static(ib)) { vel[ib] = cvt<R>(vb); om[ib] = (R)wb; }
                }
                g.sync();
            }
        };
        for (int it = (warm ? -1 : 0); it < sp.vel_iters; ++it) {
            if (it == 0 && njc > 0) joint_pass(0);
            if (it >= 0 && njc > 0) joint_pass(1);
            for (int cc = 0; cc < ncol; ++cc) {
                int s0 = coff[cc], s1 = coff[cc + 1];
                for (int j = s0 + rank; j < s1; j += g.size()) {
                    const ConsVel<R> rec = cv[j];
                    const int ia = rec.ia, ib = rec.ib;
                    Cons<R> k = vel_cons(rec, invm[ia], invm[ib], invi[ia], invi[ib]);
                    vec2<R> va = vel[ia], vb = vel[ib];
                    R wa = om[ia], wb = om[ib];
                    if (it < 0) warm_start(k, va, wa, vb, wb);
                    else {
                        solve_velocity(k, va, wa, vb, wb);
                        cv[j].ni[0] = k.ni[0]; cv[j].ni[1] = k.ni[1];
                        cv[j].ti[0] = k.ti[0]; cv[j].ti[1] = k.ti[1];
                    }
                    if (!is_static(ia)) { vel[ia] = va; om[ia] = wa; }
                    if (!is_static(ib)) { vel[ib] = vb; om[ib] = wb; }
                }
                g.sync();
            }
        }
        if (sp.vel_iters <= 0 && njc > 0) joint_pass(0);   // the set-up runs with no velocity iteration too
    }
    if (failed) {
        if (rank == 0) w.H->status |= GB_ST_WAIT_TIMEOUT;
        pipe_drain(g, pipe);   // the copies still in flight land before the block returns
        return;
    }
    if (cached) {
        for (int b = rank; b < nb; b += g.size()) { w.B.b_v[w.bb + b] = vel[b]; w.B.b_w[w.bb + b] = om[b]; }
        g.sync();
    }
    if (rank == 0) { ck.mark(4); if (ck.acc) ck.acc[10] += ncol; }
    // 7. store impulses (contact.py:801-806); the post-solve report of each
    //    solved contact (island.py:245-252)
    const EvCtx ev{sp.events, sp.step_index, GB_EV_PHASE_SOLVE};
    for (int k = rank; k < ncons; k += g.size()) {
        const ConsVel<R> &v = cv[k];
        const int ci = cpos[k].cidx;
        ContactRec<R> &c = w.con(ci);
        for (int j = 0; j < v.npts && j < c.m.count; ++j) { c.m.ni[j] = v.ni[j]; c.m.ti[j] = v.ti[j]; }
        if (ev.on) record_event<R>(w, ev, GB_EV_POST_SOLVE, ci, ci, v.npts, v.ni, v.ti);
    }
    // 8. integrate positions (island.py:120-138)
    for (int b = rank; b < nb; b += g.size()) {
        if (w.btype(b) == GB_BODY_STATIC || !(rootf[parent[b]] & R_SIM)) continue;
        int gb = w.bb + b;
        vec2<R> v = w.B.b_v[gb];
        R omg = w.B.b_w[gb];
        const R dtr = (R)dt;
        vec2<R> tr = dtr * v;
        if (dot(tr, tr) > (R)GB_MAX_TRANSLATION_SQR) {
            R ratio = (R)GB_MAX_TRANSLATION / len(tr);
            v = ratio * v;
        }
        R rotation = dtr * omg;
        if (sq(rotation) > (R)GB_MAX_ROTATION_SQR) {
            R ratio = (R)GB_MAX_ROTATION / fabs(rotation);
            omg = omg * ratio;
        }
        const vec2<double> cn = w.B.b_c[gb] + cvt<double>(dtr * v);
        const double an = w.B.b_a[gb] + (double)(dtr * omg);
        w.B.b_c[gb] = cn;
        w.B.b_a[gb] = an;
        w.B.b_v[gb] = v; w.B.b_w[gb] = omg;
        // a body whose state stopped being finite (the reference would carry
        // the NaN on, body.py:49-63 only checks arguments): flag the world
        if (!(finite_bits(cn.x) && finite_bits(cn.y) && finite_bits(an) && finite_bits(v.x) && finite_bits(v.y) &&
              finite_bits(omg)))
            atomicOr(&w.H->status, GB_ST_NONFINITE);
    }
    g.sync();
    if (rank == 0) ck.mark(5);
    // 9. position iterations with the per-island early exit (island.py:141-153)
    // float32 batches with the body cache run the passes on float32 deltas
    // (solve_position_f32d): cf | dc | ar | da in the cache's 24 bytes a body
    constexpr bool F32D = std::is_same<R, float>::value;
    const bool f32d = F32D && cached && njc == 0;   // joints take the float64 position cache
    vec2<float> *cf = nullptr, *dcv = nullptr;
    float *ar = nullptr, *dav = nullptr;
    if (cached) {
        if (f32d) {
            unsigned char *m = cache.mem;
            cf = reinterpret_cast<vec2<float> *>(m);
            dcv = reinterpret_cast<vec2<float> *>(m + 8 * (size_t)nb);
            ar = reinterpret_cast<float *>(m + 16 * (size_t)nb);
            dav = reinterpret_cast<float *>(m + 20 * (size_t)nb);
            for (int b = rank; b < nb; b += g.size()) {
                cf[b] = cvt<float>(w.B.b_c[w.bb + b]);
                ar[b] = angle_f32(w.B.b_a[w.bb + b]);
                dcv[b] = mk<float>(0.0f, 0.0f);
                dav[b] = 0.0f;
            }
        } else {
            for (int b = rank; b < nb; b += g.size()) { pc[b] = w.B.b_c[w.bb + b]; pa[b] = w.B.b_a[w.bb + b]; }
        }
        g.sync();
    }
    auto pos_one = [&](const ConsPos<R> &rec) {
        if (rootf[rec.root] & R_DONE) return;
        const int ia = rec.ia, ib = rec.ib;
        Cons<R> k = pos_cons(rec, invm[ia], invm[ib], invi[ia], invi[ib]);
        if constexpr (F32D) {
            if (f32d) {
                vec2<float> dca = dcv[ia], dcb = dcv[ib];
                float daa = dav[ia], dab = dav[ib];
                const float ms = solve_position_f32d(k, cf[ia], ar[ia], dca, daa, cf[ib], ar[ib], dcb, dab, 0.0f);
                atomicMin(&minsep[rec.root], dkey((double)ms));
                if (!is_static(ia)) { dcv[ia] = dca; dav[ia] = daa; }
                if (!is_static(ib)) { dcv[ib] = dcb; dav[ib] = dab; }
                return;
            }
        }
        vec2<double> ca = pc[ia], cb = pc[ib];
        double aa = pa[ia], ab = pa[ib];
        double ms = solve_position(k, ca, aa, cb, ab, 0.0, false, false, false);
        atomicMin(&minsep[rec.root], dkey(ms));
        if (!is_static(ia)) { pc[ia] = ca; pa[ia] = aa; }
        if (!is_static(ib)) { pc[ib] = cb; pa[ib] = ab; }
    };
    // island early exit; bits 8-15 of the root's flags keep the number of
    // iterations the island ran (the step record)
    auto pos_check = [&](int it) {
        bool pending = false;
        for (int b = rank; b < nb; b += g.size()) {
            if (parent[b] != b || !(rootf[b] & R_SIM) || (rootf[b] & R_DONE)) continue;
            if (w.btype(b) == GB_BODY_STATIC) continue;
            if (dkey_inv(minsep[b]) >= -3.0 * GB_LINEAR_SLOP && !(rootf[b] & R_JBAD))
                rootf[b] |= R_DONE | R_SOLVED | ((uint32_t)(it + 1) << 8);
            else pending = true;
        }
        return g.any(pending);
    };
    // the joints' position pass after the contacts', colour by colour; a
    // joint out of tolerance keeps its island iterating (island.py:145-153)
    auto joint_pos_pass = [&]() {
        for (int cc = 0; cc < njcol; ++cc) {
            for (int k = joff[cc] + rank; k < joff[cc + 1]; k += g.size()) {
                const JCons &q = jc[k];
                if (rootf[q.root] & R_DONE) continue;
                const int ia = q.ia, ib = q.ib;
                vec2<double> ca = pc[ia], cb = pc[ib];
                double aa = pa[ia], ab = pa[ib];
                if (!joint_position(JJ[q.j], q, ca, aa, cb, ab)) atomicOr(&rootf[q.root], R_JBAD);
                if (!is_static(ia)) { pc[ia] = ca; pa[ia] = aa; }
                if (!is_static(ib)) { pc[ib] = cb; pa[ib] = ab; }
            }
            g.sync();
        }
    };
    if (pipe.nbuf > 0 && ncons > 0 && sp.pos_iters > 0 && njc == 0) {
        int *tab = w.B.s_pref + w.cb + 1;
        const int nch = tab[-1];
        const int total = sp.pos_iters * nch;
        const int ahead = pipe.nbuf - 1;
        pipe.issued = pipe.consumed = 0;
        for (; pipe.issued < ahead && pipe.issued < total; ++pipe.issued) pipe_issue(g, pipe, pipe.issued, cpos, tab, nch);
        int q = 0;
        for (int it = 0; it < sp.pos_iters && !failed; ++it) {
            for (int b = rank; b < nb; b += g.size()) minsep[b] = dkey(0.0);
            g.sync();
            for (int j = 0; j < nch; ++j, ++q) {
                if (pipe.issued < total && pipe.issued <= q + ahead) {
                    pipe_issue(g, pipe, pipe.issued, cpos, tab, nch);
                    ++pipe.issued;
                }
                const int b = q % pipe.nbuf;
                const bool ok = mbar_wait(&pipe.bar[b], (pipe.parity >> b) & 1u, polls);
                if (ok) { pipe.parity ^= 1u << b; ++pipe.consumed; }
                else *pipe_fail = 1;
                const int e = tab[j];
                const int cnt = e >> 22;
                if (ok && rank < cnt) pos_one(reinterpret_cast<const ConsPos<R> *>(pipe.buf + (size_t)b * pipe.buf_bytes)[rank]);
                g.sync();
                if (*pipe_fail) { failed = true; break; }
            }
            if (failed) break;
            if (!pos_check(it)) break;
        }
        // the chunks issued past an early exit or a wait that gave up
        if (!pipe_drain(g, pipe)) failed = true;
        if (failed) {
            if (rank == 0) w.H->status |= GB_ST_WAIT_TIMEOUT;
            g.sync();
            return;
        }
    } else {
        for (int it = 0; it < sp.pos_iters; ++it) {
            for (int b = rank; b < nb; b += g.size()) {
                minsep[b] = dkey(0.0);
                if (njc > 0 && parent[b] == b) rootf[b] &= ~R_JBAD;
            }
            g.sync();
            for (int cc = 0; cc < ncol; ++cc) {
                int s0 = coff[cc], s1 = coff[cc + 1];
                for (int j = s0 + rank; j < s1; j += g.size()) {
                    const ConsPos<R> rec = cpos[j];
                    pos_one(rec);
                }
                g.sync();
            }
            if (njc > 0) joint_pos_pass();
            if (!pos_check(it)) break;
        }
    }
    g.sync();
    if (sp.record_order)   // step record: position iterations of each body's island
        for (int b = rank; b < nb; b += g.size()) {
            if (w.btype(b) == GB_BODY_STATIC || !(rootf[parent[b]] & R_SIM)) continue;
            const uint32_t rf = rootf[parent[b]];
            const int its = (rf & R_DONE) ? (int)((rf >> 8) & 0xffu) : sp.pos_iters;
            w.B.rec[w.bb + b] = (w.B.rec[w.bb + b] & ~0xff) | (its > 255 ? 255 : its);
            w.B.rec_island[w.bb + b] = parent[b];
        }
    if (cached) {
        if (f32d) {
            for (int b = rank; b < nb; b += g.size()) {
                const vec2<float> d = dcv[b];
                const float e = dav[b];
                if (d.x == 0.0f && d.y == 0.0f && e == 0.0f) continue;
                vec2<double> c = w.B.b_c[w.bb + b];
                if (d.x != 0.0f) c.x = c.x + (double)d.x;
                if (d.y != 0.0f) c.y = c.y + (double)d.y;
                w.B.b_c[w.bb + b] = c;
                if (e != 0.0f) w.B.b_a[w.bb + b] = w.B.b_a[w.bb + b] + (double)e;
            }
        } else {
            for (int b = rank; b < nb; b += g.size()) { w.B.b_c[w.bb + b] = pc[b]; w.B.b_a[w.bb + b] = pa[b]; }
        }
        g.sync();
    }
    if (rank == 0) ck.mark(6);
    // 10. write back the transforms of the island bodies (island.py:156-159)
    for (int b = rank; b < nb; b += g.size()) {
        if (w.btype(b) == GB_BODY_STATIC || !(rootf[parent[b]] & R_SIM)) continue;
        sync_transform(w, b);
    }
    g.sync();
}

// island.py:163-179 sleep, including the depth-first order where the
// reference's result depends on it.
template <class R, class G> __device__ void sleep_group(const G &g, const WView<R> &w, const StepParams &sp) {
    const int nb = w.H->nb, nc = w.H->nc, nf = w.H->nf;
    int *parent = w.B.s_parent + w.bb;
    uint32_t *rootf = w.B.s_root + w.bb;
    int *seed = w.B.s_seed + w.bb;
    unsigned long long *minsep = w.B.s_minsep + w.bb;
    unsigned long long *minsleep = w.B.s_minsleep + w.bb;
    unsigned long long *claim = w.B.s_claim + w.bb;
    int *cons_of = w.B.s_cons_of + w.cb;
    int *colour = w.B.s_colour + w.cb;
    int *order = w.B.s_order + w.cb;
    int *pref = w.B.s_pref + w.cb;
    Cons<R> *cons = w.B.s_cons + w.cb;
    int *coff = w.B.s_proc + w.cb;
    const double dt = sp.dt;
    const bool warm = (w.H->flags & GB_W_WARM_STARTING) != 0;
    (void)nb; (void)nc; (void)nf; (void)parent; (void)rootf; (void)seed; (void)minsep; (void)minsleep; (void)claim;
    (void)cons_of; (void)colour; (void)order; (void)pref; (void)cons; (void)coff; (void)dt; (void)warm;
    // 11. sleep (island.py:163-179)
    if (w.H->flags & GB_W_ALLOW_SLEEP) {
        bool need_dfs_all = !w.H->all_allow;
        for (int b = g.rank(); b < nb; b += g.size()) {
            if (w.btype(b) == GB_BODY_STATIC || !(rootf[parent[b]] & R_SIM)) continue;
            int gb = w.bb + b;
            R om = w.B.b_w[gb];
            vec2<R> v = w.B.b_v[gb];
            bool moving = sq(om) > (R)GB_ANGULAR_SLEEP_TOL_SQR || len2(v) > (R)GB_LINEAR_SLEEP_TOL_SQR;
            if (!need_dfs_all) {
                if (moving) { w.B.b_sleep[gb] = 0.0; atomicMin(&minsleep[parent[b]], 0ull); }
                else {
                    double st = w.B.b_sleep[gb] + dt;
                    w.B.b_sleep[gb] = st;
                    atomicMin(&minsleep[parent[b]], (unsigned long long)__double_as_longlong(st));
                }
            }
        }
        g.sync();
        // islands that may fall asleep need the depth-first order
        bool want = false;
        for (int b = g.rank(); b < nb; b += g.size()) {
            if (parent[b] != b || w.btype(b) == GB_BODY_STATIC || !(rootf[b] & R_SIM)) continue;
            bool cand = need_dfs_all || (__longlong_as_double((long long)minsleep[b]) >= GB_TIME_TO_SLEEP && (rootf[b] & R_SOLVED));
            if (cand) { rootf[b] |= R_DFS; want = true; }
        }
        want = g.any(want);
        if (want) {
            // adjacency of every body in contact-list order (Body._contacts)
            int *off = w.B.s_adjoff + w.bb + w.wi;
            int *adj = w.B.s_adj + 2 * w.cb;
            int *deg = w.B.s_stack + w.bb;
            for (int b = g.rank(); b < nb; b += g.size()) deg[b] = 0;
            g.sync();
            for (int i = g.rank(); i < nc; i += g.size()) {
                const ContactRec<R> &c = w.con(i);
                if (!qualifies(w, c)) continue;
                atomicAdd(&deg[w.fbody(c.fa)], 1);
                atomicAdd(&deg[w.fbody(c.fb)], 1);
            }
            g.sync();
            int tot = group_scan(g, nb, [&](int b) { return deg[b]; }, off);
            if (g.rank() == 0) off[nb] = tot;
            g.sync();
            for (int b = g.rank(); b < nb; b += g.size()) deg[b] = off[b];
            g.sync();
            for (int i = g.rank(); i < nc; i += g.size()) {
                const ContactRec<R> &c = w.con(i);
                if (!qualifies(w, c)) continue;
                adj[atomicAdd(&deg[w.fbody(c.fa)], 1)] = i;
                adj[atomicAdd(&deg[w.fbody(c.fb)], 1)] = i;
            }
            g.sync();
            for (int b = g.rank(); b < nb; b += g.size()) {
                for (int e = off[b] + 1; e < off[b + 1]; ++e) {   // insertion sort by contact index
                    int v = adj[e], j = e - 1;
                    while (j >= off[b] && adj[j] > v) { adj[j + 1] = adj[j]; --j; }
                    adj[j + 1] = v;
                }
                w.B.s_bvis[w.bb + b] = 0;
            }
            for (int i = g.rank(); i < nc; i += g.size()) w.B.s_cvis[w.cb + i] = 0;
            for (int j = g.rank(); j < w.H->nj; j += g.size()) w.B.s_jvis[w.H->jbase + j] = 0;
            g.sync();
            if (g.rank() == 0) {
                unsigned char *bvis = w.B.s_bvis + w.bb;
                for (int r = 0; r < nb; ++r) {
                    if (parent[r] != r || !(rootf[r] & R_DFS)) continue;
                    int last, last_ns;
                    island_dfs(w, seed[r], &last, &last_ns);
                    // static bodies may belong to several islands: clear all marks
                    for (int b = 0; b < nb; ++b) if (w.btype(b) == GB_BODY_STATIC) bvis[b] = 0;
                    if (need_dfs_all) {
                        bool allow_last = (w.B.b_flags[w.bb + last] & GB_BODY_ALLOW_SLEEP) != 0;
                        unsigned long long ms = ~0ull;
                        for (int b = 0; b < nb; ++b) {
                            if (parent[b] != r || w.btype(b) == GB_BODY_STATIC) continue;
                            int gb = w.bb + b;
                            bool moving = sq(w.B.b_w[gb]) > (R)GB_ANGULAR_SLEEP_TOL_SQR || len2(w.B.b_v[gb]) > (R)GB_LINEAR_SLEEP_TOL_SQR;
                            if (!allow_last || moving) { w.B.b_sleep[gb] = 0.0; ms = 0ull; }
                            else {
                                double st = w.B.b_sleep[gb] + dt;
                                w.B.b_sleep[gb] = st;
                                unsigned long long k = (unsigned long long)__double_as_longlong(st);
                                if (k < ms) ms = k;
                            }
                        }
                        minsleep[r] = ms;
                    }
                    if (__longlong_as_double((long long)minsleep[r]) >= GB_TIME_TO_SLEEP && (rootf[r] & R_SOLVED) && last_ns >= 0)
                        sleep_body(w, last_ns);
                }
            }
            g.sync();
        }
    }
}

// world.py:582-592: fixture sync of island bodies, move buffer in fixture
// order, pair finding.
template <class R, class G> __device__ void sync_pairs_group(const G &g, const WView<R> &w, const StepParams &sp, WShared *sh) {
    const int nb = w.H->nb, nc = w.H->nc, nf = w.H->nf;
    int *parent = w.B.s_parent + w.bb;
    uint32_t *rootf = w.B.s_root + w.bb;
    int *seed = w.B.s_seed + w.bb;
    unsigned long long *minsep = w.B.s_minsep + w.bb;
    unsigned long long *minsleep = w.B.s_minsleep + w.bb;
    unsigned long long *claim = w.B.s_claim + w.bb;
    int *cons_of = w.B.s_cons_of + w.cb;
    int *colour = w.B.s_colour + w.cb;
    int *order = w.B.s_order + w.cb;
    int *pref = w.B.s_pref + w.cb;
    Cons<R> *cons = w.B.s_cons + w.cb;
    int *coff = w.B.s_proc + w.cb;
    const double dt = sp.dt;
    const bool warm = (w.H->flags & GB_W_WARM_STARTING) != 0;
    (void)nb; (void)nc; (void)nf; (void)parent; (void)rootf; (void)seed; (void)minsep; (void)minsleep; (void)claim;
    (void)cons_of; (void)colour; (void)order; (void)pref; (void)cons; (void)coff; (void)dt; (void)warm;
    // 12. synchronise fixtures of island bodies; the move buffer is the
    //     re-fattened proxies in body order = fixture order (world.py:584-589)
    int *mv = w.B.s_move + w.fb;
    int *mflag = w.B.s_first + w.fb;
    for (int f = g.rank(); f < nf; f += g.size()) {
        int b = w.fbody(f);
        bool moved = false;
        if (w.btype(b) != GB_BODY_STATIC && (rootf[parent[b]] & R_SIM)) moved = sync_fixture(w, f);
        mflag[f] = moved ? 1 : 0;
    }
    g.sync();
    int nmove = group_scan(g, nf, [&](int f) { return mflag[f]; }, w.B.s_cnt + w.fb);
    g.sync();
    for (int f = g.rank(); f < nf; f += g.size())
        if (mflag[f]) mv[w.B.s_cnt[w.fb + f]] = f;
    if (g.rank() == 0) sh->nmove = nmove;
    g.sync();
    find_new_contacts(g, w, sh);
}

template <class R, class G> __device__ void world_solve(const G &g, const WView<R> &w, const StepParams &sp, WShared *sh,
                                                        PhaseClock &pc) {
    if (w.H->nctl) controllers_group(g, w);
    islands_group(g, w, sp);
    if (g.rank() == 0) pc.mark(2);
    constraints_group(g, w, sp);
    if (g.rank() == 0) pc.mark(3);
    for (int b = g.rank(); b < w.H->nb; b += g.size()) integrate_velocity_body(w, b, sp.dt);
    g.sync();
    for (int k = g.rank(); k < w.H->last_ncons; k += g.size()) init_constraint(w, k, sp);
    g.sync();
    if (g.rank() == 0) pc.mark(4);
    solve_group(g, w, sp);
    if (g.rank() == 0) pc.mark(6);
    sleep_group(g, w, sp);
    if (g.rank() == 0) pc.mark(7);
    sync_pairs_group(g, w, sp, sh);
    if (g.rank() == 0) pc.mark(8);
}

// gb_toi_f32.cuh -- the float32 unit's time of impact (toi.py:216-391) and
// GJK distance (distance.py:424-561): the algorithm of the float64
// functions in gb_collide.cuh, step for step, in float32 arithmetic on
// sweeps relative to sweep A's start position.  The separations the root
// finder compares with its tolerance (a quarter of the linear slop,
// 1.25e-3 m) are then good to ~1e-7 m wherever the bodies are, while
// GB300 issues float64 arithmetic at a small fraction of the float32 rate.
// The float64 unit keeps the float64 functions (bit-exact with the CPU
// restatement).
#pragma once
#include "gb_collide.cuh"

struct FProxy { vec2<float> v[GB_MAX_POLY_VERTS]; int count; float radius; };

template <class R> __device__ void fproxy_init(FProxy &p, const Shape<R> &s) {
    int n = (s.type == GB_SHAPE_CIRCLE) ? 1 : (s.type == GB_SHAPE_POLYGON ? s.count : 2);
    for (int i = 0; i < n; ++i) p.v[i] = mk<float>((float)s.v[i].x, (float)s.v[i].y);
    p.count = n;
    p.radius = (float)s.radius;
}
static __device__ __forceinline__ int fsupport(const FProxy &p, vec2<float> d) {
    int best = 0;
    float bd = 0;
    for (int i = 0; i < p.count; ++i) {
        float x = dot(p.v[i], d);
        if (i == 0 || x > bd) { bd = x; best = i; }
    }
    return best;
}

struct FCache { float metric; int count; int ia[3], ib[3]; };
struct FVert { vec2<float> wa, wb, w; float a; int ia, ib; };

// The reference simplex rebinds _v1/_v2 to copies in solve2/solve3 while new
// support points are written into the three objects captured at the start
// of fshape_distance (distance.py:469, 524-531); orig[] are those objects,
// r1o/r2o tell whether _v1/_v2 still refer to them.
struct FSimplex {
    FVert orig[3];
    FVert d1, d2;
    int r1o, r2o, count;
    __device__ FVert &v1() { return r1o ? orig[0] : d1; }
    __device__ FVert &v2() { return r2o ? orig[1] : d2; }
    __device__ FVert &v3() { return orig[2]; }
    __device__ FVert &vk(int k) { return k == 0 ? v1() : (k == 1 ? v2() : v3()); }
};

static __device__ float fsimplex_metric(FSimplex &s) {
    if (s.count == 1) return 0.0f;
    if (s.count == 2) return len(s.v1().w - s.v2().w);
    return cross(s.v2().w - s.v1().w, s.v3().w - s.v1().w);
}

static __device__ void fsimplex_solve2(FSimplex &s) {
    vec2<float> w1 = s.v1().w, w2 = s.v2().w;
    vec2<float> e12 = w2 - w1;
    float d12_2 = -dot(w1, e12);
    if (d12_2 <= 0.0f) { s.v1().a = 1.0f; s.count = 1; return; }
    float d12_1 = dot(w2, e12);
    if (d12_1 <= 0.0f) { s.v2().a = 1.0f; s.count = 1; s.d1 = s.v2(); s.r1o = 0; return; }
    float inv = 1.0f / (d12_1 + d12_2);
    s.v1().a = d12_1 * inv;
    s.v2().a = d12_2 * inv;
    s.count = 2;
}

static __device__ void fsimplex_solve3(FSimplex &s) {
    vec2<float> w1 = s.v1().w, w2 = s.v2().w, w3 = s.v3().w;
    vec2<float> e12 = w2 - w1;
    float d12_1 = dot(w2, e12), d12_2 = -dot(w1, e12);
    vec2<float> e13 = w3 - w1;
    float d13_1 = dot(w3, e13), d13_2 = -dot(w1, e13);
    vec2<float> e23 = w3 - w2;
    float d23_1 = dot(w3, e23), d23_2 = -dot(w2, e23);
    float n123 = cross(e12, e13);
    float d123_1 = n123 * cross(w2, w3);
    float d123_2 = n123 * cross(w3, w1);
    float d123_3 = n123 * cross(w1, w2);
    if (d12_2 <= 0.0f && d13_2 <= 0.0f) { s.v1().a = 1.0f; s.count = 1; return; }
    if (d12_1 > 0.0f && d12_2 > 0.0f && d123_3 <= 0.0f) {
        float inv = 1.0f / (d12_1 + d12_2);
        s.v1().a = d12_1 * inv; s.v2().a = d12_2 * inv; s.count = 2; return;
    }
    if (d13_1 > 0.0f && d13_2 > 0.0f && d123_2 <= 0.0f) {
        float inv = 1.0f / (d13_1 + d13_2);
        s.v1().a = d13_1 * inv; s.v3().a = d13_2 * inv; s.count = 2;
        s.d2 = s.v3(); s.r2o = 0; return;
    }
    if (d12_1 <= 0.0f && d23_2 <= 0.0f) { s.v2().a = 1.0f; s.count = 1; s.d1 = s.v2(); s.r1o = 0; return; }
    if (d13_1 <= 0.0f && d23_1 <= 0.0f) { s.v3().a = 1.0f; s.count = 1; s.d1 = s.v3(); s.r1o = 0; return; }
    if (d23_1 > 0.0f && d23_2 > 0.0f && d123_1 <= 0.0f) {
        float inv = 1.0f / (d23_1 + d23_2);
        s.v2().a = d23_1 * inv; s.v3().a = d23_2 * inv; s.count = 2;
        s.d1 = s.v3(); s.r1o = 0; return;
    }
    float inv = 1.0f / (d123_1 + d123_2 + d123_3);
    s.v1().a = d123_1 * inv; s.v2().a = d123_2 * inv; s.v3().a = d123_3 * inv;
    s.count = 3;
}

// distance.py:424-561 fshape_distance
static __device__ float fshape_distance(const FProxy &A, const FProxy &B, xform2<float> xa, xform2<float> xb, bool use_radii, FCache &cache) {
    FSimplex s;
    s.r1o = 1; s.r2o = 1;
    s.count = cache.count;
    for (int i = 0; i < s.count; ++i) {
        FVert &v = s.orig[i];
        v.ia = cache.ia[i]; v.ib = cache.ib[i];
        v.wa = xmul(xa, A.v[v.ia]); v.wb = xmul(xb, B.v[v.ib]);
        v.w = v.wb - v.wa; v.a = 0.0f;
    }
    for (int i = s.count; i < 3; ++i) { s.orig[i].a = 0.0f; s.orig[i].ia = 0; s.orig[i].ib = 0; }
    if (s.count > 1) {
        float m1 = cache.metric, m2 = fsimplex_metric(s);
        if (m2 < 0.5f * m1 || 2.0f * m1 < m2 || m2 < (float)GB_EPSILON) s.count = 0;
    }
    if (s.count == 0) {
        FVert &v = s.orig[0];
        v.ia = 0; v.ib = 0;
        v.wa = xmul(xa, A.v[0]); v.wb = xmul(xb, B.v[0]);
        v.w = v.wb - v.wa;
        s.count = 1;
    }
    int save_ia[3], save_ib[3], save_n;
    for (int iter = 0; iter < 20;) {
        save_n = s.count;
        for (int i = 0; i < s.count; ++i) { save_ia[i] = s.vk(i).ia; save_ib[i] = s.vk(i).ib; }
        if (s.count == 2) fsimplex_solve2(s);
        else if (s.count == 3) { fsimplex_solve3(s); break; }
        vec2<float> d;
        if (s.count == 1) d = -s.v1().w;
        else {
            vec2<float> e12 = s.v2().w - s.v1().w;
            float sgn = cross(e12, -s.v1().w);
            d = (sgn > 0.0f) ? cross(1.0f, e12) : cross(e12, 1.0f);
        }
        if (len2(d) < (float)GB_EPSILON_SQR) break;
        FVert &vx = s.orig[s.count];
        vx.ia = fsupport(A, rmul_t(xa.q, -d));
        vx.wa = xmul(xa, A.v[vx.ia]);
        vx.ib = fsupport(B, rmul_t(xb.q, d));
        vx.wb = xmul(xb, B.v[vx.ib]);
        vx.w = vx.wb - vx.wa;
        ++iter;
        bool dup = false;
        for (int i = 0; i < save_n; ++i) if (save_ia[i] == vx.ia && save_ib[i] == vx.ib) { dup = true; break; }
        if (dup) break;
        s.count += 1;
    }
    vec2<float> pa, pb;
    if (s.count == 1) { pa = s.v1().wa; pb = s.v1().wb; }
    else if (s.count == 2) {
        pa = s.v1().a * s.v1().wa + s.v2().a * s.v2().wa;
        pb = s.v1().a * s.v1().wb + s.v2().a * s.v2().wb;
    } else {
        pa = (s.v1().a * s.v1().wa + s.v2().a * s.v2().wa) + s.v3().a * s.v3().wa;
        pb = pa;
    }
    float dist = len(pa - pb);
    cache.metric = fsimplex_metric(s);
    cache.count = s.count;
    for (int i = 0; i < s.count; ++i) { cache.ia[i] = s.vk(i).ia; cache.ib[i] = s.vk(i).ib; }
    if (use_radii) {
        float ra = A.radius, rb = B.radius;
        if (dist > ra + rb && dist > (float)GB_EPSILON) dist -= ra + rb;
        else dist = 0.0f;
    }
    return dist;
}

// ------------------------------------------------------------------
// common.py:870-923 Sweep in float32 relative form: centres relative to an
// origin (sweep A's start position; the float64 differences rounded once),
// the start angle reduced to [-pi, pi] and the angle swept.  The pose at
// beta is the reference's (1 - beta) * start + beta * end.
struct FSweep {
    vec2<float> lc, c0, c;
    float a0, da;
};
static __device__ __forceinline__ FSweep fsweep_of(const Sweep &s, vec2<double> origin) {
    FSweep f;
    f.lc = cvt<float>(s.lc);
    f.c0 = cvt<float>(s.c0 - origin);
    f.c = cvt<float>(s.c - origin);
    f.a0 = angle_f32(s.a0);
    f.da = (float)(s.a - s.a0);
    return f;
}
static __device__ __forceinline__ xform2<float> fsweep_xf(const FSweep &sw, float beta) {
    xform2<float> x;
    x.p = (1.0f - beta) * sw.c0 + beta * sw.c;
    x.q = rot_f32(sw.a0 + beta * sw.da);
    x.p = x.p - rmul(x.q, sw.lc);
    return x;
}

struct FSepFn {
    const FProxy *A, *B;
    FSweep sa, sb;
    int type;
    vec2<float> axis, lp;
};

// toi.py:53-123 (the POINTS axis stays unnormalised, as in the reference)
static __device__ void fsep_init(FSepFn &f, const FCache &c, float t1) {
    xform2<float> xa = fsweep_xf(f.sa, t1), xb = fsweep_xf(f.sb, t1);
    int ia0 = c.ia[0], ib0 = c.ib[0];
    if (c.count == 1) {
        f.type = SF_POINTS;
        f.axis = xmul(xb, f.B->v[ib0]) - xmul(xa, f.A->v[ia0]);
        return;
    }
    int ia1 = c.ia[1], ib1 = c.ib[1];
    if (ia0 == ia1) {
        f.type = SF_FACE_B;
        vec2<float> lb1 = f.B->v[ib0], lb2 = f.B->v[ib1];
        f.axis = normalized(cross(lb2 - lb1, 1.0f));
        vec2<float> normal = rmul(xb.q, f.axis);
        f.lp = 0.5f * (lb1 + lb2);
        vec2<float> pb = xmul(xb, f.lp), pa = xmul(xa, f.A->v[ia0]);
        if (dot(pa - pb, normal) < 0.0f) f.axis = -f.axis;
    } else {
        f.type = SF_FACE_A;
        vec2<float> la1 = f.A->v[ia0], la2 = f.A->v[ia1];
        f.axis = normalized(cross(la2 - la1, 1.0f));
        vec2<float> normal = rmul(xa.q, f.axis);
        f.lp = 0.5f * (la1 + la2);
        vec2<float> pa = xmul(xa, f.lp), pb = xmul(xb, f.B->v[ib0]);
        if (dot(pb - pa, normal) < 0.0f) f.axis = -f.axis;
    }
}

static __device__ float fsep_find_min(FSepFn &f, float t, int *ia, int *ib) {
    xform2<float> xa = fsweep_xf(f.sa, t), xb = fsweep_xf(f.sb, t);
    if (f.type == SF_POINTS) {
        *ia = fsupport(*f.A, rmul_t(xa.q, f.axis));
        *ib = fsupport(*f.B, rmul_t(xb.q, -f.axis));
        return dot(xmul(xb, f.B->v[*ib]) - xmul(xa, f.A->v[*ia]), f.axis);
    } else if (f.type == SF_FACE_A) {
        vec2<float> normal = rmul(xa.q, f.axis);
        vec2<float> pa = xmul(xa, f.lp);
        *ia = -1;
        *ib = fsupport(*f.B, rmul_t(xb.q, -normal));
        return dot(xmul(xb, f.B->v[*ib]) - pa, normal);
    } else {
        vec2<float> normal = rmul(xb.q, f.axis);
        vec2<float> pb = xmul(xb, f.lp);
        *ib = -1;
        *ia = fsupport(*f.A, rmul_t(xa.q, -normal));
        return dot(xmul(xa, f.A->v[*ia]) - pb, normal);
    }
}

static __device__ float fsep_eval(FSepFn &f, int ia, int ib, float t) {
    xform2<float> xa = fsweep_xf(f.sa, t), xb = fsweep_xf(f.sb, t);
    if (f.type == SF_POINTS) return dot(xmul(xb, f.B->v[ib]) - xmul(xa, f.A->v[ia]), f.axis);
    if (f.type == SF_FACE_A) {
        vec2<float> normal = rmul(xa.q, f.axis);
        return dot(xmul(xb, f.B->v[ib]) - xmul(xa, f.lp), normal);
    }
    vec2<float> normal = rmul(xb.q, f.axis);
    return dot(xmul(xa, f.A->v[ia]) - xmul(xb, f.lp), normal);
}

// toi.py:216-391.  The reference's push-back loop is unbounded; here it
// stops after 1000 rounds with FAILED and sets *limit_hit.
static __device__ int time_of_impact_f32(const FProxy &A, const FProxy &B, const FSweep &swa, const FSweep &swb, float t_max,
                              float *t_out, bool *limit_hit) {
    int state = 0;
    float out_t = t_max;
    FSepFn f;
    f.A = &A; f.B = &B; f.sa = swa; f.sb = swb;
    float total_radius = A.radius + B.radius;
    float target = pymax((float)GB_LINEAR_SLOP, total_radius - 3.0f * (float)GB_LINEAR_SLOP);
    float tol = 0.25f * (float)GB_LINEAR_SLOP;
    float t1 = 0.0f;
    int iter = 0;
    FCache cache;
    cache.metric = 0.0f; cache.count = 0;
    for (int i = 0; i < 3; ++i) { cache.ia[i] = 0; cache.ib[i] = 0; }
    for (;;) {
        xform2<float> xa = fsweep_xf(f.sa, t1), xb = fsweep_xf(f.sb, t1);
        float dist = fshape_distance(A, B, xa, xb, false, cache);
        if (dist <= 0.0f) { state = TOI_OVERLAPPED; out_t = 0.0f; break; }
        if (dist < target + tol) { state = TOI_TOUCHING; out_t = t1; break; }
        fsep_init(f, cache, t1);
        bool done = false;
        float t2 = t_max;
        int push_back = 0;
        for (;;) {
            int ia, ib;
            float s2 = fsep_find_min(f, t2, &ia, &ib);
            if (s2 > target + tol) { state = TOI_SEPARATED; out_t = t_max; done = true; break; }
            if (s2 > target - tol) { t1 = t2; break; }
            float s1 = fsep_eval(f, ia, ib, t1);
            if (s1 < target - tol) { state = TOI_FAILED; out_t = t1; done = true; break; }
            if (s1 <= target + tol) { state = TOI_TOUCHING; out_t = t1; done = true; break; }
            int root_iter = 0;
            float a1 = t1, a2 = t2;
            for (;;) {
                float t;
                if (root_iter & 1) t = a1 + (target - s1) * (a2 - a1) / (s2 - s1);
                else t = 0.5f * (a1 + a2);
                float s = fsep_eval(f, ia, ib, t);
                if (fabsf(s - target) < tol) { t2 = t; break; }
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

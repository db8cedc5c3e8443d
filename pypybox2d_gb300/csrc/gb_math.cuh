// gb_math.cuh -- 2-D algebra of the world-step kernels.
//
// Every operation keeps the operation order of pypybox2d's C extension
// `_common` (pypybox2d/src/vec2module.c, mat22module.c, transform.c,
// aabbmodule.c): with R = double and no FMA contraction (the float64
// translation unit is compiled with -fmad=false) the kernels produce the
// reference's doubles bit for bit, apart from cos/sin, which come from the
// portable sincos below, and `x**2`, which is x*x.
#pragma once
#include <cstdint>
#include <cmath>

#define GB_HD __host__ __device__ __forceinline__

template <class R> struct vec2 { R x, y; };

template <class R> GB_HD vec2<R> mk(R x, R y) { vec2<R> r; r.x = x; r.y = y; return r; }
template <class R> GB_HD vec2<R> operator+(vec2<R> a, vec2<R> b) { return mk<R>(a.x + b.x, a.y + b.y); }
template <class R> GB_HD vec2<R> operator-(vec2<R> a, vec2<R> b) { return mk<R>(a.x - b.x, a.y - b.y); }
template <class R> GB_HD vec2<R> operator-(vec2<R> a) { return mk<R>(-a.x, -a.y); }
// Vec2_mul with a float operand
template <class R> GB_HD vec2<R> operator*(R s, vec2<R> a) { return mk<R>(s * a.x, s * a.y); }
template <class R> GB_HD R dot(vec2<R> a, vec2<R> b) { return a.x * b.x + a.y * b.y; }
template <class R> GB_HD R cross(vec2<R> a, vec2<R> b) { return a.x * b.y - a.y * b.x; }
// Vec2_cross(float): (s * y, -s * x)
template <class R> GB_HD vec2<R> cross(vec2<R> a, R s) { return mk<R>(s * a.y, -s * a.x); }
// scalar_cross(s, v): (-s * y, s * x)
template <class R> GB_HD vec2<R> cross(R s, vec2<R> a) { return mk<R>(-s * a.y, s * a.x); }
template <class R> GB_HD R len2(vec2<R> a) { return a.x * a.x + a.y * a.y; }
template <class R> GB_HD R len(vec2<R> a) { return sqrt(a.x * a.x + a.y * a.y); }
// Vec2_normalized: unchanged below FLT_EPSILON
template <class R> GB_HD vec2<R> normalized(vec2<R> a) {
    R l = sqrt(a.x * a.x + a.y * a.y);
    if (l < (R)1.1920928955078125e-07) return a;
    R inv = (R)1 / l;
    return mk<R>(a.x * inv, a.y * inv);
}
template <class T, class R> GB_HD vec2<T> cvt(vec2<R> a) { return mk<T>((T)a.x, (T)a.y); }

// rotation col1 = (c, s), col2 = (-s, c)
template <class R> struct rot2 { R c, s; };
// axis-aligned box: lower (lx, ly), upper (ux, uy)
struct __align__(16) dbox { double x, y, z, w; };
static GB_HD dbox mkbox(double lx, double ly, double ux, double uy) { dbox b; b.x = lx; b.y = ly; b.z = ux; b.w = uy; return b; }
// float32 copy of a fat box (each coordinate rounded to nearest)
static GB_HD float4 boxf_of(const dbox &b) { return make_float4((float)b.x, (float)b.y, (float)b.z, (float)b.w); }
template <class R> struct xform2 { vec2<R> p; rot2<R> q; };

// Mat22_mul
template <class R> GB_HD vec2<R> rmul(rot2<R> q, vec2<R> v) { return mk<R>(q.c * v.x + (-q.s) * v.y, q.s * v.x + q.c * v.y); }
// Mat22_mul_t_vec
template <class R> GB_HD vec2<R> rmul_t(rot2<R> q, vec2<R> v) { return mk<R>(q.c * v.x + q.s * v.y, (-q.s) * v.x + q.c * v.y); }
// Transform_mul: position + col1 * x + col2 * y, left to right
template <class R> GB_HD vec2<R> xmul(xform2<R> t, vec2<R> v) {
    return mk<R>(t.p.x + t.q.c * v.x + (-t.q.s) * v.y, t.p.y + t.q.s * v.x + t.q.c * v.y);
}
// Transform_mul_t_vec
template <class R> GB_HD vec2<R> xmul_t(xform2<R> t, vec2<R> v) {
    R v0 = v.x - t.p.x, v1 = v.y - t.p.y;
    return mk<R>(t.q.c * v0 + t.q.s * v1, (-t.q.s) * v0 + t.q.c * v1);
}

// CPython min()/max() of two floats: the first argument wins ties
template <class R> GB_HD R pymin(R a, R b) { return (b < a) ? b : a; }
template <class R> GB_HD R pymax(R a, R b) { return (b > a) ? b : a; }
// commonmodule.c clamp: MAX(low, MIN(value, high))
template <class R> GB_HD R cclamp(R v, R lo, R hi) { R m = (v < hi) ? v : hi; return (lo > m) ? lo : m; }
template <class R> GB_HD R cmin(R a, R b) { return (a < b) ? a : b; }
template <class R> GB_HD R cmax(R a, R b) { return (a > b) ? a : b; }
template <class R> GB_HD R sq(R x) { return x * x; }

// Portable sine/cosine of a float64 angle: Cody-Waite reduction by pi/2 in
// three parts (33 + 33 significant bits + rest, so k*P1 and k*P2 are exact
// for |k| < 2^20), Taylor series of sin and cos about 0 on [-pi/4, pi/4]
// (terms to x^17 and x^18), Horner form.  The CPU restatement evaluates the
// same expression, so both produce identical doubles.
static GB_HD rot2<double> rot_of(double a) {
    const double TWO_OVER_PI = 0.6366197723675814;
    const double P1 = 1.5707963267341256;
    const double P2 = 6.077100506303966e-11;
    const double P3 = 2.0222662487959506e-21;
    double k = rint(a * TWO_OVER_PI);
    double r = ((a - k * P1) - k * P2) - k * P3;
    double r2 = r * r;
    double sp = -1.0 / 6.0 + r2 * (1.0 / 120.0 + r2 * (-1.0 / 5040.0 + r2 * (1.0 / 362880.0 +
                r2 * (-2.505210838544172e-08 + r2 * (1.6059043836821613e-10 +
                r2 * (-7.647163731819816e-13 + r2 * 2.8114572543455206e-15))))));
    double sn = r + (r * r2) * sp;
    double cp = -0.5 + r2 * (1.0 / 24.0 + r2 * (-1.0 / 720.0 + r2 * (2.48015873015873e-05 +
                r2 * (-2.755731922398589e-07 + r2 * (2.08767569878681e-09 +
                r2 * (-1.1470745597729725e-11 + r2 * (4.779477332387385e-14 +
                r2 * -1.5619206968586225e-16)))))));
    double cs = 1.0 + r2 * cp;
    long long qi = (long long)k;
    int quad = (int)(qi & 3);
    rot2<double> q;
    if (quad == 0) { q.c = cs; q.s = sn; }
    else if (quad == 1) { q.c = -sn; q.s = cs; }
    else if (quad == 2) { q.c = -cs; q.s = -sn; }
    else { q.c = sn; q.s = -cs; }
    return q;
}

// float32 Taylor polynomials of sin and cos on [-pi/4, pi/4] (sin to x^11,
// cos to x^12; truncation below 1e-10) and the quadrant swap.
static GB_HD rot2<float> rot_poly_f32(float r, int quad) {
    float r2 = r * r;
    float sn = r + (r * r2) * (-1.0f / 6.0f + r2 * (1.0f / 120.0f + r2 * (-1.0f / 5040.0f + r2 * (2.7557319e-06f + r2 * -2.5052108e-08f))));
    float cs = 1.0f + r2 * (-0.5f + r2 * (1.0f / 24.0f + r2 * (-1.0f / 720.0f + r2 * (2.4801587e-05f + r2 * (-2.7557319e-07f + r2 * 2.0876757e-09f)))));
    rot2<float> q;
    if (quad == 0) { q.c = cs; q.s = sn; }
    else if (quad == 1) { q.c = -sn; q.s = cs; }
    else if (quad == 2) { q.c = -cs; q.s = -sn; }
    else { q.c = sn; q.s = -cs; }
    return q;
}

// float32 rotation of a float64 angle: the same reduction in float64, then
// the float32 polynomials.
static GB_HD rot2<float> rot_of_f32(double a) {
    const double TWO_OVER_PI = 0.6366197723675814;
    const double P1 = 1.5707963267341256;
    const double P2 = 6.077100506303966e-11;
    double k = rint(a * TWO_OVER_PI);
    float r = (float)((a - k * P1) - k * P2);
    return rot_poly_f32(r, (int)(((long long)k) & 3));
}

// float32 rotation of a float32 angle of a few pi at most: reduction by
// pi/2 in float32 (pi/2 = P1 + P2, P1 the float nearest pi/2, so k * P1 is
// exact for |k| <= 2), then the float32 polynomials.  No float64 arithmetic.
static GB_HD rot2<float> rot_f32(float x) {
    const float k = rintf(x * 0.63661977f);
    float r = fmaf(-k, 1.57079637f, x);
    r = fmaf(-k, -4.37113900e-08f, r);
    return rot_poly_f32(r, ((int)k) & 3);
}

// A float64 angle reduced to [-pi, pi] and rounded to float32 (the
// step-start angle of the float32 position passes).
static GB_HD float angle_f32(double a) {
    const double INV_TWO_PI = 0.15915494309189535;
    const double Q1 = 6.283185307179586;      // float64 nearest 2 pi
    const double Q2 = 2.4492935982947064e-16;  // 2 pi - Q1
    double k = rint(a * INV_TWO_PI);
    return (float)((a - k * Q1) - k * Q2);
}

// Rotation of the float64 poses (body transforms, sweeps, fat boxes).  The
// float64 unit takes the portable sincos above (bit-exact with the CPU
// restatement); the float32 unit (GB_POSE_ROT_F32) the float32 rotation,
// widened: its narrow phase and solver read float32 rotations anyway, and
// GB300 issues float64 arithmetic at a small fraction of the float32 rate.
static GB_HD rot2<double> pose_rot(double a) {
#if defined(GB_POSE_ROT_F32)
    const rot2<float> q = rot_of_f32(a);
    rot2<double> r;
    r.c = (double)q.c; r.s = (double)q.s;
    return r;
#else
    return rot_of(a);
#endif
}

template <class R> struct Rot;
// float64 rotations of the solver's positions: the portable sincos in the
// float64 unit (bit-exact with the CPU restatement); in the float32 unit the
// float32-accurate rotation of the poses (the TOI position pass, whose
// float64 arithmetic would otherwise spend most of its time in the sincos)
template <> struct Rot<double> { GB_HD static rot2<double> of(double a) { return pose_rot(a); } };
template <> struct Rot<float> { GB_HD static rot2<float> of(double a) { return rot_of_f32(a); } };

// Order-preserving map of a double to uint64 (for atomicMin over doubles).
static __device__ __forceinline__ unsigned long long dkey(double d) {
    unsigned long long b = (unsigned long long)__double_as_longlong(d);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
static __device__ __forceinline__ double dkey_inv(unsigned long long k) {
    unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
    return __longlong_as_double((long long)b);
}

/*
 * oracle_math.h -- TEST INFRASTRUCTURE: float64 vector algebra of the CPU
 * restatement of pypybox2d's World.step.  Every helper repeats the exact
 * operation order of the reference's C extension `_common`
 * (pypybox2d/src/vec2module.c, mat22module.c, transform.c, aabbmodule.c) so
 * that the restatement reproduces the reference's doubles bit for bit.
 *
 * Two spellings of the reference's libm calls exist:
 *   ORACLE_LIBM defined   -> cos/sin and `x**2` go through libm (cos, sin,
 *                            pow(x, 2.0)), exactly what CPython does; this
 *                            build is pinned against the Python reference.
 *   ORACLE_LIBM undefined -> the portable sincos below (Cody-Waite reduction,
 *                            Taylor series) and `x**2` as x*x; the GPU kernels
 *                            use the same two formulas, so this build is the
 *                            bit-exact checker of the float64 GPU path.
 */
#ifndef ORACLE_MATH_H
#define ORACLE_MATH_H

#include <math.h>
#include <float.h>

typedef struct { double x, y; } v2;
/* rotation matrix col1 = (c, s), col2 = (-s, c)  (mat22module.c Mat22_set_angle) */
typedef struct { double c, s; } rot;
typedef struct { v2 p; rot q; } xform;

static inline v2 V(double x, double y) { v2 r; r.x = x; r.y = y; return r; }
/* vec2module.c Vec2_add / Vec2_sub / Vec2_neg */
static inline v2 vadd(v2 a, v2 b) { return V(a.x + b.x, a.y + b.y); }
static inline v2 vsub(v2 a, v2 b) { return V(a.x - b.x, a.y - b.y); }
static inline v2 vneg(v2 a) { return V(-a.x, -a.y); }
/* Vec2_mul with one float operand */
static inline v2 vscale(double s, v2 a) { return V(s * a.x, s * a.y); }
/* Vec2_mul of two vectors (dot) */
static inline double vdot(v2 a, v2 b) { return a.x * b.x + a.y * b.y; }
/* Vec2_cross(vector) */
static inline double vcross(v2 a, v2 b) { return a.x * b.y - a.y * b.x; }
/* Vec2_cross(float): new_Vec2(ox * sy, -ox * sx) */
static inline v2 vcross_vs(v2 a, double s) { return V(s * a.y, -s * a.x); }
/* module scalar_cross: new_Vec2(-scalar * y, scalar * x) */
static inline v2 vcross_sv(double s, v2 a) { return V(-s * a.y, s * a.x); }
static inline double vlen2(v2 a) { return a.x * a.x + a.y * a.y; }
static inline double vlen(v2 a) { return sqrt(a.x * a.x + a.y * a.y); }
/* Vec2_normalized: threshold FLT_EPSILON (vec2module.c:447-459) */
static inline v2 vnormalized(v2 a) {
    double l = sqrt(a.x * a.x + a.y * a.y);
    if (l < FLT_EPSILON) return a;
    double inv = 1.0 / l;
    return V(a.x * inv, a.y * inv);
}
/* Mat22_mul (matrix * vector) */
static inline v2 rmul(rot q, v2 v) { return V(q.c * v.x + (-q.s) * v.y, q.s * v.x + q.c * v.y); }
/* Mat22_mul_t_vec */
static inline v2 rmul_t(rot q, v2 v) { return V(q.c * v.x + q.s * v.y, (-q.s) * v.x + q.c * v.y); }
/* Transform_mul: position + col1 * v0 + col2 * v1, left to right */
static inline v2 xmul(xform t, v2 v) {
    return V(t.p.x + t.q.c * v.x + (-t.q.s) * v.y, t.p.y + t.q.s * v.x + t.q.c * v.y);
}
/* Transform_mul_t_vec */
static inline v2 xmul_t(xform t, v2 v) {
    double v0 = v.x - t.p.x, v1 = v.y - t.p.y;
    return V(t.q.c * v0 + t.q.s * v1, (-t.q.s) * v0 + t.q.c * v1);
}
/* CPython min()/max() of two floats: the first argument wins ties */
static inline double pymin(double a, double b) { return (b < a) ? b : a; }
static inline double pymax(double a, double b) { return (b > a) ? b : a; }
/* commonmodule.c module_clamp: MAX(low, MIN(value, high)) */
static inline double cclamp(double v, double lo, double hi) {
    double m = (v < hi) ? v : hi;
    return (lo > m) ? lo : m;
}
/* common.h MIN/MAX as used by min_vector/max_vector and AABB_add */
static inline double cmin(double a, double b) { return (a < b) ? a : b; }
static inline double cmax(double a, double b) { return (a > b) ? a : b; }

#ifdef ORACLE_LIBM
/* CPython float ** 2 is libm pow(x, 2.0), which is not always x*x.  The
 * call goes through a volatile pointer so the compiler cannot fold it into
 * x*x. */
static double (*volatile or_pow_fn)(double, double) = pow;
static inline double SQ(double x) { return or_pow_fn(x, 2.0); }
static inline rot rot_of(double a) { rot q; q.c = cos(a); q.s = sin(a); return q; }
#else
static inline double SQ(double x) { return x * x; }
/*
 * Portable sine/cosine shared, formula for formula, with the GPU kernels.
 * Cody-Waite reduction by pi/2 split into three parts (the first two with 33
 * significant bits, so k*P1 and k*P2 are exact for |k| < 2^20), then the
 * Taylor series of sin and cos about 0 on [-pi/4, pi/4] (terms to x^17 and
 * x^18; the first omitted term is below 1e-19 relative), Horner form.
 */
static inline rot rot_of(double a) {
    const double TWO_OVER_PI = 0.6366197723675814;
    const double P1 = 1.5707963267341256;
    const double P2 = 6.077100506303966e-11;
    const double P3 = 2.0222662487959506e-21;
    double k = nearbyint(a * TWO_OVER_PI);
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
    rot q;
    switch (quad) {
    case 0: q.c = cs; q.s = sn; break;
    case 1: q.c = -sn; q.s = cs; break;
    case 2: q.c = -cs; q.s = -sn; break;
    default: q.c = sn; q.s = -cs; break;
    }
    return q;
}
#endif

#endif /* ORACLE_MATH_H */

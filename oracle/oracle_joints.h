/*
 * oracle_joints.h -- TEST INFRASTRUCTURE: float64 restatement of the joint
 * constraints pypybox2d's island solver runs beside the contacts
 * (island.py:107-113, 145-148): revolute (joints/revolute.py:240-453),
 * prismatic (joints/prismatic.py:238-513), distance
 * (joints/distance.py:175-311) and weld (joints/weld.py:118-257).
 *
 * Every expression keeps the reference's operation order.  Two properties of
 * the reference's C extension shape the arithmetic: Vec2 has no in-place
 * operators (vec2module.c:636-652), so `x *= s` rebinds x and leaves other
 * names bound to the old vector (the distance joint's effective mass uses
 * the unnormalised direction, distance.py:212-222); Vec3 and Mat33 are
 * Python classes (common.py:227-612) whose dot, cross and solves are
 * restated below as written there.  Included by oracle.c only.
 */
#ifndef ORACLE_JOINTS_H
#define ORACLE_JOINTS_H

#include "oracle_math.h"
#include "../include/gb2d.h"

/* settings.py:61-94 */
#define OR_LINEAR_SLOP_J 0.005
#ifndef OR_ANGULAR_SLOP
#define OR_ANGULAR_SLOP (2.0 / 180.0 * 3.141592653589793)
#endif
#define OR_MAX_LINEAR_CORRECTION_J 0.2
#define OR_MAX_ANGULAR_CORRECTION (8.0 / 180.0 * 3.141592653589793)
#define OR_PI 3.141592653589793

typedef struct { double x, y, z; } v3;
static inline v3 V3(double x, double y, double z) { v3 r; r.x = x; r.y = y; r.z = z; return r; }
/* Vec3.dot: (x * vx) + (y * vy) + (z * vz), left to right */
static inline double v3dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
/* Vec3.cross */
static inline v3 v3cross(v3 s, v3 v) { return V3(s.y * v.z - s.z * v.y, s.z * v.x - s.x * v.z, s.x * v.y - s.y * v.x); }
static inline v3 v3add(v3 a, v3 b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 v3sub(v3 a, v3 b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 v3neg(v3 a) { return V3(-a.x, -a.y, -a.z); }
/* Vec3.__mul__(number): Vec3(value * x, value * y, value * z) */
static inline v3 v3scale(double s, v3 a) { return V3(s * a.x, s * a.y, s * a.z); }

/* Mat33 (column-major, common.py:533-612) */
typedef struct { v3 c1, c2, c3; } m33;
/* Mat33.solve3x3 */
static inline v3 m33_solve3(m33 m, v3 b) {
    double det = v3dot(m.c1, v3cross(m.c2, m.c3));
    if (det != 0.0) det = 1.0 / det;
    return V3(det * v3dot(b, v3cross(m.c2, m.c3)), det * v3dot(m.c1, v3cross(b, m.c3)), det * v3dot(m.c1, v3cross(m.c2, b)));
}
/* Mat33.solve2x2 (upper 2x2 block) */
static inline v2 m33_solve2(m33 m, v2 v) {
    double a11 = m.c1.x, a12 = m.c2.x, a21 = m.c1.y, a22 = m.c2.y;
    double det = a11 * a22 - a12 * a21;
    if (det != 0.0) det = 1.0 / det;
    return V(det * (a22 * v.x - a12 * v.y), det * (a11 * v.y - a21 * v.x));
}
/* Mat22.solve (mat22module.c:500-516); K given by its columns */
static inline v2 m22_solve(v2 c1, v2 c2, v2 v) {
    double a = c1.x, b = c2.x, c = c1.y, d = c2.y;
    double det = a * d - b * c;
    if (det != 0.0) det = 1.0 / det;
    return V(det * (d * v.x - b * v.y), det * (a * v.y - c * v.x));
}

/* What _init_velocity_constraints leaves on the joint for the passes of one
 * step (the underscore attributes it sets). */
typedef struct {
    int j;                 /* joint index in the world */
    int ia, ib;            /* island indices of body_a, body_b */
    double ma, mb, iA, iB; /* _inv_mass_a/_b, _inv_Ia/_Ib */
    v2 lca, lcb;           /* _local_center_a/_b */
    v2 ra, rb;             /* _ra, _rb */
    m33 m;                 /* revolute/weld _mass, prismatic _k */
    double motor_mass;     /* revolute, prismatic */
    v2 u;                  /* distance _u */
    double dmass;          /* distance _mass */
    v2 axis, perp;         /* prismatic */
    double s1, s2, a1, a2;
} or_jcons;

static inline v2 j_la(const gb_joint *J) { return V(J->la_x, J->la_y); }
static inline v2 j_lb(const gb_joint *J) { return V(J->lb_x, J->lb_y); }

/* the carried _impulse minus its z component: `_impulse -= (0, 0, z)` */
static inline void j_drop_z(gb_joint *J) { J->impulse[2] = J->impulse[2] - J->impulse[2]; }

/* ------------------------------------------------------------ revolute */
static void revolute_init(gb_joint *J, or_jcons *k, const v2 *pc, const double *pa, v2 *vv, double *ww, double dt_ratio,
                          int warm) {
    double ma = k->ma, mb = k->mb, ia = k->iA, ib = k->iB;
    double aa = pa[k->ia], ab = pa[k->ib];
    (void)pc;
    v2 va = vv[k->ia], vb = vv[k->ib];
    double wa = ww[k->ia], wb = ww[k->ib];
    rot qa = rot_of(aa), qb = rot_of(ab);
    v2 ra = k->ra = rmul(qa, vsub(j_la(J), k->lca));
    v2 rb = k->rb = rmul(qb, vsub(j_lb(J), k->lcb));
    k->m.c3 = V3(-ra.y * ia - rb.y * ib, ra.x * ia + rb.x * ib, ia + ib);
    k->m.c2 = V3(-ra.y * ra.x * ia - rb.y * rb.x * ib, ma + mb + ra.x * ra.x * ia + rb.x * rb.x * ib, k->m.c3.y);
    k->m.c1 = V3(ma + mb + ra.y * ra.y * ia + rb.y * rb.y * ib, k->m.c2.x, k->m.c3.x);
    k->motor_mass = ia + ib;
    int fixed_rotation = (k->motor_mass == 0.0);
    if (k->motor_mass > 0.0) k->motor_mass = 1.0 / k->motor_mass;
    if (!(J->flags & GB_J_MOTOR) || fixed_rotation) J->motor_impulse = 0.0;
    if ((J->flags & GB_J_LIMIT) && !fixed_rotation) {
        double joint_angle = ab - aa - J->ref_angle;
        if (fabs(J->upper - J->lower) < 2.0 * OR_ANGULAR_SLOP) {
            J->limit_state = GB_LIMIT_EQUAL;
        } else if (joint_angle <= J->lower) {
            if (J->limit_state != GB_LIMIT_LOWER) j_drop_z(J);
            J->limit_state = GB_LIMIT_LOWER;
        } else if (joint_angle >= J->upper) {
            if (J->limit_state != GB_LIMIT_UPPER) j_drop_z(J);
            J->limit_state = GB_LIMIT_UPPER;
        } else {
            J->limit_state = GB_LIMIT_INACTIVE;
            j_drop_z(J);
        }
    } else {
        J->limit_state = GB_LIMIT_INACTIVE;
    }
    if (warm) {
        J->impulse[0] = dt_ratio * J->impulse[0];
        J->impulse[1] = dt_ratio * J->impulse[1];
        J->impulse[2] = dt_ratio * J->impulse[2];
        J->motor_impulse = J->motor_impulse * dt_ratio;
        v2 P = V(J->impulse[0], J->impulse[1]);
        va = vsub(va, vscale(ma, P));
        wa = wa - ia * (vcross(ra, P) + J->motor_impulse + J->impulse[2]);
        vb = vadd(vb, vscale(mb, P));
        wb = wb + ib * (vcross(rb, P) + J->motor_impulse + J->impulse[2]);
    } else {
        J->impulse[0] = J->impulse[1] = J->impulse[2] = 0.0;
        J->motor_impulse = 0.0;
    }
    vv[k->ia] = va; ww[k->ia] = wa;
    vv[k->ib] = vb; ww[k->ib] = wb;
}

static void revolute_solve_velocity(gb_joint *J, or_jcons *k, v2 *vv, double *ww, double dt) {
    v2 va = vv[k->ia], vb = vv[k->ib];
    double wa = ww[k->ia], wb = ww[k->ib];
    double ma = k->ma, mb = k->mb, ia = k->iA, ib = k->iB;
    v2 ra = k->ra, rb = k->rb;
    int fixed_rotation = ((ia + ib) == 0.0);
    if ((J->flags & GB_J_MOTOR) && J->limit_state != GB_LIMIT_EQUAL && !fixed_rotation) {
        double Cdot = wb - wa - J->motor_speed;
        double impulse = k->motor_mass * (-Cdot);
        double old_impulse = J->motor_impulse;
        double max_impulse = dt * J->max_motor;
        J->motor_impulse = cclamp(J->motor_impulse + impulse, -max_impulse, max_impulse);
        impulse = J->motor_impulse - old_impulse;
        wa = wa - ia * impulse;
        wb = wb + ib * impulse;
    }
    if ((J->flags & GB_J_LIMIT) && J->limit_state != GB_LIMIT_INACTIVE && !fixed_rotation) {
        v2 Cdot1 = vsub(vsub(vadd(vb, vcross_sv(wb, rb)), va), vcross_sv(wa, ra));
        double Cdot2 = wb - wa;
        v3 impulse = v3neg(m33_solve3(k->m, V3(Cdot1.x, Cdot1.y, Cdot2)));
        v3 acc = V3(J->impulse[0], J->impulse[1], J->impulse[2]);
        if (J->limit_state == GB_LIMIT_EQUAL) {
            acc = v3add(acc, impulse);
        } else if (J->limit_state == GB_LIMIT_LOWER || J->limit_state == GB_LIMIT_UPPER) {
            double new_impulse = acc.z + impulse.z;
            int clamp_it = J->limit_state == GB_LIMIT_LOWER ? (new_impulse < 0.0) : (new_impulse > 0.0);
            if (clamp_it) {
                v2 rhs = vadd(vneg(Cdot1), vscale(acc.z, V(k->m.c3.x, k->m.c3.y)));
                v2 reduced = m33_solve2(k->m, rhs);
                impulse = V3(reduced.x, reduced.y, -acc.z);
                acc = v3add(acc, V3(reduced.x, reduced.y, -acc.z));
            } else {
                acc = v3add(acc, impulse);
            }
        }
        J->impulse[0] = acc.x; J->impulse[1] = acc.y; J->impulse[2] = acc.z;
        v2 P = V(impulse.x, impulse.y);
        va = vsub(va, vscale(ma, P));
        wa = wa - ia * (vcross(ra, P) + impulse.z);
        vb = vadd(vb, vscale(mb, P));
        wb = wb + ib * (vcross(rb, P) + impulse.z);
    } else {
        v2 Cdot = vsub(vsub(vadd(vb, vcross_sv(wb, rb)), va), vcross_sv(wa, ra));
        v2 impulse = m33_solve2(k->m, vneg(Cdot));
        J->impulse[0] = J->impulse[0] + impulse.x;
        J->impulse[1] = J->impulse[1] + impulse.y;
        J->impulse[2] = J->impulse[2] + 0.0;
        va = vsub(va, vscale(ma, impulse));
        wa = wa - ia * vcross(ra, impulse);
        vb = vadd(vb, vscale(mb, impulse));
        wb = wb + ib * vcross(rb, impulse);
    }
    vv[k->ia] = va; ww[k->ia] = wa;
    vv[k->ib] = vb; ww[k->ib] = wb;
}

static int revolute_solve_position(gb_joint *J, or_jcons *k, v2 *pc, double *pa) {
    v2 ca = pc[k->ia], cb = pc[k->ib];
    double aa = pa[k->ia], ab = pa[k->ib];
    double ma = k->ma, mb = k->mb, ia = k->iA, ib = k->iB;
    int fixed_rotation = ((ia + ib) == 0.0);
    double angular_error = 0.0, position_error = 0.0;
    if ((J->flags & GB_J_LIMIT) && J->limit_state != GB_LIMIT_INACTIVE && !fixed_rotation) {
        double angle = ab - aa - J->ref_angle;
        double limit_impulse = 0.0;
        if (J->limit_state == GB_LIMIT_EQUAL) {
            double C = cclamp(angle - J->lower, -OR_MAX_ANGULAR_CORRECTION, OR_MAX_ANGULAR_CORRECTION);
            limit_impulse = -k->motor_mass * C;
            angular_error = fabs(C);
        } else if (J->limit_state == GB_LIMIT_LOWER) {
            double C = angle - J->lower;
            angular_error = -C;
            C = cclamp(C + OR_ANGULAR_SLOP, -OR_MAX_ANGULAR_CORRECTION, 0.0);
            limit_impulse = -k->motor_mass * C;
        } else if (J->limit_state == GB_LIMIT_UPPER) {
            double C = angle - J->upper;
            angular_error = C;
            C = cclamp(C - OR_ANGULAR_SLOP, 0.0, OR_MAX_ANGULAR_CORRECTION);
            limit_impulse = -k->motor_mass * C;
        }
        aa = aa - ia * limit_impulse;
        ab = ab + ib * limit_impulse;
    }
    rot qa = rot_of(aa), qb = rot_of(ab);
    v2 ra = rmul(qa, vsub(j_la(J), k->lca));
    v2 rb = rmul(qb, vsub(j_lb(J), k->lcb));
    v2 C = vsub(vsub(vadd(cb, rb), ca), ra);
    position_error = vlen(C);
    double rax = ra.x, ray = ra.y, rbx = rb.x, rby = rb.y;
    v2 c1 = V(ma + mb + ia * ray * ray + ib * rby * rby, -ia * rax * ray - ib * rbx * rby);
    v2 c2 = V(c1.y, ma + mb + ia * rax * rax + ib * rbx * rbx);
    v2 impulse = vneg(m22_solve(c1, c2, C));
    ca = vsub(ca, vscale(ma, impulse));
    aa = aa - ia * vcross(ra, impulse);
    cb = vadd(cb, vscale(mb, impulse));
    ab = ab + ib * vcross(rb, impulse);
    pc[k->ia] = ca; pa[k->ia] = aa;
    pc[k->ib] = cb; pa[k->ib] = ab;
    return position_error <= OR_LINEAR_SLOP_J && angular_error <= OR_ANGULAR_SLOP;
}

/* ------------------------------------------------------------ prismatic */
/* prismatic.py:82-85: local y axis = scalar_cross(1.0, local x axis) */
static inline v2 j_ly(const gb_joint *J) { return vcross_sv(1.0, V(J->ax_x, J->ax_y)); }

static void prismatic_init(gb_joint *J, or_jcons *k, const v2 *pc, const double *pa, v2 *vv, double *ww, double dt_ratio,
                           int warm) {
    double ma = k->ma, mb = k->mb, ia = k->iA, ib = k->iB;
    v2 ca = pc[k->ia], cb = pc[k->ib];
    double aa = pa[k->ia], ab = pa[k->ib];
    v2 va = vv[k->ia], vb = vv[k->ib];
    double wa = ww[k->ia], wb = ww[k->ib];
    rot qa = rot_of(aa), qb = rot_of(ab);
    v2 ra = k->ra = rmul(qa, vsub(j_la(J), k->lca));
    v2 rb = k->rb = rmul(qb, vsub(j_lb(J), k->lcb));
    v2 d = vsub(vsub(vadd(cb, rb), ca), ra);
    v2 axis = k->axis = rmul(qa, V(J->ax_x, J->ax_y));
    double a1 = k->a1 = vcross(vadd(d, ra), axis);
    double a2 = k->a2 = vcross(rb, axis);
    k->motor_mass = ma + mb + ia * SQ(a1) + ib * SQ(a2);
    if (k->motor_mass > 0.0) k->motor_mass = 1.0 / k->motor_mass;
    v2 perp = k->perp = rmul(qa, j_ly(J));
    double s1 = k->s1 = vcross(vadd(d, ra), perp);
    double s2 = k->s2 = vcross(rb, perp);
    double k11 = ma + mb + ia * SQ(s1) + ib * SQ(s2);
    double k12 = ia * s1 + ib * s2;
    double k13 = ia * s1 * a1 + ib * s2 * a2;
    double k22 = ia + ib;
    if (k22 == 0.0) k22 = 1.0;
    double k23 = ia * a1 + ib * a2;
    double k33 = ma + mb + ia * SQ(a1) + ib * SQ(a2);
    k->m.c1 = V3(k11, k12, k13);
    k->m.c2 = V3(k12, k22, k23);
    k->m.c3 = V3(k13, k23, k33);
    if (J->flags & GB_J_LIMIT) {
        double joint_translation = vdot(axis, d);
        if (fabs(J->upper - J->lower) < 2.0 * OR_LINEAR_SLOP_J) {
            J->limit_state = GB_LIMIT_EQUAL;
        } else if (joint_translation <= J->lower) {
            if (J->limit_state != GB_LIMIT_LOWER) { J->limit_state = GB_LIMIT_LOWER; j_drop_z(J); }
        } else if (joint_translation >= J->upper) {
            if (J->limit_state != GB_LIMIT_UPPER) { J->limit_state = GB_LIMIT_UPPER; j_drop_z(J); }
        } else {
            J->limit_state = GB_LIMIT_INACTIVE;
            j_drop_z(J);
        }
    } else {
        J->limit_state = GB_LIMIT_INACTIVE;
        j_drop_z(J);
    }
    if (!(J->flags & GB_J_MOTOR)) J->motor_impulse = 0.0;
    if (warm) {
        J->impulse[0] = dt_ratio * J->impulse[0];
        J->impulse[1] = dt_ratio * J->impulse[1];
        J->impulse[2] = dt_ratio * J->impulse[2];
        J->motor_impulse = J->motor_impulse * dt_ratio;
        double ix = J->impulse[0], iy = J->impulse[1], iz = J->impulse[2], mi = J->motor_impulse;
        v2 P = vadd(vscale(ix, perp), vscale(mi + iz, axis));
        double L1 = ix * s1 + iy + (mi + iz) * a1;
        double L2 = ix * s2 + iy + (mi + iz) * a2;
        va = vsub(va, vscale(ma, P));
        wa = wa - ia * L1;
        vb = vadd(vb, vscale(mb, P));
        wb = wb + ib * L2;
    } else {
        J->impulse[0] = J->impulse[1] = J->impulse[2] = 0.0;
        J->motor_impulse = 0.0;
    }
    J->ux = axis.x; J->uy = axis.y;
    J->perp_x = perp.x; J->perp_y = perp.y;
    vv[k->ia] = va; ww[k->ia] = wa;
    vv[k->ib] = vb; ww[k->ib] = wb;
}

static void prismatic_solve_velocity(gb_joint *J, or_jcons *k, v2 *vv, double *ww, double dt) {
    v2 va = vv[k->ia], vb = vv[k->ib];
    double wa = ww[k->ia], wb = ww[k->ib];
    double ma = k->ma, mb = k->mb, ia = k->iA, ib = k->iB;
    double a1 = k->a1, a2 = k->a2, s1 = k->s1, s2 = k->s2;
    v2 perp = k->perp, axis = k->axis;
    if ((J->flags & GB_J_MOTOR) && J->limit_state != GB_LIMIT_EQUAL) {
        double Cdot = vdot(axis, vsub(vb, va)) + a2 * wb - a1 * wa;
        double impulse = k->motor_mass * (J->motor_speed - Cdot);
        double old_impulse = J->motor_impulse;
        double max_impulse = dt * J->max_motor;
        J->motor_impulse = cclamp(J->motor_impulse + impulse, -max_impulse, max_impulse);
        impulse = J->motor_impulse - old_impulse;
        v2 P = vscale(impulse, axis);
        double L1 = impulse * a1, L2 = impulse * a2;
        va = vsub(va, vscale(ma, P));
        wa = wa - ia * L1;
        vb = vadd(vb, vscale(mb, P));
        wb = wb + ib * L2;
    }
    v2 Cdot1 = V(vdot(perp, vsub(vb, va)) + s2 * wb - s1 * wa, wb - wa);
    v2 P;
    double L1, L2;
    if ((J->flags & GB_J_LIMIT) && J->limit_state != GB_LIMIT_INACTIVE) {
        double Cdot2 = vdot(axis, vsub(vb, va)) + a2 * wb - a1 * wa;
        v3 Cdot = V3(Cdot1.x, Cdot1.y, Cdot2);
        v3 old = V3(J->impulse[0], J->impulse[1], J->impulse[2]);
        v3 df = m33_solve3(k->m, v3neg(Cdot));
        v3 acc = v3add(old, df);
        double iz;
        if (J->limit_state == GB_LIMIT_LOWER) iz = pymax(acc.z, 0.0);
        else if (J->limit_state == GB_LIMIT_UPPER) iz = pymin(acc.z, 0.0);
        else iz = acc.z;
        v2 b = vsub(vneg(Cdot1), vscale(acc.z - old.z, V(k->m.c3.x, k->m.c3.y)));
        v2 f2r = vadd(m33_solve2(k->m, b), V(old.x, old.y));
        acc = V3(f2r.x, f2r.y, iz);
        J->impulse[0] = acc.x; J->impulse[1] = acc.y; J->impulse[2] = acc.z;
        df = v3sub(acc, old);
        P = vadd(vscale(df.x, perp), vscale(df.z, axis));
        L1 = df.x * s1 + df.y + df.z * a1;
        L2 = df.x * s2 + df.y + df.z * a2;
    } else {
        v2 df = m33_solve2(k->m, vneg(Cdot1));
        J->impulse[0] = J->impulse[0] + df.x;
        J->impulse[1] = J->impulse[1] + df.y;
        J->impulse[2] = J->impulse[2] + 0.0;
        P = vscale(df.x, perp);
        L1 = df.x * s1 + df.y;
        L2 = df.x * s2 + df.y;
    }
    va = vsub(va, vscale(ma, P));
    wa = wa - ia * L1;
    vb = vadd(vb, vscale(mb, P));
    wb = wb + ib * L2;
    vv[k->ia] = va; ww[k->ia] = wa;
    vv[k->ib] = vb; ww[k->ib] = wb;
}

static int prismatic_solve_position(gb_joint *J, or_jcons *k, v2 *pc, double *pa) {
    v2 ca = pc[k->ia], cb = pc[k->ib];
    double aa = pa[k->ia], ab = pa[k->ib];
    double ma = k->ma, mb = k->mb, ia = k->iA, ib = k->iB;
    rot qa = rot_of(aa), qb = rot_of(ab);
    v2 ra = rmul(qa, vsub(j_la(J), k->lca));
    v2 rb = rmul(qb, vsub(j_lb(J), k->lcb));
    v2 d = vsub(vsub(vadd(cb, rb), ca), ra);
    v2 axis = rmul(qa, V(J->ax_x, J->ax_y));
    double a1 = vcross(vadd(d, ra), axis);
    double a2 = vcross(rb, axis);
    v2 perp = rmul(qa, j_ly(J));
    double s1 = vcross(vadd(d, ra), perp);
    double s2 = vcross(rb, perp);
    v2 C1 = V(vdot(perp, d), ab - aa - J->ref_angle);
    double linear_error = fabs(C1.x), angular_error = fabs(C1.y);
    int active = 0;
    double C2 = 0.0;
    if (J->flags & GB_J_LIMIT) {
        double translation = vdot(axis, d);
        if (fabs(J->upper - J->lower) < 2.0 * OR_LINEAR_SLOP_J) {
            C2 = cclamp(translation, -OR_MAX_LINEAR_CORRECTION_J, OR_MAX_LINEAR_CORRECTION_J);
            linear_error = pymax(linear_error, translation);
            active = 1;
        } else if (translation <= J->lower) {
            C2 = cclamp(translation - J->lower + OR_LINEAR_SLOP_J, -OR_MAX_LINEAR_CORRECTION_J, 0.0);
            linear_error = pymax(linear_error, J->lower - translation);
            active = 1;
        } else if (translation >= J->upper) {
            C2 = cclamp(translation - J->upper - OR_LINEAR_SLOP_J, 0.0, OR_MAX_LINEAR_CORRECTION_J);
            linear_error = pymax(linear_error, translation - J->upper);
            active = 1;
        }
    }
    double ix, iy, iz;
    if (active) {
        double k11 = ma + mb + ia * SQ(s1) + ib * SQ(s2);
        double k12 = ia * s1 + ib * s2;
        double k13 = ia * s1 * a1 + ib * s2 * a2;
        double k22 = ia + ib;
        if (k22 == 0.0) k22 = 1.0;
        double k23 = ia * a1 + ib * a2;
        double k33 = ma + mb + ia * SQ(a1) + ib * SQ(a2);
        m33 K;
        K.c1 = V3(k11, k12, k13); K.c2 = V3(k12, k22, k23); K.c3 = V3(k13, k23, k33);
        v3 impulse = m33_solve3(K, v3neg(V3(C1.x, C1.y, C2)));
        ix = impulse.x; iy = impulse.y; iz = impulse.z;
    } else {
        double k11 = ma + mb + ia * s1 * s1 + ib * s2 * s2;
        double k12 = ia * s1 + ib * s2;
        double k22 = ia + ib;
        if (k22 == 0.0) k22 = 1.0;
        m33 K = k->m;   /* the step's _k with its first two columns replaced (prismatic.py:493-494) */
        K.c1 = V3(k11, k12, 0.0);
        K.c2 = V3(k12, k22, 0.0);
        v2 impulse1 = m33_solve2(K, vneg(C1));
        ix = impulse1.x; iy = impulse1.y; iz = 0.0;
    }
    v2 P = vadd(vscale(ix, perp), vscale(iz, axis));
    double L1 = ix * s1 + iy + iz * a1;
    double L2 = ix * s2 + iy + iz * a2;
    ca = vsub(ca, vscale(ma, P));
    cb = vadd(cb, vscale(mb, P));
    aa = aa - ia * L1;
    ab = ab + ib * L2;
    pc[k->ia] = ca; pa[k->ia] = aa;
    pc[k->ib] = cb; pa[k->ib] = ab;
    return (linear_error <= OR_LINEAR_SLOP_J) && (angular_error <= OR_ANGULAR_SLOP);
}

/* ------------------------------------------------------------ distance */
static void distance_init(gb_joint *J, or_jcons *k, const v2 *pc, const double *pa, v2 *vv, double *ww, double dt,
                          double dt_ratio, int warm) {
    double ma = k->ma, mb = k->mb, iA = k->iA, iB = k->iB;
    v2 ca = pc[k->ia], cb = pc[k->ib];
    double aa = pa[k->ia], ab = pa[k->ib];
    v2 va = vv[k->ia], vb = vv[k->ib];
    double wa = ww[k->ia], wb = ww[k->ib];
    rot qa = rot_of(aa), qb = rot_of(ab);
    v2 ra = k->ra = rmul(qa, vsub(j_la(J), k->lca));
    v2 rb = k->rb = rmul(qb, vsub(j_lb(J), k->lcb));
    v2 u = vsub(vsub(vadd(cb, rb), ca), ra);   /* `u` keeps this vector: `self._u *= ...` rebinds only _u */
    double length = vlen(u);
    if (length > OR_LINEAR_SLOP_J) k->u = vscale(1.0 / length, u);
    else k->u = V(0.0, 0.0);
    double cr_au = SQ(vcross(ra, u));
    double cr_bu = SQ(vcross(rb, u));
    double inv_mass = ma + iA * cr_au + mb + iB * cr_bu;
    k->dmass = inv_mass != 0.0 ? 1.0 / inv_mass : 0.0;
    if (J->frequency > 0.0) {
        double C = length - J->length;
        double omega = 2.0 * OR_PI * J->frequency;
        double dd = 2.0 * k->dmass * J->damping_ratio * omega;
        double kk = k->dmass * SQ(omega);
        double gamma = dt * (dd + dt * kk);
        J->gamma = gamma != 0.0 ? 1.0 / gamma : 0.0;
        J->bias = C * dt * kk * J->gamma;
        double mass = inv_mass + J->gamma;
        k->dmass = mass != 0.0 ? 1.0 / mass : 0.0;
    }
    if (warm) {
        J->impulse[0] = J->impulse[0] * dt_ratio;
        v2 P = vscale(J->impulse[0], k->u);
        va = vsub(va, vscale(ma, P));
        wa = wa - iA * vcross(ra, P);
        vb = vadd(vb, vscale(mb, P));
        wb = wb + iB * vcross(rb, P);
    } else {
        J->impulse[0] = 0.0;
    }
    J->ux = k->u.x; J->uy = k->u.y;
    vv[k->ia] = va; ww[k->ia] = wa;
    vv[k->ib] = vb; ww[k->ib] = wb;
}

static void distance_solve_velocity(gb_joint *J, or_jcons *k, v2 *vv, double *ww) {
    v2 va = vv[k->ia], vb = vv[k->ib];
    double wa = ww[k->ia], wb = ww[k->ib];
    v2 ra = k->ra, rb = k->rb;
    double ma = k->ma, mb = k->mb, ia = k->iA, ib = k->iB;
    v2 vpa = vadd(va, vcross_sv(wa, ra));
    v2 vpb = vadd(vb, vcross_sv(wb, rb));
    double Cdot = vdot(k->u, vsub(vpb, vpa));
    double impulse = -k->dmass * (Cdot + J->bias + J->gamma * J->impulse[0]);
    J->impulse[0] = J->impulse[0] + impulse;
    v2 P = vscale(impulse, k->u);
    va = vsub(va, vscale(ma, P));
    wa = wa - ia * vcross(ra, P);
    vb = vadd(vb, vscale(mb, P));
    wb = wb + ib * vcross(rb, P);
    vv[k->ia] = va; ww[k->ia] = wa;
    vv[k->ib] = vb; ww[k->ib] = wb;
}

static int distance_solve_position(gb_joint *J, or_jcons *k, v2 *pc, double *pa) {
    if (J->frequency > 0.0) return 1;   /* soft constraints have no position correction */
    v2 ca = pc[k->ia], cb = pc[k->ib];
    double aa = pa[k->ia], ab = pa[k->ib];
    rot qa = rot_of(aa), qb = rot_of(ab);
    double ma = k->ma, mb = k->mb, ia = k->iA, ib = k->iB;
    v2 ra = rmul(qa, vsub(j_la(J), k->lca));
    v2 rb = rmul(qb, vsub(j_lb(J), k->lcb));
    v2 u = vsub(vsub(vadd(cb, rb), ca), ra);
    double length = vlen(u);
    u = vnormalized(u);
    double C = length - J->length;
    double impulse = -k->dmass * cclamp(C, -OR_MAX_LINEAR_CORRECTION_J, OR_MAX_LINEAR_CORRECTION_J);
    v2 P = vscale(impulse, u);
    ca = vsub(ca, vscale(ma, P));
    aa = aa - ia * vcross(ra, P);
    cb = vadd(cb, vscale(mb, P));
    ab = ab + ib * vcross(rb, P);
    pc[k->ia] = ca; pa[k->ia] = aa;
    pc[k->ib] = cb; pa[k->ib] = ab;
    return fabs(C) < OR_LINEAR_SLOP_J;
}

/* ------------------------------------------------------------ weld */
static void weld_init(gb_joint *J, or_jcons *k, const v2 *pc, const double *pa, v2 *vv, double *ww, double dt_ratio,
                      int warm) {
    double ma = k->ma, mb = k->mb, ia = k->iA, ib = k->iB;
    double aa = pa[k->ia], ab = pa[k->ib];
    (void)pc;
    v2 va = vv[k->ia], vb = vv[k->ib];
    double wa = ww[k->ia], wb = ww[k->ib];
    rot qa = rot_of(aa), qb = rot_of(ab);
    v2 ra = k->ra = rmul(qa, vsub(j_la(J), k->lca));
    v2 rb = k->rb = rmul(qb, vsub(j_lb(J), k->lcb));
    double c2x = -ra.y * ra.x * ia - rb.y * rb.x * ib;
    double c3x = -ra.y * ia - rb.y * ib;
    k->m.c1 = V3(ma + mb + ra.y * ra.y * ia + rb.y * rb.y * ib, c2x, c3x);
    /* weld.py:163-165: the velocity mass keeps c3x in col2.z */
    k->m.c2 = V3(c2x, ma + mb + ra.x * ra.x * ia + rb.x * rb.x * ib, c3x);
    k->m.c3 = V3(c3x, ra.x * ia + rb.x * ib, ia + ib);
    if (warm) {
        J->impulse[0] = dt_ratio * J->impulse[0];
        J->impulse[1] = dt_ratio * J->impulse[1];
        J->impulse[2] = dt_ratio * J->impulse[2];
        double ix = J->impulse[0], iy = J->impulse[1], iz = J->impulse[2];
        v2 P = V(ix, iy);
        va = vsub(va, vscale(ma, P));
        wa = wa - ia * (vcross(ra, P) + iz);
        vb = vadd(vb, vscale(mb, P));
        wb = wb + ib * (vcross(rb, P) + iz);
    } else {
        J->impulse[0] = J->impulse[1] = J->impulse[2] = 0.0;
    }
    vv[k->ia] = va; ww[k->ia] = wa;
    vv[k->ib] = vb; ww[k->ib] = wb;
}

static void weld_solve_velocity(gb_joint *J, or_jcons *k, v2 *vv, double *ww) {
    v2 va = vv[k->ia], vb = vv[k->ib];
    double wa = ww[k->ia], wb = ww[k->ib];
    v2 ra = k->ra, rb = k->rb;
    double ma = k->ma, mb = k->mb, ia = k->iA, ib = k->iB;
    v2 Cdot1 = vsub(vsub(vadd(vb, vcross_sv(wb, rb)), va), vcross_sv(wa, ra));
    double Cdot2 = wb - wa;
    v3 impulse = m33_solve3(k->m, v3neg(V3(Cdot1.x, Cdot1.y, Cdot2)));
    J->impulse[0] = J->impulse[0] + impulse.x;
    J->impulse[1] = J->impulse[1] + impulse.y;
    J->impulse[2] = J->impulse[2] + impulse.z;
    v2 P = V(impulse.x, impulse.y);
    va = vsub(va, vscale(ma, P));
    wa = wa - ia * (vcross(ra, P) + impulse.z);
    vb = vadd(vb, vscale(mb, P));
    wb = wb + ib * (vcross(rb, P) + impulse.z);
    vv[k->ia] = va; ww[k->ia] = wa;
    vv[k->ib] = vb; ww[k->ib] = wb;
}

static int weld_solve_position(gb_joint *J, or_jcons *k, v2 *pc, double *pa) {
    v2 ca = pc[k->ia], cb = pc[k->ib];
    double aa = pa[k->ia], ab = pa[k->ib];
    rot qa = rot_of(aa), qb = rot_of(ab);
    double ma = k->ma, mb = k->mb, ia = k->iA, ib = k->iB;
    v2 ra = rmul(qa, vsub(j_la(J), k->lca));
    v2 rb = rmul(qb, vsub(j_lb(J), k->lcb));
    v2 C1 = vsub(vsub(vadd(cb, rb), ca), ra);
    double C2 = ab - aa - J->ref_angle;
    double position_error = vlen(C1);
    double angular_error = fabs(C2);
    double c2x = -ra.y * ra.x * ia - rb.y * rb.x * ib;
    double c3x = -ra.y * ia - rb.y * ib;
    double c3y = ra.x * ia + rb.x * ib;
    m33 mass;
    mass.c1 = V3(ma + mb + ra.y * ra.y * ia + rb.y * rb.y * ib, c2x, c3x);
    mass.c2 = V3(c2x, ma + mb + ra.x * ra.x * ia + rb.x * rb.x * ib, c3y);
    mass.c3 = V3(-ra.y * ia - rb.y * ib, ra.x * ia + rb.x * ib, ia + ib);
    v3 impulse = v3neg(m33_solve3(mass, V3(C1.x, C1.y, C2)));
    v2 P = V(impulse.x, impulse.y);
    ca = vsub(ca, vscale(ma, P));
    aa = aa - ia * (vcross(ra, P) + impulse.z);
    cb = vadd(cb, vscale(mb, P));
    ab = ab + ib * (vcross(rb, P) + impulse.z);
    pc[k->ia] = ca; pa[k->ia] = aa;
    pc[k->ib] = cb; pa[k->ib] = ab;
    return position_error <= OR_LINEAR_SLOP_J && angular_error <= OR_ANGULAR_SLOP;
}

/* ------------------------------------------------------------ friction
 * joints/friction.py:107-233.  Its _solve_velocity_constraints writes the
 * positions back instead of the velocities (friction.py:228-229), so the
 * passes change only the accumulated impulses; the warm start of the set-up
 * is the only velocity change the joint makes. */
static void friction_init(gb_joint *J, or_jcons *k, const double *pa, v2 *vv, double *ww, double dt_ratio, int warm) {
    double ma = k->ma, mb = k->mb, iA = k->iA, iB = k->iB;
    v2 va = vv[k->ia], vb = vv[k->ib];
    double wa = ww[k->ia], wb = ww[k->ib];
    rot qa = rot_of(pa[k->ia]), qb = rot_of(pa[k->ib]);
    v2 ra = k->ra = rmul(qa, vsub(j_la(J), k->lca));
    v2 rb = k->rb = rmul(qb, vsub(j_lb(J), k->lcb));
    double a = ma + mb + iA * ra.y * ra.y + iB * rb.y * rb.y;
    double c = -iA * ra.x * ra.y - iB * rb.x * rb.y;
    double b = c;
    double d = ma + mb + iA * ra.x * ra.x + iB * rb.x * rb.x;
    double det = a * d - b * c;                    /* Mat22.inverse (mat22module.c) */
    if (det != 0.0) det = 1.0 / det;
    k->m.c1 = V3(det * d, -det * c, 0.0);
    k->m.c2 = V3(-det * b, det * a, 0.0);
    k->motor_mass = iA + iB;
    if (k->motor_mass > 0.0) k->motor_mass = 1.0 / k->motor_mass;
    if (warm) {
        J->impulse[0] = J->impulse[0] * dt_ratio;
        J->impulse[1] = J->impulse[1] * dt_ratio;
        J->impulse[2] = J->impulse[2] * dt_ratio;
        v2 P = V(J->impulse[0], J->impulse[1]);
        va = vsub(va, vscale(ma, P));
        wa = wa - iA * (vcross(ra, P) + J->impulse[2]);
        vb = vadd(vb, vscale(mb, P));
        wb = wb + iB * (vcross(rb, P) + J->impulse[2]);
    } else {
        J->impulse[0] = J->impulse[1] = J->impulse[2] = 0.0;
    }
    vv[k->ia] = va; ww[k->ia] = wa;
    vv[k->ib] = vb; ww[k->ib] = wb;
}

static void friction_solve_velocity(gb_joint *J, or_jcons *k, const v2 *vv, const double *ww, double dt) {
    v2 va = vv[k->ia], vb = vv[k->ib];
    double wa = ww[k->ia], wb = ww[k->ib];
    v2 ra = k->ra, rb = k->rb;
    double iA = k->iA, iB = k->iB;
    double Cdot = wb - wa;
    double impulse = -k->motor_mass * Cdot;
    double old_impulse = J->impulse[2];
    double max_impulse = dt * J->max_torque;
    J->impulse[2] = cclamp(J->impulse[2] + impulse, -max_impulse, max_impulse);
    impulse = J->impulse[2] - old_impulse;
    wa = wa - iA * impulse;
    wb = wb + iB * impulse;
    v2 Cdot2 = vsub(vsub(vadd(vb, vcross_sv(wb, rb)), va), vcross_sv(wa, ra));
    v2 li = V(-(k->m.c1.x * Cdot2.x + k->m.c2.x * Cdot2.y), -(k->m.c1.y * Cdot2.x + k->m.c2.y * Cdot2.y));
    v2 acc = V(J->impulse[0] + li.x, J->impulse[1] + li.y);
    double max_force_impulse = dt * J->max_force;
    if (acc.x * acc.x + acc.y * acc.y > SQ(max_force_impulse)) acc = vscale(max_force_impulse, vnormalized(acc));
    J->impulse[0] = acc.x;
    J->impulse[1] = acc.y;
}

/* ------------------------------------------------------------ rope
 * joints/rope.py:106-248.  `u /= length` rebinds the local name only, so the
 * kept `_u` is the unnormalised anchor difference: the velocity passes and
 * the warm start project on it (rope.py:140-149, 186-196). */
static void rope_init(gb_joint *J, or_jcons *k, const v2 *pc, const double *pa, v2 *vv, double *ww, double dt_ratio,
                      int warm) {
    double ma = k->ma, mb = k->mb, ia = k->iA, ib = k->iB;
    v2 ca = pc[k->ia], cb = pc[k->ib];
    v2 va = vv[k->ia], vb = vv[k->ib];
    double wa = ww[k->ia], wb = ww[k->ib];
    rot qa = rot_of(pa[k->ia]), qb = rot_of(pa[k->ib]);
    v2 ra = k->ra = rmul(qa, vsub(j_la(J), k->lca));
    v2 rb = k->rb = rmul(qb, vsub(j_lb(J), k->lcb));
    v2 u = vsub(vsub(vadd(cb, rb), ca), ra);
    J->ux = u.x; J->uy = u.y;
    J->cur_length = vlen(u);
    double C = J->cur_length - J->max_length;
    J->limit_state = C > 0.0 ? GB_LIMIT_UPPER : GB_LIMIT_INACTIVE;
    if (J->cur_length > OR_LINEAR_SLOP_J) {
        u = V(u.x / J->cur_length, u.y / J->cur_length);
    } else {
        k->dmass = 0.0;
        J->impulse[0] = 0.0;
        return;
    }
    double cra = vcross(ra, u), crb = vcross(rb, u);
    double inv_mass = ma + ia * cra * cra + mb + ib * crb * crb;
    k->dmass = inv_mass != 0.0 ? 1.0 / inv_mass : 0.0;
    if (warm) {
        J->impulse[0] = J->impulse[0] * dt_ratio;
        v2 P = vscale(J->impulse[0], V(J->ux, J->uy));
        va = vsub(va, vscale(ma, P));
        wa = wa - ia * vcross(ra, P);
        vb = vadd(vb, vscale(mb, P));
        wb = wb + ib * vcross(rb, P);
    } else {
        J->impulse[0] = 0.0;
    }
    vv[k->ia] = va; ww[k->ia] = wa;
    vv[k->ib] = vb; ww[k->ib] = wb;
}

static void rope_solve_velocity(gb_joint *J, or_jcons *k, v2 *vv, double *ww, double inv_dt) {
    v2 va = vv[k->ia], vb = vv[k->ib];
    double wa = ww[k->ia], wb = ww[k->ib];
    v2 ra = k->ra, rb = k->rb;
    double ma = k->ma, mb = k->mb, ia = k->iA, ib = k->iB;
    v2 u = V(J->ux, J->uy);
    v2 vpa = vadd(va, vcross_sv(wa, ra));
    v2 vpb = vadd(vb, vcross_sv(wb, rb));
    double C = J->cur_length - J->max_length;
    double Cdot = vdot(u, vsub(vpb, vpa));
    if (C < 0.0) Cdot += inv_dt * C;
    double impulse = -k->dmass * Cdot;
    double old_impulse = J->impulse[0];
    J->impulse[0] = pymin(0.0, J->impulse[0] + impulse);
    impulse = J->impulse[0] - old_impulse;
    v2 P = vscale(impulse, u);
    va = vsub(va, vscale(ma, P));
    wa = wa - ia * vcross(ra, P);
    vb = vadd(vb, vscale(mb, P));
    wb = wb + ib * vcross(rb, P);
    vv[k->ia] = va; ww[k->ia] = wa;
    vv[k->ib] = vb; ww[k->ib] = wb;
}

static int rope_solve_position(gb_joint *J, or_jcons *k, v2 *pc, double *pa) {
    v2 ca = pc[k->ia], cb = pc[k->ib];
    double aa = pa[k->ia], ab = pa[k->ib];
    rot qa = rot_of(aa), qb = rot_of(ab);
    double ma = k->ma, mb = k->mb, ia = k->iA, ib = k->iB;
    v2 ra = rmul(qa, vsub(j_la(J), k->lca));
    v2 rb = rmul(qb, vsub(j_lb(J), k->lcb));
    v2 u = vsub(vsub(vadd(cb, rb), ca), ra);
    double length = vlen(u);
    u = vnormalized(u);
    double C = cclamp(length - J->max_length, 0.0, OR_MAX_LINEAR_CORRECTION_J);
    double impulse = -k->dmass * C;
    v2 P = vscale(impulse, u);
    ca = vsub(ca, vscale(ma, P));
    aa = aa - ia * vcross(ra, P);
    cb = vadd(cb, vscale(mb, P));
    ab = ab + ib * vcross(rb, P);
    pc[k->ia] = ca; pa[k->ia] = aa;
    pc[k->ib] = cb; pa[k->ib] = ab;
    return length - J->max_length < OR_LINEAR_SLOP_J;
}

/* ------------------------------------------------------------ wheel
 * joints/wheel.py:202-417.  The spring's axis and arms (_ax, _s_ax, _s_bx)
 * are set only by a set-up with a positive frequency and kept otherwise,
 * and the velocity passes always run the spring and motor rows
 * (wheel.py:329-355); the position pass takes its effective mass from the
 * set-up's arms (wheel.py:397). */
static void wheel_init(gb_joint *J, or_jcons *k, const v2 *pc, const double *pa, v2 *vv, double *ww, double dt,
                       double dt_ratio, int warm) {
    double ma = k->ma, mb = k->mb, ia = k->iA, ib = k->iB;
    v2 ca = pc[k->ia], cb = pc[k->ib];
    v2 va = vv[k->ia], vb = vv[k->ib];
    double wa = ww[k->ia], wb = ww[k->ib];
    rot qa = rot_of(pa[k->ia]), qb = rot_of(pa[k->ib]);
    v2 ra = k->ra = rmul(qa, vsub(j_la(J), k->lca));
    v2 rb = k->rb = rmul(qb, vsub(j_lb(J), k->lcb));
    v2 d = vsub(vsub(vadd(cb, rb), ca), ra);
    v2 ay = k->axis = rmul(qa, j_ly(J));
    J->perp_x = ay.x; J->perp_y = ay.y;            /* _ay, kept for the reaction force */
    double s_ay = k->s1 = vcross(vadd(d, ra), ay);
    double s_by = k->s2 = vcross(rb, ay);
    k->dmass = ma + mb + ia * SQ(s_ay) + ib * SQ(s_by);
    if (k->dmass > 0.0) k->dmass = 1.0 / k->dmass;
    k->a1 = 0.0;                                   /* _spring_mass */
    J->bias = 0.0;
    J->gamma = 0.0;
    if (J->frequency > 0.0) {
        v2 ax = rmul(qa, V(J->ax_x, J->ax_y));
        J->sax_x = ax.x; J->sax_y = ax.y;
        J->s_ax = vcross(vadd(d, ra), ax);
        J->s_bx = vcross(rb, ax);
        double inv_mass = ma + mb + ia * SQ(J->s_ax) + ib * SQ(J->s_bx);
        if (inv_mass > 0.0) {
            k->a1 = 1.0 / inv_mass;
            double C = vdot(d, ax);
            double omega = 2.0 * OR_PI * J->frequency;
            double dd = 2.0 * k->a1 * J->damping_ratio * omega;
            double kk = k->a1 * SQ(omega);
            J->gamma = dt * (dd + dt * kk);
            if (J->gamma > 0.0) J->gamma = 1.0 / J->gamma;
            J->bias = C * dt * kk * J->gamma;
            k->a1 = inv_mass + J->gamma;
            if (k->a1 > 0.0) k->a1 = 1.0 / k->a1;
        }
    } else {
        J->spring_impulse = 0.0;
    }
    if (J->flags & GB_J_MOTOR) {
        k->motor_mass = ia + ib;
        if (k->motor_mass > 0.0) k->motor_mass = 1.0 / k->motor_mass;
    } else {
        k->motor_mass = 0.0;
        J->motor_impulse = 0.0;
    }
    if (warm) {
        J->impulse[0] = J->impulse[0] * dt_ratio;
        J->spring_impulse = J->spring_impulse * dt_ratio;
        J->motor_impulse = J->motor_impulse * dt_ratio;
        double imp = J->impulse[0], si = J->spring_impulse, mi = J->motor_impulse;
        v2 P = vadd(vscale(imp, ay), vscale(si, V(J->sax_x, J->sax_y)));
        double La = imp * s_ay + si * J->s_ax + mi;
        double Lb = imp * s_by + si * J->s_bx + mi;
        va = vsub(va, vscale(ma, P));
        wa = wa - ia * La;
        vb = vadd(vb, vscale(mb, P));
        wb = wb + ib * Lb;
    } else {
        J->impulse[0] = 0.0;
        J->spring_impulse = 0.0;
        J->motor_impulse = 0.0;
    }
    vv[k->ia] = va; ww[k->ia] = wa;
    vv[k->ib] = vb; ww[k->ib] = wb;
}

static void wheel_solve_velocity(gb_joint *J, or_jcons *k, v2 *vv, double *ww, double dt) {
    v2 va = vv[k->ia], vb = vv[k->ib];
    double wa = ww[k->ia], wb = ww[k->ib];
    double ma = k->ma, mb = k->mb, ia = k->iA, ib = k->iB;
    v2 ax = V(J->sax_x, J->sax_y);
    double Cdot = vdot(ax, vsub(vb, va)) + J->s_bx * wb - J->s_ax * wa;
    double impulse = -k->a1 * (Cdot + J->bias + J->gamma * J->spring_impulse);
    J->spring_impulse = J->spring_impulse + impulse;
    v2 P = vscale(impulse, ax);
    double La = impulse * J->s_ax, Lb = impulse * J->s_bx;
    va = vsub(va, vscale(ma, P));
    wa = wa - ia * La;
    vb = vadd(vb, vscale(mb, P));
    wb = wb + ib * Lb;
    Cdot = wb - wa - J->motor_speed;
    impulse = -k->motor_mass * Cdot;
    double old_impulse = J->motor_impulse;
    double max_impulse = dt * J->max_motor;
    J->motor_impulse = cclamp(J->motor_impulse + impulse, -max_impulse, max_impulse);
    impulse = J->motor_impulse - old_impulse;
    wa = wa - ia * impulse;
    wb = wb + ib * impulse;
    Cdot = vdot(k->axis, vsub(vb, va)) + k->s2 * wb - k->s1 * wa;
    impulse = -k->dmass * Cdot;
    J->impulse[0] = J->impulse[0] + impulse;
    P = vscale(impulse, k->axis);
    La = impulse * k->s1; Lb = impulse * k->s2;
    va = vsub(va, vscale(ma, P));
    wa = wa - ia * La;
    vb = vadd(vb, vscale(mb, P));
    wb = wb + ib * Lb;
    vv[k->ia] = va; ww[k->ia] = wa;
    vv[k->ib] = vb; ww[k->ib] = wb;
}

static int wheel_solve_position(gb_joint *J, or_jcons *k, v2 *pc, double *pa) {
    v2 ca = pc[k->ia], cb = pc[k->ib];
    double aa = pa[k->ia], ab = pa[k->ib];
    rot qa = rot_of(aa), qb = rot_of(ab);
    double ma = k->ma, mb = k->mb, ia = k->iA, ib = k->iB;
    v2 ra = rmul(qa, vsub(j_la(J), k->lca));
    v2 rb = rmul(qb, vsub(j_lb(J), k->lcb));
    v2 d = vsub(vadd(vsub(cb, ca), rb), ra);
    double kk = ma + mb + ia * SQ(k->s1) + ib * SQ(k->s2);
    v2 ay = rmul(qa, j_ly(J));
    double s_ay = vcross(vadd(d, ra), ay);
    double s_by = vcross(rb, ay);
    double C = vdot(d, ay);
    double impulse = kk != 0.0 ? -C / kk : 0.0;
    v2 P = vscale(impulse, ay);
    double La = impulse * s_ay, Lb = impulse * s_by;
    ca = vsub(ca, vscale(ma, P));
    aa = aa - ia * La;
    cb = vadd(cb, vscale(mb, P));
    ab = ab + ib * Lb;
    pc[k->ia] = ca; pa[k->ia] = aa;
    pc[k->ib] = cb; pa[k->ib] = ab;
    return fabs(C) <= OR_LINEAR_SLOP_J;
}

/* ------------------------------------------------------------ pulley
 * joints/pulley.py:156-320.  The set-up's warm start and the position pass
 * apply the impulses with the effective masses ma + ia * (ra x ua)^2 (the
 * local names are rebound, pulley.py:190-193, 292-295); the velocity passes
 * take the inverse masses. */
static void pulley_arms(const gb_joint *J, v2 ca, v2 ra, v2 cb, v2 rb, v2 *ua, v2 *ub, double *la, double *lb) {
    v2 a = vsub(vadd(ca, ra), V(J->ga_x, J->ga_y));
    v2 b = vsub(vadd(cb, rb), V(J->gb_x, J->gb_y));
    *la = vlen(a);
    *lb = vlen(b);
    *ua = *la > 10.0 * OR_LINEAR_SLOP_J ? V(a.x / *la, a.y / *la) : V(0.0, 0.0);
    *ub = *lb > 10.0 * OR_LINEAR_SLOP_J ? V(b.x / *lb, b.y / *lb) : V(0.0, 0.0);
}

static void pulley_init(gb_joint *J, or_jcons *k, const v2 *pc, const double *pa, v2 *vv, double *ww, double dt_ratio,
                        int warm) {
    double ia = k->iA, ib = k->iB;
    v2 va = vv[k->ia], vb = vv[k->ib];
    double wa = ww[k->ia], wb = ww[k->ib];
    rot qa = rot_of(pa[k->ia]), qb = rot_of(pa[k->ib]);
    v2 ra = k->ra = rmul(qa, vsub(j_la(J), k->lca));
    v2 rb = k->rb = rmul(qb, vsub(j_lb(J), k->lcb));
    double la, lb;
    pulley_arms(J, pc[k->ia], ra, pc[k->ib], rb, &k->u, &k->perp, &la, &lb);
    double rua = vcross(ra, k->u), rub = vcross(rb, k->perp);
    double ma = k->ma + ia * SQ(rua);
    double mb = k->mb + ib * SQ(rub);
    k->dmass = ma + J->ratio * J->ratio * mb;
    if (k->dmass > 0.0) k->dmass = 1.0 / k->dmass;
    if (warm) {
        J->impulse[0] = J->impulse[0] * dt_ratio;
        v2 Pa = vscale(-J->impulse[0], k->u);
        v2 Pb = vscale(-J->ratio * J->impulse[0], k->perp);
        va = vadd(va, vscale(ma, Pa));
        wa = wa + ia * vcross(ra, Pa);
        vb = vadd(vb, vscale(mb, Pb));
        wb = wb + ib * vcross(rb, Pb);
    } else {
        J->impulse[0] = 0.0;
    }
    vv[k->ia] = va; ww[k->ia] = wa;
    vv[k->ib] = vb; ww[k->ib] = wb;
}

static void pulley_solve_velocity(gb_joint *J, or_jcons *k, v2 *vv, double *ww) {
    v2 va = vv[k->ia], vb = vv[k->ib];
    double wa = ww[k->ia], wb = ww[k->ib];
    v2 ra = k->ra, rb = k->rb;
    double ma = k->ma, mb = k->mb, ia = k->iA, ib = k->iB;
    v2 vpa = vadd(va, vcross_sv(wa, ra));
    v2 vpb = vadd(vb, vcross_sv(wb, rb));
    double Cdot = -vdot(k->u, vpa) - J->ratio * vdot(k->perp, vpb);
    double impulse = -k->dmass * Cdot;
    J->impulse[0] = J->impulse[0] + impulse;
    v2 Pa = vscale(-impulse, k->u);
    v2 Pb = vscale(-J->ratio * impulse, k->perp);
    va = vadd(va, vscale(ma, Pa));
    wa = wa + ia * vcross(ra, Pa);
    vb = vadd(vb, vscale(mb, Pb));
    wb = wb + ib * vcross(rb, Pb);
    vv[k->ia] = va; ww[k->ia] = wa;
    vv[k->ib] = vb; ww[k->ib] = wb;
}

static int pulley_solve_position(gb_joint *J, or_jcons *k, v2 *pc, double *pa) {
    v2 ca = pc[k->ia], cb = pc[k->ib];
    double aa = pa[k->ia], ab = pa[k->ib];
    rot qa = rot_of(aa), qb = rot_of(ab);
    double ia = k->iA, ib = k->iB;
    v2 ra = rmul(qa, vsub(j_la(J), k->lca));
    v2 rb = rmul(qb, vsub(j_lb(J), k->lcb));
    v2 ua, ub;
    double la, lb;
    pulley_arms(J, ca, ra, cb, rb, &ua, &ub, &la, &lb);
    double rua = vcross(ra, ua), rub = vcross(rb, ub);
    double ma = k->ma + ia * SQ(rua);
    double mb = k->mb + ib * SQ(rub);
    double mass = ma + SQ(J->ratio) * mb;
    if (mass > 0.0) mass = 1.0 / mass;
    double C = J->constant - la - J->ratio * lb;
    double linear_error = fabs(C);
    double impulse = -mass * C;
    v2 Pa = vscale(-impulse, ua);
    v2 Pb = vscale(-J->ratio * impulse, ub);
    ca = vadd(ca, vscale(ma, Pa));
    aa = aa + ia * vcross(ra, Pa);
    cb = vadd(cb, vscale(mb, Pb));
    ab = ab + ib * vcross(rb, Pb);
    pc[k->ia] = ca; pa[k->ia] = aa;
    pc[k->ib] = cb; pa[k->ib] = ab;
    return linear_error < OR_LINEAR_SLOP_J;
}

/* ------------------------------------------------------------ mouse
 * joints/mouse.py:138-229: body B pulled towards a target by a soft
 * constraint with a force limit; the record's body_a is body B (the
 * reference's is None), so the island indices coincide and only B's slots
 * are written.  The set-up damps B's angular velocity by 0.98
 * (mouse.py:183). */
static void mouse_init(gb_joint *J, or_jcons *k, const v2 *pc, const double *pa, v2 *vv, double *ww, double dt,
                       double dt_ratio, double body_mass, int warm) {
    double mb = k->mb, ib = k->iB;
    v2 cb = pc[k->ib];
    v2 vb = vv[k->ib];
    double wb = ww[k->ib];
    rot qb = rot_of(pa[k->ib]);
    double mass = body_mass;
    double omega = 2.0 * OR_PI * J->frequency;
    double d = 2.0 * mass * J->damping_ratio * omega;
    double kk = mass * SQ(omega);
    J->gamma = dt * (d + dt * kk);
    if (J->gamma != 0.0) J->gamma = 1.0 / J->gamma;
    J->bias = dt * kk * J->gamma;                 /* _beta */
    v2 rb = k->rb = rmul(qb, vsub(j_lb(J), k->lcb));
    double a = mb + ib * SQ(rb.y) + J->gamma;
    double c = -ib * rb.x * rb.y;
    double b = c;
    double dd = mb + ib * SQ(rb.x) + J->gamma;
    double det = a * dd - b * c;                  /* Mat22.inverse */
    if (det != 0.0) det = 1.0 / det;
    k->m.c1 = V3(det * dd, -det * c, 0.0);
    k->m.c2 = V3(-det * b, det * a, 0.0);
    k->u = vscale(J->bias, vsub(vadd(cb, rb), V(J->target_x, J->target_y)));   /* _c */
    wb = wb * 0.98;
    if (warm) {
        J->impulse[0] = J->impulse[0] * dt_ratio;
        J->impulse[1] = J->impulse[1] * dt_ratio;
        v2 P = V(J->impulse[0], J->impulse[1]);
        vb = vadd(vb, vscale(mb, P));
        wb = wb + ib * vcross(rb, P);
    } else {
        J->impulse[0] = J->impulse[1] = 0.0;
    }
    vv[k->ib] = vb; ww[k->ib] = wb;
}

static void mouse_solve_velocity(gb_joint *J, or_jcons *k, v2 *vv, double *ww, double dt) {
    v2 vb = vv[k->ib];
    double wb = ww[k->ib];
    v2 rb = k->rb;
    v2 Cdot = vadd(vb, vcross_sv(wb, rb));
    v2 acc = V(J->impulse[0], J->impulse[1]);
    v2 e = vneg(vadd(vadd(Cdot, k->u), vscale(J->gamma, acc)));
    v2 impulse = V(k->m.c1.x * e.x + k->m.c2.x * e.y, k->m.c1.y * e.x + k->m.c2.y * e.y);
    v2 old_impulse = acc;
    acc = vadd(acc, impulse);
    double max_impulse = dt * J->max_force;
    if (acc.x * acc.x + acc.y * acc.y > SQ(max_impulse)) {
        double s = max_impulse / sqrt(acc.x * acc.x + acc.y * acc.y);
        acc = V(acc.x * s, acc.y * s);
    }
    J->impulse[0] = acc.x; J->impulse[1] = acc.y;
    impulse = vsub(acc, old_impulse);
    vb = vadd(vb, vscale(k->mb, impulse));
    wb = wb + k->iB * vcross(rb, impulse);
    vv[k->ib] = vb; ww[k->ib] = wb;
}

/* ------------------------------------------------------------ dispatch */
static void joint_init(gb_joint *J, or_jcons *k, const v2 *pc, const double *pa, v2 *vv, double *ww, double dt,
                       double dt_ratio, double body_b_mass, int warm) {
    switch (J->type) {
    case GB_JOINT_MOUSE: mouse_init(J, k, pc, pa, vv, ww, dt, dt_ratio, body_b_mass, warm); break;
    case GB_JOINT_REVOLUTE: revolute_init(J, k, pc, pa, vv, ww, dt_ratio, warm); break;
    case GB_JOINT_PRISMATIC: prismatic_init(J, k, pc, pa, vv, ww, dt_ratio, warm); break;
    case GB_JOINT_DISTANCE: distance_init(J, k, pc, pa, vv, ww, dt, dt_ratio, warm); break;
    case GB_JOINT_FRICTION: friction_init(J, k, pa, vv, ww, dt_ratio, warm); break;
    case GB_JOINT_ROPE: rope_init(J, k, pc, pa, vv, ww, dt_ratio, warm); break;
    case GB_JOINT_WHEEL: wheel_init(J, k, pc, pa, vv, ww, dt, dt_ratio, warm); break;
    case GB_JOINT_PULLEY: pulley_init(J, k, pc, pa, vv, ww, dt_ratio, warm); break;
    default: weld_init(J, k, pc, pa, vv, ww, dt_ratio, warm); break;
    }
}
static void joint_solve_velocity(gb_joint *J, or_jcons *k, v2 *vv, double *ww, double dt) {
    switch (J->type) {
    case GB_JOINT_REVOLUTE: revolute_solve_velocity(J, k, vv, ww, dt); break;
    case GB_JOINT_PRISMATIC: prismatic_solve_velocity(J, k, vv, ww, dt); break;
    case GB_JOINT_DISTANCE: distance_solve_velocity(J, k, vv, ww); break;
    case GB_JOINT_FRICTION: friction_solve_velocity(J, k, vv, ww, dt); break;
    case GB_JOINT_ROPE: rope_solve_velocity(J, k, vv, ww, 1.0 / dt); break;
    case GB_JOINT_WHEEL: wheel_solve_velocity(J, k, vv, ww, dt); break;
    case GB_JOINT_PULLEY: pulley_solve_velocity(J, k, vv, ww); break;
    case GB_JOINT_MOUSE: mouse_solve_velocity(J, k, vv, ww, dt); break;
    default: weld_solve_velocity(J, k, vv, ww); break;
    }
}
static int joint_solve_position(gb_joint *J, or_jcons *k, v2 *pc, double *pa) {
    switch (J->type) {
    case GB_JOINT_REVOLUTE: return revolute_solve_position(J, k, pc, pa);
    case GB_JOINT_PRISMATIC: return prismatic_solve_position(J, k, pc, pa);
    case GB_JOINT_DISTANCE: return distance_solve_position(J, k, pc, pa);
    case GB_JOINT_FRICTION: return 1;
    case GB_JOINT_ROPE: return rope_solve_position(J, k, pc, pa);
    case GB_JOINT_WHEEL: return wheel_solve_position(J, k, pc, pa);
    case GB_JOINT_PULLEY: return pulley_solve_position(J, k, pc, pa);
    case GB_JOINT_MOUSE: return 1;
    default: return weld_solve_position(J, k, pc, pa);
    }
}

#endif /* ORACLE_JOINTS_H */

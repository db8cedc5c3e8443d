// gb_joints.cuh -- the joint constraints the island solver runs beside the
// contacts (island.py:107-113, 145-148): revolute (joints/revolute.py:240-453),
// prismatic (joints/prismatic.py:238-513), distance (joints/distance.py:175-311),
// weld (joints/weld.py:118-257), friction (joints/friction.py:107-233), rope
// (joints/rope.py:106-248), wheel (joints/wheel.py:202-417), pulley
// (joints/pulley.py:156-320) and mouse (joints/mouse.py:138-229).
//
// Joints are few next to contacts, so they are solved in float64 in both
// precision units: the float32 unit widens the bodies' velocities for the
// joint passes and rounds them back.  Every expression keeps the reference's
// operation order (with -fmad=false the float64 unit reproduces it bit for
// bit).  Two properties of the reference's math types fix that arithmetic:
// its C Vec2 has no in-place operators, so `u *= s` rebinds the name and the
// distance joint's effective mass is formed with the unnormalised direction
// (distance.py:212-222); Vec3 and Mat33 are Python classes whose dot, cross
// and solves (common.py:227-612) are written out below as they are there.
#pragma once
#include "gb_world.cuh"

#define GB_ANGULAR_SLOP_J (2.0 / 180.0 * 3.141592653589793)       // settings.py:65
#define GB_MAX_ANGULAR_CORRECTION (8.0 / 180.0 * 3.141592653589793) // settings.py:94
#define GB_LINEAR_SLOP_J 0.005
#define GB_MAX_LINEAR_CORRECTION_J 0.2

static __device__ __forceinline__ d3 mk3(double x, double y, double z) { d3 r; r.x = x; r.y = y; r.z = z; return r; }
static __device__ __forceinline__ double dot3(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static __device__ __forceinline__ d3 cross3(d3 s, d3 v) {
    return mk3(s.y * v.z - s.z * v.y, s.z * v.x - s.x * v.z, s.x * v.y - s.y * v.x);
}
static __device__ __forceinline__ d3 add3(d3 a, d3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
static __device__ __forceinline__ d3 sub3(d3 a, d3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
static __device__ __forceinline__ d3 neg3(d3 a) { return mk3(-a.x, -a.y, -a.z); }
// Mat33.solve3x3
static __device__ __forceinline__ d3 solve33(const m33d &m, d3 b) {
    double det = dot3(m.c1, cross3(m.c2, m.c3));
    if (det != 0.0) det = 1.0 / det;
    return mk3(det * dot3(b, cross3(m.c2, m.c3)), det * dot3(m.c1, cross3(b, m.c3)), det * dot3(m.c1, cross3(m.c2, b)));
}
// Mat33.solve2x2 (upper-left block); Mat22.solve has the same form
static __device__ __forceinline__ vec2<double> solve22(double a11, double a21, double a12, double a22, vec2<double> v) {
    double det = a11 * a22 - a12 * a21;
    if (det != 0.0) det = 1.0 / det;
    return mk<double>(det * (a22 * v.x - a12 * v.y), det * (a11 * v.y - a21 * v.x));
}
static __device__ __forceinline__ vec2<double> solve22(const m33d &m, vec2<double> v) {
    return solve22(m.c1.x, m.c1.y, m.c2.x, m.c2.y, v);
}

static __device__ __forceinline__ vec2<double> j_la(const gb_joint &J) { return mk<double>(J.la_x, J.la_y); }
static __device__ __forceinline__ vec2<double> j_lb(const gb_joint &J) { return mk<double>(J.lb_x, J.lb_y); }
// `_impulse -= (0, 0, _impulse.z)`
static __device__ __forceinline__ void j_drop_z(gb_joint &J) { J.impulse[2] = J.impulse[2] - J.impulse[2]; }
// prismatic.py:85: local y axis = scalar_cross(1.0, local x axis)
static __device__ __forceinline__ vec2<double> j_ly(const gb_joint &J) { return cross(1.0, mk<double>(J.ax_x, J.ax_y)); }

// ------------------------------------------------------------ revolute
static __device__ void revolute_init(gb_joint &J, JCons &k, double aa, double ab, vec2<double> &va, double &wa,
                                     vec2<double> &vb, double &wb, double dt_ratio, bool warm) {
    const double ma = k.ma, mb = k.mb, ia = k.iA, ib = k.iB;
    const rot2<double> qa = pose_rot(aa), qb = pose_rot(ab);
    const vec2<double> ra = k.ra = rmul(qa, j_la(J) - k.lca);
    const vec2<double> rb = k.rb = rmul(qb, j_lb(J) - k.lcb);
    k.m.c3 = mk3(-ra.y * ia - rb.y * ib, ra.x * ia + rb.x * ib, ia + ib);
    k.m.c2 = mk3(-ra.y * ra.x * ia - rb.y * rb.x * ib, ma + mb + ra.x * ra.x * ia + rb.x * rb.x * ib, k.m.c3.y);
    k.m.c1 = mk3(ma + mb + ra.y * ra.y * ia + rb.y * rb.y * ib, k.m.c2.x, k.m.c3.x);
    k.motor_mass = ia + ib;
    const bool fixed_rotation = k.motor_mass == 0.0;
    if (k.motor_mass > 0.0) k.motor_mass = 1.0 / k.motor_mass;
    if (!(J.flags & GB_J_MOTOR) || fixed_rotation) J.motor_impulse = 0.0;
    if ((J.flags & GB_J_LIMIT) && !fixed_rotation) {
        const double joint_angle = ab - aa - J.ref_angle;
        if (fabs(J.upper - J.lower) < 2.0 * GB_ANGULAR_SLOP_J) {
            J.limit_state = GB_LIMIT_EQUAL;
        } else if (joint_angle <= J.lower) {
            if (J.limit_state != GB_LIMIT_LOWER) j_drop_z(J);
            J.limit_state = GB_LIMIT_LOWER;
        } else if (joint_angle >= J.upper) {
            if (J.limit_state != GB_LIMIT_UPPER) j_drop_z(J);
            J.limit_state = GB_LIMIT_UPPER;
        } else {
            J.limit_state = GB_LIMIT_INACTIVE;
            j_drop_z(J);
        }
    } else {
        J.limit_state = GB_LIMIT_INACTIVE;
    }
    if (warm) {
        J.impulse[0] = dt_ratio * J.impulse[0];
        J.impulse[1] = dt_ratio * J.impulse[1];
        J.impulse[2] = dt_ratio * J.impulse[2];
        J.motor_impulse = J.motor_impulse * dt_ratio;
        const vec2<double> P = mk<double>(J.impulse[0], J.impulse[1]);
        va = va - ma * P;
        wa = wa - ia * (cross(ra, P) + J.motor_impulse + J.impulse[2]);
        vb = vb + mb * P;
        wb = wb + ib * (cross(rb, P) + J.motor_impulse + J.impulse[2]);
    } else {
        J.impulse[0] = J.impulse[1] = J.impulse[2] = 0.0;
        J.motor_impulse = 0.0;
    }
}

static __device__ void revolute_velocity(gb_joint &J, const JCons &k, vec2<double> &va, double &wa, vec2<double> &vb,
                                         double &wb, double dt) {
    const double ma = k.ma, mb = k.mb, ia = k.iA, ib = k.iB;
    const vec2<double> ra = k.ra, rb = k.rb;
    const bool fixed_rotation = (ia + ib) == 0.0;
    if ((J.flags & GB_J_MOTOR) && J.limit_state != GB_LIMIT_EQUAL && !fixed_rotation) {
        const double Cdot = wb - wa - J.motor_speed;
        double impulse = k.motor_mass * (-Cdot);
        const double old_impulse = J.motor_impulse;
        const double max_impulse = dt * J.max_motor;
        J.motor_impulse = cclamp(J.motor_impulse + impulse, -max_impulse, max_impulse);
        impulse = J.motor_impulse - old_impulse;
        wa = wa - ia * impulse;
        wb = wb + ib * impulse;
    }
    if ((J.flags & GB_J_LIMIT) && J.limit_state != GB_LIMIT_INACTIVE && !fixed_rotation) {
        const vec2<double> Cdot1 = vb + cross(wb, rb) - va - cross(wa, ra);
        const double Cdot2 = wb - wa;
        d3 impulse = neg3(solve33(k.m, mk3(Cdot1.x, Cdot1.y, Cdot2)));
        d3 acc = mk3(J.impulse[0], J.impulse[1], J.impulse[2]);
        if (J.limit_state == GB_LIMIT_EQUAL) {
            acc = add3(acc, impulse);
        } else {
            const double new_impulse = acc.z + impulse.z;
            const bool clip = J.limit_state == GB_LIMIT_LOWER ? new_impulse < 0.0 : new_impulse > 0.0;
            if (clip) {
                const vec2<double> rhs = -Cdot1 + acc.z * mk<double>(k.m.c3.x, k.m.c3.y);
                const vec2<double> reduced = solve22(k.m, rhs);
                impulse = mk3(reduced.x, reduced.y, -acc.z);
                acc = add3(acc, mk3(reduced.x, reduced.y, -acc.z));
            } else {
                acc = add3(acc, impulse);
            }
        }
        J.impulse[0] = acc.x; J.impulse[1] = acc.y; J.impulse[2] = acc.z;
        const vec2<double> P = mk<double>(impulse.x, impulse.y);
        va = va - ma * P;
        wa = wa - ia * (cross(ra, P) + impulse.z);
        vb = vb + mb * P;
        wb = wb + ib * (cross(rb, P) + impulse.z);
    } else {
        const vec2<double> Cdot = vb + cross(wb, rb) - va - cross(wa, ra);
        const vec2<double> impulse = solve22(k.m, -Cdot);
        J.impulse[0] = J.impulse[0] + impulse.x;
        J.impulse[1] = J.impulse[1] + impulse.y;
        J.impulse[2] = J.impulse[2] + 0.0;
        va = va - ma * impulse;
        wa = wa - ia * cross(ra, impulse);
        vb = vb + mb * impulse;
        wb = wb + ib * cross(rb, impulse);
    }
}

static __device__ bool revolute_position(const gb_joint &J, const JCons &k, vec2<double> &ca, double &aa,
                                         vec2<double> &cb, double &ab) {
    const double ma = k.ma, mb = k.mb, ia = k.iA, ib = k.iB;
    const bool fixed_rotation = (ia + ib) == 0.0;
    double angular_error = 0.0, position_error = 0.0;
    if ((J.flags & GB_J_LIMIT) && J.limit_state != GB_LIMIT_INACTIVE && !fixed_rotation) {
        const double angle = ab - aa - J.ref_angle;
        double limit_impulse = 0.0;
        if (J.limit_state == GB_LIMIT_EQUAL) {
            const double C = cclamp(angle - J.lower, -GB_MAX_ANGULAR_CORRECTION, GB_MAX_ANGULAR_CORRECTION);
            limit_impulse = -k.motor_mass * C;
            angular_error = fabs(C);
        } else if (J.limit_state == GB_LIMIT_LOWER) {
            double C = angle - J.lower;
            angular_error = -C;
            C = cclamp(C + GB_ANGULAR_SLOP_J, -GB_MAX_ANGULAR_CORRECTION, 0.0);
            limit_impulse = -k.motor_mass * C;
        } else {
            double C = angle - J.upper;
            angular_error = C;
            C = cclamp(C - GB_ANGULAR_SLOP_J, 0.0, GB_MAX_ANGULAR_CORRECTION);
            limit_impulse = -k.motor_mass * C;
        }
        aa = aa - ia * limit_impulse;
        ab = ab + ib * limit_impulse;
    }
    const rot2<double> qa = pose_rot(aa), qb = pose_rot(ab);
    const vec2<double> ra = rmul(qa, j_la(J) - k.lca);
    const vec2<double> rb = rmul(qb, j_lb(J) - k.lcb);
    const vec2<double> C = cb + rb - ca - ra;
    position_error = len(C);
    const double rax = ra.x, ray = ra.y, rbx = rb.x, rby = rb.y;
    const double k11 = ma + mb + ia * ray * ray + ib * rby * rby;
    const double k21 = -ia * rax * ray - ib * rbx * rby;
    const double k22 = ma + mb + ia * rax * rax + ib * rbx * rbx;
    const vec2<double> impulse = -solve22(k11, k21, k21, k22, C);   // Mat22.solve (mat22module.c:500-516)
    ca = ca - ma * impulse;
    aa = aa - ia * cross(ra, impulse);
    cb = cb + mb * impulse;
    ab = ab + ib * cross(rb, impulse);
    return position_error <= GB_LINEAR_SLOP_J && angular_error <= GB_ANGULAR_SLOP_J;
}

// ------------------------------------------------------------ prismatic
static __device__ void prismatic_init(gb_joint &J, JCons &k, vec2<double> ca, double aa, vec2<double> cb, double ab,
                                      vec2<double> &va, double &wa, vec2<double> &vb, double &wb, double dt_ratio,
                                      bool warm) {
    const double ma = k.ma, mb = k.mb, ia = k.iA, ib = k.iB;
    const rot2<double> qa = pose_rot(aa), qb = pose_rot(ab);
    const vec2<double> ra = k.ra = rmul(qa, j_la(J) - k.lca);
    const vec2<double> rb = k.rb = rmul(qb, j_lb(J) - k.lcb);
    const vec2<double> d = cb + rb - ca - ra;
    const vec2<double> axis = k.axis = rmul(qa, mk<double>(J.ax_x, J.ax_y));
    const double a1 = k.a1 = cross(d + ra, axis);
    const double a2 = k.a2 = cross(rb, axis);
    k.motor_mass = ma + mb + ia * sq(a1) + ib * sq(a2);
    if (k.motor_mass > 0.0) k.motor_mass = 1.0 / k.motor_mass;
    const vec2<double> perp = k.perp = rmul(qa, j_ly(J));
    const double s1 = k.s1 = cross(d + ra, perp);
    const double s2 = k.s2 = cross(rb, perp);
    const double k11 = ma + mb + ia * sq(s1) + ib * sq(s2);
    const double k12 = ia * s1 + ib * s2;
    const double k13 = ia * s1 * a1 + ib * s2 * a2;
    double k22 = ia + ib;
    if (k22 == 0.0) k22 = 1.0;
    const double k23 = ia * a1 + ib * a2;
    const double k33 = ma + mb + ia * sq(a1) + ib * sq(a2);
    k.m.c1 = mk3(k11, k12, k13);
    k.m.c2 = mk3(k12, k22, k23);
    k.m.c3 = mk3(k13, k23, k33);
    if (J.flags & GB_J_LIMIT) {
        const double joint_translation = dot(axis, d);
        if (fabs(J.upper - J.lower) < 2.0 * GB_LINEAR_SLOP_J) {
            J.limit_state = GB_LIMIT_EQUAL;
        } else if (joint_translation <= J.lower) {
            if (J.limit_state != GB_LIMIT_LOWER) { J.limit_state = GB_LIMIT_LOWER; j_drop_z(J); }
        } else if (joint_translation >= J.upper) {
            if (J.limit_state != GB_LIMIT_UPPER) { J.limit_state = GB_LIMIT_UPPER; j_drop_z(J); }
        } else {
            J.limit_state = GB_LIMIT_INACTIVE;
            j_drop_z(J);
        }
    } else {
        J.limit_state = GB_LIMIT_INACTIVE;
        j_drop_z(J);
    }
    if (!(J.flags & GB_J_MOTOR)) J.motor_impulse = 0.0;
    if (warm) {
        J.impulse[0] = dt_ratio * J.impulse[0];
        J.impulse[1] = dt_ratio * J.impulse[1];
        J.impulse[2] = dt_ratio * J.impulse[2];
        J.motor_impulse = J.motor_impulse * dt_ratio;
        const double ix = J.impulse[0], iy = J.impulse[1], iz = J.impulse[2], mi = J.motor_impulse;
        const vec2<double> P = ix * perp + (mi + iz) * axis;
        const double L1 = ix * s1 + iy + (mi + iz) * a1;
        const double L2 = ix * s2 + iy + (mi + iz) * a2;
        va = va - ma * P;
        wa = wa - ia * L1;
        vb = vb + mb * P;
        wb = wb + ib * L2;
    } else {
        J.impulse[0] = J.impulse[1] = J.impulse[2] = 0.0;
        J.motor_impulse = 0.0;
    }
    J.ux = axis.x; J.uy = axis.y;
    J.perp_x = perp.x; J.perp_y = perp.y;
}

static __device__ void prismatic_velocity(gb_joint &J, const JCons &k, vec2<double> &va, double &wa, vec2<double> &vb,
                                          double &wb, double dt) {
    const double ma = k.ma, mb = k.mb, ia = k.iA, ib = k.iB;
    const double a1 = k.a1, a2 = k.a2, s1 = k.s1, s2 = k.s2;
    const vec2<double> perp = k.perp, axis = k.axis;
    if ((J.flags & GB_J_MOTOR) && J.limit_state != GB_LIMIT_EQUAL) {
        const double Cdot = dot(axis, vb - va) + a2 * wb - a1 * wa;
        double impulse = k.motor_mass * (J.motor_speed - Cdot);
        const double old_impulse = J.motor_impulse;
        const double max_impulse = dt * J.max_motor;
        J.motor_impulse = cclamp(J.motor_impulse + impulse, -max_impulse, max_impulse);
        impulse = J.motor_impulse - old_impulse;
        const vec2<double> P = impulse * axis;
        const double L1 = impulse * a1, L2 = impulse * a2;
        va = va - ma * P;
        wa = wa - ia * L1;
        vb = vb + mb * P;
        wb = wb + ib * L2;
    }
    const vec2<double> Cdot1 = mk<double>(dot(perp, vb - va) + s2 * wb - s1 * wa, wb - wa);
    vec2<double> P;
    double L1, L2;
    if ((J.flags & GB_J_LIMIT) && J.limit_state != GB_LIMIT_INACTIVE) {
        const double Cdot2 = dot(axis, vb - va) + a2 * wb - a1 * wa;
        const d3 old = mk3(J.impulse[0], J.impulse[1], J.impulse[2]);
        d3 df = solve33(k.m, neg3(mk3(Cdot1.x, Cdot1.y, Cdot2)));
        d3 acc = add3(old, df);
        double iz;
        if (J.limit_state == GB_LIMIT_LOWER) iz = pymax(acc.z, 0.0);
        else if (J.limit_state == GB_LIMIT_UPPER) iz = pymin(acc.z, 0.0);
        else iz = acc.z;
        const vec2<double> b = -Cdot1 - (acc.z - old.z) * mk<double>(k.m.c3.x, k.m.c3.y);
        const vec2<double> f2r = solve22(k.m, b) + mk<double>(old.x, old.y);
        acc = mk3(f2r.x, f2r.y, iz);
        J.impulse[0] = acc.x; J.impulse[1] = acc.y; J.impulse[2] = acc.z;
        df = sub3(acc, old);
        P = df.x * perp + df.z * axis;
        L1 = df.x * s1 + df.y + df.z * a1;
        L2 = df.x * s2 + df.y + df.z * a2;
    } else {
        const vec2<double> df = solve22(k.m, -Cdot1);
        J.impulse[0] = J.impulse[0] + df.x;
        J.impulse[1] = J.impulse[1] + df.y;
        J.impulse[2] = J.impulse[2] + 0.0;
        P = df.x * perp;
        L1 = df.x * s1 + df.y;
        L2 = df.x * s2 + df.y;
    }
    va = va - ma * P;
    wa = wa - ia * L1;
    vb = vb + mb * P;
    wb = wb + ib * L2;
}

static __device__ bool prismatic_position(const gb_joint &J, const JCons &k, vec2<double> &ca, double &aa,
                                          vec2<double> &cb, double &ab) {
    const double ma = k.ma, mb = k.mb, ia = k.iA, ib = k.iB;
    const rot2<double> qa = pose_rot(aa), qb = pose_rot(ab);
    const vec2<double> ra = rmul(qa, j_la(J) - k.lca);
    const vec2<double> rb = rmul(qb, j_lb(J) - k.lcb);
    const vec2<double> d = cb + rb - ca - ra;
    const vec2<double> axis = rmul(qa, mk<double>(J.ax_x, J.ax_y));
    const double a1 = cross(d + ra, axis);
    const double a2 = cross(rb, axis);
    const vec2<double> perp = rmul(qa, j_ly(J));
    const double s1 = cross(d + ra, perp);
    const double s2 = cross(rb, perp);
    const vec2<double> C1 = mk<double>(dot(perp, d), ab - aa - J.ref_angle);
    double linear_error = fabs(C1.x);
    const double angular_error = fabs(C1.y);
    bool active = false;
    double C2 = 0.0;
    if (J.flags & GB_J_LIMIT) {
        const double translation = dot(axis, d);
        if (fabs(J.upper - J.lower) < 2.0 * GB_LINEAR_SLOP_J) {
            C2 = cclamp(translation, -GB_MAX_LINEAR_CORRECTION_J, GB_MAX_LINEAR_CORRECTION_J);
            linear_error = pymax(linear_error, translation);
            active = true;
        } else if (translation <= J.lower) {
            C2 = cclamp(translation - J.lower + GB_LINEAR_SLOP_J, -GB_MAX_LINEAR_CORRECTION_J, 0.0);
            linear_error = pymax(linear_error, J.lower - translation);
            active = true;
        } else if (translation >= J.upper) {
            C2 = cclamp(translation - J.upper - GB_LINEAR_SLOP_J, 0.0, GB_MAX_LINEAR_CORRECTION_J);
            linear_error = pymax(linear_error, translation - J.upper);
            active = true;
        }
    }
    double ix, iy, iz;
    if (active) {
        const double k11 = ma + mb + ia * sq(s1) + ib * sq(s2);
        const double k12 = ia * s1 + ib * s2;
        const double k13 = ia * s1 * a1 + ib * s2 * a2;
        double k22 = ia + ib;
        if (k22 == 0.0) k22 = 1.0;
        const double k23 = ia * a1 + ib * a2;
        const double k33 = ma + mb + ia * sq(a1) + ib * sq(a2);
        m33d K;
        K.c1 = mk3(k11, k12, k13); K.c2 = mk3(k12, k22, k23); K.c3 = mk3(k13, k23, k33);
        const d3 impulse = solve33(K, neg3(mk3(C1.x, C1.y, C2)));
        ix = impulse.x; iy = impulse.y; iz = impulse.z;
    } else {
        const double k11 = ma + mb + ia * s1 * s1 + ib * s2 * s2;
        const double k12 = ia * s1 + ib * s2;
        double k22 = ia + ib;
        if (k22 == 0.0) k22 = 1.0;
        const vec2<double> impulse1 = solve22(k11, k12, k12, k22, -C1);
        ix = impulse1.x; iy = impulse1.y; iz = 0.0;
    }
    const vec2<double> P = ix * perp + iz * axis;
    const double L1 = ix * s1 + iy + iz * a1;
    const double L2 = ix * s2 + iy + iz * a2;
    ca = ca - ma * P;
    cb = cb + mb * P;
    aa = aa - ia * L1;
    ab = ab + ib * L2;
    return (linear_error <= GB_LINEAR_SLOP_J) && (angular_error <= GB_ANGULAR_SLOP_J);
}

// ------------------------------------------------------------ distance
static __device__ void distance_init(gb_joint &J, JCons &k, vec2<double> ca, double aa, vec2<double> cb, double ab,
                                     vec2<double> &va, double &wa, vec2<double> &vb, double &wb, double dt,
                                     double dt_ratio, bool warm) {
    const double ma = k.ma, mb = k.mb, iA = k.iA, iB = k.iB;
    const rot2<double> qa = pose_rot(aa), qb = pose_rot(ab);
    const vec2<double> ra = k.ra = rmul(qa, j_la(J) - k.lca);
    const vec2<double> rb = k.rb = rmul(qb, j_lb(J) - k.lcb);
    const vec2<double> u = cb + rb - ca - ra;   // the mass below uses this unnormalised vector
    const double length = len(u);
    k.u = length > GB_LINEAR_SLOP_J ? (1.0 / length) * u : mk<double>(0.0, 0.0);
    const double cr_au = sq(cross(ra, u));
    const double cr_bu = sq(cross(rb, u));
    const double inv_mass = ma + iA * cr_au + mb + iB * cr_bu;
    k.dmass = inv_mass != 0.0 ? 1.0 / inv_mass : 0.0;
    if (J.frequency > 0.0) {
        const double C = length - J.length;
        const double omega = 2.0 * 3.141592653589793 * J.frequency;
        const double dd = 2.0 * k.dmass * J.damping_ratio * omega;
        const double kk = k.dmass * sq(omega);
        const double gamma = dt * (dd + dt * kk);
        J.gamma = gamma != 0.0 ? 1.0 / gamma : 0.0;
        J.bias = C * dt * kk * J.gamma;
        const double mass = inv_mass + J.gamma;
        k.dmass = mass != 0.0 ? 1.0 / mass : 0.0;
    }
    if (warm) {
        J.impulse[0] = J.impulse[0] * dt_ratio;
        const vec2<double> P = J.impulse[0] * k.u;
        va = va - ma * P;
        wa = wa - iA * cross(ra, P);
        vb = vb + mb * P;
        wb = wb + iB * cross(rb, P);
    } else {
        J.impulse[0] = 0.0;
    }
    J.ux = k.u.x; J.uy = k.u.y;
}

static __device__ void distance_velocity(gb_joint &J, const JCons &k, vec2<double> &va, double &wa, vec2<double> &vb,
                                         double &wb) {
    const vec2<double> vpa = va + cross(wa, k.ra);
    const vec2<double> vpb = vb + cross(wb, k.rb);
    const double Cdot = dot(k.u, vpb - vpa);
    const double impulse = -k.dmass * (Cdot + J.bias + J.gamma * J.impulse[0]);
    J.impulse[0] = J.impulse[0] + impulse;
    const vec2<double> P = impulse * k.u;
    va = va - k.ma * P;
    wa = wa - k.iA * cross(k.ra, P);
    vb = vb + k.mb * P;
    wb = wb + k.iB * cross(k.rb, P);
}

static __device__ bool distance_position(const gb_joint &J, const JCons &k, vec2<double> &ca, double &aa,
                                         vec2<double> &cb, double &ab) {
    if (J.frequency > 0.0) return true;   // soft constraints have no position correction
    const rot2<double> qa = pose_rot(aa), qb = pose_rot(ab);
    const vec2<double> ra = rmul(qa, j_la(J) - k.lca);
    const vec2<double> rb = rmul(qb, j_lb(J) - k.lcb);
    vec2<double> u = cb + rb - ca - ra;
    const double length = len(u);
    u = normalized(u);
    const double C = length - J.length;
    const double impulse = -k.dmass * cclamp(C, -GB_MAX_LINEAR_CORRECTION_J, GB_MAX_LINEAR_CORRECTION_J);
    const vec2<double> P = impulse * u;
    ca = ca - k.ma * P;
    aa = aa - k.iA * cross(ra, P);
    cb = cb + k.mb * P;
    ab = ab + k.iB * cross(rb, P);
    return fabs(C) < GB_LINEAR_SLOP_J;
}

// ------------------------------------------------------------ weld
static __device__ void weld_init(gb_joint &J, JCons &k, double aa, double ab, vec2<double> &va, double &wa,
                                 vec2<double> &vb, double &wb, double dt_ratio, bool warm) {
    const double ma = k.ma, mb = k.mb, ia = k.iA, ib = k.iB;
    const rot2<double> qa = pose_rot(aa), qb = pose_rot(ab);
    const vec2<double> ra = k.ra = rmul(qa, j_la(J) - k.lca);
    const vec2<double> rb = k.rb = rmul(qb, j_lb(J) - k.lcb);
    const double c2x = -ra.y * ra.x * ia - rb.y * rb.x * ib;
    const double c3x = -ra.y * ia - rb.y * ib;
    k.m.c1 = mk3(ma + mb + ra.y * ra.y * ia + rb.y * rb.y * ib, c2x, c3x);
    k.m.c2 = mk3(c2x, ma + mb + ra.x * ra.x * ia + rb.x * rb.x * ib, c3x);   // weld.py:163-165 keeps c3x here
    k.m.c3 = mk3(c3x, ra.x * ia + rb.x * ib, ia + ib);
    if (warm) {
        J.impulse[0] = dt_ratio * J.impulse[0];
        J.impulse[1] = dt_ratio * J.impulse[1];
        J.impulse[2] = dt_ratio * J.impulse[2];
        const vec2<double> P = mk<double>(J.impulse[0], J.impulse[1]);
        va = va - ma * P;
        wa = wa - ia * (cross(ra, P) + J.impulse[2]);
        vb = vb + mb * P;
        wb = wb + ib * (cross(rb, P) + J.impulse[2]);
    } else {
        J.impulse[0] = J.impulse[1] = J.impulse[2] = 0.0;
    }
}

static __device__ void weld_velocity(gb_joint &J, const JCons &k, vec2<double> &va, double &wa, vec2<double> &vb,
                                     double &wb) {
    const vec2<double> Cdot1 = vb + cross(wb, k.rb) - va - cross(wa, k.ra);
    const double Cdot2 = wb - wa;
    const d3 impulse = solve33(k.m, neg3(mk3(Cdot1.x, Cdot1.y, Cdot2)));
    J.impulse[0] = J.impulse[0] + impulse.x;
    J.impulse[1] = J.impulse[1] + impulse.y;
    J.impulse[2] = J.impulse[2] + impulse.z;
    const vec2<double> P = mk<double>(impulse.x, impulse.y);
    va = va - k.ma * P;
    wa = wa - k.iA * (cross(k.ra, P) + impulse.z);
    vb = vb + k.mb * P;
    wb = wb + k.iB * (cross(k.rb, P) + impulse.z);
}

static __device__ bool weld_position(const gb_joint &J, const JCons &k, vec2<double> &ca, double &aa, vec2<double> &cb,
                                     double &ab) {
    const double ma = k.ma, mb = k.mb, ia = k.iA, ib = k.iB;
    const rot2<double> qa = pose_rot(aa), qb = pose_rot(ab);
    const vec2<double> ra = rmul(qa, j_la(J) - k.lca);
    const vec2<double> rb = rmul(qb, j_lb(J) - k.lcb);
    const vec2<double> C1 = cb + rb - ca - ra;
    const double C2 = ab - aa - J.ref_angle;
    const double position_error = len(C1);
    const double angular_error = fabs(C2);
    const double c2x = -ra.y * ra.x * ia - rb.y * rb.x * ib;
    const double c3x = -ra.y * ia - rb.y * ib;
    const double c3y = ra.x * ia + rb.x * ib;
    m33d mass;
    mass.c1 = mk3(ma + mb + ra.y * ra.y * ia + rb.y * rb.y * ib, c2x, c3x);
    mass.c2 = mk3(c2x, ma + mb + ra.x * ra.x * ia + rb.x * rb.x * ib, c3y);
    mass.c3 = mk3(-ra.y * ia - rb.y * ib, ra.x * ia + rb.x * ib, ia + ib);
    const d3 impulse = neg3(solve33(mass, mk3(C1.x, C1.y, C2)));
    const vec2<double> P = mk<double>(impulse.x, impulse.y);
    ca = ca - ma * P;
    aa = aa - ia * (cross(ra, P) + impulse.z);
    cb = cb + mb * P;
    ab = ab + ib * (cross(rb, P) + impulse.z);
    return position_error <= GB_LINEAR_SLOP_J && angular_error <= GB_ANGULAR_SLOP_J;
}

// ------------------------------------------------------------ friction
// Mat22.inverse of the symmetric effective mass (mat22module.c); the velocity
// passes change only the accumulated impulses: the reference writes the
// positions back where the velocities belong (friction.py:228-229).
static __device__ void friction_init(gb_joint &J, JCons &k, double aa, double ab, vec2<double> &va, double &wa,
                                     vec2<double> &vb, double &wb, double dt_ratio, bool warm) {
    const double ma = k.ma, mb = k.mb, iA = k.iA, iB = k.iB;
    const rot2<double> qa = pose_rot(aa), qb = pose_rot(ab);
    const vec2<double> ra = k.ra = rmul(qa, j_la(J) - k.lca);
    const vec2<double> rb = k.rb = rmul(qb, j_lb(J) - k.lcb);
    const double a = ma + mb + iA * ra.y * ra.y + iB * rb.y * rb.y;
    const double c = -iA * ra.x * ra.y - iB * rb.x * rb.y;
    const double b = c;
    const double d = ma + mb + iA * ra.x * ra.x + iB * rb.x * rb.x;
    double det = a * d - b * c;
    if (det != 0.0) det = 1.0 / det;
    k.m.c1 = mk3(det * d, -det * c, 0.0);
    k.m.c2 = mk3(-det * b, det * a, 0.0);
    k.motor_mass = iA + iB;
    if (k.motor_mass > 0.0) k.motor_mass = 1.0 / k.motor_mass;
    if (warm) {
        J.impulse[0] = J.impulse[0] * dt_ratio;
        J.impulse[1] = J.impulse[1] * dt_ratio;
        J.impulse[2] = J.impulse[2] * dt_ratio;
        const vec2<double> P = mk<double>(J.impulse[0], J.impulse[1]);
        va = va - ma * P;
        wa = wa - iA * (cross(ra, P) + J.impulse[2]);
        vb = vb + mb * P;
        wb = wb + iB * (cross(rb, P) + J.impulse[2]);
    } else {
        J.impulse[0] = J.impulse[1] = J.impulse[2] = 0.0;
    }
}

static __device__ void friction_velocity(gb_joint &J, const JCons &k, vec2<double> va, double wa, vec2<double> vb,
                                         double wb, double dt) {
    const double Cdot = wb - wa;
    double impulse = -k.motor_mass * Cdot;
    const double old_impulse = J.impulse[2];
    const double max_impulse = dt * J.max_torque;
    J.impulse[2] = cclamp(J.impulse[2] + impulse, -max_impulse, max_impulse);
    impulse = J.impulse[2] - old_impulse;
    wa = wa - k.iA * impulse;
    wb = wb + k.iB * impulse;
    const vec2<double> Cdot2 = vb + cross(wb, k.rb) - va - cross(wa, k.ra);
    const vec2<double> li = mk<double>(-(k.m.c1.x * Cdot2.x + k.m.c2.x * Cdot2.y), -(k.m.c1.y * Cdot2.x + k.m.c2.y * Cdot2.y));
    vec2<double> acc = mk<double>(J.impulse[0] + li.x, J.impulse[1] + li.y);
    const double max_force_impulse = dt * J.max_force;
    if (acc.x * acc.x + acc.y * acc.y > sq(max_force_impulse)) acc = max_force_impulse * normalized(acc);
    J.impulse[0] = acc.x;
    J.impulse[1] = acc.y;
}

// ------------------------------------------------------------ rope
// `u /= length` rebinds the local name: the kept _u (ux, uy) is the
// unnormalised anchor difference, on which the warm start and the velocity
// passes project (rope.py:140-149, 186-196).
static __device__ void rope_init(gb_joint &J, JCons &k, vec2<double> ca, double aa, vec2<double> cb, double ab,
                                 vec2<double> &va, double &wa, vec2<double> &vb, double &wb, double dt_ratio, bool warm) {
    const double ma = k.ma, mb = k.mb, ia = k.iA, ib = k.iB;
    const rot2<double> qa = pose_rot(aa), qb = pose_rot(ab);
    const vec2<double> ra = k.ra = rmul(qa, j_la(J) - k.lca);
    const vec2<double> rb = k.rb = rmul(qb, j_lb(J) - k.lcb);
    vec2<double> u = cb + rb - ca - ra;
    J.ux = u.x; J.uy = u.y;
    J.cur_length = len(u);
    const double C = J.cur_length - J.max_length;
    J.limit_state = C > 0.0 ? GB_LIMIT_UPPER : GB_LIMIT_INACTIVE;
    if (J.cur_length > GB_LINEAR_SLOP_J) {
        u = mk<double>(u.x / J.cur_length, u.y / J.cur_length);
    } else {
        k.dmass = 0.0;
        J.impulse[0] = 0.0;
        return;
    }
    const double cra = cross(ra, u), crb = cross(rb, u);
    const double inv_mass = ma + ia * cra * cra + mb + ib * crb * crb;
    k.dmass = inv_mass != 0.0 ? 1.0 / inv_mass : 0.0;
    if (warm) {
        J.impulse[0] = J.impulse[0] * dt_ratio;
        const vec2<double> P = J.impulse[0] * mk<double>(J.ux, J.uy);
        va = va - ma * P;
        wa = wa - ia * cross(ra, P);
        vb = vb + mb * P;
        wb = wb + ib * cross(rb, P);
    } else {
        J.impulse[0] = 0.0;
    }
}

static __device__ void rope_velocity(gb_joint &J, const JCons &k, vec2<double> &va, double &wa, vec2<double> &vb,
                                     double &wb, double inv_dt) {
    const vec2<double> u = mk<double>(J.ux, J.uy);
    const vec2<double> vpa = va + cross(wa, k.ra);
    const vec2<double> vpb = vb + cross(wb, k.rb);
    const double C = J.cur_length - J.max_length;
    double Cdot = dot(u, vpb - vpa);
    if (C < 0.0) Cdot += inv_dt * C;
    double impulse = -k.dmass * Cdot;
    const double old_impulse = J.impulse[0];
    J.impulse[0] = pymin(0.0, J.impulse[0] + impulse);
    impulse = J.impulse[0] - old_impulse;
    const vec2<double> P = impulse * u;
    va = va - k.ma * P;
    wa = wa - k.iA * cross(k.ra, P);
    vb = vb + k.mb * P;
    wb = wb + k.iB * cross(k.rb, P);
}

static __device__ bool rope_position(const gb_joint &J, const JCons &k, vec2<double> &ca, double &aa, vec2<double> &cb,
                                     double &ab) {
    const rot2<double> qa = pose_rot(aa), qb = pose_rot(ab);
    const vec2<double> ra = rmul(qa, j_la(J) - k.lca);
    const vec2<double> rb = rmul(qb, j_lb(J) - k.lcb);
    vec2<double> u = cb + rb - ca - ra;
    const double length = len(u);
    u = normalized(u);
    const double C = cclamp(length - J.max_length, 0.0, GB_MAX_LINEAR_CORRECTION_J);
    const double impulse = -k.dmass * C;
    const vec2<double> P = impulse * u;
    ca = ca - k.ma * P;
    aa = aa - k.iA * cross(ra, P);
    cb = cb + k.mb * P;
    ab = ab + k.iB * cross(rb, P);
    return length - J.max_length < GB_LINEAR_SLOP_J;
}

// ------------------------------------------------------------ wheel
// The spring's axis and arms (sax, s_ax, s_bx) are set only by a set-up with
// a positive frequency and kept otherwise; the velocity passes always run the
// spring and motor rows (wheel.py:329-355); the position pass takes its
// effective mass from the set-up's arms (wheel.py:397).
static __device__ void wheel_init(gb_joint &J, JCons &k, vec2<double> ca, double aa, vec2<double> cb, double ab,
                                  vec2<double> &va, double &wa, vec2<double> &vb, double &wb, double dt, double dt_ratio,
                                  bool warm) {
    const double ma = k.ma, mb = k.mb, ia = k.iA, ib = k.iB;
    const rot2<double> qa = pose_rot(aa), qb = pose_rot(ab);
    const vec2<double> ra = k.ra = rmul(qa, j_la(J) - k.lca);
    const vec2<double> rb = k.rb = rmul(qb, j_lb(J) - k.lcb);
    const vec2<double> d = cb + rb - ca - ra;
    const vec2<double> ay = k.axis = rmul(qa, j_ly(J));
    J.perp_x = ay.x; J.perp_y = ay.y;   // _ay, kept for the reaction force
    const double s_ay = k.s1 = cross(d + ra, ay);
    const double s_by = k.s2 = cross(rb, ay);
    k.dmass = ma + mb + ia * sq(s_ay) + ib * sq(s_by);
    if (k.dmass > 0.0) k.dmass = 1.0 / k.dmass;
    k.a1 = 0.0;   // _spring_mass
    J.bias = 0.0;
    J.gamma = 0.0;
    if (J.frequency > 0.0) {
        const vec2<double> ax = rmul(qa, mk<double>(J.ax_x, J.ax_y));
        J.sax_x = ax.x; J.sax_y = ax.y;
        J.s_ax = cross(d + ra, ax);
        J.s_bx = cross(rb, ax);
        const double inv_mass = ma + mb + ia * sq(J.s_ax) + ib * sq(J.s_bx);
        if (inv_mass > 0.0) {
            k.a1 = 1.0 / inv_mass;
            const double C = dot(d, ax);
            const double omega = 2.0 * 3.141592653589793 * J.frequency;
            const double dd = 2.0 * k.a1 * J.damping_ratio * omega;
            const double kk = k.a1 * sq(omega);
            J.gamma = dt * (dd + dt * kk);
            if (J.gamma > 0.0) J.gamma = 1.0 / J.gamma;
            J.bias = C * dt * kk * J.gamma;
            k.a1 = inv_mass + J.gamma;
            if (k.a1 > 0.0) k.a1 = 1.0 / k.a1;
        }
    } else {
        J.spring_impulse = 0.0;
    }
    if (J.flags & GB_J_MOTOR) {
        k.motor_mass = ia + ib;
        if (k.motor_mass > 0.0) k.motor_mass = 1.0 / k.motor_mass;
    } else {
        k.motor_mass = 0.0;
        J.motor_impulse = 0.0;
    }
    if (warm) {
        J.impulse[0] = J.impulse[0] * dt_ratio;
        J.spring_impulse = J.spring_impulse * dt_ratio;
        J.motor_impulse = J.motor_impulse * dt_ratio;
        const double imp = J.impulse[0], si = J.spring_impulse, mi = J.motor_impulse;
        const vec2<double> P = imp * ay + si * mk<double>(J.sax_x, J.sax_y);
        const double La = imp * s_ay + si * J.s_ax + mi;
        const double Lb = imp * s_by + si * J.s_bx + mi;
        va = va - ma * P;
        wa = wa - ia * La;
        vb = vb + mb * P;
        wb = wb + ib * Lb;
    } else {
        J.impulse[0] = 0.0;
        J.spring_impulse = 0.0;
        J.motor_impulse = 0.0;
    }
}

static __device__ void wheel_velocity(gb_joint &J, const JCons &k, vec2<double> &va, double &wa, vec2<double> &vb,
                                      double &wb, double dt) {
    const double ma = k.ma, mb = k.mb, ia = k.iA, ib = k.iB;
    const vec2<double> ax = mk<double>(J.sax_x, J.sax_y);
    double Cdot = dot(ax, vb - va) + J.s_bx * wb - J.s_ax * wa;
    double impulse = -k.a1 * (Cdot + J.bias + J.gamma * J.spring_impulse);
    J.spring_impulse = J.spring_impulse + impulse;
    vec2<double> P = impulse * ax;
    double La = impulse * J.s_ax, Lb = impulse * J.s_bx;
    va = va - ma * P;
    wa = wa - ia * La;
    vb = vb + mb * P;
    wb = wb + ib * Lb;
    Cdot = wb - wa - J.motor_speed;
    impulse = -k.motor_mass * Cdot;
    const double old_impulse = J.motor_impulse;
    const double max_impulse = dt * J.max_motor;
    J.motor_impulse = cclamp(J.motor_impulse + impulse, -max_impulse, max_impulse);
    impulse = J.motor_impulse - old_impulse;
    wa = wa - ia * impulse;
    wb = wb + ib * impulse;
    Cdot = dot(k.axis, vb - va) + k.s2 * wb - k.s1 * wa;
    impulse = -k.dmass * Cdot;
    J.impulse[0] = J.impulse[0] + impulse;
    P = impulse * k.axis;
    La = impulse * k.s1; Lb = impulse * k.s2;
    va = va - ma * P;
    wa = wa - ia * La;
    vb = vb + mb * P;
    wb = wb + ib * Lb;
}

static __device__ bool wheel_position(const gb_joint &J, const JCons &k, vec2<double> &ca, double &aa, vec2<double> &cb,
                                      double &ab) {
    const double ma = k.ma, mb = k.mb, ia = k.iA, ib = k.iB;
    const rot2<double> qa = pose_rot(aa), qb = pose_rot(ab);
    const vec2<double> ra = rmul(qa, j_la(J) - k.lca);
    const vec2<double> rb = rmul(qb, j_lb(J) - k.lcb);
    const vec2<double> d = (cb - ca) + rb - ra;
    const double kk = ma + mb + ia * sq(k.s1) + ib * sq(k.s2);
    const vec2<double> ay = rmul(qa, j_ly(J));
    const double s_ay = cross(d + ra, ay);
    const double s_by = cross(rb, ay);
    const double C = dot(d, ay);
    const double impulse = kk != 0.0 ? -C / kk : 0.0;
    const vec2<double> P = impulse * ay;
    const double La = impulse * s_ay, Lb = impulse * s_by;
    ca = ca - ma * P;
    aa = aa - ia * La;
    cb = cb + mb * P;
    ab = ab + ib * Lb;
    return fabs(C) <= GB_LINEAR_SLOP_J;
}

// ------------------------------------------------------------ pulley
// The warm start and the position pass apply the impulses with the effective
// masses ma + ia * (ra x ua)^2 (the local names are rebound, pulley.py:190-193,
// 292-295); the velocity passes take the inverse masses.
static __device__ void pulley_arms(const gb_joint &J, vec2<double> ca, vec2<double> ra, vec2<double> cb, vec2<double> rb,
                                   vec2<double> &ua, vec2<double> &ub, double &la, double &lb) {
    const vec2<double> a = ca + ra - mk<double>(J.ga_x, J.ga_y);
    const vec2<double> b = cb + rb - mk<double>(J.gb_x, J.gb_y);
    la = len(a);
    lb = len(b);
    ua = la > 10.0 * GB_LINEAR_SLOP_J ? mk<double>(a.x / la, a.y / la) : mk<double>(0.0, 0.0);
    ub = lb > 10.0 * GB_LINEAR_SLOP_J ? mk<double>(b.x / lb, b.y / lb) : mk<double>(0.0, 0.0);
}

static __device__ void pulley_init(gb_joint &J, JCons &k, vec2<double> ca, double aa, vec2<double> cb, double ab,
                                   vec2<double> &va, double &wa, vec2<double> &vb, double &wb, double dt_ratio, bool warm) {
    const double ia = k.iA, ib = k.iB;
    const rot2<double> qa = pose_rot(aa), qb = pose_rot(ab);
    const vec2<double> ra = k.ra = rmul(qa, j_la(J) - k.lca);
    const vec2<double> rb = k.rb = rmul(qb, j_lb(J) - k.lcb);
    double la, lb;
    pulley_arms(J, ca, ra, cb, rb, k.u, k.perp, la, lb);
    const double rua = cross(ra, k.u), rub = cross(rb, k.perp);
    const double ma = k.ma + ia * sq(rua);
    const double mb = k.mb + ib * sq(rub);
    k.dmass = ma + J.ratio * J.ratio * mb;
    if (k.dmass > 0.0) k.dmass = 1.0 / k.dmass;
    if (warm) {
        J.impulse[0] = J.impulse[0] * dt_ratio;
        const vec2<double> Pa = (-J.impulse[0]) * k.u;
        const vec2<double> Pb = (-J.ratio * J.impulse[0]) * k.perp;
        va = va + ma * Pa;
        wa = wa + ia * cross(ra, Pa);
        vb = vb + mb * Pb;
        wb = wb + ib * cross(rb, Pb);
    } else {
        J.impulse[0] = 0.0;
    }
}

static __device__ void pulley_velocity(gb_joint &J, const JCons &k, vec2<double> &va, double &wa, vec2<double> &vb,
                                       double &wb) {
    const vec2<double> vpa = va + cross(wa, k.ra);
    const vec2<double> vpb = vb + cross(wb, k.rb);
    const double Cdot = -dot(k.u, vpa) - J.ratio * dot(k.perp, vpb);
    const double impulse = -k.dmass * Cdot;
    J.impulse[0] = J.impulse[0] + impulse;
    const vec2<double> Pa = (-impulse) * k.u;
    const vec2<double> Pb = (-J.ratio * impulse) * k.perp;
    va = va + k.ma * Pa;
    wa = wa + k.iA * cross(k.ra, Pa);
    vb = vb + k.mb * Pb;
    wb = wb + k.iB * cross(k.rb, Pb);
}

static __device__ bool pulley_position(const gb_joint &J, const JCons &k, vec2<double> &ca, double &aa, vec2<double> &cb,
                                       double &ab) {
    const double ia = k.iA, ib = k.iB;
    const rot2<double> qa = pose_rot(aa), qb = pose_rot(ab);
    const vec2<double> ra = rmul(qa, j_la(J) - k.lca);
    const vec2<double> rb = rmul(qb, j_lb(J) - k.lcb);
    vec2<double> ua, ub;
    double la, lb;
    pulley_arms(J, ca, ra, cb, rb, ua, ub, la, lb);
    const double rua = cross(ra, ua), rub = cross(rb, ub);
    const double ma = k.ma + ia * sq(rua);
    const double mb = k.mb + ib * sq(rub);
    double mass = ma + sq(J.ratio) * mb;
    if (mass > 0.0) mass = 1.0 / mass;
    const double C = J.constant - la - J.ratio * lb;
    const double linear_error = fabs(C);
    const double impulse = -mass * C;
    const vec2<double> Pa = (-impulse) * ua;
    const vec2<double> Pb = (-J.ratio * impulse) * ub;
    ca = ca + ma * Pa;
    aa = aa + ia * cross(ra, Pa);
    cb = cb + mb * Pb;
    ab = ab + ib * cross(rb, Pb);
    return linear_error < GB_LINEAR_SLOP_J;
}

// ------------------------------------------------------------ mouse
// Body B pulled towards a target by a soft constraint with a force limit.
// The record's body_a is body B (the reference's is None), so the caller's
// A and B values are the same body's and only B's are changed; the set-up
// damps B's angular velocity by 0.98 (mouse.py:183).
static __device__ void mouse_init(gb_joint &J, JCons &k, vec2<double> cb, double ab, vec2<double> &vb, double &wb,
                                  double dt, double dt_ratio, double body_mass, bool warm) {
    const double mb = k.mb, ib = k.iB;
    const rot2<double> qb = pose_rot(ab);
    const double mass = body_mass;
    const double omega = 2.0 * 3.141592653589793 * J.frequency;
    const double d = 2.0 * mass * J.damping_ratio * omega;
    const double kk = mass * sq(omega);
    J.gamma = dt * (d + dt * kk);
    if (J.gamma != 0.0) J.gamma = 1.0 / J.gamma;
    J.bias = dt * kk * J.gamma;   // _beta
    const vec2<double> rb = k.rb = rmul(qb, j_lb(J) - k.lcb);
    const double a = mb + ib * sq(rb.y) + J.gamma;
    const double c = -ib * rb.x * rb.y;
    const double b = c;
    const double dd = mb + ib * sq(rb.x) + J.gamma;
    double det = a * dd - b * c;
    if (det != 0.0) det = 1.0 / det;
    k.m.c1 = mk3(det * dd, -det * c, 0.0);
    k.m.c2 = mk3(-det * b, det * a, 0.0);
    k.u = J.bias * (cb + rb - mk<double>(J.target_x, J.target_y));   // _c
    wb = wb * 0.98;
    if (warm) {
        J.impulse[0] = J.impulse[0] * dt_ratio;
        J.impulse[1] = J.impulse[1] * dt_ratio;
        const vec2<double> P = mk<double>(J.impulse[0], J.impulse[1]);
        vb = vb + mb * P;
        wb = wb + ib * cross(rb, P);
    } else {
        J.impulse[0] = J.impulse[1] = 0.0;
    }
}

static __device__ void mouse_velocity(gb_joint &J, const JCons &k, vec2<double> &vb, double &wb, double dt) {
    const vec2<double> Cdot = vb + cross(wb, k.rb);
    vec2<double> acc = mk<double>(J.impulse[0], J.impulse[1]);
    const vec2<double> e = -(Cdot + k.u + J.gamma * acc);
    vec2<double> impulse = mk<double>(k.m.c1.x * e.x + k.m.c2.x * e.y, k.m.c1.y * e.x + k.m.c2.y * e.y);
    const vec2<double> old_impulse = acc;
    acc = acc + impulse;
    const double max_impulse = dt * J.max_force;
    if (acc.x * acc.x + acc.y * acc.y > sq(max_impulse)) {
        const double s = max_impulse / sqrt(acc.x * acc.x + acc.y * acc.y);
        acc = mk<double>(acc.x * s, acc.y * s);
    }
    J.impulse[0] = acc.x; J.impulse[1] = acc.y;
    impulse = acc - old_impulse;
    vb = vb + k.mb * impulse;
    wb = wb + k.iB * cross(k.rb, impulse);
}

// ------------------------------------------------------------ dispatch
static __device__ void joint_init(gb_joint &J, JCons &k, vec2<double> ca, double aa, vec2<double> cb, double ab,
                                  vec2<double> &va, double &wa, vec2<double> &vb, double &wb, double dt, double dt_ratio,
                                  double body_b_mass, bool warm) {
    switch (J.type) {
    case GB_JOINT_MOUSE: mouse_init(J, k, cb, ab, vb, wb, dt, dt_ratio, body_b_mass, warm); break;
    case GB_JOINT_REVOLUTE: revolute_init(J, k, aa, ab, va, wa, vb, wb, dt_ratio, warm); break;
    case GB_JOINT_PRISMATIC: prismatic_init(J, k, ca, aa, cb, ab, va, wa, vb, wb, dt_ratio, warm); break;
    case GB_JOINT_DISTANCE: distance_init(J, k, ca, aa, cb, ab, va, wa, vb, wb, dt, dt_ratio, warm); break;
    case GB_JOINT_FRICTION: friction_init(J, k, aa, ab, va, wa, vb, wb, dt_ratio, warm); break;
    case GB_JOINT_ROPE: rope_init(J, k, ca, aa, cb, ab, va, wa, vb, wb, dt_ratio, warm); break;
    case GB_JOINT_WHEEL: wheel_init(J, k, ca, aa, cb, ab, va, wa, vb, wb, dt, dt_ratio, warm); break;
    case GB_JOINT_PULLEY: pulley_init(J, k, ca, aa, cb, ab, va, wa, vb, wb, dt_ratio, warm); break;
    default: weld_init(J, k, aa, ab, va, wa, vb, wb, dt_ratio, warm); break;
    }
}
static __device__ void joint_velocity(gb_joint &J, const JCons &k, vec2<double> &va, double &wa, vec2<double> &vb,
                                      double &wb, double dt) {
    switch (J.type) {
    case GB_JOINT_REVOLUTE: revolute_velocity(J, k, va, wa, vb, wb, dt); break;
    case GB_JOINT_PRISMATIC: prismatic_velocity(J, k, va, wa, vb, wb, dt); break;
    case GB_JOINT_DISTANCE: distance_velocity(J, k, va, wa, vb, wb); break;
    case GB_JOINT_FRICTION: friction_velocity(J, k, va, wa, vb, wb, dt); break;
    case GB_JOINT_ROPE: rope_velocity(J, k, va, wa, vb, wb, 1.0 / dt); break;
    case GB_JOINT_WHEEL: wheel_velocity(J, k, va, wa, vb, wb, dt); break;
    case GB_JOINT_PULLEY: pulley_velocity(J, k, va, wa, vb, wb); break;
    case GB_JOINT_MOUSE: mouse_velocity(J, k, vb, wb, dt); break;
    default: weld_velocity(J, k, va, wa, vb, wb); break;
    }
}
static __device__ bool joint_position(const gb_joint &J, const JCons &k, vec2<double> &ca, double &aa, vec2<double> &cb,
                                      double &ab) {
    switch (J.type) {
    case GB_JOINT_REVOLUTE: return revolute_position(J, k, ca, aa, cb, ab);
    case GB_JOINT_PRISMATIC: return prismatic_position(J, k, ca, aa, cb, ab);
    case GB_JOINT_DISTANCE: return distance_position(J, k, ca, aa, cb, ab);
    case GB_JOINT_FRICTION: return true;
    case GB_JOINT_ROPE: return rope_position(J, k, ca, aa, cb, ab);
    case GB_JOINT_WHEEL: return wheel_position(J, k, ca, aa, cb, ab);
    case GB_JOINT_PULLEY: return pulley_position(J, k, ca, aa, cb, ab);
    case GB_JOINT_MOUSE: return true;
    default: return weld_position(J, k, ca, aa, cb, ab);
    }
}

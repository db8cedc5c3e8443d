/*
 * oracle_collide.h -- TEST INFRASTRUCTURE: float64 CPU restatement of the
 * reference narrow phase, distance and time-of-impact code.  Every function
 * names the reference function it restates (file:line inside the pypybox2d
 * package); the operation order is the reference's, so results are the
 * reference's doubles.  Used only by the oracle (oracle.c).
 */
#ifndef ORACLE_COLLIDE_H
#define ORACLE_COLLIDE_H

#include <stdint.h>
#include "oracle_math.h"
#include "../include/gb2d.h"

#define OR_LINEAR_SLOP 0.005
#define OR_POLYGON_RADIUS (2.0 * 0.005)
#define OR_ANGULAR_SLOP 0.03490658503988659
#define OR_MAX_FLOAT 1.7976931348623157e+308
#define OR_EPSILON 2.220446049250313e-16
#define OR_EPSILON_SQR 4.930380657631324e-32
#define OR_RELATIVE_TOL 0.98
#define OR_ABSOLUTE_TOL 0.001

#define OR_VERTEX 0
#define OR_FACE 1

typedef struct {
    int type, count;
    v2 ln, lp;
    v2 plp[2];
    double ni[2], ti[2];
    uint32_t id[2];
} or_manifold;

static inline uint32_t or_id(int ia, int ib, int ta, int tb) {
    return (uint32_t)(ia & 0xff) | ((uint32_t)(ib & 0xff) << 8) | ((uint32_t)(ta & 0xff) << 16) |
           ((uint32_t)(tb & 0xff) << 24);
}

static inline v2 fx_v(const gb_fixture *f, int i) { return V(f->vx[i], f->vy[i]); }
static inline v2 fx_n(const gb_fixture *f, int i) { return V(f->nx[i], f->ny[i]); }

/* contact_util.ClipVertex */
typedef struct { v2 v; int ia, ib, ta, tb; } clipv;

/* collision.py:46-66 collide_circles */
static void or_collide_circles(or_manifold *m, const gb_fixture *a, xform xa, const gb_fixture *b, xform xb) {
    m->count = 0;
    v2 pa = xmul(xa, fx_v(a, 0));
    v2 pb = xmul(xb, fx_v(b, 0));
    v2 d = vsub(pb, pa);
    double dist_sqr = vlen2(d);
    double radius = a->radius + b->radius;
    if (dist_sqr > SQ(radius)) return;
    m->type = GB_M_CIRCLES;
    m->lp = fx_v(a, 0);
    m->ln = V(0.0, 0.0);
    m->count = 1;
    m->plp[0] = fx_v(b, 0);
    m->id[0] = or_id(0, 0, 0, 0);
}

/* collision.py:68-141 collide_polygon_circle */
static void or_collide_polygon_circle(or_manifold *m, const gb_fixture *pa_, xform xa, const gb_fixture *cb, xform xb) {
    m->count = 0;
    v2 c = xmul(xb, fx_v(cb, 0));
    v2 cl = xmul_t(xa, c);
    int normal_index = 0;
    double separation = -OR_MAX_FLOAT;
    double radius = pa_->radius + cb->radius;
    int n = pa_->vertex_count;
    for (int i = 0; i < n; ++i) {
        double s = vdot(fx_n(pa_, i), vsub(cl, fx_v(pa_, i)));
        if (s > radius) return;
        if (s > separation) { separation = s; normal_index = i; }
    }
    int i1 = normal_index, i2 = (i1 + 1) % n;
    v2 v1 = fx_v(pa_, i1), v2_ = fx_v(pa_, i2);
    if (separation < OR_EPSILON) {
        m->count = 1;
        m->type = GB_M_FACE_A;
        m->ln = fx_n(pa_, normal_index);
        m->lp = vscale(0.5, vadd(v1, v2_));
        m->plp[0] = fx_v(cb, 0);
        m->id[0] = 0;
        return;
    }
    double u1 = vdot(vsub(cl, v1), vsub(v2_, v1));
    double u2 = vdot(vsub(cl, v2_), vsub(v1, v2_));
    if (u1 < 0.0) {
        v2 dd = vsub(cl, v1);
        if (vdot(dd, dd) > SQ(radius)) return;
        m->ln = vnormalized(vsub(cl, v1));
        m->lp = v1;
    } else if (u2 < 0.0) {
        v2 dd = vsub(cl, v2_);
        if (vdot(dd, dd) > SQ(radius)) return;
        m->ln = vnormalized(vsub(cl, v2_));
        m->lp = v2_;
    } else {
        v2 face_center = vscale(0.5, vadd(v1, v2_));
        double sep = vdot(vsub(cl, face_center), fx_n(pa_, i1));
        if (sep > radius) return;
        m->ln = fx_n(pa_, i1);
        m->lp = face_center;
    }
    m->count = 1;
    m->type = GB_M_FACE_A;
    m->plp[0] = fx_v(cb, 0);
    m->id[0] = 0;
}

/* collision_util.py:31-52 edge_separation */
static double or_edge_separation(const gb_fixture *p1, xform x1, int edge1, const gb_fixture *p2, xform x2) {
    v2 n1w = rmul(x1.q, fx_n(p1, edge1));
    v2 n1 = rmul_t(x2.q, n1w);
    int index = 0;
    double min_dot = 0.0;
    for (int i = 0; i < p2->vertex_count; ++i) {
        double d = vdot(fx_v(p2, i), n1);
        if (i == 0 || d < min_dot) { min_dot = d; index = i; }
    }
    v2 v1 = xmul(x1, fx_v(p1, edge1));
    v2 v2_ = xmul(x2, fx_v(p2, index));
    return vdot(vsub(v2_, v1), n1w);
}

/* collision_util.py:54-109 max_separation; the polygon centroid used for the
 * initial direction is the body origin because Polygon._centroid is never
 * assigned (shapes.py:244). */
static double or_max_separation(const gb_fixture *p1, xform x1, const gb_fixture *p2, xform x2, int *edge_out) {
    int count1 = p1->vertex_count;
    v2 d = vsub(xmul(x2, V(0.0, 0.0)), xmul(x1, V(0.0, 0.0)));
    v2 dl = rmul_t(x1.q, d);
    int edge = 0;
    double max_dot = 0.0;
    for (int i = 0; i < count1; ++i) {
        double dd = vdot(fx_n(p1, i), dl);
        if (i == 0 || dd > max_dot) { max_dot = dd; edge = i; }
    }
    double s = or_edge_separation(p1, x1, edge, p2, x2);
    int prev_edge = (edge - 1 + count1) % count1;
    double s_prev = or_edge_separation(p1, x1, prev_edge, p2, x2);
    int next_edge = (edge + 1) % count1;
    double s_next = or_edge_separation(p1, x1, next_edge, p2, x2);
    int increment, best_edge;
    double best_sep;
    if (s_prev > s && s_prev > s_next) {
        increment = -1; best_edge = prev_edge; best_sep = s_prev;
    } else if (s_next > s) {
        increment = 1; best_edge = next_edge; best_sep = s_next;
    } else {
        *edge_out = edge;
        return s;
    }
    for (;;) {
        if (increment == -1) edge = (best_edge - 1 + count1) % count1;
        else edge = (best_edge + 1) % count1;
        s = or_edge_separation(p1, x1, edge, p2, x2);
        if (s > best_sep) { best_edge = edge; best_sep = s; }
        else break;
    }
    *edge_out = best_edge;
    return best_sep;
}

/* collision_util.py:111-133 find_incident_edge */
static void or_find_incident_edge(clipv c[2], const gb_fixture *p1, xform x1, int edge1, const gb_fixture *p2, xform x2) {
    v2 n1 = rmul_t(x2.q, rmul(x1.q, fx_n(p1, edge1)));
    int index = 0;
    double min_dot = 0.0;
    for (int i = 0; i < p2->vertex_count; ++i) {
        double d = vdot(n1, fx_n(p2, i));
        if (i == 0 || d < min_dot) { min_dot = d; index = i; }
    }
    int i1 = index, i2 = (i1 + 1) % p2->vertex_count;
    c[0].v = xmul(x2, fx_v(p2, i1)); c[0].ia = edge1; c[0].ib = i1; c[0].ta = OR_FACE; c[0].tb = OR_VERTEX;
    c[1].v = xmul(x2, fx_v(p2, i2)); c[1].ia = edge1; c[1].ib = i2; c[1].ta = OR_FACE; c[1].tb = OR_VERTEX;
}

/* collision_util.py:135-164 clip_segment_to_line */
static int or_clip_segment(clipv out[2], const clipv in[2], v2 normal, double offset, int vertex_index_a) {
    int n = 0;
    double d0 = vdot(normal, in[0].v) - offset;
    double d1 = vdot(normal, in[1].v) - offset;
    if (d0 <= 0.0) out[n++] = in[0];
    if (d1 <= 0.0) out[n++] = in[1];
    if (d0 * d1 < 0.0) {
        double interp = d0 / (d0 - d1);
        clipv cv;
        cv.v = vadd(in[0].v, vscale(interp, vsub(in[1].v, in[0].v)));
        cv.ia = vertex_index_a; cv.ib = in[0].ib; cv.ta = OR_VERTEX; cv.tb = OR_FACE;
        if (n < 2) out[n] = cv;
        n++;
    }
    return n;
}

/* collision.py:144-241 collide_polygons */
static void or_collide_polygons(or_manifold *m, const gb_fixture *pa, xform xa, const gb_fixture *pb, xform xb) {
    m->count = 0;
    double total_radius = pa->radius + pb->radius;
    int edge_a, edge_b;
    double sep_a = or_max_separation(pa, xa, pb, xb, &edge_a);
    if (sep_a > total_radius) return;
    double sep_b = or_max_separation(pb, xb, pa, xa, &edge_b);
    if (sep_b > total_radius) return;
    const gb_fixture *poly1, *poly2;
    xform x1, x2;
    int edge1, flip;
    if (sep_b > (OR_RELATIVE_TOL * sep_a + OR_ABSOLUTE_TOL)) {
        poly1 = pb; poly2 = pa; x1 = xb; x2 = xa; edge1 = edge_b; m->type = GB_M_FACE_B; flip = 1;
    } else {
        poly1 = pa; poly2 = pb; x1 = xa; x2 = xb; edge1 = edge_a; m->type = GB_M_FACE_A; flip = 0;
    }
    clipv inc[2];
    or_find_incident_edge(inc, poly1, x1, edge1, poly2, x2);
    int iv1 = edge1, iv2 = (edge1 + 1) % poly1->vertex_count;
    v2 v11 = fx_v(poly1, iv1), v12 = fx_v(poly1, iv2);
    v2 local_tangent = vnormalized(vsub(v12, v11));
    v2 local_normal = vcross_vs(local_tangent, 1.0);
    v2 plane_point = vscale(0.5, vadd(v11, v12));
    v2 tangent = rmul(x1.q, local_tangent);
    v2 normal = vcross_vs(tangent, 1.0);
    v11 = xmul(x1, v11);
    v12 = xmul(x1, v12);
    double front_offset = vdot(normal, v11);
    double side1 = -vdot(tangent, v11) + total_radius;
    double side2 = vdot(tangent, v12) + total_radius;
    clipv cp1[2], cp2[2];
    int n1 = or_clip_segment(cp1, inc, vneg(tangent), side1, iv1);
    if (n1 < 2) return;
    int n2 = or_clip_segment(cp2, cp1, tangent, side2, iv2);
    if (n2 < 2) return;
    m->ln = local_normal;
    m->lp = plane_point;
    int pc = 0;
    for (int i = 0; i < 2; ++i) {
        double separation = vdot(normal, cp2[i].v) - front_offset;
        if (separation <= total_radius) {
            m->plp[pc] = xmul_t(x2, cp2[i].v);
            if (flip) m->id[pc] = or_id(cp2[i].ib, cp2[i].ia, cp2[i].tb, cp2[i].ta);
            else m->id[pc] = or_id(cp2[i].ia, cp2[i].ib, cp2[i].ta, cp2[i].tb);
            pc++;
        }
    }
    m->count = pc;
}

/* collision.py:245-353 collide_edge_circle */
static void or_collide_edge_circle(or_manifold *m, const gb_fixture *ea, xform xa, const gb_fixture *cb, xform xb) {
    m->count = 0;
    v2 Q = xmul_t(xa, xmul(xb, fx_v(cb, 0)));
    v2 A = fx_v(ea, 0), B = fx_v(ea, 1);
    v2 e = vsub(B, A);
    double u = vdot(e, vsub(B, Q));
    double v = vdot(e, vsub(Q, A));
    double radius = ea->radius + cb->radius;
    if (v <= 0.0) {
        v2 P = A;
        v2 d = vsub(Q, P);
        double dd = vdot(d, d);
        if (dd > SQ(radius)) return;
        if (ea->flags & GB_FIX_EDGE_HAS_V0) {
            v2 A1 = fx_v(ea, 2), B1 = A;
            v2 e1 = vsub(B1, A1);
            double u1 = vdot(e1, vsub(B1, Q));
            if (u1 > 0.0) return;
        }
        m->count = 1; m->type = GB_M_CIRCLES; m->ln = V(0.0, 0.0); m->lp = P;
        m->id[0] = or_id(0, 0, OR_VERTEX, OR_VERTEX);
        m->plp[0] = fx_v(cb, 0);
        return;
    }
    if (u <= 0.0) {
        v2 P = B;
        v2 d = vsub(Q, P);
        double dd = vdot(d, d);
        if (dd > SQ(radius)) return;
        if (ea->flags & GB_FIX_EDGE_HAS_V3) {
            v2 B2 = fx_v(ea, 3), A2 = B;
            v2 e2 = vsub(B2, A2);
            double v2_ = vdot(e2, vsub(Q, A2));
            if (v2_ > 0.0) return;
        }
        m->count = 1; m->type = GB_M_CIRCLES; m->ln = V(0.0, 0.0); m->lp = P;
        m->id[0] = or_id(1, 0, OR_VERTEX, OR_VERTEX);
        m->plp[0] = fx_v(cb, 0);
        return;
    }
    double den = vdot(e, e);
    v2 P = vscale(1.0 / den, vadd(vscale(u, A), vscale(v, B)));
    v2 d = vsub(Q, P);
    double dd = vdot(d, d);
    if (dd > SQ(radius)) return;
    v2 n = V(-e.y, e.x);
    if (vdot(n, vsub(Q, A)) < 0.0) n = V(-n.x, -n.y);
    n = vnormalized(n);
    m->count = 1; m->type = GB_M_FACE_A; m->ln = n; m->lp = A;
    m->id[0] = or_id(0, 0, OR_FACE, OR_VERTEX);
    m->plp[0] = fx_v(cb, 0);
}

/* collision.py:385-690 EPCollider (edge versus polygon with adjacency) */
typedef struct { int type, index; double separation; } ep_axis;
#define EP_UNKNOWN 0
#define EP_EDGE_A 1
#define EP_EDGE_B 2

typedef struct {
    v2 v[GB_MAX_POLY_VERTS], n[GB_MAX_POLY_VERTS];
    int count;
    v2 centroid;
} ep_proxy;

static void or_ep_incident(clipv c[2], const ep_proxy *p1, int edge1, const ep_proxy *p2) {
    v2 n1 = p1->n[edge1];
    int index = 0;
    double min_dot = 0.0;
    for (int i = 0; i < p2->count; ++i) {
        double d = vdot(n1, p2->n[i]);
        if (i == 0 || d < min_dot) { min_dot = d; index = i; }
    }
    int i1 = index, i2 = (i1 + 1) % p2->count;
    c[0].v = p2->v[i1]; c[0].ia = edge1; c[0].ib = i1; c[0].ta = OR_FACE; c[0].tb = OR_VERTEX;
    c[1].v = p2->v[i2]; c[1].ia = edge1; c[1].ib = i2; c[1].ta = OR_FACE; c[1].tb = OR_VERTEX;
}

static void or_collide_edge_polygon(or_manifold *m, const gb_fixture *ea, xform xa, const gb_fixture *pb, xform xb) {
    /* EPCollider.__init__: xa.mul_t(xb) is (pb - pa, Ra^T Rb) in the C
     * extension (transform.c Transform_mul_t: the position is not rotated). */
    xform xf;
    xf.p = vsub(xb.p, xa.p);
    xf.q.c = xa.q.c * xb.q.c + xa.q.s * xb.q.s;
    xf.q.s = (-xa.q.s) * xb.q.c + xa.q.c * xb.q.s;
    int has_v0 = (ea->flags & GB_FIX_EDGE_HAS_V0) != 0, has_v3 = (ea->flags & GB_FIX_EDGE_HAS_V3) != 0;
    v2 v0 = fx_v(ea, 2), v1 = fx_v(ea, 0), v2e = fx_v(ea, 1), v3 = fx_v(ea, 3);
    v2 e = vsub(v2e, v1);
    v2 enormal = vnormalized(V(e.y, -e.x));
    ep_proxy pxa, pxb;
    pxa.count = 2; pxa.v[0] = v1; pxa.v[1] = v2e; pxa.n[0] = enormal; pxa.n[1] = vneg(enormal);
    pxa.centroid = vscale(0.5, vadd(v1, v2e));
    pxb.centroid = xmul(xf, V(0.0, 0.0));
    pxb.count = pb->vertex_count;
    for (int i = 0; i < pb->vertex_count; ++i) {
        pxb.v[i] = xmul(xf, fx_v(pb, i));
        pxb.n[i] = rmul(xf.q, fx_n(pb, i));
    }
    double radius = 2.0 * OR_POLYGON_RADIUS;
    v2 l11 = V(0, 0), l12 = V(0, 0), l21 = V(0, 0), l22 = V(0, 0);
    m->count = 0;
    /* compute_adjacency (collision.py:546-610) */
    v2 center_b = pxb.centroid;
    if (has_v0) {
        v2 e0 = vsub(v1, v0), e1 = vsub(v2e, v1);
        v2 n0 = vnormalized(V(e0.y, -e0.x)), n1 = vnormalized(V(e1.y, -e1.x));
        int convex = vcross(n0, n1) >= 0.0;
        int front0 = vdot(n0, vsub(center_b, v0)) >= 0.0;
        int front1 = vdot(n1, vsub(center_b, v1)) >= 0.0;
        if (convex) {
            if (front0 || front1) { l11 = n1; l12 = n0; } else { l11 = vneg(n1); l12 = vneg(n0); }
        } else {
            if (front0 && front1) { l11 = n0; l12 = n1; } else { l11 = vneg(n0); l12 = vneg(n1); }
        }
    }
    if (has_v3) {
        v2 e1 = vsub(v2e, v1), e2 = vsub(v3, v2e);
        v2 n1 = vnormalized(V(e1.y, -e1.x)), n2 = vnormalized(V(e2.y, -e2.x));
        int convex = vcross(n1, n2) >= 0.0;
        int front1 = vdot(n1, vsub(center_b, v1)) >= 0.0;
        int front2 = vdot(n2, vsub(center_b, v2e)) >= 0.0;
        if (convex) {
            if (front1 || front2) { l21 = n2; l22 = n1; } else { l21 = vneg(n2); l22 = vneg(n1); }
        } else {
            if (front1 && front2) { l21 = n1; l22 = n2; } else { l21 = vneg(n1); l22 = vneg(n2); }
        }
    }
    /* compute_edge_separation (collision.py:612-639) */
    ep_axis edge_axis;
    edge_axis.type = EP_UNKNOWN; edge_axis.index = -1; edge_axis.separation = -OR_MAX_FLOAT;
    {
        v2 normals[2] = {enormal, vneg(enormal)};
        for (int i = 0; i < 2; ++i) {
            v2 n = normals[i];
            int valid1 = (vcross(n, l11) >= -OR_ANGULAR_SLOP) && (vcross(l12, n) >= -OR_ANGULAR_SLOP);
            int valid2 = (vcross(n, l21) >= -OR_ANGULAR_SLOP) && (vcross(l22, n) >= -OR_ANGULAR_SLOP);
            if (!valid1 || !valid2) continue;
            ep_axis ax; ax.type = EP_EDGE_A; ax.index = i;
            double mn = 0.0;
            for (int k = 0; k < pxb.count; ++k) {
                double d = vdot(n, vsub(pxb.v[k], v1));
                if (k == 0 || d < mn) mn = d;
            }
            ax.separation = mn;
            if (ax.separation > radius) { edge_axis = ax; goto edge_done; }
            if (ax.separation > edge_axis.separation) edge_axis = ax;
        }
    }
edge_done:
    if (edge_axis.type == EP_UNKNOWN) return;
    if (edge_axis.separation > radius) return;
    /* compute_polygon_separation (collision.py:641-668) */
    ep_axis poly_axis;
    poly_axis.type = EP_UNKNOWN; poly_axis.index = -1; poly_axis.separation = -OR_MAX_FLOAT;
    for (int i = 0; i < pxb.count; ++i) {
        v2 n = vneg(pxb.n[i]);
        int valid1 = (vcross(n, l11) >= -OR_ANGULAR_SLOP) && (vcross(l12, n) >= -OR_ANGULAR_SLOP);
        int valid2 = (vcross(n, l21) >= -OR_ANGULAR_SLOP) && (vcross(l22, n) >= -OR_ANGULAR_SLOP);
        if (!valid1 || !valid2) continue;
        double s1 = vdot(n, vsub(pxb.v[i], v1));
        double s2 = vdot(n, vsub(pxb.v[i], v2e));
        double s = pymin(s1, s2);
        if (s > radius) { poly_axis.type = EP_EDGE_B; poly_axis.index = i; poly_axis.separation = s; }
        if (s > poly_axis.separation) { poly_axis.type = EP_EDGE_B; poly_axis.index = i; poly_axis.separation = s; }
    }
    if (poly_axis.type != EP_UNKNOWN && poly_axis.separation > radius) return;
    ep_axis primary;
    if (poly_axis.type == EP_UNKNOWN) primary = edge_axis;
    else if (poly_axis.separation > OR_RELATIVE_TOL * edge_axis.separation + OR_ABSOLUTE_TOL) primary = poly_axis;
    else primary = edge_axis;
    const ep_proxy *p1, *p2;
    if (primary.type == EP_EDGE_A) { p1 = &pxa; p2 = &pxb; m->type = GB_M_FACE_A; }
    else { p1 = &pxb; p2 = &pxa; m->type = GB_M_FACE_B; }
    int edge1 = primary.index;
    clipv inc[2];
    or_ep_incident(inc, p1, edge1, p2);
    int iv1 = edge1, iv2 = (edge1 + 1) % p1->count;
    v2 v11 = p1->v[iv1], v12 = p1->v[iv2];
    v2 tangent = vnormalized(vsub(v12, v11));
    v2 normal = vcross_vs(tangent, 1.0);
    v2 plane_point = vscale(0.5, vadd(v11, v12));
    double front_offset = vdot(normal, v11);
    double side1 = -vdot(tangent, v11) + radius;
    double side2 = vdot(tangent, v12) + radius;
    clipv cp1[2], cp2[2];
    int n1 = or_clip_segment(cp1, inc, vneg(tangent), side1, iv1);
    if (n1 < 2) return;
    int n2 = or_clip_segment(cp2, cp1, tangent, side2, iv2);
    if (n2 < 2) return;
    if (primary.type == EP_EDGE_A) { m->ln = normal; m->lp = plane_point; }
    else { m->ln = rmul_t(xf.q, normal); m->lp = xmul_t(xf, plane_point); }
    int pc = 0;
    for (int i = 0; i < 2; ++i) {
        double separation = vdot(normal, cp2[i].v) - front_offset;
        if (separation <= radius) {
            if (primary.type == EP_EDGE_A) {
                m->plp[pc] = xmul_t(xf, cp2[i].v);
                m->id[pc] = or_id(cp2[i].ia, cp2[i].ib, cp2[i].ta, cp2[i].tb);
            } else {
                /* the reference stores (type_b, type_a, index_b, index_a) here (collision.py:532) */
                m->plp[pc] = cp2[i].v;
                m->id[pc] = or_id(cp2[i].tb, cp2[i].ta, cp2[i].ib, cp2[i].ia);
            }
            pc++;
        }
    }
    m->count = pc;
}

/* contact.py:294-311 dispatch: evaluate the manifold of (A, B) where A is the
 * primary shape of the registered pair. */
static void or_evaluate(or_manifold *m, const gb_fixture *a, xform xa, const gb_fixture *b, xform xb) {
    int ta = a->shape_type, tb = b->shape_type;
    if (ta == GB_SHAPE_CIRCLE && tb == GB_SHAPE_CIRCLE) or_collide_circles(m, a, xa, b, xb);
    else if (ta == GB_SHAPE_POLYGON && tb == GB_SHAPE_POLYGON) or_collide_polygons(m, a, xa, b, xb);
    else if (ta == GB_SHAPE_POLYGON && tb == GB_SHAPE_CIRCLE) or_collide_polygon_circle(m, a, xa, b, xb);
    else if (ta == GB_SHAPE_EDGE && tb == GB_SHAPE_CIRCLE) or_collide_edge_circle(m, a, xa, b, xb);
    else if (ta == GB_SHAPE_EDGE && tb == GB_SHAPE_POLYGON) or_collide_edge_polygon(m, a, xa, b, xb);
    else m->count = 0;
}

/* contact.py:294-311: which (type1, type2) pairs have an evaluate function,
 * and whether the first fixture is the primary (A) shape. */
static int or_pair_registered(int t1, int t2, int *primary) {
    int reg = 0, prim = 0;
    if (t1 == GB_SHAPE_CIRCLE && t2 == GB_SHAPE_CIRCLE) { reg = 1; prim = 1; }
    else if (t1 == GB_SHAPE_POLYGON && t2 == GB_SHAPE_POLYGON) { reg = 1; prim = 1; }
    else if (t1 == GB_SHAPE_POLYGON && t2 == GB_SHAPE_CIRCLE) { reg = 1; prim = 1; }
    else if (t1 == GB_SHAPE_CIRCLE && t2 == GB_SHAPE_POLYGON) { reg = 1; prim = 0; }
    else if (t1 == GB_SHAPE_EDGE && t2 == GB_SHAPE_CIRCLE) { reg = 1; prim = 1; }
    else if (t1 == GB_SHAPE_CIRCLE && t2 == GB_SHAPE_EDGE) { reg = 1; prim = 0; }
    else if (t1 == GB_SHAPE_EDGE && t2 == GB_SHAPE_POLYGON) { reg = 1; prim = 1; }
    else if (t1 == GB_SHAPE_POLYGON && t2 == GB_SHAPE_EDGE) { reg = 1; prim = 0; }
    *primary = prim;
    return reg;
}

/* ------------------------------------------------------------------ */
/* distance.py: GJK with the simplex cache                             */
/* ------------------------------------------------------------------ */
typedef struct { v2 v[GB_MAX_POLY_VERTS]; int count; double radius; } or_dproxy;

/* distance.py:352-391 DistanceProxy */
static void or_dproxy_init(or_dproxy *p, const gb_fixture *f) {
    if (f->shape_type == GB_SHAPE_CIRCLE) { p->v[0] = fx_v(f, 0); p->count = 1; }
    else if (f->shape_type == GB_SHAPE_POLYGON) {
        for (int i = 0; i < f->vertex_count; ++i) p->v[i] = fx_v(f, i);
        p->count = f->vertex_count;
    } else { p->v[0] = fx_v(f, 0); p->v[1] = fx_v(f, 1); p->count = 2; }
    p->radius = f->radius;
}
/* distance.py:393-396 get_support: first index of the maximum dot */
static int or_support(const or_dproxy *p, v2 d) {
    int best = 0;
    double bd = 0.0;
    for (int i = 0; i < p->count; ++i) {
        double x = vdot(p->v[i], d);
        if (i == 0 || x > bd) { bd = x; best = i; }
    }
    return best;
}

typedef struct { double metric; int count; int ia[3], ib[3]; } or_scache;
typedef struct { v2 wa, wb, w; double a; int ia, ib; } or_svert;

/* The reference's Simplex keeps three vertex objects; Simplex.solve2/solve3
 * rebind _v1/_v2 to fresh copies while the iteration writes new support
 * points into the list captured at the start (distance.py:469, 524-531).
 * orig[] are the three captured objects; r1/r2 say whether _v1/_v2 still
 * refer to them, d1/d2 hold the rebound copies.  _v3 is never rebound. */
typedef struct {
    or_svert orig[3];
    or_svert d1, d2;
    int r1_orig, r2_orig;
    int count;
} or_simplex;

static inline or_svert *sv1(or_simplex *s) { return s->r1_orig ? &s->orig[0] : &s->d1; }
static inline or_svert *sv2(or_simplex *s) { return s->r2_orig ? &s->orig[1] : &s->d2; }
static inline or_svert *sv3(or_simplex *s) { return &s->orig[2]; }
static inline or_svert *svk(or_simplex *s, int k) { return k == 0 ? sv1(s) : (k == 1 ? sv2(s) : sv3(s)); }

/* distance.py:177-189 Simplex.metric */
static double or_simplex_metric(or_simplex *s) {
    if (s->count == 1) return 0.0;
    if (s->count == 2) return vlen(vsub(sv1(s)->w, sv2(s)->w));
    return vcross(vsub(sv2(s)->w, sv1(s)->w), vsub(sv3(s)->w, sv1(s)->w));
}

/* distance.py:105-135 read_cache */
static void or_read_cache(or_simplex *s, const or_scache *c, const or_dproxy *pa, xform xa, const or_dproxy *pb, xform xb) {
    memset(s, 0, sizeof(*s));
    s->r1_orig = 1; s->r2_orig = 1;
    s->count = c->count;
    for (int i = 0; i < s->count; ++i) {
        or_svert *v = &s->orig[i];
        v->ia = c->ia[i]; v->ib = c->ib[i];
        v->wa = xmul(xa, pa->v[v->ia]);
        v->wb = xmul(xb, pb->v[v->ib]);
        v->w = vsub(v->wb, v->wa);
        v->a = 0.0;
    }
    if (s->count > 1) {
        double m1 = c->metric, m2 = or_simplex_metric(s);
        if (m2 < 0.5 * m1 || 2.0 * m1 < m2 || m2 < OR_EPSILON) s->count = 0;
    }
    if (s->count == 0) {
        or_svert *v = &s->orig[0];
        v->ia = 0; v->ib = 0;
        v->wa = xmul(xa, pa->v[0]);
        v->wb = xmul(xb, pb->v[0]);
        v->w = vsub(v->wb, v->wa);
        s->count = 1;
    }
}

static void or_write_cache(or_simplex *s, or_scache *c) {
    c->metric = or_simplex_metric(s);
    c->count = s->count;
    for (int i = 0; i < s->count; ++i) { c->ia[i] = svk(s, i)->ia; c->ib[i] = svk(s, i)->ib; }
}

static v2 or_closest_point(or_simplex *s) {
    if (s->count == 1) return sv1(s)->w;
    if (s->count == 2) return vadd(vscale(sv1(s)->a, sv1(s)->w), vscale(sv2(s)->a, sv2(s)->w));
    return V(0.0, 0.0);
}

static v2 or_search_direction(or_simplex *s) {
    if (s->count == 1) return vneg(sv1(s)->w);
    v2 e12 = vsub(sv2(s)->w, sv1(s)->w);
    double sgn = vcross(e12, vneg(sv1(s)->w));
    if (sgn > 0.0) return vcross_sv(1.0, e12);
    return vcross_vs(e12, 1.0);
}

static void or_witness(or_simplex *s, v2 *pa, v2 *pb) {
    if (s->count == 1) { *pa = sv1(s)->wa; *pb = sv1(s)->wb; }
    else if (s->count == 2) {
        *pa = vadd(vscale(sv1(s)->a, sv1(s)->wa), vscale(sv2(s)->a, sv2(s)->wa));
        *pb = vadd(vscale(sv1(s)->a, sv1(s)->wb), vscale(sv2(s)->a, sv2(s)->wb));
    } else {
        v2 v = vadd(vadd(vscale(sv1(s)->a, sv1(s)->wa), vscale(sv2(s)->a, sv2(s)->wa)), vscale(sv3(s)->a, sv3(s)->wa));
        *pa = v; *pb = v;
    }
}

/* distance.py:222-245 solve2 */
static void or_solve2(or_simplex *s) {
    v2 w1 = sv1(s)->w, w2 = sv2(s)->w;
    v2 e12 = vsub(w2, w1);
    double d12_2 = -vdot(w1, e12);
    if (d12_2 <= 0.0) { sv1(s)->a = 1.0; s->count = 1; return; }
    double d12_1 = vdot(w2, e12);
    if (d12_1 <= 0.0) {
        sv2(s)->a = 1.0; s->count = 1;
        s->d1 = *sv2(s); s->r1_orig = 0;
        return;
    }
    double inv = 1.0 / (d12_1 + d12_2);
    sv1(s)->a = d12_1 * inv;
    sv2(s)->a = d12_2 * inv;
    s->count = 2;
}

/* distance.py:247-338 solve3 */
static void or_solve3(or_simplex *s) {
    v2 w1 = sv1(s)->w, w2 = sv2(s)->w, w3 = sv3(s)->w;
    v2 e12 = vsub(w2, w1);
    double w1e12 = vdot(w1, e12), w2e12 = vdot(w2, e12);
    double d12_1 = w2e12, d12_2 = -w1e12;
    v2 e13 = vsub(w3, w1);
    double w1e13 = vdot(w1, e13), w3e13 = vdot(w3, e13);
    double d13_1 = w3e13, d13_2 = -w1e13;
    v2 e23 = vsub(w3, w2);
    double w2e23 = vdot(w2, e23), w3e23 = vdot(w3, e23);
    double d23_1 = w3e23, d23_2 = -w2e23;
    double n123 = vcross(e12, e13);
    double d123_1 = n123 * vcross(w2, w3);
    double d123_2 = n123 * vcross(w3, w1);
    double d123_3 = n123 * vcross(w1, w2);
    if (d12_2 <= 0.0 && d13_2 <= 0.0) { sv1(s)->a = 1.0; s->count = 1; return; }
    if (d12_1 > 0.0 && d12_2 > 0.0 && d123_3 <= 0.0) {
        double inv = 1.0 / (d12_1 + d12_2);
        sv1(s)->a = d12_1 * inv; sv2(s)->a = d12_2 * inv; s->count = 2; return;
    }
    if (d13_1 > 0.0 && d13_2 > 0.0 && d123_2 <= 0.0) {
        double inv = 1.0 / (d13_1 + d13_2);
        sv1(s)->a = d13_1 * inv; sv3(s)->a = d13_2 * inv; s->count = 2;
        s->d2 = *sv3(s); s->r2_orig = 0;
        return;
    }
    if (d12_1 <= 0.0 && d23_2 <= 0.0) {
        sv2(s)->a = 1.0; s->count = 1;
        s->d1 = *sv2(s); s->r1_orig = 0;
        return;
    }
    if (d13_1 <= 0.0 && d23_1 <= 0.0) {
        sv3(s)->a = 1.0; s->count = 1;
        s->d1 = *sv3(s); s->r1_orig = 0;
        return;
    }
    if (d23_1 > 0.0 && d23_2 > 0.0 && d123_1 <= 0.0) {
        double inv = 1.0 / (d23_1 + d23_2);
        sv2(s)->a = d23_1 * inv; sv3(s)->a = d23_2 * inv; s->count = 2;
        s->d1 = *sv3(s); s->r1_orig = 0;
        return;
    }
    double inv = 1.0 / (d123_1 + d123_2 + d123_3);
    sv1(s)->a = d123_1 * inv; sv2(s)->a = d123_2 * inv; sv3(s)->a = d123_3 * inv;
    s->count = 3;
}

/* distance.py:424-561 shape_distance; returns the distance, the witness
 * points (pa_out, pb_out) and updates the cache. */
static double or_shape_distance(const or_dproxy *A, const or_dproxy *B, xform xa, xform xb, int use_radii,
                                or_scache *cache, v2 *pa_out, v2 *pb_out) {
    or_simplex s;
    or_read_cache(&s, cache, A, xa, B, xb);
    int save_ia[3], save_ib[3], save_n;
    int iter = 0;
    while (iter < 20) {
        save_n = s.count;
        for (int i = 0; i < s.count; ++i) { save_ia[i] = svk(&s, i)->ia; save_ib[i] = svk(&s, i)->ib; }
        if (s.count == 2) or_solve2(&s);
        else if (s.count == 3) { or_solve3(&s); break; }
        (void)or_closest_point(&s);
        v2 d = or_search_direction(&s);
        if (vlen2(d) < OR_EPSILON_SQR) break;
        or_svert *vx = &s.orig[s.count]; /* the captured list, not the rebound attribute */
        vx->ia = or_support(A, rmul_t(xa.q, vneg(d)));
        vx->wa = xmul(xa, A->v[vx->ia]);
        vx->ib = or_support(B, rmul_t(xb.q, d));
        vx->wb = xmul(xb, B->v[vx->ib]);
        vx->w = vsub(vx->wb, vx->wa);
        ++iter;
        int dup = 0;
        for (int i = 0; i < save_n; ++i)
            if (save_ia[i] == vx->ia && save_ib[i] == vx->ib) { dup = 1; break; }
        if (dup) break;
        s.count += 1;
    }
    v2 pa, pb;
    or_witness(&s, &pa, &pb);
    double dist = vlen(vsub(pa, pb));
    or_write_cache(&s, cache);
    if (use_radii) {
        double ra = A->radius, rb = B->radius;
        if (dist > ra + rb && dist > OR_EPSILON) {
            dist -= ra + rb;
            v2 normal = vnormalized(vsub(pb, pa));
            pa = vadd(pa, vscale(ra, normal));
            pb = vsub(pb, vscale(rb, normal));
        } else {
            v2 p = vscale(0.5, vadd(pa, pb));
            pa = p; pb = p;
            dist = 0.0;
        }
    }
    if (pa_out) *pa_out = pa;
    if (pb_out) *pb_out = pb;
    return dist;
}

/* ------------------------------------------------------------------ */
/* common.py:870-923 Sweep                                             */
/* ------------------------------------------------------------------ */
typedef struct { v2 lc, c0, c; double a0, a, alpha0; } or_sweep;

static xform or_sweep_xf(const or_sweep *sw, double beta) {
    xform x;
    x.p = vadd(vscale(1.0 - beta, sw->c0), vscale(beta, sw->c));
    x.q = rot_of((1.0 - beta) * sw->a0 + beta * sw->a);
    x.p = vsub(x.p, rmul(x.q, sw->lc));
    return x;
}
static void or_sweep_advance(or_sweep *sw, double alpha) {
    double beta = (alpha - sw->alpha0) / (1.0 - sw->alpha0);
    sw->c0 = vadd(vscale(1.0 - beta, sw->c0), vscale(beta, sw->c));
    sw->a0 = (1.0 - beta) * sw->a0 + beta * sw->a;
    sw->alpha0 = alpha;
}
static void or_sweep_normalize(or_sweep *sw) {
    const double TWO_PI = 2.0 * 3.141592653589793;
    double d = TWO_PI * floor(sw->a0 / TWO_PI);
    sw->a0 -= d;
    sw->a -= d;
}

/* ------------------------------------------------------------------ */
/* toi.py:45-391                                                        */
/* ------------------------------------------------------------------ */
#define SF_POINTS 0
#define SF_FACE_A 1
#define SF_FACE_B 2
#define TOI_UNKNOWN 0
#define TOI_FAILED 1
#define TOI_OVERLAPPED 2
#define TOI_TOUCHING 3
#define TOI_SEPARATED 4

typedef struct {
    const or_dproxy *A, *B;
    or_sweep sa, sb;
    int type;
    v2 axis, lp;
} or_sepfn;

/* toi.py:53-123 SeparationFunction.initialize.  For POINTS the reference
 * keeps the unnormalised axis (it assigns `.normalized` to a local). */
static void or_sep_init(or_sepfn *f, const or_scache *c, double t1) {
    xform xa = or_sweep_xf(&f->sa, t1), xb = or_sweep_xf(&f->sb, t1);
    int ia0 = c->ia[0], ib0 = c->ib[0];
    if (c->count == 1) {
        f->type = SF_POINTS;
        v2 pa = xmul(xa, f->A->v[ia0]);
        v2 pb = xmul(xb, f->B->v[ib0]);
        f->axis = vsub(pb, pa);
        return;
    }
    int ia1 = c->ia[1], ib1 = c->ib[1];
    if (ia0 == ia1) {
        f->type = SF_FACE_B;
        v2 lb1 = f->B->v[ib0], lb2 = f->B->v[ib1];
        f->axis = vnormalized(vcross_vs(vsub(lb2, lb1), 1.0));
        v2 normal = rmul(xb.q, f->axis);
        f->lp = vscale(0.5, vadd(lb1, lb2));
        v2 pb = xmul(xb, f->lp);
        v2 pa = xmul(xa, f->A->v[ia0]);
        double s = vdot(vsub(pa, pb), normal);
        if (s < 0.0) f->axis = vneg(f->axis);
    } else {
        f->type = SF_FACE_A;
        v2 la1 = f->A->v[ia0], la2 = f->A->v[ia1];
        f->axis = vnormalized(vcross_vs(vsub(la2, la1), 1.0));
        v2 normal = rmul(xa.q, f->axis);
        f->lp = vscale(0.5, vadd(la1, la2));
        v2 pa = xmul(xa, f->lp);
        v2 pb = xmul(xb, f->B->v[ib0]);
        double s = vdot(vsub(pb, pa), normal);
        if (s < 0.0) f->axis = vneg(f->axis);
    }
}

static double or_sep_find_min(or_sepfn *f, double t, int *ia, int *ib) {
    xform xa = or_sweep_xf(&f->sa, t), xb = or_sweep_xf(&f->sb, t);
    if (f->type == SF_POINTS) {
        v2 axa = rmul_t(xa.q, f->axis);
        v2 axb = rmul_t(xb.q, vneg(f->axis));
        *ia = or_support(f->A, axa);
        *ib = or_support(f->B, axb);
        v2 pa = xmul(xa, f->A->v[*ia]);
        v2 pb = xmul(xb, f->B->v[*ib]);
        return vdot(vsub(pb, pa), f->axis);
    } else if (f->type == SF_FACE_A) {
        v2 normal = rmul(xa.q, f->axis);
        v2 pa = xmul(xa, f->lp);
        v2 axb = rmul_t(xb.q, vneg(normal));
        *ia = -1;
        *ib = or_support(f->B, axb);
        v2 pb = xmul(xb, f->B->v[*ib]);
        return vdot(vsub(pb, pa), normal);
    } else {
        v2 normal = rmul(xb.q, f->axis);
        v2 pb = xmul(xb, f->lp);
        v2 axa = rmul_t(xa.q, vneg(normal));
        *ib = -1;
        *ia = or_support(f->A, axa);
        v2 pa = xmul(xa, f->A->v[*ia]);
        return vdot(vsub(pa, pb), normal);
    }
}

static double or_sep_eval(or_sepfn *f, int ia, int ib, double t) {
    xform xa = or_sweep_xf(&f->sa, t), xb = or_sweep_xf(&f->sb, t);
    if (f->type == SF_POINTS) {
        v2 pa = xmul(xa, f->A->v[ia]);
        v2 pb = xmul(xb, f->B->v[ib]);
        return vdot(vsub(pb, pa), f->axis);
    } else if (f->type == SF_FACE_A) {
        v2 normal = rmul(xa.q, f->axis);
        v2 pa = xmul(xa, f->lp);
        v2 pb = xmul(xb, f->B->v[ib]);
        return vdot(vsub(pb, pa), normal);
    } else {
        v2 normal = rmul(xb.q, f->axis);
        v2 pb = xmul(xb, f->lp);
        v2 pa = xmul(xa, f->A->v[ia]);
        return vdot(vsub(pa, pb), normal);
    }
}

/* toi.py:216-391 time_of_impact.  The inner push-back loop has no bound in
 * the reference; the restatement stops it after 1000 rounds and reports
 * FAILED (never reached in the test scenes). */
static int or_time_of_impact(const or_dproxy *A, const or_dproxy *B, const or_sweep *swa, const or_sweep *swb,
                             double t_max, double *t_out) {
    int state = TOI_UNKNOWN;
    double output_t = t_max;
    or_sepfn f;
    f.A = A; f.B = B;
    f.sa = *swa; f.sb = *swb;
    or_sweep_normalize(&f.sa);
    or_sweep_normalize(&f.sb);
    double total_radius = A->radius + B->radius;
    double target = pymax(OR_LINEAR_SLOP, total_radius - 3.0 * OR_LINEAR_SLOP);
    double tolerance = 0.25 * OR_LINEAR_SLOP;
    double t1 = 0.0;
    int iter = 0;
    or_scache cache;
    memset(&cache, 0, sizeof(cache));
    for (;;) {
        xform xa = or_sweep_xf(&f.sa, t1), xb = or_sweep_xf(&f.sb, t1);
        double dist = or_shape_distance(A, B, xa, xb, 0, &cache, NULL, NULL);
        if (dist <= 0.0) { state = TOI_OVERLAPPED; output_t = 0.0; break; }
        if (dist < target + tolerance) { state = TOI_TOUCHING; output_t = t1; break; }
        or_sep_init(&f, &cache, t1);
        int done = 0;
        double t2 = t_max;
        int push_back = 0;
        for (;;) {
            int ia, ib;
            double s2 = or_sep_find_min(&f, t2, &ia, &ib);
            if (s2 > target + tolerance) { state = TOI_SEPARATED; output_t = t_max; done = 1; break; }
            if (s2 > target - tolerance) { t1 = t2; break; }
            double s1 = or_sep_eval(&f, ia, ib, t1);
            if (s1 < target - tolerance) { state = TOI_FAILED; output_t = t1; done = 1; break; }
            if (s1 <= target + tolerance) { state = TOI_TOUCHING; output_t = t1; done = 1; break; }
            int root_iter = 0;
            double a1 = t1, a2 = t2;
            for (;;) {
                double t;
                if (root_iter & 1) t = a1 + (target - s1) * (a2 - a1) / (s2 - s1);
                else t = 0.5 * (a1 + a2);
                double s = or_sep_eval(&f, ia, ib, t);
                if (fabs(s - target) < tolerance) { t2 = t; break; }
                if (s > target) { a1 = t; s1 = s; }
                else { a2 = t; s2 = s; }
                ++root_iter;
                if (root_iter == 50) break;
            }
            ++push_back;
            if (push_back == 1000) { state = TOI_FAILED; output_t = t1; done = 1; break; }
        }
        ++iter;
        if (done) break;
        if (iter == 20) { state = TOI_FAILED; output_t = t1; break; }
    }
    *t_out = output_t;
    return state;
}

#endif /* ORACLE_COLLIDE_H */

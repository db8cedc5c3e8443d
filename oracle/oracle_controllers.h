/*
 * oracle_controllers.h -- TEST INFRASTRUCTURE: float64 restatement of
 * pypybox2d's controllers (pypybox2d/controllers.py), run at the start of
 * every solve (world.py:476-479), and of the shapes' submerged areas they
 * use (shapes.py:219-236 circle, :538-616 polygon, :751-778 edge, :866-882
 * loop).  Included by oracle.c after the world structure.
 *
 * The circle's submerged segment calls asin and pow(y, 1.5): libm's in the
 * ORACLE_LIBM build (what CPython's math.asin and ** call), and in the
 * portable build the Maclaurin-series arcsine and y * sqrt(y) that the GPU
 * kernels spell the same way.
 */
#ifndef ORACLE_CONTROLLERS_H
#define ORACLE_CONTROLLERS_H

#define OR_PI 3.141592653589793

#ifdef ORACLE_LIBM
static double (*volatile or_asin_fn)(double) = asin;
static inline double or_asin(double x) { return or_asin_fn(x); }
static inline double or_pow15(double y) { return or_pow_fn(y, 1.5); }
#else
/* asin: Maclaurin series of asin on [0, 1/2], sum (2n)! / (4^n (n!)^2 (2n+1))
 * x^(2n+1) to n = 23 in Horner form, and pi/2 - 2 asin(sqrt((1 - x) / 2))
 * above 1/2 */
static inline double or_asin_series(double x) {
    static const double c[24] = {
        1.0, 0.16666666666666666, 0.075, 0.044642857142857144, 0.030381944444444444, 0.022372159090909092,
        0.017352764423076924, 0.01396484375, 0.011551800896139705, 0.009761609529194078, 0.008390335809616815,
        0.0073125258735988454, 0.006447210311889649, 0.005740037670841924, 0.005153309682319905,
        0.004660143486915096, 0.004240907093679363, 0.003880964558837669, 0.0035692053938259347,
        0.003297059503473485, 0.0030578216492580306, 0.002846178401108942, 0.00265787063820729,
        0.0024894486782468836};
    double x2 = x * x;
    double p = c[23];
    for (int n = 22; n >= 1; --n) p = c[n] + x2 * p;
    return x + (x * x2) * p;
}
static inline double or_asin(double x) {
    double a = x < 0.0 ? -x : x;
    double r = a <= 0.5 ? or_asin_series(a) : 1.5707963267948966 - 2.0 * or_asin_series(sqrt((1.0 - a) * 0.5));
    return x < 0.0 ? -r : r;
}
static inline double or_pow15(double y) { return y * sqrt(y); }
#endif

typedef struct { double area; v2 c; } or_sub;

/* Circle.compute_submerged_area */
static or_sub sub_circle(const gb_fixture *f, xform x, v2 n, double off) {
    v2 p = xmul(x, V(f->vx[0], f->vy[0]));
    double r = f->radius;
    double l = -(vdot(n, p) - off);
    or_sub s;
    s.c = p;
    if (l < -r + OR_EPSILON) { s.area = 0.0; return s; }
    if (l > r) { s.area = OR_PI * SQ(r); return s; }
    double r2 = SQ(r), l2 = SQ(l);
    double area = r2 * (or_asin(l / r) + OR_PI / 2.0) + l * sqrt(r2 - l2);
    double com = -2.0 / 3.0 * or_pow15(r2 - l2) / area;
    s.area = area;
    s.c = vadd(p, vscale(com, n));
    return s;
}

/* Polygon.compute_submerged_area; dry or submerged, compute_mass(density) */
static or_sub sub_polygon(const gb_fixture *f, xform x, v2 n, double off, double density) {
    int cnt = f->vertex_count;
    double depth[GB_MAX_POLY_VERTS];
    v2 nl = rmul_t(x.q, n);
    double offl = off - vdot(n, x.p);
    int last = 0, into = -1, outof = -1, dives = 0;
    for (int i = 0; i < cnt; ++i) {
        depth[i] = vdot(nl, V(f->vx[i], f->vy[i])) - offl;
        int sub = depth[i] < OR_EPSILON;
        if (i > 0) {
            if (sub) {
                if (!last) { into = i - 1; dives++; }
            } else if (last) {
                outof = i - 1; dives++;
            }
        }
        last = sub;
    }
    or_sub s;
    if (dives == 0) {
        v2 sref = V(f->vx[0], f->vy[0]);
        for (int i = 1; i < cnt; ++i) sref = vadd(sref, V(f->vx[i], f->vy[i]));
        sref = V(sref.x / (double)cnt, sref.y / (double)cnt);
        v2 center = V(0.0, 0.0);
        double area = 0.0;
        double inv3 = 1.0 / 3.0;
        for (int i = 0; i < cnt; ++i) {
            int j = (i + 1) % cnt;
            v2 e1 = vsub(V(f->vx[i], f->vy[i]), sref), e2 = vsub(V(f->vx[j], f->vy[j]), sref);
            double D = vcross(e1, e2);
            double tri = 0.5 * D;
            area += tri;
            center = vadd(center, vscale(tri * inv3, vadd(e1, e2)));
        }
        double mass = density * area;
        center = V(center.x / area, center.y / area);
        s.c = xmul(x, vadd(center, sref));
        s.area = last ? mass / density : 0.0;
        return s;
    }
    if (dives == 1) {
        if (into < 0) into = cnt - 1;
        else outof = cnt - 1;
    }
    int into2 = (into + 1) % cnt, outof2 = (outof + 1) % cnt;
    double il = -depth[into] / (depth[into2] - depth[into]);
    double ol = -depth[outof] / (depth[outof2] - depth[outof]);
    v2 iv = vadd(vscale(1.0 - il, V(f->vx[into], f->vy[into])), vscale(il, V(f->vx[into2], f->vy[into2])));
    v2 ov = vadd(vscale(1.0 - ol, V(f->vx[outof], f->vy[outof])), vscale(ol, V(f->vx[outof2], f->vy[outof2])));
    double area = 0.0;
    v2 center = V(0.0, 0.0);
    v2 p2 = V(f->vx[into2], f->vy[into2]);
    int i = into2;
    while (i != outof2) {
        i = (i + 1) % cnt;
        v2 p3 = (i == outof2) ? ov : V(f->vx[i], f->vy[i]);
        v2 e1 = vsub(p2, iv), e2 = vsub(p3, iv);
        double d = vcross(e1, e2);
        double tri = 0.5 * d;
        area += tri;
        v2 t = vscale(tri, vadd(vadd(iv, p2), p3));
        center = vadd(center, V(t.x / 3.0, t.y / 3.0));
        p2 = p3;
    }
    s.area = area;
    s.c = xmul(x, vscale(1.0 / area, center));
    return s;
}

/* Edge.compute_submerged_area */
static or_sub sub_edge(const gb_fixture *f, xform x, v2 n, double off) {
    v2 v0 = vscale(off, n);
    v2 v1 = xmul(x, V(f->vx[0], f->vy[0]));
    v2 v2_ = xmul(x, V(f->vx[1], f->vy[1]));
    double d1 = vdot(n, v1) - off, d2 = vdot(n, v2_) - off;
    or_sub s;
    if (d1 > 0.0) {
        if (d2 > 0.0) { s.area = 0.0; s.c = v1; return s; }
        v1 = vadd(vscale(-d2 / (d1 - d2), v1), vscale(d1 / (d1 - d2), v2_));
    } else if (d2 > 0.0) {
        v2_ = vadd(vscale(-d2 / (d1 - d2), v1), vscale(d1 / (d1 - d2), v2_));
    }
    v2 e1 = vsub(v1, v0), e2 = vsub(v2_, v0);
    s.area = 0.5 * vcross(e1, e2);
    s.c = vscale(1.0 / 3.0, vadd(vadd(v0, v1), v2_));
    return s;
}

/* Body.apply_force (body.py:477-491) */
static void ctl_apply_force(gb_body *b, v2 force, v2 point) {
    if (b->type != GB_BODY_DYNAMIC) return;
    if (!body_awake(b)) set_awake(b, 1);
    b->fx = b->fx + force.x;
    b->fy = b->fy + force.y;
    b->torque += vcross(vsub(point, V(b->cx, b->cy)), force);
}

/* BuoyancyController.step (controllers.py:173-222) */
static void buoyancy_step(or_world *w, const gb_controller *C, const int *list) {
    v2 gravity = (C->flags & GB_CTRL_OWN_GRAVITY) ? V(C->gravity_x, C->gravity_y) : w->gravity;
    v2 n = V(C->normal_x, C->normal_y);
    double off = C->offset;
    int nl = C->body_count;
    int *awake = (int *)malloc(sizeof(int) * (size_t)(nl ? nl : 1));
    for (int i = 0; i < nl; ++i) awake[i] = body_awake(&w->b[list[i]]);   /* the list is taken first */
    for (int i = 0; i < nl; ++i) {
        if (!awake[i]) continue;
        gb_body *b = &w->b[list[i]];
        xform x = body_xf(b);
        v2 area_c = V(0.0, 0.0), mass_c = V(0.0, 0.0);
        double area = 0.0, mass = 0.0, dens = 1.0;
        for (int k = 0; k < b->fixture_count;) {
            const gb_fixture *f = &w->f[b->fixture_start + k];
            or_sub s;
            if (f->flags & GB_FIX_LOOP_CHILD) {
                /* the children of one loop, summed (the centre not divided) */
                double ta = 0.0;
                v2 tc = V(0.0, 0.0);
                int c = 0;
                do {
                    or_sub e = sub_edge(&w->f[b->fixture_start + k + c], x, n, off);
                    tc = vadd(tc, vscale(e.area, e.c));
                    ta += e.area;
                    ++c;
                } while (k + c < b->fixture_count &&
                         (w->f[b->fixture_start + k + c].flags & (GB_FIX_LOOP_CHILD | GB_FIX_LOOP_FIRST)) == GB_FIX_LOOP_CHILD);
                s.area = ta;
                s.c = tc;
                k += c;
            } else {
                if (f->shape_type == GB_SHAPE_CIRCLE) s = sub_circle(f, x, n, off);
                else if (f->shape_type == GB_SHAPE_POLYGON) s = sub_polygon(f, x, n, off, dens);
                else s = sub_edge(f, x, n, off);
                k += 1;
            }
            area += s.area;
            area_c = vadd(area_c, vscale(s.area, s.c));
            mass += s.area * dens;
            mass_c = vadd(mass_c, vscale(s.area * dens, s.c));
        }
        if (!(area >= OR_EPSILON)) continue;
        area_c = V(area_c.x / area, area_c.y / area);
        mass_c = V(mass_c.x / mass, mass_c.y / mass);
        ctl_apply_force(b, vscale(-C->density * area, gravity), mass_c);
        v2 lin_vel = vadd(V(b->vx, b->vy), vcross_sv(b->w, vsub(area_c, V(b->cx, b->cy))));
        v2 drag = vscale(-C->linear_drag * area, vsub(lin_vel, V(C->velocity_x, C->velocity_y)));
        ctl_apply_force(b, drag, area_c);
        if (b->type == GB_BODY_DYNAMIC) {
            double inertia = b->I + b->mass * vlen2(V(b->lcx, b->lcy));
            b->torque += -inertia / b->mass * area * b->w * C->angular_drag;
        }
    }
    free(awake);
}

/* GravityController.step (controllers.py:263-280) */
static void gravity_step(or_world *w, const gb_controller *C, const int *list) {
    int nl = C->body_count;
    int inv_sqr = (C->flags & GB_CTRL_INV_SQR) != 0;
    for (int i = 0; i < nl; ++i)
        for (int j = 0; j < nl; ++j) {
            if (i == j) continue;
            gb_body *b1 = &w->b[list[i]], *b2 = &w->b[list[j]];
            v2 c1 = V(b1->cx, b1->cy), c2 = V(b2->cx, b2->cy);
            v2 d = vsub(c2, c1);
            double r2 = vlen2(d);
            v2 f = vscale(C->G / r2 * b1->mass * b2->mass, d);
            if (inv_sqr) {
                double r = sqrt(r2);
                f = V(f.x / r, f.y / r);
            }
            ctl_apply_force(b1, f, c1);
            ctl_apply_force(b2, vneg(f), c2);
        }
}

/* the world's controllers, in World.controllers order (world.py:476-479) */
static void controllers_step(or_world *w) {
    for (int k = 0; k < w->nctl; ++k) {
        const gb_controller *C = &w->ctl[k];
        const int *list = w->ctl_bodies + C->body_start;
        if (C->type == GB_CONTROLLER_BUOYANCY) buoyancy_step(w, C, list);
        else if (C->type == GB_CONTROLLER_GRAVITY) gravity_step(w, C, list);
    }
}

#endif /* ORACLE_CONTROLLERS_H */

// Controllers (pypybox2d/controllers.py): force rules that run over their
// bodies at the start of every solve (world.py:476-479), before the islands
// are built.  A world's controllers run in World.controllers order, one after
// the other (a group barrier between them); within a controller each body is
// one thread, which alone writes that body's force, torque and awake state.
//
// Everything is float64 in the reference's operation order (the Vec2
// arithmetic of vec2module.c: a float times a vector scales both components,
// a vector over a float divides both).  The circle's submerged segment takes
// asin and pow(y, 1.5); the float64 unit spells them as gb_asin below and
// y * sqrt(y), as the CPU restatement's portable build does.
#pragma once

#define GB_PI 3.141592653589793

// asin: the Maclaurin series sum_n (2n)! / (4^n (n!)^2 (2n + 1)) x^(2n+1) on
// [0, 1/2] (24 terms, Horner form in x^2; the first omitted term is below
// 1e-17 relative), and asin(x) = pi/2 - 2 asin(sqrt((1 - x) / 2)) above 1/2.
// Within 5e-16 relative of a correctly rounded asin.
GB_HD double gb_asin_series(double x) {
    const double x2 = x * x;
    double p = 0.0024894486782468836;
    p = 0.00265787063820729 + x2 * p;
    p = 0.002846178401108942 + x2 * p;
    p = 0.0030578216492580306 + x2 * p;
    p = 0.003297059503473485 + x2 * p;
    p = 0.0035692053938259347 + x2 * p;
    p = 0.003880964558837669 + x2 * p;
    p = 0.004240907093679363 + x2 * p;
    p = 0.004660143486915096 + x2 * p;
    p = 0.005153309682319905 + x2 * p;
    p = 0.005740037670841924 + x2 * p;
    p = 0.006447210311889649 + x2 * p;
    p = 0.0073125258735988454 + x2 * p;
    p = 0.008390335809616815 + x2 * p;
    p = 0.009761609529194078 + x2 * p;
    p = 0.011551800896139705 + x2 * p;
    p = 0.01396484375 + x2 * p;
    p = 0.017352764423076924 + x2 * p;
    p = 0.022372159090909092 + x2 * p;
    p = 0.030381944444444444 + x2 * p;
    p = 0.044642857142857144 + x2 * p;
    p = 0.075 + x2 * p;
    p = 0.16666666666666666 + x2 * p;
    return x + (x * x2) * p;
}
GB_HD double gb_asin(double x) {
    const double a = x < 0.0 ? -x : x;
    double r;
    if (a <= 0.5) r = gb_asin_series(a);
    else r = 1.5707963267948966 - 2.0 * gb_asin_series(sqrt((1.0 - a) * 0.5));
    return x < 0.0 ? -r : r;
}

struct SubArea { double area, cx, cy; };

// Transform_mul (transform.c): position + col1 * v.x + col2 * v.y, left to right
__device__ __forceinline__ void ctl_xmul(const xform2<double> &x, double vx, double vy, double *ox, double *oy) {
    *ox = x.p.x + x.q.c * vx + (-x.q.s) * vy;
    *oy = x.p.y + x.q.s * vx + x.q.c * vy;
}

// Circle.compute_submerged_area (shapes.py:219-236)
template <class R> __device__ SubArea submerged_circle(const Shape<R> &s, const xform2<double> &x, double nx, double ny,
                                                       double off) {
    double px, py;
    ctl_xmul(x, (double)s.v[0].x, (double)s.v[0].y, &px, &py);
    const double r = (double)s.radius;
    const double l = -((nx * px + ny * py) - off);
    if (l < -r + GB_EPSILON) return SubArea{0.0, px, py};
    if (l > r) return SubArea{GB_PI * (r * r), px, py};
    const double r2 = r * r, l2 = l * l;
    const double area = r2 * (gb_asin(l / r) + GB_PI / 2.0) + l * sqrt(r2 - l2);
    const double y = r2 - l2;
    const double com = -2.0 / 3.0 * (y * sqrt(y)) / area;
    return SubArea{area, px + nx * com, py + ny * com};
}

// Polygon.compute_submerged_area (shapes.py:538-616); a dry or submerged
// polygon takes compute_mass's area and centroid (shapes.py:336-419)
template <class R> __device__ SubArea submerged_polygon(const Shape<R> &s, const xform2<double> &x, double nx, double ny,
                                                        double off, double density) {
    const int n = s.count;
    double vx[GB_MAX_POLY_VERTS], vy[GB_MAX_POLY_VERTS], depth[GB_MAX_POLY_VERTS];
    for (int i = 0; i < n; ++i) { vx[i] = (double)s.v[i].x; vy[i] = (double)s.v[i].y; }
    // the plane in shape coordinates (Mat22_mul_t_vec)
    const double nlx = x.q.c * nx + x.q.s * ny;
    const double nly = (-x.q.s) * nx + x.q.c * ny;
    const double offl = off - (nx * x.p.x + ny * x.p.y);
    bool last = false;
    int into = -1, outof = -1, dives = 0;
    for (int i = 0; i < n; ++i) {
        depth[i] = (nlx * vx[i] + nly * vy[i]) - offl;
        const bool sub = depth[i] < GB_EPSILON;
        if (i > 0) {
            if (sub) {
                if (!last) { into = i - 1; ++dives; }
            } else if (last) {
                outof = i - 1; ++dives;
            }
        }
        last = sub;
    }
    if (dives == 0) {
        // compute_mass(density): reference point s = mean of the vertices
        double sx = vx[0], sy = vy[0];
        for (int i = 1; i < n; ++i) { sx = sx + vx[i]; sy = sy + vy[i]; }
        sx = sx / (double)n; sy = sy / (double)n;
        double cx = 0.0, cy = 0.0, area = 0.0;
        const double inv3 = 1.0 / 3.0;
        for (int i = 0; i < n; ++i) {
            const int j = (i + 1) % n;
            const double e1x = vx[i] - sx, e1y = vy[i] - sy, e2x = vx[j] - sx, e2y = vy[j] - sy;
            const double D = e1x * e2y - e1y * e2x;
            const double tri = 0.5 * D;
            area += tri;
            const double k = tri * inv3;
            cx = cx + k * (e1x + e2x);
            cy = cy + k * (e1y + e2y);
        }
        const double mass = density * area;
        cx = cx / area; cy = cy / area;
        double wx, wy;
        ctl_xmul(x, cx + sx, cy + sy, &wx, &wy);
        return SubArea{last ? mass / density : 0.0, wx, wy};
    }
    if (dives == 1) {
        if (into < 0) into = n - 1;
        else outof = n - 1;
    }
    const int into2 = (into + 1) % n, outof2 = (outof + 1) % n;
    const double il = -depth[into] / (depth[into2] - depth[into]);
    const double ol = -depth[outof] / (depth[outof2] - depth[outof]);
    const double ivx = vx[into] * (1.0 - il) + vx[into2] * il, ivy = vy[into] * (1.0 - il) + vy[into2] * il;
    const double ovx = vx[outof] * (1.0 - ol) + vx[outof2] * ol, ovy = vy[outof] * (1.0 - ol) + vy[outof2] * ol;
    double area = 0.0, cx = 0.0, cy = 0.0;
    double p2x = vx[into2], p2y = vy[into2];
    int i = into2;
    while (i != outof2) {
        i = (i + 1) % n;
        double p3x, p3y;
        if (i == outof2) { p3x = ovx; p3y = ovy; }
        else { p3x = vx[i]; p3y = vy[i]; }
        const double e1x = p2x - ivx, e1y = p2y - ivy, e2x = p3x - ivx, e2y = p3y - ivy;
        const double d = e1x * e2y - e1y * e2x;
        const double tri = 0.5 * d;
        area += tri;
        cx = cx + (tri * ((ivx + p2x) + p3x)) / 3.0;
        cy = cy + (tri * ((ivy + p2y) + p3y)) / 3.0;
        p2x = p3x; p2y = p3y;
    }
    const double inv = 1.0 / area;
    double wx, wy;
    ctl_xmul(x, cx * inv, cy * inv, &wx, &wy);
    return SubArea{area, wx, wy};
}

// Edge.compute_submerged_area (shapes.py:751-778): the triangle between the
// plane point offset * normal and the edge's submerged part
template <class R> __device__ SubArea submerged_edge(const Shape<R> &s, const xform2<double> &x, double nx, double ny,
                                                     double off) {
    const double v0x = off * nx, v0y = off * ny;
    double v1x, v1y, v2x, v2y;
    ctl_xmul(x, (double)s.v[0].x, (double)s.v[0].y, &v1x, &v1y);
    ctl_xmul(x, (double)s.v[1].x, (double)s.v[1].y, &v2x, &v2y);
    const double d1 = (nx * v1x + ny * v1y) - off;
    const double d2 = (nx * v2x + ny * v2y) - off;
    if (d1 > 0.0) {
        if (d2 > 0.0) return SubArea{0.0, v1x, v1y};
        const double a = -d2 / (d1 - d2), b = d1 / (d1 - d2);
        const double tx = a * v1x + b * v2x, ty = a * v1y + b * v2y;
        v1x = tx; v1y = ty;
    } else if (d2 > 0.0) {
        const double a = -d2 / (d1 - d2), b = d1 / (d1 - d2);
        const double tx = a * v1x + b * v2x, ty = a * v1y + b * v2y;
        v2x = tx; v2y = ty;
    }
    const double e1x = v1x - v0x, e1y = v1y - v0y, e2x = v2x - v0x, e2y = v2y - v0y;
    const double third = 1.0 / 3.0;
    return SubArea{0.5 * (e1x * e2y - e1y * e2x), third * ((v0x + v1x) + v2x), third * ((v0y + v1y) + v2y)};
}

// Body.apply_force (body.py:477-491): dynamic bodies only; wakes the body
template <class R> __device__ __forceinline__ void ctl_apply_force(const WView<R> &w, int b, double fx, double fy,
                                                                   double px, double py) {
    const int g = w.bb + b;
    wake_body(w, b);
    const vec2<double> c = w.B.b_c[g];
    const vec2<R> f = w.B.b_f[g];
    w.B.b_f[g] = mk<R>((R)((double)f.x + fx), (R)((double)f.y + fy));
    w.B.b_torque[g] = (R)((double)w.B.b_torque[g] + ((px - c.x) * fy - (py - c.y) * fx));
}

// BuoyancyController.step for one body (controllers.py:173-222)
template <class R> __device__ void buoyancy_body(const WView<R> &w, const gb_controller &C, int b) {
    if (!w.awake(b) || w.btype(b) != GB_BODY_DYNAMIC) return;   // asleep: skipped; others: apply_* do nothing
    const int g = w.bb + b;
    const xform2<double> x = w.xfd(b);
    const double nx = C.normal_x, ny = C.normal_y, off = C.offset;
    const double dens = 1.0;   // use_density is not supported (shapes carry no density attribute)
    double area = 0.0, mass = 0.0, acx = 0.0, acy = 0.0, mcx = 0.0, mcy = 0.0;
    const int f0 = w.B.b_fstart[g], nf = w.B.b_fcount[g];
    for (int k = 0; k < nf;) {
        const Shape<R> s = w.shape(f0 + k);
        SubArea sa;
        if (s.flags & GB_FIX_LOOP_CHILD) {
            // Loop.compute_submerged_area (shapes.py:866-882): the children's
            // areas and area-weighted centres summed, the centre not divided
            double ta = 0.0, tcx = 0.0, tcy = 0.0;
            int c = 0;
            do {
                const SubArea e = submerged_edge(w.shape(f0 + k + c), x, nx, ny, off);
                tcx = tcx + e.area * e.cx;
                tcy = tcy + e.area * e.cy;
                ta += e.area;
                ++c;
            } while (k + c < nf && (w.B.f_flags[w.fb + f0 + k + c] & (GB_FIX_LOOP_CHILD | GB_FIX_LOOP_FIRST)) == GB_FIX_LOOP_CHILD);
            sa = SubArea{ta, tcx, tcy};
            k += c;
        } else {
            if (s.type == GB_SHAPE_CIRCLE) sa = submerged_circle(s, x, nx, ny, off);
            else if (s.type == GB_SHAPE_POLYGON) sa = submerged_polygon(s, x, nx, ny, off, dens);
            else sa = submerged_edge(s, x, nx, ny, off);
            k += 1;
        }
        area += sa.area;
        acx = acx + sa.area * sa.cx;
        acy = acy + sa.area * sa.cy;
        mass += sa.area * dens;
        const double m = sa.area * dens;
        mcx = mcx + m * sa.cx;
        mcy = mcy + m * sa.cy;
    }
    if (!(area >= GB_EPSILON)) return;
    acx = acx / area; acy = acy / area;
    mcx = mcx / mass; mcy = mcy / mass;
    double gx = w.H->gx, gy = w.H->gy;
    if (C.flags & GB_CTRL_OWN_GRAVITY) { gx = C.gravity_x; gy = C.gravity_y; }
    const double kb = -C.density * area;
    ctl_apply_force(w, b, kb * gx, kb * gy, mcx, mcy);
    // linear drag at the submerged centroid (Body.get_linear_velocity_from_world_point)
    const vec2<double> c = w.B.b_c[g];
    const double wv = (double)w.B.b_w[g];
    const vec2<R> v = w.B.b_v[g];
    const double lvx = (double)v.x + (-wv) * (acy - c.y), lvy = (double)v.y + wv * (acx - c.x);
    const double kd = -C.linear_drag * area;
    ctl_apply_force(w, b, (lvx - C.velocity_x) * kd, (lvy - C.velocity_y) * kd, acx, acy);
    // angular drag (Body.inertia: I + mass * |local centre|^2)
    const vec2<double> lc = w.B.b_lc[g];
    const double bm = w.B.b_mass[g];
    const double inertia = w.B.b_I[g] + bm * (lc.x * lc.x + lc.y * lc.y);
    const double t = -inertia / bm * area * wv * C.angular_drag;
    w.B.b_torque[g] = (R)((double)w.B.b_torque[g] + t);
}

// GravityController.step for one body (controllers.py:263-280): the pair loop
// over (body1, body2) in list order applies +f to body1 and -f to body2; this
// body's share of it, in that order
template <class R> __device__ void gravity_body(const WView<R> &w, const gb_controller &C, const int *list, int pk) {
    const int n = C.body_count;
    const int b = list[pk];
    if (w.btype(b) != GB_BODY_DYNAMIC || n < 2) return;
    const bool inv_sqr = (C.flags & GB_CTRL_INV_SQR) != 0;
    const vec2<double> cb = w.B.b_c[w.bb + b];
    const double mb = w.B.b_mass[w.bb + b];
    auto force = [&](int i, int j, double mi, double mj, vec2<double> ci, vec2<double> cj, double *fx, double *fy) {
        (void)i; (void)j;
        const double dx = cj.x - ci.x, dy = cj.y - ci.y;
        const double r2 = dx * dx + dy * dy;
        const double s = C.G / r2 * mi * mj;
        *fx = s * dx; *fy = s * dy;
        if (inv_sqr) { const double r = sqrt(r2); *fx = *fx / r; *fy = *fy / r; }
    };
    double fx, fy;
    for (int i = 0; i < n; ++i) {
        if (i == pk) {      // pairs (b, j) for every other j: +f to b
            for (int j = 0; j < n; ++j) {
                if (j == pk) continue;
                const int q = list[j];
                force(b, q, mb, w.B.b_mass[w.bb + q], cb, w.B.b_c[w.bb + q], &fx, &fy);
                ctl_apply_force(w, b, fx, fy, cb.x, cb.y);
            }
        } else {            // pair (o, b): -f to b
            const int o = list[i];
            force(o, b, w.B.b_mass[w.bb + o], mb, w.B.b_c[w.bb + o], cb, &fx, &fy);
            ctl_apply_force(w, b, -fx, -fy, cb.x, cb.y);
        }
    }
}

// The world's controllers, in order (world.py:476-479)
template <class R, class G> __device__ __noinline__ void controllers_group(const G &g, const WView<R> &w) {
    const int n = w.H->nctl;
    for (int k = 0; k < n; ++k) {
        const gb_controller &C = w.B.ctl[w.H->ctlbase + k];
        const int *list = w.B.ctl_bodies + C.body_start;
        for (int i = g.rank(); i < C.body_count; i += g.size()) {
            if (C.type == GB_CONTROLLER_BUOYANCY) buoyancy_body(w, C, list[i]);
            else gravity_body(w, C, list, i);
        }
        g.sync();
    }
}

/*
 * oracle.c -- TEST INFRASTRUCTURE, not product code.
 *
 * Sequential float64 CPU restatement of pypybox2d's World.step
 * (pypybox2d/world.py:307-354) and everything below it: contact update
 * (contact_manager.py:174-223, contact.py:210-268), island search and solve
 * (world.py:475-592, island.py:65-179, contact.py:375-864), fixture
 * synchronisation and pair finding (body.py:879-885, fixture.py:287-298,
 * dynamictree.py:152-188, broadphase.py:83-109, contact_manager.py:102-158)
 * and continuous collision (world.py:594-821, island.py:181-243,
 * contact.py:866-933, toi.py, distance.py).
 *
 * It is the checker of the GPU library: tests, the smoke check and the CPU
 * baseline of the benchmark call it; the product never does.  Its
 * correctness is pinned against the reference itself through the golden
 * vectors under tests/golden/ (made by tests/golden/make_golden.py with the
 * ORACLE_LIBM build, which uses libm cos/sin/pow like CPython).
 *
 * Two deliberate, documented hooks exist:
 *   - pair order: the reference keeps new broad-phase pairs in a Python set
 *     (broadphase.py:41), so contacts are created in hash order.  Here (and
 *     in the reference run by the golden script) new pairs are created in a
 *     fixed order: by the first position of the moved proxy in the move
 *     buffer, then by the other proxy's index.  The pair SET and each pair's
 *     orientation are the reference's.
 *   - solver order: or_set_solver_order() permutes each island's contact
 *     list before the contact solver is built (island.py:98), so the
 *     restatement can be run in the constraint order of the GPU solver.
 */
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#include <stdint.h>
#include <pthread.h>
#include "oracle_collide.h"
#include "oracle_joints.h"
#include "oracle.h"

#define MAX_TRANSLATION 2.0
#define MAX_TRANSLATION_SQR 4.0
#define MAX_ROTATION (0.5 * 3.141592653589793)
#define MAX_ROTATION_SQR 2.4674011002723395
#define BAUMGARTE 0.2
#define TOI_BAUMGARTE 0.75
#define MAX_LINEAR_CORRECTION 0.2
#define VELOCITY_THRESHOLD 1.0
#define TIME_TO_SLEEP 0.5
#define LINEAR_SLEEP_TOL_SQR 0.0001
#define ANGULAR_SLEEP_TOL_SQR 0.0012184696791468343
#define AABB_EXTENSION 0.1
#define AABB_MULTIPLIER 2.0
#define MAX_SUB_STEPS 8
#define MAX_TOI_CONTACTS 32

typedef struct {
    int fa, fb, ia, ib;
    uint32_t flags;
    int toi_count;
    double toi;
    double friction, restitution;
    or_manifold m;
    int alive;
} or_contact;

typedef struct { int *d; int n, cap; } ivec;
static void iv_push(ivec *v, int x) {
    if (v->n == v->cap) { v->cap = v->cap ? v->cap * 2 : 8; v->d = (int *)realloc(v->d, sizeof(int) * v->cap); }
    v->d[v->n++] = x;
}
static void iv_remove(ivec *v, int x) {
    for (int i = 0; i < v->n; ++i)
        if (v->d[i] == x) { memmove(v->d + i, v->d + i + 1, sizeof(int) * (v->n - i - 1)); v->n--; return; }
}

/* velocity / position constraint of contact.py ContactSolver */
typedef struct {
    int cid;                  /* contact id */
    int ia, ib;               /* island indices */
    double ma, mb, ia_, ib_;  /* inv masses, inv inertias */
    v2 lca, lcb;
    double ra, rb;            /* shape radii */
    double friction, restitution;
    int npts;                 /* velocity points (may drop to 1) */
    int mcount;               /* manifold points */
    v2 normal;
    v2 rA[2], rB[2];
    double ni[2], ti[2], nm[2], tm[2], bias[2];
    double k11, k12, k22, nm11, nm12, nm21, nm22;
    int mtype;
    v2 ln, lp, lpts[2];
    int dec;                  /* set-up decisions: restitution bias of point 0/1 (bits 0/1), block dropped (bit 2) */
} or_cons;

struct or_world {
    int nb, nf;
    gb_body *b;
    gb_fixture *f;
    or_contact *c;
    int nc_pool, cap_pool;
    ivec order;     /* ContactManager.contacts: contact ids in creation order */
    ivec *bcon;     /* Body._contacts */
    ivec move;      /* BroadPhase._move_buffer (fixture ids) */
    int *island_flag_b;
    int *island_index;
    uint32_t wflags;
    v2 gravity;
    double inv_dt0;
    /* solver order hook */
    int *hook_rank;   /* rank per contact id */
    int *hook_pending;
    int hook_pending_n;
    int hook_set;
    int *pos_of;      /* contact-list position per contact id during _solve */
    ivec last_order;  /* contact list positions in solver order, last _solve */
    /* counters */
    long long n_toi_calls, n_toi_events;
    int status;
    /* step record of the last step, per body: position iterations of its
     * island (bits 0-7), TOI position-pass iterations (8-15) and TOI events
     * (16-23), each capped at 255; set-up decision parities (24-27) */
    int *rec;
    int *rec_island;  /* island of each body in the last solve: its smallest non-static body id (-1: none) */
    /* joints (World.joints order) and each body's joint list (Body.joints) */
    gb_joint *j;
    int nj;
    ivec *bjoint;
    int *jflag;           /* Joint._island_flag */
    int *jhook_rank;      /* joint solver order hook: rank per joint */
    int jhook_set;
    ivec last_jorder;     /* joints in solver order, last _solve */
    /* controllers (World.controllers order) and their body lists */
    gb_controller *ctl;
    int nctl;
    int *ctl_bodies;
    /* a custom contact filter (world.py:123-136) as its answers for every
     * ordered pair of fixture records: accept[a * accept_n + b], or NULL for
     * the default rule */
    unsigned char *accept;
    int accept_n;
};

static void rec_add(int *x, int shift, int v) {
    int cur = (*x >> shift) & 0xff;
    int nv = cur + v > 255 ? 255 : cur + v;
    *x = (*x & ~(0xff << shift)) | (nv << shift);
}

/* ------------------------------------------------------------------ */
static inline xform body_xf(const gb_body *b) { xform x; x.p = V(b->px, b->py); x.q.c = b->qc; x.q.s = b->qs; return x; }
static inline int body_awake(const gb_body *b) { return (b->flags & GB_BODY_AWAKE) != 0; }

/* body.py:781-793 Body.awake setter */
static void set_awake(gb_body *b, int awake) {
    if (awake) {
        if (!(b->flags & GB_BODY_AWAKE)) b->sleep_time = 0.0;
        b->flags |= GB_BODY_AWAKE;
    } else {
        b->sleep_time = 0.0;
        b->vx = 0.0; b->vy = 0.0; b->w = 0.0;
        b->fx = 0.0; b->fy = 0.0; b->torque = 0.0;
        b->flags &= ~GB_BODY_AWAKE;
    }
}

/* body.py:887-889 _synchronize_transform */
static void sync_transform(gb_body *b) {
    rot q = rot_of(b->a);
    v2 p = vsub(V(b->cx, b->cy), rmul(q, V(b->lcx, b->lcy)));
    b->px = p.x; b->py = p.y; b->qc = q.c; b->qs = q.s;
}

static or_sweep get_sweep(const gb_body *b) {
    or_sweep s;
    s.lc = V(b->lcx, b->lcy); s.c0 = V(b->c0x, b->c0y); s.c = V(b->cx, b->cy);
    s.a0 = b->a0; s.a = b->a; s.alpha0 = b->alpha0;
    return s;
}
static void put_sweep(gb_body *b, const or_sweep *s) {
    b->lcx = s->lc.x; b->lcy = s->lc.y; b->c0x = s->c0.x; b->c0y = s->c0.y;
    b->cx = s->c.x; b->cy = s->c.y; b->a0 = s->a0; b->a = s->a; b->alpha0 = s->alpha0;
}

/* body.py:911-918 _advance */
static void body_advance(gb_body *b, double alpha) {
    or_sweep s = get_sweep(b);
    or_sweep_advance(&s, alpha);
    s.c = s.c0;
    s.a = s.a0;
    put_sweep(b, &s);
    rot q = rot_of(s.a);
    v2 p = vsub(s.c, rmul(q, s.lc));
    b->qc = q.c; b->qs = q.s; b->px = p.x; b->py = p.y;
}

/* shapes.py compute_aabb for child 0 */
static void shape_aabb(const gb_fixture *f, xform x, double out[4]) {
    if (f->shape_type == GB_SHAPE_CIRCLE) {
        /* Circle.compute_aabb: p = xf._position + xf._rotation * position */
        v2 p = vadd(x.p, rmul(x.q, fx_v(f, 0)));
        out[0] = p.x - f->radius; out[1] = p.y - f->radius;
        out[2] = p.x + f->radius; out[3] = p.y + f->radius;
    } else if (f->shape_type == GB_SHAPE_POLYGON) {
        v2 lower = xmul(x, fx_v(f, 0));
        v2 upper = lower;
        for (int i = 0; i < f->vertex_count; ++i) {
            v2 v = xmul(x, fx_v(f, i));
            lower = V(cmin(lower.x, v.x), cmin(lower.y, v.y));
            upper = V(cmax(upper.x, v.x), cmax(upper.y, v.y));
        }
        out[0] = lower.x - f->radius; out[1] = lower.y - f->radius;
        out[2] = upper.x + f->radius; out[3] = upper.y + f->radius;
    } else {
        v2 v1 = xmul(x, fx_v(f, 0)), v2_ = xmul(x, fx_v(f, 1));
        v2 lower = V(cmin(v1.x, v2_.x), cmin(v1.y, v2_.y));
        v2 upper = V(cmax(v1.x, v2_.x), cmax(v1.y, v2_.y));
        if (f->flags & GB_FIX_LOOP_CHILD) {   /* Loop.compute_aabb: no radius (shapes.py:822-837) */
            out[0] = lower.x; out[1] = lower.y; out[2] = upper.x; out[3] = upper.y;
            return;
        }
        out[0] = lower.x - f->radius; out[1] = lower.y - f->radius;
        out[2] = upper.x + f->radius; out[3] = upper.y + f->radius;
    }
}

/* aabbmodule.c AABB_test_overlap */
static int aabb_overlap(const double a[4], const double b[4]) {
    if ((b[0] - a[2]) > 0.0 || (b[1] - a[3]) > 0.0 || (a[0] - b[2]) > 0.0 || (a[1] - b[3]) > 0.0) return 0;
    return 1;
}

/* body.py:879-885 _synchronize_fixtures + fixture.py:287-298 _synchronize +
 * dynamictree.py:152-188 move_proxy */
static void sync_fixtures(or_world *w, int bi) {
    gb_body *b = &w->b[bi];
    xform x1;
    x1.q = rot_of(b->a0);
    x1.p = vsub(V(b->c0x, b->c0y), rmul(x1.q, V(b->lcx, b->lcy)));
    xform x2 = body_xf(b);
    for (int k = 0; k < b->fixture_count; ++k) {
        int fi = b->fixture_start + k;
        gb_fixture *f = &w->f[fi];
        double a1[4], a2[4], aabb[4];
        shape_aabb(f, x1, a1);
        shape_aabb(f, x2, a2);
        aabb[0] = cmin(a1[0], a2[0]); aabb[1] = cmin(a1[1], a2[1]);
        aabb[2] = cmax(a1[2], a2[2]); aabb[3] = cmax(a1[3], a2[3]);
        v2 disp = vsub(x2.p, x1.p);
        double *fat = f->aabb;
        if (fat[0] <= aabb[0] && fat[1] <= aabb[1] && aabb[2] <= fat[2] && aabb[3] <= fat[3]) continue;
        double nb[4];
        nb[0] = aabb[0] - AABB_EXTENSION; nb[1] = aabb[1] - AABB_EXTENSION;
        nb[2] = aabb[2] + AABB_EXTENSION; nb[3] = aabb[3] + AABB_EXTENSION;
        v2 d = vscale(AABB_MULTIPLIER, disp);
        if (d.x < 0.0) nb[0] = nb[0] + d.x; else nb[2] = nb[2] + d.x;
        if (d.y < 0.0) nb[1] = nb[1] + d.y; else nb[3] = nb[3] + d.y;
        /* b.lower_bound += (d.x, 0) also adds 0.0 to the other coordinate */
        if (d.x < 0.0) nb[1] = nb[1] + 0.0; else nb[3] = nb[3] + 0.0;
        if (d.y < 0.0) nb[0] = nb[0] + 0.0; else nb[2] = nb[2] + 0.0;
        memcpy(fat, nb, sizeof(nb));
        iv_push(&w->move, fi);
    }
}

/* world.py:958-970 default_contact_filter */
static int default_filter(const gb_fixture *a, const gb_fixture *b) {
    if (a->group_index == b->group_index && a->group_index != 0) return a->group_index > 0;
    return ((a->mask_bits & b->category_bits) != 0) && ((a->category_bits & b->mask_bits) != 0);
}

/* contact_manager.py:145,202: the world's contact filter, the default rule
 * (world.py:958-970) unless a custom filter's answers were given */
static int pair_filter(const or_world *w, int fa, int fb) {
    if (w->accept && fa < w->accept_n && fb < w->accept_n) return w->accept[(size_t)fa * w->accept_n + fb] != 0;
    return default_filter(&w->f[fa], &w->f[fb]);
}

/* body.py:912-927 _should_collide of body `a` with body `b`: one of them
 * dynamic, and no joint between them that turns collision off */
static int should_collide(const or_world *w, int a, int b) {
    if (w->b[a].type != GB_BODY_DYNAMIC && w->b[b].type != GB_BODY_DYNAMIC) return 0;
    const ivec *lst = &w->bjoint[a];
    for (int i = 0; i < lst->n; ++i) {
        const gb_joint *J = &w->j[lst->d[i]];
        if ((J->body_a == a && J->body_b == b) || (J->body_b == a && J->body_a == b))
            if (!(J->flags & GB_J_COLLIDE_CONNECTED)) return 0;
    }
    return 1;
}

static int contact_new(or_world *w) {
    if (w->nc_pool == w->cap_pool) {
        w->cap_pool = w->cap_pool ? w->cap_pool * 2 : 64;
        w->c = (or_contact *)realloc(w->c, sizeof(or_contact) * w->cap_pool);
    }
    int id = w->nc_pool++;
    memset(&w->c[id], 0, sizeof(or_contact));
    return id;
}

/* contact.py:313-326 Contact._create + contact_manager.py:150-158 */
static void create_contact(or_world *w, int fa, int ia, int fb, int ib) {
    int prim;
    if (!or_pair_registered(w->f[fa].shape_type, w->f[fb].shape_type, &prim)) return;
    int id = contact_new(w);
    or_contact *c = &w->c[id];
    if (!prim) { int t = fa; fa = fb; fb = t; t = ia; ia = ib; ib = t; }
    c->fa = fa; c->fb = fb; c->ia = ia; c->ib = ib;
    c->alive = 1;
    c->toi = 0.0; c->toi_count = 0;
    c->friction = sqrt(w->f[fa].friction * w->f[fb].friction);
    c->restitution = pymax(w->f[fa].restitution, w->f[fb].restitution);
    c->flags = 0;
    c->m.type = GB_M_CIRCLES; c->m.count = 0;
    c->m.ln = V(0, 0); c->m.lp = V(0, 0);
    iv_push(&w->order, id);
    iv_push(&w->bcon[w->f[fa].body], id);
    iv_push(&w->bcon[w->f[fb].body], id);
}

/* broadphase.py:83-109 update_pairs in the fixed pair order, followed by
 * contact_manager.py:102-158 find_new_contacts */
typedef struct { int pos, q, p; } pair_rec;
static int pair_cmp(const void *x, const void *y) {
    const pair_rec *a = (const pair_rec *)x, *b = (const pair_rec *)y;
    if (a->pos != b->pos) return a->pos < b->pos ? -1 : 1;
    if (a->q != b->q) return a->q < b->q ? -1 : 1;
    return 0;
}

static void find_new_contacts(or_world *w) {
    int nf = w->nf;
    int *first = (int *)malloc(sizeof(int) * (nf ? nf : 1));
    for (int i = 0; i < nf; ++i) first[i] = -1;
    for (int i = 0; i < w->move.n; ++i)
        if (first[w->move.d[i]] < 0) first[w->move.d[i]] = i;
    int np = 0, pcap = 64;
    pair_rec *pairs = (pair_rec *)malloc(sizeof(pair_rec) * pcap);
    for (int p = 0; p < nf; ++p) {
        if (first[p] < 0) continue;
        const double *ap = w->f[p].aabb;
        for (int q = 0; q < nf; ++q) {
            if (q == p) continue;
            if (first[q] >= 0 && first[q] < first[p]) continue;
            if (!aabb_overlap(w->f[q].aabb, ap)) continue;
            if (np == pcap) { pcap *= 2; pairs = (pair_rec *)realloc(pairs, sizeof(pair_rec) * pcap); }
            pairs[np].pos = first[p]; pairs[np].q = q; pairs[np].p = p; np++;
        }
    }
    w->move.n = 0;
    qsort(pairs, np, sizeof(pair_rec), pair_cmp);
    for (int k = 0; k < np; ++k) {
        int fa = pairs[k].p, fb = pairs[k].q;
        int ba = w->f[fa].body, bb = w->f[fb].body;
        if (ba == bb) continue;
        /* an inactive body's fixtures have no proxies (body.py:848-872) */
        if (!(w->b[ba].flags & w->b[bb].flags & GB_BODY_ACTIVE)) continue;
        int exists = 0;
        ivec *lst = &w->bcon[bb];
        for (int i = 0; i < lst->n; ++i) {
            or_contact *c = &w->c[lst->d[i]];
            int other = (w->f[c->fa].body == bb) ? w->f[c->fb].body : w->f[c->fa].body;
            if (other != ba) continue;
            if (c->fa == fa && c->fb == fb && c->ia == 0 && c->ib == 0) { exists = 1; break; }
            if (c->fa == fb && c->fb == fa && c->ia == 0 && c->ib == 0) { exists = 1; break; }
        }
        if (exists) continue;
        if (!should_collide(w, bb, ba)) continue;
        if (!pair_filter(w, fa, fb)) continue;
        create_contact(w, fa, 0, fb, 0);
    }
    free(pairs);
    free(first);
}

/* contact_manager.py:160-172 destroy */
static void destroy_contact(or_world *w, int id) {
    or_contact *c = &w->c[id];
    iv_remove(&w->order, id);
    iv_remove(&w->bcon[w->f[c->fa].body], id);
    iv_remove(&w->bcon[w->f[c->fb].body], id);
    c->alive = 0;
}

/* contact.py:210-268 Contact.update (no listeners in the restatement) */
static void contact_update(or_world *w, int id) {
    or_contact *c = &w->c[id];
    or_manifold old = c->m;
    c->flags |= GB_C_ENABLED;
    int was_touching = (c->flags & GB_C_TOUCHING) != 0;
    const gb_fixture *fa = &w->f[c->fa], *fb = &w->f[c->fb];
    gb_body *ba = &w->b[fa->body], *bb = &w->b[fb->body];
    int sensor = ((fa->flags | fb->flags) & GB_FIX_SENSOR) != 0;
    int touching;
    if (sensor) {
        or_dproxy pa, pb;
        or_dproxy_init(&pa, fa); or_dproxy_init(&pb, fb);
        or_scache cache; memset(&cache, 0, sizeof(cache));
        double d = or_shape_distance(&pa, &pb, body_xf(ba), body_xf(bb), 1, &cache, NULL, NULL);
        touching = d < 10.0 * OR_EPSILON;
        c->m.count = 0;
    } else {
        or_evaluate(&c->m, fa, body_xf(ba), fb, body_xf(bb));
        touching = c->m.count > 0;
        for (int i = 0; i < c->m.count; ++i) {
            int found = -1;
            for (int j = old.count - 1; j >= 0; --j)
                if (old.id[j] == c->m.id[i]) { found = j; break; }
            if (found >= 0) { c->m.ni[i] = old.ni[found]; c->m.ti[i] = old.ti[found]; }
            else { c->m.ni[i] = 0.0; c->m.ti[i] = 0.0; }
        }
        if (touching != was_touching) { set_awake(ba, 1); set_awake(bb, 1); }
    }
    if (touching) c->flags |= GB_C_TOUCHING; else c->flags &= ~GB_C_TOUCHING;
}

/* contact_manager.py:174-223 collide */
static void collide(or_world *w) {
    int n = w->order.n;
    int *ids = (int *)malloc(sizeof(int) * (n ? n : 1));
    memcpy(ids, w->order.d, sizeof(int) * n);
    int *rm = (int *)malloc(sizeof(int) * (n ? n : 1));
    int nrm = 0;
    for (int k = 0; k < n; ++k) {
        int id = ids[k];
        or_contact *c = &w->c[id];
        gb_body *ba = &w->b[w->f[c->fa].body], *bb = &w->b[w->f[c->fb].body];
        int act_a = body_awake(ba) && ba->type != GB_BODY_STATIC;
        int act_b = body_awake(bb) && bb->type != GB_BODY_STATIC;
        if (!act_a && !act_b) continue;
        if (c->flags & GB_C_FILTER) {
            if (!should_collide(w, w->f[c->fb].body, w->f[c->fa].body) || !pair_filter(w, c->fa, c->fb)) {
                rm[nrm++] = id;
                continue;
            }
            c->flags &= ~GB_C_FILTER;
        }
        if (!aabb_overlap(w->f[c->fa].aabb, w->f[c->fb].aabb)) { rm[nrm++] = id; continue; }
        contact_update(w, id);
    }
    for (int k = 0; k < nrm; ++k) destroy_contact(w, rm[k]);
    free(ids);
    free(rm);
}

/* ------------------------------------------------------------------ */
/* contact.py:375-412 ContactSolver.__init__                           */
static void build_constraint(or_world *w, or_cons *k, int cid, int warm, double dt_ratio) {
    or_contact *c = &w->c[cid];
    const gb_fixture *fa = &w->f[c->fa], *fb = &w->f[c->fb];
    const gb_body *ba = &w->b[fa->body], *bb = &w->b[fb->body];
    k->cid = cid;
    k->ia = w->island_index[fa->body]; k->ib = w->island_index[fb->body];
    k->ma = ba->inv_mass; k->mb = bb->inv_mass; k->ia_ = ba->inv_I; k->ib_ = bb->inv_I;
    k->lca = V(ba->lcx, ba->lcy); k->lcb = V(bb->lcx, bb->lcy);
    k->ra = fa->radius; k->rb = fb->radius;
    k->friction = c->friction; k->restitution = c->restitution;
    k->mcount = c->m.count; k->npts = c->m.count;
    k->mtype = c->m.type; k->ln = c->m.ln; k->lp = c->m.lp;
    for (int i = 0; i < c->m.count; ++i) {
        k->lpts[i] = c->m.plp[i];
        if (warm) { k->ni[i] = dt_ratio * c->m.ni[i]; k->ti[i] = dt_ratio * c->m.ti[i]; }
        else { k->ni[i] = c->m.ni[i]; k->ti[i] = c->m.ti[i]; }
    }
}

/* contact.py:414-496 initialize_velocity_constraints (+ contact_util.py:195-245 WorldManifold) */
static void init_velocity(or_cons *k, const v2 *pc, const double *pa, const v2 *vv, const double *ww) {
    k->dec = 0;
    v2 ca = pc[k->ia], cb = pc[k->ib];
    double aa = pa[k->ia], ab = pa[k->ib];
    v2 va = vv[k->ia], vb = vv[k->ib];
    double wa = ww[k->ia], wb = ww[k->ib];
    xform xa, xb;
    xa.q = rot_of(aa); xb.q = rot_of(ab);
    xa.p = vsub(ca, rmul(xa.q, k->lca));
    xb.p = vsub(cb, rmul(xb.q, k->lcb));
    v2 normal, pts[2];
    if (k->mtype == GB_M_CIRCLES) {
        normal = V(1.0, 0.0);
        v2 pA = xmul(xa, k->lp), pB = xmul(xb, k->lpts[0]);
        v2 dd = vsub(pA, pB);
        if (vdot(dd, dd) > OR_EPSILON_SQR) normal = vnormalized(vsub(pB, pA));
        v2 cA = vadd(pA, vscale(k->ra, normal));
        v2 cB = vsub(pB, vscale(k->rb, normal));
        pts[0] = vscale(0.5, vadd(cA, cB));
    } else if (k->mtype == GB_M_FACE_A) {
        normal = rmul(xa.q, k->ln);
        v2 plane = xmul(xa, k->lp);
        for (int i = 0; i < k->mcount; ++i) {
            v2 clip = xmul(xb, k->lpts[i]);
            v2 cA = vadd(clip, vscale(k->ra - vdot(vsub(clip, plane), normal), normal));
            v2 cB = vsub(clip, vscale(k->rb, normal));
            pts[i] = vscale(0.5, vadd(cA, cB));
        }
    } else {
        normal = rmul(xb.q, k->ln);
        v2 plane = xmul(xb, k->lp);
        for (int i = 0; i < k->mcount; ++i) {
            v2 clip = xmul(xa, k->lpts[i]);
            v2 cB = vadd(clip, vscale(k->rb - vdot(vsub(clip, plane), normal), normal));
            v2 cA = vsub(clip, vscale(k->ra, normal));
            pts[i] = vscale(0.5, vadd(cA, cB));
        }
        normal = vneg(normal);
    }
    k->normal = normal;
    for (int i = 0; i < k->npts; ++i) {
        v2 ra = vsub(pts[i], ca), rb = vsub(pts[i], cb);
        k->rA[i] = ra; k->rB[i] = rb;
        double rna = SQ(vcross(ra, normal)), rnb = SQ(vcross(rb, normal));
        double kn = k->ma + k->mb + k->ia_ * rna + k->ib_ * rnb;
        k->nm[i] = kn > 0.0 ? 1.0 / kn : 0.0;
        v2 tangent = vcross_vs(normal, 1.0);
        double rta = SQ(vcross(ra, tangent)), rtb = SQ(vcross(rb, tangent));
        double kt = k->ma + k->mb + k->ia_ * rta + k->ib_ * rtb;
        k->tm[i] = kt > 0.0 ? 1.0 / kt : 0.0;
        k->bias[i] = 0.0;
        double vrel = vdot(normal, vsub(vsub(vadd(vb, vcross_sv(wb, rb)), va), vcross_sv(wa, ra)));
        if (vrel < -VELOCITY_THRESHOLD) { k->bias[i] = -k->restitution * vrel; k->dec |= 1 << i; }
    }
    if (k->npts == 2) {
        double rn1a = vcross(k->rA[0], normal), rn1b = vcross(k->rB[0], normal);
        double rn2a = vcross(k->rA[1], normal), rn2b = vcross(k->rB[1], normal);
        double k11 = k->ma + k->mb + k->ia_ * rn1a * rn1a + k->ib_ * rn1b * rn1b;
        double k22 = k->ma + k->mb + k->ia_ * rn2a * rn2a + k->ib_ * rn2b * rn2b;
        double k12 = k->ma + k->mb + k->ia_ * rn1a * rn2a + k->ib_ * rn1b * rn2b;
        if (SQ(k11) < 1000.0 * (k11 * k22 - SQ(k12))) {
            k->k11 = k11; k->k12 = k12; k->k22 = k22;
            double det = k11 * k22 - k12 * k12;
            if (det != 0.0) det = 1.0 / det;
            k->nm11 = det * k22; k->nm12 = -det * k12; k->nm21 = -det * k12; k->nm22 = det * k11;
        } else {
            k->npts = 1;
            k->dec |= 4;
        }
    }
}

/* contact.py:498-525 warm_start */
static void warm_start(or_cons *k, v2 *vv, double *ww) {
    v2 normal = k->normal, tangent = vcross_vs(normal, 1.0);
    v2 va = vv[k->ia], vb = vv[k->ib];
    double wa = ww[k->ia], wb = ww[k->ib];
    for (int i = 0; i < k->npts; ++i) {
        v2 P = vadd(vscale(k->ni[i], normal), vscale(k->ti[i], tangent));
        wa = wa - k->ia_ * vcross(k->rA[i], P);
        va = vsub(va, vscale(k->ma, P));
        wb = wb + k->ib_ * vcross(k->rB[i], P);
        vb = vadd(vb, vscale(k->mb, P));
    }
    vv[k->ia] = va; ww[k->ia] = wa;
    vv[k->ib] = vb; ww[k->ib] = wb;
}

/* contact.py:527-799 solve_velocity_constraints (one constraint) */
static void solve_velocity(or_cons *k, v2 *vv, double *ww) {
    v2 va = vv[k->ia], vb = vv[k->ib];
    double wa = ww[k->ia], wb = ww[k->ib];
    double ma = k->ma, mb = k->mb, iA = k->ia_, iB = k->ib_;
    v2 normal = k->normal, tangent = vcross_vs(normal, 1.0);
    double friction = k->friction;
    for (int i = 0; i < k->npts; ++i) {
        v2 ra = k->rA[i], rb = k->rB[i];
        v2 dv = vsub(vsub(vadd(vb, vcross_sv(wb, rb)), va), vcross_sv(wa, ra));
        double vt = vdot(dv, tangent);
        double lambda = k->tm[i] * (-vt);
        double maxf = friction * k->ni[i];
        double ni = cclamp(k->ti[i] + lambda, -maxf, maxf);
        lambda = ni - k->ti[i];
        v2 P = vscale(lambda, tangent);
        va = vsub(va, vscale(ma, P));
        wa = wa - iA * vcross(ra, P);
        vb = vadd(vb, vscale(mb, P));
        wb = wb + iB * vcross(rb, P);
        k->ti[i] = ni;
    }
    if (k->npts == 1) {
        v2 ra = k->rA[0], rb = k->rB[0];
        v2 dv = vsub(vsub(vadd(vb, vcross_sv(wb, rb)), va), vcross_sv(wa, ra));
        double vn = vdot(dv, normal);
        double lambda = -k->nm[0] * (vn - k->bias[0]);
        double ni = pymax(k->ni[0] + lambda, 0.0);
        lambda = ni - k->ni[0];
        v2 P = vscale(lambda, normal);
        va = vsub(va, vscale(ma, P));
        wa = wa - iA * vcross(ra, P);
        vb = vadd(vb, vscale(mb, P));
        wb = wb + iB * vcross(rb, P);
        k->ni[0] = ni;
    } else {
        v2 a = V(k->ni[0], k->ni[1]);
        v2 ra1 = k->rA[0], rb1 = k->rB[0], ra2 = k->rA[1], rb2 = k->rB[1];
        v2 dv1 = vsub(vsub(vadd(vb, vcross_sv(wb, rb1)), va), vcross_sv(wa, ra1));
        v2 dv2 = vsub(vsub(vadd(vb, vcross_sv(wb, rb2)), va), vcross_sv(wa, ra2));
        double vn1 = vdot(dv1, normal), vn2 = vdot(dv2, normal);
        v2 b = V(vn1 - k->bias[0], vn2 - k->bias[1]);
        b = vsub(b, V(k->k11 * a.x + k->k12 * a.y, k->k12 * a.x + k->k22 * a.y));
        v2 x;
        int solved = 0;
        /* case 1: x = -inv(K) b */
        x = V(-(k->nm11 * b.x + k->nm12 * b.y), -(k->nm21 * b.x + k->nm22 * b.y));
        if (x.x >= 0.0 && x.y >= 0.0) solved = 1;
        if (!solved) {
            x = V(-k->nm[0] * b.x, 0.0);
            vn2 = k->k12 * x.x + b.y;
            if (x.x >= 0.0 && vn2 >= 0.0) solved = 1;
        }
        if (!solved) {
            x = V(0.0, -k->nm[1] * b.y);
            vn1 = k->k12 * x.y + b.x;
            if (x.y >= 0.0 && vn1 >= 0.0) solved = 1;
        }
        if (!solved) {
            x = V(0.0, 0.0);
            vn1 = b.x; vn2 = b.y;
            if (vn1 >= 0.0 && vn2 >= 0.0) solved = 1;
        }
        if (solved) {
            v2 d = vsub(x, a);
            v2 p1 = vscale(d.x, normal), p2 = vscale(d.y, normal);
            va = vsub(va, vscale(ma, vadd(p1, p2)));
            wa = wa - iA * (vcross(ra1, p1) + vcross(ra2, p2));
            vb = vadd(vb, vscale(mb, vadd(p1, p2)));
            wb = wb + iB * (vcross(rb1, p1) + vcross(rb2, p2));
            k->ni[0] = x.x; k->ni[1] = x.y;
        }
    }
    vv[k->ia] = va; ww[k->ia] = wa;
    vv[k->ib] = vb; ww[k->ib] = wb;
}

/* contact_util.py:323-360 solver_manifold */
static void solver_manifold(const or_cons *k, xform xa, xform xb, int idx, v2 *normal, v2 *point, double *sep) {
    if (k->mtype == GB_M_CIRCLES) {
        v2 pA = xmul(xa, k->lp), pB = xmul(xb, k->lpts[0]);
        *normal = vnormalized(vsub(pB, pA));
        *point = vscale(0.5, vadd(pA, pB));
        *sep = vdot(vsub(pB, pA), *normal) - k->ra - k->rb;
    } else if (k->mtype == GB_M_FACE_A) {
        *normal = rmul(xa.q, k->ln);
        v2 plane = xmul(xa, k->lp);
        v2 clip = xmul(xb, k->lpts[idx]);
        *sep = vdot(vsub(clip, plane), *normal) - k->ra - k->rb;
        *point = clip;
    } else {
        *normal = rmul(xb.q, k->ln);
        v2 plane = xmul(xb, k->lp);
        v2 clip = xmul(xa, k->lpts[idx]);
        *sep = vdot(vsub(clip, plane), *normal) - k->ra - k->rb;
        *point = clip;
        *normal = vneg(*normal);
    }
}

/* contact.py:809-864 / 866-933 position solver for one constraint; returns
 * the running minimum separation.  toi_a/toi_b < 0 selects the discrete form. */
static double solve_position(const or_cons *k, v2 *pc, double *pa, double minsep, int toi_a, int toi_b) {
    double ma = k->ma, mb = k->mb, iA = k->ia_, iB = k->ib_;
    double baum = BAUMGARTE;
    if (toi_a >= 0) {
        baum = TOI_BAUMGARTE;
        if (!(k->ia == toi_a || k->ia == toi_b)) { ma = 0.0; iA = 0.0; }
        if (!(k->ib == toi_a || k->ib == toi_b)) { mb = 0.0; iB = 0.0; }
    }
    v2 ca = pc[k->ia], cb = pc[k->ib];
    double aa = pa[k->ia], ab = pa[k->ib];
    for (int j = 0; j < k->mcount; ++j) {
        xform xa, xb;
        xa.q = rot_of(aa); xb.q = rot_of(ab);
        xa.p = vsub(ca, rmul(xa.q, k->lca));
        xb.p = vsub(cb, rmul(xb.q, k->lcb));
        v2 normal, point;
        double sep;
        solver_manifold(k, xa, xb, j, &normal, &point, &sep);
        v2 ra = vsub(point, ca), rb = vsub(point, cb);
        minsep = pymin(minsep, sep);
        double C = cclamp(baum * (sep + OR_LINEAR_SLOP), -MAX_LINEAR_CORRECTION, 0.0);
        double rna = SQ(vcross(ra, normal)), rnb = SQ(vcross(rb, normal));
        double K = ma + mb + (iA * rna) + (iB * rnb);
        double impulse = K > 0.0 ? -C / K : 0.0;
        v2 P = vscale(impulse, normal);
        ca = vsub(ca, vscale(ma, P));
        aa = aa - iA * vcross(ra, P);
        cb = vadd(cb, vscale(mb, P));
        ab = ab + iB * vcross(rb, P);
    }
    pc[k->ia] = ca; pa[k->ia] = aa;
    pc[k->ib] = cb; pa[k->ib] = ab;
    return minsep;
}

static __thread or_world *rank_w;
static int cmp_rank(const void *x, const void *y) {
    int a = *(const int *)x, b = *(const int *)y;
    int ra = rank_w->hook_rank[a], rb = rank_w->hook_rank[b];
    return (ra < rb) ? -1 : (ra > rb ? 1 : 0);
}
static int cmp_jrank(const void *x, const void *y) {
    int a = *(const int *)x, b = *(const int *)y;
    int ra = rank_w->jhook_rank[a], rb = rank_w->jhook_rank[b];
    return (ra < rb) ? -1 : (ra > rb ? 1 : 0);
}

/* Step record: parity of the restitution-bias points (bit `shift`) and of
 * the block solver's drop to one point (bit shift + 1) of a constraint,
 * toggled on its non-static bodies (`bodies`: island body ids). */
static void rec_decisions(or_world *w, const int *bodies, const or_cons *k, int shift) {
    int bits = ((((k->dec & 1) + ((k->dec >> 1) & 1)) & 1) << shift) | (((k->dec >> 2) & 1) << (shift + 1));
    if (!bits) return;
    if (w->b[bodies[k->ia]].type != GB_BODY_STATIC) w->rec[bodies[k->ia]] ^= bits;
    if (w->b[bodies[k->ib]].type != GB_BODY_STATIC) w->rec[bodies[k->ib]] ^= bits;
}

/* island.py:65-179 Island.solve */
static void island_solve(or_world *w, const int *bodies, int nbi, int *contacts, int nci, int *joints, int nji, double dt,
                         double inv_dt, double dt_ratio, int vel_iters, int pos_iters, int warm) {
    (void)inv_dt;
    v2 *pc = (v2 *)malloc(sizeof(v2) * nbi);
    double *pa = (double *)malloc(sizeof(double) * nbi);
    v2 *vv = (v2 *)malloc(sizeof(v2) * nbi);
    double *ww = (double *)malloc(sizeof(double) * nbi);
    for (int i = 0; i < nbi; ++i) {
        gb_body *b = &w->b[bodies[i]];
        v2 c = V(b->cx, b->cy);
        double a = b->a;
        v2 v = V(b->vx, b->vy);
        double om = b->w;
        b->c0x = c.x; b->c0y = c.y; b->a0 = a;
        if (b->type == GB_BODY_DYNAMIC) {
            v = vadd(v, vscale(dt, vadd(vscale(b->gravity_scale, w->gravity), vscale(b->inv_mass, V(b->fx, b->fy)))));
            om = om + dt * b->inv_I * b->torque;
            v = vscale(cclamp(1.0 - dt * b->linear_damping, 0.0, 1.0), v);
            om = om * cclamp(1.0 - dt * b->angular_damping, 0.0, 1.0);
        }
        pc[i] = c; pa[i] = a; vv[i] = v; ww[i] = om;
    }
    if (w->hook_set) {
        rank_w = w;
        qsort(contacts, nci, sizeof(int), cmp_rank);
    }
    /* record the contact-list position of each constraint in solver order */
    for (int i = 0; i < nci; ++i) iv_push(&w->last_order, w->pos_of[contacts[i]]);
    or_cons *ks = (or_cons *)malloc(sizeof(or_cons) * (size_t)(nci > 0 ? nci : 1));
    for (int i = 0; i < nci; ++i) build_constraint(w, &ks[i], contacts[i], warm, dt_ratio);
    for (int i = 0; i < nci; ++i) init_velocity(&ks[i], pc, pa, vv, ww);
    for (int i = 0; i < nci; ++i) rec_decisions(w, bodies, &ks[i], 24);
    if (warm)
        for (int i = 0; i < nci; ++i) warm_start(&ks[i], vv, ww);
    /* joints: set-up with their warm start after the contacts' (island.py:107-108) */
    if (w->jhook_set) {
        rank_w = w;
        qsort(joints, nji, sizeof(int), cmp_jrank);
    }
    for (int i = 0; i < nji; ++i) iv_push(&w->last_jorder, joints[i]);
    or_jcons *jk = (or_jcons *)malloc(sizeof(or_jcons) * (size_t)(nji > 0 ? nji : 1));
    for (int i = 0; i < nji; ++i) {
        gb_joint *J = &w->j[joints[i]];
        const gb_body *ba = &w->b[J->body_a], *bb = &w->b[J->body_b];
        or_jcons *k = &jk[i];
        k->j = joints[i];
        k->ia = w->island_index[J->body_a];
        k->ib = w->island_index[J->body_b];
        k->lca = V(ba->lcx, ba->lcy);
        k->lcb = V(bb->lcx, bb->lcy);
        k->ma = ba->inv_mass; k->mb = bb->inv_mass;
        k->iA = ba->inv_I; k->iB = bb->inv_I;
        joint_init(J, k, pc, pa, vv, ww, dt, dt_ratio, bb->mass, warm);
    }
    /* velocity iterations: the joints, then the contacts (island.py:110-113) */
    for (int it = 0; it < vel_iters; ++it) {
        for (int i = 0; i < nji; ++i) joint_solve_velocity(&w->j[jk[i].j], &jk[i], vv, ww, dt);
        for (int i = 0; i < nci; ++i) solve_velocity(&ks[i], vv, ww);
    }
    /* store_impulses */
    for (int i = 0; i < nci; ++i) {
        or_contact *c = &w->c[ks[i].cid];
        for (int j = 0; j < ks[i].npts && j < c->m.count; ++j) { c->m.ni[j] = ks[i].ni[j]; c->m.ti[j] = ks[i].ti[j]; }
    }
    for (int i = 0; i < nbi; ++i) {
        v2 v = vv[i];
        double om = ww[i];
        v2 tr = vscale(dt, v);
        if (vdot(tr, tr) > MAX_TRANSLATION_SQR) {
            double ratio = MAX_TRANSLATION / vlen(tr);
            v = vscale(ratio, v);
        }
        double rotation = dt * om;
        if (SQ(rotation) > MAX_ROTATION_SQR) {
            double ratio = MAX_ROTATION / fabs(rotation);
            om = om * ratio;
        }
        pc[i] = vadd(pc[i], vscale(dt, v));
        pa[i] = pa[i] + dt * om;
        vv[i] = v; ww[i] = om;
    }
    int position_solved = 0, its = pos_iters;
    for (int it = 0; it < pos_iters; ++it) {
        double minsep = 0.0;
        for (int i = 0; i < nci; ++i) minsep = solve_position(&ks[i], pc, pa, minsep, -1, -1);
        /* the contacts, then every joint (island.py:141-153) */
        int joints_okay = 1;
        for (int i = 0; i < nji; ++i) {
            int ok = joint_solve_position(&w->j[jk[i].j], &jk[i], pc, pa);
            joints_okay = joints_okay && ok;
        }
        if (minsep >= -3.0 * OR_LINEAR_SLOP && joints_okay) { position_solved = 1; its = it + 1; break; }
    }
    free(jk);
    int root = -1;
    for (int i = 0; i < nbi; ++i)
        if (w->b[bodies[i]].type != GB_BODY_STATIC && (root < 0 || bodies[i] < root)) root = bodies[i];
    for (int i = 0; i < nbi; ++i)
        if (w->b[bodies[i]].type != GB_BODY_STATIC) {
            w->rec[bodies[i]] = (w->rec[bodies[i]] & ~0xff) | (its > 255 ? 255 : its);
            w->rec_island[bodies[i]] = root;
        }
    for (int i = 0; i < nbi; ++i) {
        gb_body *b = &w->b[bodies[i]];
        b->cx = pc[i].x; b->cy = pc[i].y; b->a = pa[i];
        b->vx = vv[i].x; b->vy = vv[i].y; b->w = ww[i];
        sync_transform(b);
    }
    if (w->wflags & GB_W_ALLOW_SLEEP) {
        /* island.py:163-179; `body` is the last island body, `b` the last
         * non-static one (loop variables leaking out of their loops). */
        const gb_body *last = &w->b[bodies[nbi - 1]];
        double min_sleep = OR_MAX_FLOAT;
        int blast = -1;
        for (int i = 0; i < nbi; ++i) {
            gb_body *b = &w->b[bodies[i]];
            if (b->type == GB_BODY_STATIC) continue;
            blast = bodies[i];
            if (!(last->flags & GB_BODY_ALLOW_SLEEP) || SQ(b->w) > ANGULAR_SLEEP_TOL_SQR ||
                vlen2(V(b->vx, b->vy)) > LINEAR_SLEEP_TOL_SQR) {
                b->sleep_time = 0.0;
                min_sleep = 0.0;
            } else {
                b->sleep_time += dt;
                min_sleep = pymin(min_sleep, b->sleep_time);
            }
        }
        if (min_sleep >= TIME_TO_SLEEP && position_solved && blast >= 0) set_awake(&w->b[blast], 0);
    }
    free(ks);
    free(pc); free(pa); free(vv); free(ww);
}

/* world.py:475-592 World._solve */
#include "oracle_controllers.h"

static void world_solve(or_world *w, double dt, double inv_dt, double dt_ratio, int vel_iters, int pos_iters) {
    controllers_step(w);   /* world.py:476-479 */
    int nb = w->nb;
    int *bflag = w->island_flag_b;
    for (int i = 0; i < nb; ++i) bflag[i] = 0;
    for (int k = 0; k < w->order.n; ++k) w->c[w->order.d[k]].flags &= ~GB_C_ISLAND;
    for (int k = 0; k < w->nj; ++k) w->jflag[k] = 0;
    int *ijoints = (int *)malloc(sizeof(int) * (w->nj ? w->nj : 1));
    w->last_jorder.n = 0;
    int *stack = (int *)malloc(sizeof(int) * (nb ? nb : 1));
    int *ibodies = (int *)malloc(sizeof(int) * (nb ? nb : 1));
    int *icontacts = (int *)malloc(sizeof(int) * (w->order.n ? w->order.n : 1));
    int *tmp = (int *)malloc(sizeof(int) * (w->order.n ? w->order.n : 1));
    w->last_order.n = 0;
    w->pos_of = (int *)realloc(w->pos_of, sizeof(int) * (w->nc_pool ? w->nc_pool : 1));
    for (int k = 0; k < w->order.n; ++k) w->pos_of[w->order.d[k]] = k;
    if (w->hook_set) {
        w->hook_rank = (int *)realloc(w->hook_rank, sizeof(int) * (w->nc_pool ? w->nc_pool : 1));
        for (int k = 0; k < w->order.n; ++k) w->hook_rank[w->order.d[k]] = w->hook_pending_n + k;
        for (int i = 0; i < w->hook_pending_n; ++i) {
            int p = w->hook_pending[i];
            if (p >= 0 && p < w->order.n) w->hook_rank[w->order.d[p]] = i;
        }
    }
    for (int seed = 0; seed < nb; ++seed) {
        gb_body *sb = &w->b[seed];
        if (bflag[seed]) continue;
        if (!body_awake(sb) || !(sb->flags & GB_BODY_ACTIVE)) continue;
        if (sb->type == GB_BODY_STATIC) continue;
        int nbi = 0, nci = 0, nji = 0, sp = 0;
        stack[sp++] = seed;
        bflag[seed] = 1;
        while (sp > 0) {
            int bi = stack[--sp];
            gb_body *b = &w->b[bi];
            w->island_index[bi] = nbi;
            ibodies[nbi++] = bi;
            set_awake(b, 1);
            if (b->type == GB_BODY_STATIC) continue;
            ivec *lst = &w->bcon[bi];
            int nt = 0;
            for (int i = 0; i < lst->n; ++i) {
                or_contact *c = &w->c[lst->d[i]];
                if (c->flags & GB_C_ISLAND) continue;
                if (!(c->flags & GB_C_ENABLED) || !(c->flags & GB_C_TOUCHING)) continue;
                if ((w->f[c->fa].flags | w->f[c->fb].flags) & GB_FIX_SENSOR) continue;
                tmp[nt++] = lst->d[i];
            }
            for (int i = 0; i < nt; ++i) {
                or_contact *c = &w->c[tmp[i]];
                icontacts[nci++] = tmp[i];
                c->flags |= GB_C_ISLAND;
                int ob = (w->f[c->fa].body == bi) ? w->f[c->fb].body : w->f[c->fa].body;
                if (bflag[ob]) continue;
                stack[sp++] = ob;
                bflag[ob] = 1;
            }
            /* the body's joints (world.py:547-567); joints to inactive bodies are not simulated */
            ivec *jl = &w->bjoint[bi];
            for (int i = 0; i < jl->n; ++i) {
                int jj = jl->d[i];
                if (w->jflag[jj]) continue;
                const gb_joint *J = &w->j[jj];
                int ob = (J->body_a == bi) ? J->body_b : J->body_a;
                if (!(w->b[ob].flags & GB_BODY_ACTIVE)) continue;
                ijoints[nji++] = jj;
                w->jflag[jj] = 1;
                if (bflag[ob]) continue;
                stack[sp++] = ob;
                bflag[ob] = 1;
            }
        }
        island_solve(w, ibodies, nbi, icontacts, nci, ijoints, nji, dt, inv_dt, dt_ratio, vel_iters, pos_iters,
                     (w->wflags & GB_W_WARM_STARTING) != 0);
        for (int i = 0; i < nbi; ++i)
            if (w->b[ibodies[i]].type == GB_BODY_STATIC) bflag[ibodies[i]] = 0;
    }
    for (int i = 0; i < nb; ++i)
        if (bflag[i] && w->b[i].type != GB_BODY_STATIC) sync_fixtures(w, i);
    find_new_contacts(w);
    free(stack); free(ibodies); free(icontacts); free(tmp); free(ijoints);
}

/* island.py:181-243 Island.solve_toi */
static void island_solve_toi(or_world *w, const int *bodies, int nbi, int *contacts, int nci, double sub_dt,
                             int vel_iters, int toi_a, int toi_b) {
    v2 *pc = (v2 *)malloc(sizeof(v2) * nbi);
    double *pa = (double *)malloc(sizeof(double) * nbi);
    v2 *vv = (v2 *)malloc(sizeof(v2) * nbi);
    double *ww = (double *)malloc(sizeof(double) * nbi);
    for (int i = 0; i < nbi; ++i) {
        gb_body *b = &w->b[bodies[i]];
        pc[i] = V(b->cx, b->cy); pa[i] = b->a; vv[i] = V(b->vx, b->vy); ww[i] = b->w;
    }
    or_cons *ks = (or_cons *)malloc(sizeof(or_cons) * (size_t)(nci > 0 ? nci : 1));
    for (int i = 0; i < nci; ++i) build_constraint(w, &ks[i], contacts[i], 0, 1.0);
    int its = 0;
    for (int it = 0; it < 20; ++it) {
        double minsep = 0.0;
        for (int i = 0; i < nci; ++i) minsep = solve_position(&ks[i], pc, pa, minsep, toi_a, toi_b);
        its = it + 1;
        if (minsep >= -1.5 * OR_LINEAR_SLOP) break;
    }
    rec_add(&w->rec[bodies[toi_a]], 8, its); rec_add(&w->rec[bodies[toi_a]], 16, 1);
    rec_add(&w->rec[bodies[toi_b]], 8, its); rec_add(&w->rec[bodies[toi_b]], 16, 1);
    gb_body *ba = &w->b[bodies[toi_a]], *bb = &w->b[bodies[toi_b]];
    ba->c0x = pc[toi_a].x; ba->c0y = pc[toi_a].y; ba->a0 = pa[toi_a];
    bb->c0x = pc[toi_b].x; bb->c0y = pc[toi_b].y; bb->a0 = pa[toi_b];
    for (int i = 0; i < nci; ++i) init_velocity(&ks[i], pc, pa, vv, ww);
    for (int i = 0; i < nci; ++i) rec_decisions(w, bodies, &ks[i], 26);
    for (int it = 0; it < vel_iters; ++it)
        for (int i = 0; i < nci; ++i) solve_velocity(&ks[i], vv, ww);
    for (int i = 0; i < nbi; ++i) {
        gb_body *b = &w->b[bodies[i]];
        v2 v = vv[i];
        double om = ww[i];
        v2 tr = vscale(sub_dt, v);
        if (vlen2(tr) > MAX_TRANSLATION_SQR) {
            double ratio = MAX_TRANSLATION / vlen(tr);
            v = vscale(ratio, v);
        }
        double rotation = sub_dt * om;
        if (SQ(rotation) > MAX_ROTATION_SQR) {
            double ratio = MAX_ROTATION / fabs(rotation);
            om = om * ratio;
        }
        v2 c = vadd(pc[i], vscale(sub_dt, v));
        double a = pa[i] + sub_dt * om;
        pc[i] = c; pa[i] = a; vv[i] = v; ww[i] = om;
        b->cx = c.x; b->cy = c.y; b->a = a;
        b->vx = v.x; b->vy = v.y; b->w = om;
        sync_transform(b);
    }
    free(ks);
    free(pc); free(pa); free(vv); free(ww);
}

/* world.py:594-821 World.solve_toi */
static void world_solve_toi(or_world *w, double dt, int vel_iters) {
    int nb = w->nb;
    int *bflag = w->island_flag_b;
    if (w->wflags & GB_W_STEP_COMPLETE) {
        for (int i = 0; i < nb; ++i) { bflag[i] = 0; w->b[i].alpha0 = 0.0; }
        for (int k = 0; k < w->order.n; ++k) {
            or_contact *c = &w->c[w->order.d[k]];
            c->flags &= ~(GB_C_TOI | GB_C_ISLAND);
            c->toi_count = 0;
            c->toi = 1.0;
        }
    }
    int ibodies[2 * MAX_TOI_CONTACTS];
    int icontacts[MAX_TOI_CONTACTS];
    for (;;) {
        int min_contact = -1;
        double min_alpha = 1.0;
        int n = w->order.n;
        int *snap = (int *)malloc(sizeof(int) * (n ? n : 1));
        int ns = 0;
        for (int k = 0; k < n; ++k) {
            or_contact *c = &w->c[w->order.d[k]];
            if ((c->flags & GB_C_ENABLED) && c->toi_count <= MAX_SUB_STEPS) snap[ns++] = w->order.d[k];
        }
        for (int k = 0; k < ns; ++k) {
            or_contact *c = &w->c[snap[k]];
            double alpha = 1.0;
            if (c->flags & GB_C_TOI) {
                alpha = c->toi;
            } else {
                const gb_fixture *fa = &w->f[c->fa], *fb = &w->f[c->fb];
                if ((fa->flags | fb->flags) & GB_FIX_SENSOR) continue;
                gb_body *ba = &w->b[fa->body], *bb = &w->b[fb->body];
                int act_a = body_awake(ba) && ba->type != GB_BODY_STATIC;
                int act_b = body_awake(bb) && bb->type != GB_BODY_STATIC;
                if (!act_a && !act_b) continue;
                int col_a = (ba->flags & GB_BODY_BULLET) || ba->type != GB_BODY_DYNAMIC;
                int col_b = (bb->flags & GB_BODY_BULLET) || bb->type != GB_BODY_DYNAMIC;
                if (!col_a && !col_b) continue;
                double alpha0 = ba->alpha0;
                if (ba->alpha0 < bb->alpha0) {
                    alpha0 = bb->alpha0;
                    or_sweep s = get_sweep(ba); or_sweep_advance(&s, alpha0); put_sweep(ba, &s);
                } else if (bb->alpha0 < ba->alpha0) {
                    or_sweep s = get_sweep(bb); or_sweep_advance(&s, alpha0); put_sweep(bb, &s);
                }
                or_dproxy pa, pb;
                or_dproxy_init(&pa, fa); or_dproxy_init(&pb, fb);
                or_sweep sa = get_sweep(ba), sb = get_sweep(bb);
                double beta;
                int state = or_time_of_impact(&pa, &pb, &sa, &sb, 1.0, &beta);
                w->n_toi_calls++;
                if (state == TOI_TOUCHING) alpha = pymin(alpha0 + (1.0 - alpha0) * beta, 1.0);
                else alpha = 1.0;
                c->toi = alpha;
                c->flags |= GB_C_TOI;
            }
            if (alpha < min_alpha) { min_contact = snap[k]; min_alpha = alpha; }
        }
        free(snap);
        if (min_contact < 0 || (1.0 - (10.0 * OR_EPSILON)) < min_alpha) {
            w->wflags |= GB_W_STEP_COMPLETE;
            break;
        }
        w->n_toi_events++;
        or_contact *mc = &w->c[min_contact];
        int bia = w->f[mc->fa].body, bib = w->f[mc->fb].body;
        gb_body *ba = &w->b[bia], *bb = &w->b[bib];
        gb_body backup_a = *ba, backup_b = *bb;
        body_advance(ba, min_alpha);
        body_advance(bb, min_alpha);
        contact_update(w, min_contact);
        mc = &w->c[min_contact];
        mc->flags &= ~GB_C_TOI;
        mc->toi_count += 1;
        if (!(mc->flags & GB_C_ENABLED) || !(mc->flags & GB_C_TOUCHING)) {
            mc->flags &= ~GB_C_ENABLED;
            or_sweep s = get_sweep(&backup_a); put_sweep(ba, &s);
            s = get_sweep(&backup_b); put_sweep(bb, &s);
            sync_transform(ba); sync_transform(bb);
            continue;
        }
        set_awake(ba, 1); set_awake(bb, 1);
        int nbi = 0, nci = 0;
        w->island_index[bia] = nbi; ibodies[nbi++] = bia;
        w->island_index[bib] = nbi; ibodies[nbi++] = bib;
        icontacts[nci++] = min_contact;
        bflag[bia] = 1; bflag[bib] = 1;
        mc->flags |= GB_C_ISLAND;
        int dyn[2], nd = 0;
        if (ba->type == GB_BODY_DYNAMIC) dyn[nd++] = bia;
        if (bb->type == GB_BODY_DYNAMIC) dyn[nd++] = bib;
        for (int di = 0; di < nd; ++di) {
            int bi = dyn[di];
            gb_body *body = &w->b[bi];
            ivec *lst = &w->bcon[bi];
            for (int li = 0; li < lst->n; ++li) {
                if (nbi == 2 * MAX_TOI_CONTACTS) { w->status |= GB_ST_TOI_ISLAND_CAP; break; }
                if (nci == MAX_TOI_CONTACTS) { w->status |= GB_ST_TOI_ISLAND_CAP; break; }
                int cid = lst->d[li];
                or_contact *c = &w->c[cid];
                if (c->flags & GB_C_ISLAND) continue;
                int oi = (w->f[c->fa].body == bi) ? w->f[c->fb].body : w->f[c->fa].body;
                gb_body *other = &w->b[oi];
                if (other->type == GB_BODY_DYNAMIC && !(body->flags & GB_BODY_BULLET) && !(other->flags & GB_BODY_BULLET))
                    continue;
                if ((w->f[c->fa].flags | w->f[c->fb].flags) & GB_FIX_SENSOR) continue;
                gb_body backup = *other;
                if (!bflag[oi]) body_advance(other, min_alpha);
                contact_update(w, cid);
                c = &w->c[cid];
                if (!(c->flags & GB_C_ENABLED) || !(c->flags & GB_C_TOUCHING)) {
                    or_sweep s = get_sweep(&backup); put_sweep(other, &s);
                    sync_transform(other);
                    continue;
                }
                c->flags |= GB_C_ISLAND;
                icontacts[nci++] = cid;
                if (bflag[oi]) continue;
                bflag[oi] = 1;
                if (other->type != GB_BODY_STATIC) set_awake(other, 1);
                w->island_index[oi] = nbi;
                ibodies[nbi++] = oi;
            }
        }
        double sub_dt = (1.0 - min_alpha) * dt;
        island_solve_toi(w, ibodies, nbi, icontacts, nci, sub_dt, vel_iters, w->island_index[bia], w->island_index[bib]);
        for (int i = 0; i < nbi; ++i) {
            int bi = ibodies[i];
            bflag[bi] = 0;
            if (w->b[bi].type == GB_BODY_DYNAMIC) {
                sync_fixtures(w, bi);
                ivec *lst = &w->bcon[bi];
                for (int li = 0; li < lst->n; ++li) w->c[lst->d[li]].flags &= ~(GB_C_TOI | GB_C_ISLAND);
            }
        }
        find_new_contacts(w);
    }
}

/* world.py:307-354 World.step */
void or_step(or_world *w, double dt, int vel_iters, int pos_iters) {
    memset(w->rec, 0, sizeof(int) * (size_t)(w->nb ? w->nb : 1));
    for (int i = 0; i < w->nb; ++i) w->rec_island[i] = -1;
    if (w->wflags & GB_W_NEW_FIXTURE) {
        find_new_contacts(w);
        w->wflags &= ~GB_W_NEW_FIXTURE;
    }
    double inv_dt = dt > 0.0 ? 1.0 / dt : 0.0;
    double dt_ratio = w->inv_dt0 * dt;
    collide(w);
    if ((w->wflags & GB_W_STEP_COMPLETE) && dt > 0.0) world_solve(w, dt, inv_dt, dt_ratio, vel_iters, pos_iters);
    if ((w->wflags & GB_W_CONTINUOUS) && dt > 0.0) world_solve_toi(w, dt, vel_iters);
    if (dt > 0.0) w->inv_dt0 = inv_dt;
    if (w->wflags & GB_W_AUTO_CLEAR_FORCES)
        for (int i = 0; i < w->nb; ++i) { w->b[i].fx = 0.0; w->b[i].fy = 0.0; w->b[i].torque = 0.0; }
    w->hook_set = 0;
    w->jhook_set = 0;
}

/* ------------------------------------------------------------------ */
or_world *or_create(const gb_world_desc *wd, const gb_body *bodies, const gb_fixture *fixtures, const gb_contact *contacts,
                    const int32_t *moves) {
    or_world *w = (or_world *)calloc(1, sizeof(or_world));
    w->nb = wd->body_count;
    w->nf = wd->fixture_count;
    w->b = (gb_body *)malloc(sizeof(gb_body) * (w->nb ? w->nb : 1));
    w->f = (gb_fixture *)malloc(sizeof(gb_fixture) * (w->nf ? w->nf : 1));
    memcpy(w->b, bodies + wd->body_start, sizeof(gb_body) * w->nb);
    memcpy(w->f, fixtures + wd->fixture_start, sizeof(gb_fixture) * w->nf);
    w->bcon = (ivec *)calloc(w->nb ? w->nb : 1, sizeof(ivec));
    w->island_flag_b = (int *)calloc(w->nb ? w->nb : 1, sizeof(int));
    w->island_index = (int *)calloc(w->nb ? w->nb : 1, sizeof(int));
    w->rec = (int *)calloc(w->nb ? w->nb : 1, sizeof(int));
    w->rec_island = (int *)calloc(w->nb ? w->nb : 1, sizeof(int));
    w->bjoint = (ivec *)calloc(w->nb ? w->nb : 1, sizeof(ivec));
    w->wflags = wd->flags;
    w->gravity = V(wd->gx, wd->gy);
    w->inv_dt0 = wd->inv_dt0;
    if (contacts) {
        for (int k = 0; k < wd->contact_count; ++k) {
            const gb_contact *g = &contacts[wd->contact_start + k];
            int id = contact_new(w);
            or_contact *c = &w->c[id];
            c->fa = g->fixture_a; c->fb = g->fixture_b; c->ia = g->child_a; c->ib = g->child_b;
            c->flags = g->flags; c->toi_count = g->toi_count; c->toi = g->toi;
            c->friction = g->friction; c->restitution = g->restitution;
            c->m.type = g->m_type; c->m.count = g->m_point_count;
            c->m.ln = V(g->m_lnx, g->m_lny); c->m.lp = V(g->m_lpx, g->m_lpy);
            for (int i = 0; i < 2; ++i) {
                c->m.plp[i] = V(g->p_lx[i], g->p_ly[i]);
                c->m.ni[i] = g->p_ni[i]; c->m.ti[i] = g->p_ti[i]; c->m.id[i] = g->p_id[i];
            }
            c->alive = 1;
            iv_push(&w->order, id);
            iv_push(&w->bcon[w->f[c->fa].body], id);
            iv_push(&w->bcon[w->f[c->fb].body], id);
        }
    }
    if (wd->move_count > 0 && moves)
        for (int i = 0; i < wd->move_count; ++i) iv_push(&w->move, moves[wd->move_start + i]);
    else if (w->wflags & GB_W_NEW_FIXTURE)
        for (int i = 0; i < w->nf; ++i) iv_push(&w->move, i);
    return w;
}

void or_destroy(or_world *w) {
    if (!w) return;
    for (int i = 0; i < w->nb; ++i) free(w->bcon[i].d);
    free(w->bcon);
    free(w->order.d); free(w->move.d); free(w->last_order.d);
    free(w->island_flag_b); free(w->island_index); free(w->hook_rank);
    free(w->hook_pending); free(w->pos_of); free(w->rec); free(w->rec_island);
    if (w->bjoint)
        for (int i = 0; i < w->nb; ++i) free(w->bjoint[i].d);
    free(w->bjoint); free(w->j); free(w->jflag); free(w->jhook_rank); free(w->last_jorder.d);
    free(w->ctl); free(w->ctl_bodies); free(w->accept);
    free(w->c); free(w->b); free(w->f);
    free(w);
}

int or_body_count(const or_world *w) { return w->nb; }
int or_contact_count(const or_world *w) { return w->order.n; }
uint32_t or_world_flags(const or_world *w) { return w->wflags; }
double or_inv_dt0(const or_world *w) { return w->inv_dt0; }
int or_status(const or_world *w) { return w->status; }

void or_get_bodies(const or_world *w, gb_body *out) { memcpy(out, w->b, sizeof(gb_body) * w->nb); }
void or_set_bodies(or_world *w, const gb_body *in) { memcpy(w->b, in, sizeof(gb_body) * w->nb); }
void or_get_fixtures(const or_world *w, gb_fixture *out) { memcpy(out, w->f, sizeof(gb_fixture) * w->nf); }

int or_get_contacts(const or_world *w, gb_contact *out, int cap) {
    int n = w->order.n;
    for (int k = 0; k < n && k < cap; ++k) {
        const or_contact *c = &w->c[w->order.d[k]];
        gb_contact *g = &out[k];
        memset(g, 0, sizeof(*g));
        g->fixture_a = c->fa; g->fixture_b = c->fb; g->child_a = c->ia; g->child_b = c->ib;
        g->flags = c->flags; g->toi_count = c->toi_count; g->toi = c->toi;
        g->friction = c->friction; g->restitution = c->restitution;
        g->m_type = c->m.type; g->m_point_count = c->m.count;
        g->m_lnx = c->m.ln.x; g->m_lny = c->m.ln.y; g->m_lpx = c->m.lp.x; g->m_lpy = c->m.lp.y;
        for (int i = 0; i < 2; ++i) {
            g->p_lx[i] = c->m.plp[i].x; g->p_ly[i] = c->m.plp[i].y;
            g->p_ni[i] = c->m.ni[i]; g->p_ti[i] = c->m.ti[i]; g->p_id[i] = c->m.id[i];
        }
    }
    return n;
}

/* Solver order hook: `order` lists contact-list positions (at the time of
 * the next step's _solve) in the order the constraints must be solved. */
void or_set_solver_order(or_world *w, const int *order, int n) {
    w->hook_pending_n = n;
    free(w->hook_pending);
    w->hook_pending = (int *)malloc(sizeof(int) * (n ? n : 1));
    memcpy(w->hook_pending, order, sizeof(int) * n);
    w->hook_set = 1;
}

int or_get_solver_order(const or_world *w, int *out, int cap) {
    for (int i = 0; i < w->last_order.n && i < cap; ++i) out[i] = w->last_order.d[i];
    return w->last_order.n;
}

long long or_toi_calls(const or_world *w) { return w->n_toi_calls; }
void or_clear_status(or_world *w) { w->status = 0; }

/* The joints of a world (World.joints order, each added by World.add_joint,
 * world.py:252-283); replaces any joints given before.  Returns -1 (and
 * keeps the old joints) for a joint with a bad body index or type. */
int or_set_joints(or_world *w, const gb_joint *joints, int n) {
    for (int i = 0; i < n; ++i) {
        const gb_joint *J = &joints[i];
        if (J->body_a < 0 || J->body_a >= w->nb || J->body_b < 0 || J->body_b >= w->nb ||
            (J->type == GB_JOINT_MOUSE ? J->body_a != J->body_b : J->body_a == J->body_b) ||
            J->type < GB_JOINT_REVOLUTE || J->type > GB_JOINT_MOUSE)
            return -1;
    }
    for (int i = 0; i < w->nb; ++i) w->bjoint[i].n = 0;
    w->j = (gb_joint *)realloc(w->j, sizeof(gb_joint) * (size_t)(n ? n : 1));
    w->jflag = (int *)realloc(w->jflag, sizeof(int) * (size_t)(n ? n : 1));
    w->jhook_rank = (int *)realloc(w->jhook_rank, sizeof(int) * (size_t)(n ? n : 1));
    if (n) memcpy(w->j, joints, sizeof(gb_joint) * (size_t)n);
    w->nj = n;
    for (int i = 0; i < n; ++i) {
        iv_push(&w->bjoint[w->j[i].body_a], i);
        if (w->j[i].body_b != w->j[i].body_a) iv_push(&w->bjoint[w->j[i].body_b], i);   /* mouse: one body */
    }
    return 0;
}
/* World.add_joint's flagging of the contacts between a new joint's bodies
 * (world.py:275-281), for a joint that turns collision off */
void or_flag_joint_contacts(or_world *w, int j) {
    const gb_joint *J = &w->j[j];
    if (J->flags & GB_J_COLLIDE_CONNECTED) return;
    ivec *lst = &w->bcon[J->body_b];
    for (int i = 0; i < lst->n; ++i) {
        or_contact *c = &w->c[lst->d[i]];
        int other = (w->f[c->fa].body == J->body_b) ? w->f[c->fb].body : w->f[c->fa].body;
        if (other == J->body_a) c->flags |= GB_C_FILTER;
    }
}
int or_joint_count(const or_world *w) { return w->nj; }
void or_get_joints(const or_world *w, gb_joint *out) { if (w->nj) memcpy(out, w->j, sizeof(gb_joint) * (size_t)w->nj); }
/* Solve the next step's joints in this order (world joint indices); joints
 * not listed come after the listed ones, in index order. */
void or_set_joint_order(or_world *w, const int *order, int n) {
    for (int k = 0; k < w->nj; ++k) w->jhook_rank[k] = n + k;
    for (int i = 0; i < n; ++i)
        if (order[i] >= 0 && order[i] < w->nj) w->jhook_rank[order[i]] = i;
    w->jhook_set = 1;
}
int or_get_joint_order(const or_world *w, int *out, int cap) {
    for (int i = 0; i < w->last_jorder.n && i < cap; ++i) out[i] = w->last_jorder.d[i];
    return w->last_jorder.n;
}
void or_get_step_record(const or_world *w, int *out) {
    memcpy(out, w->rec, sizeof(int) * (size_t)w->nb);
    memcpy(out + w->nb, w->rec_island, sizeof(int) * (size_t)w->nb);
}
long long or_toi_events(const or_world *w) { return w->n_toi_events; }

/* ------------------------------------------------------------------ */
/* multi-threaded driver used as the CPU baseline                       */
#include <time.h>
typedef struct {
    const gb_scene *scene;
    double dt;
    int vi, pi, steps;
    gb_body *out;
    int next;
    pthread_mutex_t mu;
} or_job;

/* A custom contact filter's answers for every ordered pair of the world's
 * fixture records (n must be the record count), or accept = NULL for the
 * default rule again; returns -1 for a wrong count. */
int or_set_pair_filter(or_world *w, const unsigned char *accept, int n) {
    if (!accept) { free(w->accept); w->accept = NULL; w->accept_n = 0; return 0; }
    if (n != w->nf) return -1;
    unsigned char *m = (unsigned char *)malloc((size_t)n * (size_t)n + 1u);
    if (!m) return -1;
    memcpy(m, accept, (size_t)n * (size_t)n);
    free(w->accept);
    w->accept = m;
    w->accept_n = n;
    return 0;
}

/* The controllers of a world (World.controllers order) with their body
 * lists: controller k's bodies are bodies[ctl[k].body_start ..
 * + ctl[k].body_count), world-local.  Replaces any controllers given before;
 * returns -1 (keeping the old ones) for a bad kind or body index. */
int or_set_controllers(or_world *w, const gb_controller *ctl, int n, const int32_t *bodies, int nbodies) {
    if (n < 0) return -1;
    size_t total = 0;
    for (int k = 0; k < n; ++k) {
        const gb_controller *C = &ctl[k];
        if (C->type < GB_CONTROLLER_BUOYANCY || C->type > GB_CONTROLLER_GRAVITY || C->body_count < 0 || C->body_start < 0 ||
            C->body_start + C->body_count > nbodies)
            return -1;
        for (int i = 0; i < C->body_count; ++i)
            if (bodies[C->body_start + i] < 0 || bodies[C->body_start + i] >= w->nb) return -1;
        total += (size_t)C->body_count;
    }
    w->ctl = (gb_controller *)realloc(w->ctl, sizeof(gb_controller) * (n > 0 ? (size_t)n : 1u));
    w->ctl_bodies = (int *)realloc(w->ctl_bodies, sizeof(int) * (total ? total : 1));
    int at = 0;
    for (int k = 0; k < n; ++k) {
        w->ctl[k] = ctl[k];
        for (int i = 0; i < ctl[k].body_count; ++i) w->ctl_bodies[at + i] = bodies[ctl[k].body_start + i];
        w->ctl[k].body_start = at;
        at += ctl[k].body_count;
    }
    w->nctl = n;
    return 0;
}

/* the controllers of world `wi` of a scene (sorted by world) */
static void scene_controllers(or_world *w, const gb_scene *scene, int wi) {
    if (scene->n_controllers <= 0 || !scene->controllers) return;
    int s0 = 0;
    while (s0 < scene->n_controllers && scene->controllers[s0].world < wi) ++s0;
    int s1 = s0;
    while (s1 < scene->n_controllers && scene->controllers[s1].world == wi) ++s1;
    if (s1 > s0) or_set_controllers(w, scene->controllers + s0, s1 - s0, scene->controller_bodies, scene->n_controller_bodies);
}

/* the joints of world `wi` of a scene (sorted by world) */
static void scene_joints(or_world *w, const gb_scene *scene, int wi) {
    if (scene->n_joints <= 0 || !scene->joints) return;
    int s0 = 0;
    while (s0 < scene->n_joints && scene->joints[s0].world < wi) ++s0;
    int s1 = s0;
    while (s1 < scene->n_joints && scene->joints[s1].world == wi) ++s1;
    if (s1 > s0) or_set_joints(w, scene->joints + s0, s1 - s0);
}

static void *or_worker(void *arg) {
    or_job *j = (or_job *)arg;
    for (;;) {
        pthread_mutex_lock(&j->mu);
        int wi = j->next++;
        pthread_mutex_unlock(&j->mu);
        if (wi >= j->scene->n_worlds) break;
        const gb_world_desc *wd = &j->scene->worlds[wi];
        or_world *w = or_create(wd, j->scene->bodies, j->scene->fixtures, j->scene->contacts, j->scene->moves);
        scene_joints(w, j->scene, wi);
        scene_controllers(w, j->scene, wi);
        for (int s = 0; s < j->steps; ++s) or_step(w, j->dt, j->vi, j->pi);
        if (j->out) or_get_bodies(w, j->out + wd->body_start);
        or_destroy(w);
    }
    return NULL;
}

double or_run_scene(const gb_scene *scene, double dt, int vel_iters, int pos_iters, int n_steps, int threads,
                    gb_body *bodies_out) {
    or_job j;
    j.scene = scene; j.dt = dt; j.vi = vel_iters; j.pi = pos_iters; j.steps = n_steps;
    j.out = bodies_out; j.next = 0;
    pthread_mutex_init(&j.mu, NULL);
    if (threads < 1) threads = 1;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * threads);
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    for (int i = 0; i < threads; ++i) pthread_create(&th[i], NULL, or_worker, &j);
    for (int i = 0; i < threads; ++i) pthread_join(th[i], NULL);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    free(th);
    pthread_mutex_destroy(&j.mu);
    return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}

/* Persistent batch of worlds stepped by a pool of POSIX threads (the CPU
 * baseline steps the same worlds repeatedly, as a simulation loop does). */
struct or_batch {
    int n;
    or_world **w;
};

or_batch *or_batch_create(const gb_scene *scene) {
    or_batch *b = (or_batch *)calloc(1, sizeof(or_batch));
    b->n = scene->n_worlds;
    b->w = (or_world **)calloc(b->n ? b->n : 1, sizeof(or_world *));
    for (int i = 0; i < b->n; ++i) {
        b->w[i] = or_create(&scene->worlds[i], scene->bodies, scene->fixtures, scene->contacts, scene->moves);
        scene_joints(b->w[i], scene, i);
        scene_controllers(b->w[i], scene, i);
    }
    return b;
}

void or_batch_destroy(or_batch *b) {
    if (!b) return;
    for (int i = 0; i < b->n; ++i) or_destroy(b->w[i]);
    free(b->w);
    free(b);
}

typedef struct {
    or_batch *b;
    double dt;
    int vi, pi, steps, next;
    pthread_mutex_t mu;
} or_bjob;

static void *or_bworker(void *arg) {
    or_bjob *j = (or_bjob *)arg;
    for (;;) {
        pthread_mutex_lock(&j->mu);
        int wi = j->next++;
        pthread_mutex_unlock(&j->mu);
        if (wi >= j->b->n) break;
        for (int s = 0; s < j->steps; ++s) or_step(j->b->w[wi], j->dt, j->vi, j->pi);
    }
    return NULL;
}

double or_batch_step(or_batch *b, double dt, int vel_iters, int pos_iters, int n_steps, int threads) {
    or_bjob j;
    j.b = b; j.dt = dt; j.vi = vel_iters; j.pi = pos_iters; j.steps = n_steps; j.next = 0;
    pthread_mutex_init(&j.mu, NULL);
    if (threads < 1) threads = 1;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * threads);
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    for (int i = 0; i < threads; ++i) pthread_create(&th[i], NULL, or_bworker, &j);
    for (int i = 0; i < threads; ++i) pthread_join(th[i], NULL);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    free(th);
    pthread_mutex_destroy(&j.mu);
    return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}

int or_batch_get_bodies(const or_batch *b, int wi, gb_body *out) {
    if (wi < 0 || wi >= b->n) return -1;
    or_get_bodies(b->w[wi], out);
    return b->w[wi]->nb;
}

/* ------------------------------------------------------------------ queries
 * World.ray_cast with a closest-hit callback (world.py:387-440) and
 * World.query_aabb (world.py:371-385) over one world's host records
 * (fixture.body indexes `bodies`, fixtures world-local). */

/* AABB.test_overlap (aabbmodule.c AABB_test_overlap): node box a, other box b */
static int or_box_overlap(const double *a, double blx, double bly, double bhx, double bhy) {
    return !((blx - a[2]) > 0.0 || (bly - a[3]) > 0.0 || (a[0] - bhx) > 0.0 || (a[1] - bhy) > 0.0);
}

/* Circle.ray_cast (shapes.py:147-171), max_fraction 1 */
static int or_ray_circle(const gb_fixture *f, xform xf, v2 p1, v2 p2, v2 *normal, double *fraction) {
    v2 position = vadd(xf.p, rmul(xf.q, V(f->vx[0], f->vy[0])));
    v2 s = vsub(p1, position);
    double b = vdot(s, s) - SQ(f->radius);
    v2 r = vsub(p2, p1);
    double c = vdot(s, r);
    double rr = vdot(r, r);
    double sigma = c * c - rr * b;
    if (sigma < 0.0 || rr < DBL_EPSILON) return 0;
    double a = -(c + sqrt(sigma));
    if (0.0 <= a && a <= 1.0 * rr) {
        a /= rr;
        *fraction = a;
        *normal = vnormalized(vadd(s, vscale(a, r)));
        return 1;
    }
    return 0;
}

/* Polygon.ray_cast (shapes.py:265-314), max_fraction 1 */
static int or_ray_polygon(const gb_fixture *f, xform xf, v2 p1, v2 p2, v2 *normal, double *fraction) {
    v2 q1 = rmul_t(xf.q, vsub(p1, xf.p));
    v2 q2 = rmul_t(xf.q, vsub(p2, xf.p));
    v2 d = vsub(q2, q1);
    double lower = 0.0, upper = 1.0;
    int tagged = -1;
    for (int k = 0; k < f->vertex_count; ++k) {
        v2 nk = V(f->nx[k], f->ny[k]);
        double numerator = vdot(nk, vsub(V(f->vx[k], f->vy[k]), q1));
        double denominator = vdot(nk, d);
        if (denominator == 0.0) {
            if (numerator < 0.0) return 0;
        } else {
            if (denominator < 0.0 && numerator < lower * denominator) {
                lower = numerator / denominator;
                tagged = k;
            } else if (denominator > 0.0 && numerator < upper * denominator) {
                upper = numerator / denominator;
            }
        }
        if (upper < lower) return 0;
    }
    if (tagged < 0) return 0;
    *normal = rmul(xf.q, V(f->nx[tagged], f->ny[tagged]));
    *fraction = lower;
    return 1;
}

/* Edge.ray_cast (shapes.py:655-702); the normal stays in the edge's frame */
static int or_ray_edge(const gb_fixture *f, xform xf, v2 p1, v2 p2, v2 *normal, double *fraction) {
    v2 q1 = rmul_t(xf.q, vsub(p1, xf.p));
    v2 q2 = rmul_t(xf.q, vsub(p2, xf.p));
    v2 d = vsub(q2, q1);
    v2 v1 = V(f->vx[0], f->vy[0]), v2_ = V(f->vx[1], f->vy[1]);
    v2 e = vsub(v2_, v1);
    v2 nn = vnormalized(V(e.y, -e.x));
    double numerator = vdot(nn, vsub(v1, q1));
    double denominator = vdot(nn, d);
    if (denominator == 0.0) return 0;
    double t = numerator / denominator;
    if (t < 0.0 || 1.0 < t) return 0;
    v2 q = vadd(q1, vscale(t, d));
    v2 r = vsub(v2_, v1);
    double rr = vdot(r, r);
    if (rr == 0.0) return 0;
    double s = vdot(vsub(q, v1), r) / rr;
    if (s < 0.0 || 1.0 < s) return 0;
    *fraction = t;
    *normal = numerator > 0.0 ? vneg(nn) : nn;
    return 1;
}

/* DynamicTree.ray_cast's segment tests (dynamictree.py:222-250) at
 * max_fraction 1, then the fixture's shape ray cast */
typedef struct { v2 p1, p2, v, abs_v; double slx, sly, shx, shy; } or_seg;
static or_seg or_ray_seg(const gb_ray *ray) {
    or_seg s;
    s.p1 = V(ray->p1x, ray->p1y);
    s.p2 = V(ray->p2x, ray->p2y);
    v2 r = vnormalized(vsub(s.p2, s.p1));
    s.v = vcross_sv(1.0, r);
    s.abs_v = V(fabs(s.v.x), fabs(s.v.y));
    v2 t = vadd(s.p1, vscale(1.0, vsub(s.p2, s.p1)));
    s.slx = pymin(s.p1.x, t.x); s.sly = pymin(s.p1.y, t.y); s.shx = pymax(s.p1.x, t.x); s.shy = pymax(s.p1.y, t.y);
    return s;
}
static int or_ray_fixture(const gb_body *bodies, const gb_fixture *f, const or_seg *s, v2 *nrm, double *fr) {
    if (!(bodies[f->body].flags & GB_BODY_ACTIVE)) return 0;   /* no proxy */
    const double *a = f->aabb;
    if (!or_box_overlap(a, s->slx, s->sly, s->shx, s->shy)) return 0;
    v2 c = V(0.5 * (a[2] + a[0]), 0.5 * (a[3] + a[1]));
    v2 h = V(0.5 * (a[2] - a[0]), 0.5 * (a[3] - a[1]));
    double separation = fabs(vdot(s->v, vsub(s->p1, c))) - vdot(s->abs_v, h);
    if (separation > 0.0) return 0;
    const gb_body *b = &bodies[f->body];
    xform xf;
    xf.p = V(b->px, b->py);
    xf.q.c = b->qc;
    xf.q.s = b->qs;
    if (f->shape_type == GB_SHAPE_CIRCLE) return or_ray_circle(f, xf, s->p1, s->p2, nrm, fr);
    if (f->shape_type == GB_SHAPE_POLYGON) return or_ray_polygon(f, xf, s->p1, s->p2, nrm, fr);
    if (f->shape_type == GB_SHAPE_EDGE) return or_ray_edge(f, xf, s->p1, s->p2, nrm, fr);
    return 0;
}
static gb_ray_hit or_make_hit(const or_seg *s, int k, v2 n, double fr) {
    gb_ray_hit o;
    memset(&o, 0, sizeof(o));
    v2 pt = vadd(vscale(1.0 - fr, s->p1), vscale(fr, s->p2));   /* world.py:431 */
    o.fixture = k; o.px = pt.x; o.py = pt.y; o.nx = n.x; o.ny = n.y; o.fraction = fr;
    return o;
}

/* every hit of each ray, in fixture order: the generator form of
 * World.ray_cast with each fraction left at 1 */
void or_ray_cast_all_records(const gb_body *bodies, const gb_fixture *fixtures, int nf, const gb_ray *rays, int n,
                             gb_ray_hit *hits, int cap, int32_t *counts) {
    for (int q = 0; q < n; ++q) {
        or_seg s = or_ray_seg(&rays[q]);
        int found = 0;
        for (int k = 0; k < nf; ++k) {
            v2 nrm;
            double fr = 0.0;
            if (!or_ray_fixture(bodies, &fixtures[k], &s, &nrm, &fr)) continue;
            if (found < cap) hits[(size_t)q * cap + found] = or_make_hit(&s, k, nrm, fr);
            ++found;
        }
        counts[q] = found;
    }
}

void or_ray_cast_records(const gb_body *bodies, const gb_fixture *fixtures, int nf, const gb_ray *rays, int n,
                         gb_ray_hit *hits) {
    for (int q = 0; q < n; ++q) {
        v2 p1 = V(rays[q].p1x, rays[q].p1y), p2 = V(rays[q].p2x, rays[q].p2y);
        /* DynamicTree.ray_cast's segment tests (dynamictree.py:222-250) */
        v2 r = vnormalized(vsub(p2, p1));
        v2 v = vcross_sv(1.0, r);
        v2 abs_v = V(fabs(v.x), fabs(v.y));
        v2 t = vadd(p1, vscale(1.0, vsub(p2, p1)));
        double slx = pymin(p1.x, t.x), sly = pymin(p1.y, t.y), shx = pymax(p1.x, t.x), shy = pymax(p1.y, t.y);
        gb_ray_hit o;
        memset(&o, 0, sizeof(o));
        o.fixture = -1;
        o.fraction = 1.0;
        double best = 2.0;
        v2 best_n = V(0.0, 0.0);
        for (int k = 0; k < nf; ++k) {
            const gb_fixture *f = &fixtures[k];
            const double *a = f->aabb;
            if (!or_box_overlap(a, slx, sly, shx, shy)) continue;
            v2 c = V(0.5 * (a[2] + a[0]), 0.5 * (a[3] + a[1]));
            v2 h = V(0.5 * (a[2] - a[0]), 0.5 * (a[3] - a[1]));
            double separation = fabs(vdot(v, vsub(p1, c))) - vdot(abs_v, h);
            if (separation > 0.0) continue;
            const gb_body *b = &bodies[f->body];
            xform xf;
            xf.p = V(b->px, b->py);
            xf.q.c = b->qc;
            xf.q.s = b->qs;
            v2 nrm;
            double fr = 0.0;
            int hit = 0;
            if (f->shape_type == GB_SHAPE_CIRCLE) hit = or_ray_circle(f, xf, p1, p2, &nrm, &fr);
            else if (f->shape_type == GB_SHAPE_POLYGON) hit = or_ray_polygon(f, xf, p1, p2, &nrm, &fr);
            else if (f->shape_type == GB_SHAPE_EDGE) hit = or_ray_edge(f, xf, p1, p2, &nrm, &fr);
            if (hit && fr < best) { best = fr; o.fixture = k; best_n = nrm; }
        }
        if (o.fixture >= 0) {
            /* world.py:431: (1 - fraction) * point1 + fraction * point2 */
            v2 pt = vadd(vscale(1.0 - best, p1), vscale(best, p2));
            o.px = pt.x; o.py = pt.y; o.nx = best_n.x; o.ny = best_n.y; o.fraction = best;
        }
        hits[q] = o;
    }
}

void or_query_aabb_records(const gb_fixture *fixtures, int nf, const gb_aabb_query *qs, int n, int32_t *out, int cap,
                           int32_t *counts) {
    for (int q = 0; q < n; ++q) {
        int found = 0;
        for (int k = 0; k < nf; ++k)
            if (or_box_overlap(fixtures[k].aabb, qs[q].lx, qs[q].ly, qs[q].ux, qs[q].uy)) {
                if (found < cap) out[(size_t)q * cap + found] = k;
                ++found;
            }
        counts[q] = found;
    }
}

// gb_toi.cuh -- continuous collision (pypybox2d/world.py:594-821) and the
// per-step driver World.step (world.py:307-354) for one world.
//
// The time-of-impact event loop is sequential in the reference: the earliest
// event over all contacts is resolved, bodies are advanced, a sub-island is
// solved and the loop repeats.  Here the first pass over the contacts (every
// sweep still starts at alpha0 = 0, so no contact changes another's input)
// computes all times of impact in parallel; each event and every later pass
// run on the group's rank 0 in contact-list order, as the reference does,
// because a pass there advances sweeps in place.  Pair finding after an
// event is group-parallel.
#pragma once
#include "gb_step.cuh"

// world.py:617-653 for contact i at the start of a TOI pass: 0 = skipped
// (disabled, sub-stepped too often, sensor, inactive, no bullet or
// non-dynamic body), 1 = cached time of impact, 2 = needs a fresh one.
template <class R> __device__ int toi_status(const WView<R> &w, int i) {
    const ContactRec<R> &c = w.con(i);
    if (!(c.flags & GB_C_ENABLED) || c.toi_count > GB_MAX_SUB_STEPS) return 0;
    if (c.flags & GB_C_TOI) return 1;
    if (fx_sensor(w, c.fa) || fx_sensor(w, c.fb)) return 0;
    int ba = w.fbody(c.fa), bb = w.fbody(c.fb);
    int ta = w.btype(ba), tb = w.btype(bb);
    bool act_a = w.awake(ba) && ta != GB_BODY_STATIC;
    bool act_b = w.awake(bb) && tb != GB_BODY_STATIC;
    if (!act_a && !act_b) return 0;
    bool col_a = (w.B.b_flags[w.bb + ba] & GB_BODY_BULLET) || ta != GB_BODY_DYNAMIC;
    bool col_b = (w.B.b_flags[w.bb + bb] & GB_BODY_BULLET) || tb != GB_BODY_DYNAMIC;
    if (!col_a && !col_b) return 0;
    return 2;
}

// world.py:656-661: put both sweeps on the same time interval, advancing
// the lagging body's sweep in place; returns alpha0 and the two sweeps.
template <class R> __device__ double toi_align(const WView<R> &w, int i, Sweep *sa, Sweep *sb) {
    const ContactRec<R> &c = w.con(i);
    int ba = w.fbody(c.fa), bb = w.fbody(c.fb);
    double al_a = w.B.b_alpha0[w.bb + ba], al_b = w.B.b_alpha0[w.bb + bb];
    double alpha0 = al_a;
    if (al_a < al_b) {
        alpha0 = al_b;
        Sweep s = w.sweep(ba); sweep_advance(s, alpha0); w.put_sweep(ba, s);
    } else if (al_b < al_a) {
        Sweep s = w.sweep(bb); sweep_advance(s, alpha0); w.put_sweep(bb, s);
    }
    *sa = w.sweep(ba);
    *sb = w.sweep(bb);
    return alpha0;
}

// world.py:669-681: the time of impact from the aligned sweeps.  Float64 in
// both units: the root finder stops anywhere inside its tolerance band
// (a quarter of the linear slop, toi.py:233-234) and the TOI position pass
// stops at -1.5 slop (contact.py:931), which is where the TOI target leaves
// the separation, so float32 arithmetic here moves the bodies by up to
// ~1e-3 m against the float64 step.
template <class R, bool XF_CACHE = false>
__device__ void toi_compute(const WView<R> &w, int i, double alpha0, const Sweep &sa, const Sweep &sb) {
    ContactRec<R> &c = w.con(i);
    double beta;
    bool lim = false;
    DProxy pa, pb;
    dproxy_init(pa, w.shape(c.fa));
    dproxy_init(pb, w.shape(c.fb));
    int state = time_of_impact<XF_CACHE>(pa, pb, sa, sb, 1.0, &beta, &lim);
    if (lim) atomicOr(&w.H->status, GB_ST_ITER_LIMIT);
    double alpha = (state == TOI_TOUCHING) ? pymin(alpha0 + (1.0 - alpha0) * beta, 1.0) : 1.0;
    c.toi = alpha;
    c.flags |= GB_C_TOI;
}

// One contact of a TOI pass (status, alignment, computation); false when
// the contact does not take part.
template <class R> __device__ bool toi_of_contact(const WView<R> &w, int i) {
    int st = toi_status(w, i);
    if (st == 0) return false;
    if (st == 2) {
        Sweep sa, sb;
        double a0 = toi_align(w, i, &sa, &sb);
        toi_compute(w, i, a0, sa, sb);
    }
    return true;
}

// island.py:181-243 Island.solve_toi on rank 0 (island of at most 64
// bodies and 32 contacts).
template <class R> __device__ void island_solve_toi(const WView<R> &w, const int *ib, int nbi, const int *ic, int nci,
                                                    double sub_dt, int vel_iters, int toi_a, int toi_b, const EvCtx *ev = nullptr,
                                                    PhaseClock *ck = nullptr) {
    vec2<double> pc[2 * GB_MAX_TOI_CONTACTS];
    double pa[2 * GB_MAX_TOI_CONTACTS];
    vec2<R> vv[2 * GB_MAX_TOI_CONTACTS];
    R ww[2 * GB_MAX_TOI_CONTACTS];
    int idx[2 * GB_MAX_TOI_CONTACTS][2];
    Cons<R> *ks = w.B.s_cons + (size_t)w.wi * GB_MAX_TOI_CONTACTS;
    for (int i = 0; i < nbi; ++i) {
        int g = w.bb + ib[i];
        pc[i] = w.B.b_c[g]; pa[i] = w.B.b_a[g]; vv[i] = w.B.b_v[g]; ww[i] = w.B.b_w[g];
    }
    for (int k = 0; k < nci; ++k) {
        build_cons(w, ks[k], ic[k], false, 1.0);
        int la = -1, lb = -1;
        for (int i = 0; i < nbi; ++i) { if (ib[i] == ks[k].ia) la = i; if (ib[i] == ks[k].ib) lb = i; }
        if (la < 0 || lb < 0) {   // both bodies of an island contact are island bodies; never index with -1
            w.H->status |= GB_ST_ITER_LIMIT;
            la = 0; lb = 0;
        }
        idx[k][0] = la; idx[k][1] = lb;
    }
    // the position passes in float64 in both units (their early exit at
    // -1.5 slop is where the TOI leaves the separation: see toi_compute)
    int its = 0;
    for (int it = 0; it < 20; ++it) {
        double minsep = 0.0;
        for (int k = 0; k < nci; ++k) {
            int la = idx[k][0], lb = idx[k][1];
            const Cons<double> kd = pos_cons_f64(ks[k]);
            minsep = solve_position(kd, pc[la], pa[la], pc[lb], pa[lb], minsep, true, la == toi_a || la == toi_b,
                                    lb == toi_a || lb == toi_b);
        }
        its = it + 1;
        if (minsep >= -1.5 * GB_LINEAR_SLOP) break;
    }
    if (ck) ck->mark(20);
    if (ev && ev->rec)
        for (int t : {toi_a, toi_b}) {
            rec_add_byte(&ev->rec[ib[t]], GB_REC_TOI_ITERS_SHIFT, its);
            rec_add_byte(&ev->rec[ib[t]], GB_REC_TOI_EVENTS_SHIFT, 1);
        }
    w.B.b_c0[w.bb + ib[toi_a]] = pc[toi_a]; w.B.b_a0[w.bb + ib[toi_a]] = pa[toi_a];
    w.B.b_c0[w.bb + ib[toi_b]] = pc[toi_b]; w.B.b_a0[w.bb + ib[toi_b]] = pa[toi_b];
    for (int k = 0; k < nci; ++k) {
        int la = idx[k][0], lb = idx[k][1];
        init_velocity(ks[k], pc[la], pa[la], pc[lb], pa[lb], vv[la], ww[la], vv[lb], ww[lb]);
        if (ev && ev->rec) {   // step record: the sub-step's set-up decisions
            const int bits = rec_setup_bits(ks[k].dec, GB_REC_SETUP_SHIFT + 2);
            if (w.btype(ib[la]) != GB_BODY_STATIC) ev->rec[ib[la]] ^= bits;
            if (w.btype(ib[lb]) != GB_BODY_STATIC) ev->rec[ib[lb]] ^= bits;
        }
    }
    for (int it = 0; it < vel_iters; ++it)
        for (int k = 0; k < nci; ++k) {
            int la = idx[k][0], lb = idx[k][1];
            vec2<R> va = vv[la], vb = vv[lb];
            R wa = ww[la], wb = ww[lb];
            solve_velocity(ks[k], va, wa, vb, wb);
            vv[la] = va; ww[la] = wa;
            vv[lb] = vb; ww[lb] = wb;
        }
    if (ev && ev->on)   // island.py:243 report of the sub-step's impulses
        for (int k = 0; k < nci; ++k) record_event<R>(w, *ev, GB_EV_POST_SOLVE, ic[k], -1, ks[k].npts, ks[k].ni, ks[k].ti);
    const R dtr = (R)sub_dt;
    for (int i = 0; i < nbi; ++i) {
        vec2<R> v = vv[i];
        R om = ww[i];
        vec2<R> tr = dtr * v;
        if (len2(tr) > (R)GB_MAX_TRANSLATION_SQR) {
            R ratio = (R)GB_MAX_TRANSLATION / len(tr);
            v = ratio * v;
        }
        R rotation = dtr * om;
        if (sq(rotation) > (R)GB_MAX_ROTATION_SQR) {
            R ratio = (R)GB_MAX_ROTATION / fabs(rotation);
            om = om * ratio;
        }
        int g = w.bb + ib[i];
        if (w.btype(ib[i]) != GB_BODY_STATIC) {
            const vec2<double> cn = pc[i] + cvt<double>(dtr * v);
            const double an = pa[i] + (double)(dtr * om);
            w.B.b_c[g] = cn;
            w.B.b_a[g] = an;
            w.B.b_v[g] = v; w.B.b_w[g] = om;
            sync_transform(w, ib[i]);
            if (!(finite_bits(cn.x) && finite_bits(cn.y) && finite_bits(an) && finite_bits(v.x) && finite_bits(v.y) &&
                  finite_bits(om)))
                atomicOr(&w.H->status, GB_ST_NONFINITE);
        }
    }
    if (ck) ck->mark(21);
}

// One TOI event (world.py:693-817) on rank 0.  Appends the re-fattened
// proxies to the move buffer (sh->nmove).
// la/lb: the contacts of the TOI contact's bodies A and B in list order
// (Body._contacts).  The island bodies are left in s_stack[0..sh->nisland)
// with their s_bvis marks set; the caller invalidates and clears them.
template <class R> __device__ void toi_event(const WView<R> &w, int mi, double min_alpha, double dt, int vel_iters, WShared *sh,
                                             const int *la, int na, const int *lb, int nlb, const EvCtx *ev = nullptr,
                                             PhaseClock *ck = nullptr) {
    ContactRec<R> &mc = w.con(mi);
    unsigned char *bflag = w.B.s_bvis + w.bb;
    int bia = w.fbody(mc.fa), bib = w.fbody(mc.fb);
    Sweep back_a = w.sweep(bia), back_b = w.sweep(bib);
    body_advance(w, bia, min_alpha);
    body_advance(w, bib, min_alpha);
    contact_update(w, mi, ev, -1);
    mc.flags &= ~GB_C_TOI;
    mc.toi_count += 1;
    sh->nisland = 0;
    if (!(mc.flags & GB_C_ENABLED) || !(mc.flags & GB_C_TOUCHING)) {
        mc.flags &= ~GB_C_ENABLED;
        w.put_sweep(bia, back_a); w.put_sweep(bib, back_b);
        sync_transform(w, bia); sync_transform(w, bib);
        return;
    }
    wake_body(w, bia); wake_body(w, bib);
    int ib[2 * GB_MAX_TOI_CONTACTS], ic[GB_MAX_TOI_CONTACTS];
    int nbi = 0, nci = 0;
    ib[nbi++] = bia; ib[nbi++] = bib;
    ic[nci++] = mi;
    bflag[bia] = 1; bflag[bib] = 1;
    mc.flags |= GB_C_ISLAND;
    int dyn[2], nd = 0;
    if (w.btype(bia) == GB_BODY_DYNAMIC) dyn[nd++] = bia;
    if (w.btype(bib) == GB_BODY_DYNAMIC) dyn[nd++] = bib;
    for (int di = 0; di < nd; ++di) {
        int bi = dyn[di];
        bool bullet = (w.B.b_flags[w.bb + bi] & GB_BODY_BULLET) != 0;
        const int *lst = (bi == bia) ? la : lb;
        const int nl = (bi == bia) ? na : nlb;
        for (int li = 0; li < nl; ++li) {   // Body._contacts in contact-list order
            int ci = lst[li];
            ContactRec<R> &c = w.con(ci);
            int fa = w.fbody(c.fa), fbb = w.fbody(c.fb);
            if (nbi == 2 * GB_MAX_TOI_CONTACTS || nci == GB_MAX_TOI_CONTACTS) { w.H->status |= GB_ST_TOI_ISLAND_CAP; break; }
            if (c.flags & GB_C_ISLAND) continue;
            int oi = (fa == bi) ? fbb : fa;
            if (w.btype(oi) == GB_BODY_DYNAMIC && !bullet && !(w.B.b_flags[w.bb + oi] & GB_BODY_BULLET)) continue;
            if (fx_sensor(w, c.fa) || fx_sensor(w, c.fb)) continue;
            Sweep backup = w.sweep(oi);
            if (!bflag[oi]) body_advance(w, oi, min_alpha);
            contact_update(w, ci, ev, -1);
            if (!(c.flags & GB_C_ENABLED) || !(c.flags & GB_C_TOUCHING)) {
                w.put_sweep(oi, backup);
                sync_transform(w, oi);
                continue;
            }
            c.flags |= GB_C_ISLAND;
            ic[nci++] = ci;
            if (bflag[oi]) continue;
            bflag[oi] = 1;
            if (w.btype(oi) != GB_BODY_STATIC) wake_body(w, oi);
            ib[nbi++] = oi;
        }
    }
    double sub_dt = (1.0 - min_alpha) * dt;
    if (ck) ck->mark(19);
    island_solve_toi(w, ib, nbi, ic, nci, sub_dt, vel_iters, 0, 1, ev, ck);
    int *mv = w.B.s_move + w.fb;
    for (int i = 0; i < nbi; ++i) {
        int bi = ib[i];
        if (w.btype(bi) == GB_BODY_DYNAMIC) {
            int fs = w.B.b_fstart[w.bb + bi], fcn = w.B.b_fcount[w.bb + bi];
            for (int f = fs; f < fs + fcn; ++f)
                if (sync_fixture(w, f)) {
                    if (sh->nmove < w.H->nf) mv[sh->nmove++] = f;
                    else w.H->status |= GB_ST_PAIR_OVERFLOW;
                }
        }
    }
    int *isl = w.B.s_stack + w.bb;
    for (int i = 0; i < nbi; ++i) isl[i] = ib[i];
    sh->nisland = nbi;
    if (ck) ck->mark(22);
}

// world.py:599-609 reset of the TOI state of one contact
template <class R> __device__ __forceinline__ void toi_reset_contact(const WView<R> &w, int i) {
    ContactRec<R> &c = w.con(i);
    c.flags &= ~(GB_C_TOI | GB_C_ISLAND);
    c.toi_count = 0;
    c.toi = 1.0;
}

// First pass of the TOI loop for contact i (every sweep at alpha0 = 0, so
// contacts are independent): proc = whether the contact takes part.
template <class R> __device__ __forceinline__ void toi_first_pass_contact(const WView<R> &w, int i, int *proc) {
    proc[i] = toi_of_contact(w, i) ? 1 : 0;
}

// The contacts of dynamic body b in list order (Body._contacts): its
// adjacency entries from the start of the loop, then the contacts created
// since (indices >= nc0).  Calls fn(contact) in that order.
template <class R, class F> __device__ __forceinline__ void body_contacts(const WView<R> &w, const int *off, const int *adj,
                                                                         int nc0, int nc, int b, F fn) {
    for (int e = off[b]; e < off[b + 1]; ++e) fn(adj[e]);
    for (int i = nc0; i < nc; ++i) {
        const ContactRec<R> &c = w.con(i);
        if (w.fbody(c.fa) == b || w.fbody(c.fb) == b) fn(i);
    }
}

// Hash set of the world's contact pairs (unordered fixture pairs), open
// addressing; the TOI loop keeps one for its whole run.
static __device__ __forceinline__ unsigned long long pair_key(int p, int q) {
    return (((unsigned long long)(unsigned)min(p, q) << 32) | (unsigned)max(p, q)) + 1ull;
}
static __device__ __forceinline__ bool pair_hash_has(const unsigned long long *hash, int hmask, int p, int q) {
    const unsigned long long key = pair_key(p, q);
    unsigned h = (unsigned)((key * 0x9E3779B97F4A7C15ull) >> 32) & hmask;
    for (int probe = 0; probe <= hmask; ++probe) {
        unsigned long long k = hash[h];
        if (k == key) return true;
        if (k == 0ull) return false;
        h = (h + 1) & hmask;
    }
    return false;
}
static __device__ __forceinline__ void pair_hash_put(unsigned long long *hash, int hmask, int p, int q) {
    const unsigned long long key = pair_key(p, q);
    unsigned h = (unsigned)((key * 0x9E3779B97F4A7C15ull) >> 32) & hmask;
    for (int probe = 0; probe <= hmask; ++probe) {
        unsigned long long prev = atomicCAS(&hash[h], 0ull, key);
        if (prev == 0ull || prev == key) return;
        h = (h + 1) & hmask;
    }
}

// Pair finding after a TOI event (broadphase.py:83-109 +
// contact_manager.py:102-158 for the few proxies the event re-fattened):
// every (moved proxy, proxy) pair is tested in parallel, existing pairs come
// from the loop's pair hash, and each moved proxy's new pairs are sorted by
// the other proxy's index -- the pairs and the order of find_new_contacts,
// without its passes over every contact and proxy of the world.
// Slots for a pair hash of n contacts: a power of two of at least 2 (n + 64),
// at most the largest power of two in the world's 4 x ccap scratch slots.
template <class R> __device__ __forceinline__ int pair_hash_cap(const WView<R> &w, int n) {
    int hmax = 16;
    while (2 * hmax <= 4 * w.H->ccap) hmax <<= 1;
    int hcap = 16;
    while (hcap < 2 * (n + 64) && hcap < hmax) hcap <<= 1;
    return hcap;
}
// (Re)build the loop's pair hash over contacts [0, nc).
template <class R, class G> __device__ void build_loop_hash(const G &g, const WView<R> &w, WShared *sh, unsigned long long *hash, int nc,
                                                            int n_expected) {
    const int hcap = pair_hash_cap(w, n_expected);
    for (int k = g.rank(); k < hcap; k += g.size()) hash[k] = 0ull;
    g.sync();
    for (int i = g.rank(); i < nc; i += g.size()) pair_hash_put(hash, hcap - 1, w.con(i).fa, w.con(i).fb);
    if (g.rank() == 0) sh->lhcap = hcap;
    g.sync();
}

template <class R, class G> __device__ void toi_find_pairs(const G &g, const WView<R> &w, WShared *sh, unsigned long long *hash) {
    const int nmove = sh->nmove;
    if (nmove == 0) return;
    int hmask = sh->lhcap - 1;
    const int nf = w.H->nf;
    const int *mv = w.B.s_move + w.fb;
    int *cnt = w.B.s_cnt + w.fb;      // new pairs per move-buffer entry, then their start
    int *cur = w.B.s_first + w.fb;    // fill counters
    int *pq = w.B.s_colour + w.cb;    // other proxy of new pair t (free during the TOI loop)
    int *pp = w.B.s_order + w.cb;     // moved proxy of new pair t
    const int nc = w.H->nc, ccap = w.H->ccap, room = ccap - nc;
    for (int i = g.rank(); i < nmove; i += g.size()) { cnt[i] = 0; cur[i] = 0; }
    g.sync();
    auto earlier = [&](int i, int f) {
        for (int j = 0; j < i; ++j)
            if (mv[j] == f) return true;
        return false;
    };
    auto new_pair = [&](int i, int q) -> bool {
        const int p = mv[i];
        if (q == p || earlier(i, q)) return false;   // a proxy moved earlier made this pair
        if (!aabb_overlap(w.B.f_aabb[w.fb + q], w.B.f_aabb[w.fb + p])) return false;
        const int ba = w.fbody(p), bb = w.fbody(q);
        if (ba == bb) return false;
        if (!(w.B.b_flags[w.bb + ba] & w.B.b_flags[w.bb + bb] & GB_BODY_ACTIVE)) return false;   // no proxy
        if (pair_hash_has(hash, hmask, p, q)) return false;
        if (!should_collide(w, bb, ba)) return false;
        if (!pair_filter(w, p, q)) return false;
        bool prim;
        return pair_registered(w.B.f_type[w.fb + p], w.B.f_type[w.fb + q], &prim);
    };
    const long long items = (long long)nmove * nf;
    for (long long t = g.rank(); t < items; t += g.size()) {
        const int i = (int)(t / nf), q = (int)(t - (long long)i * nf);
        if (!earlier(i, mv[i]) && new_pair(i, q)) atomicAdd(&cnt[i], 1);
    }
    g.sync();
    if (g.rank() == 0) {
        int acc = 0;
        for (int i = 0; i < nmove; ++i) { int c = cnt[i]; cnt[i] = acc; acc += c; }
        sh->red = (unsigned long long)acc;
    }
    g.sync();
    const int total = (int)sh->red;
    for (long long t = g.rank(); t < items; t += g.size()) {
        const int i = (int)(t / nf), q = (int)(t - (long long)i * nf);
        if (!earlier(i, mv[i]) && new_pair(i, q)) {
            const int k = cnt[i] + atomicAdd(&cur[i], 1);
            if (k < room) { pq[k] = q; pp[k] = mv[i]; }
        }
    }
    g.sync();
    for (int i = g.rank(); i < nmove; i += g.size()) {   // by the other proxy's index
        const int b0 = cnt[i], b1 = min(b0 + cur[i], room);
        for (int a = b0 + 1; a < b1; ++a) {
            int v = pq[a], b = a - 1;
            while (b >= b0 && pq[b] > v) { pq[b + 1] = pq[b]; --b; }
            pq[b + 1] = v;
        }
    }
    g.sync();
    const int ncreate = total < room ? total : room;
    if (2 * (nc + ncreate) > sh->lhcap) {   // keep the hash at most half full
        build_loop_hash(g, w, sh, hash, nc, 2 * (nc + ncreate));
        hmask = sh->lhcap - 1;
    }
    for (int t = g.rank(); t < ncreate; t += g.size()) {
        const int p = pp[t], q = pq[t];
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
        pair_hash_put(hash, hmask, p, q);
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

// Set-up of the event loop: the per-body adjacency of the dynamic bodies
// (Body._contacts in list order), the loop's pair hash over every contact
// and the candidate list in list order.  Returns the number of candidates;
// the hash's slot count is left in sh->lhcap.  Run by the loop itself, or
// ahead of it by a wider group (the set-up kernel), whose results the loop
// then reads (WorldHdr::toi_ready).
template <class R, class G> __device__ int toi_setup(const G &g, const WView<R> &w, WShared *sh) {
    int *ids = w.B.s_pref + w.cb;
    int *cand = w.B.s_cons_of + w.cb;
    int *off = w.B.s_adjoff + w.bb + w.wi;
    int *adj = reinterpret_cast<int *>(w.B.s_kb + w.cb);
    int *cursor = w.B.s_seed + w.bb;
    const int nb = w.H->nb;
    const int nc0 = w.H->nc;
    // adjacency: count, scan, scatter, sort each body's entries by index
    for (int b = g.rank(); b < nb; b += g.size()) cursor[b] = 0;
    g.sync();
    for (int i = g.rank(); i < nc0; i += g.size()) {
        const ContactRec<R> &c = w.con(i);
        int ba = w.fbody(c.fa), bb = w.fbody(c.fb);
        if (w.btype(ba) == GB_BODY_DYNAMIC) atomicAdd(&cursor[ba], 1);
        if (w.btype(bb) == GB_BODY_DYNAMIC) atomicAdd(&cursor[bb], 1);
    }
    g.sync();
    int tot = group_scan(g, nb, [&](int b) { return cursor[b]; }, off);
    g.sync();
    if (g.rank() == 0) off[nb] = tot;
    for (int b = g.rank(); b < nb; b += g.size()) cursor[b] = off[b];
    g.sync();
    for (int i = g.rank(); i < nc0; i += g.size()) {
        const ContactRec<R> &c = w.con(i);
        int ba = w.fbody(c.fa), bb = w.fbody(c.fb);
        if (w.btype(ba) == GB_BODY_DYNAMIC) adj[atomicAdd(&cursor[ba], 1)] = i;
        if (w.btype(bb) == GB_BODY_DYNAMIC) adj[atomicAdd(&cursor[bb], 1)] = i;
    }
    g.sync();
    for (int b = g.rank(); b < nb; b += g.size())
        for (int e = off[b] + 1; e < off[b + 1]; ++e) {
            int v = adj[e], j = e - 1;
            while (j >= off[b] && adj[j] > v) { adj[j + 1] = adj[j]; --j; }
            adj[j + 1] = v;
        }
    // the pair hash of the loop (every contact, then those events create)
    unsigned long long *lhash = w.B.s_hash + 4 * (size_t)w.cb;
    build_loop_hash(g, w, sh, lhash, nc0, nc0);
    // candidates in list order
    int ncand = group_scan(g, nc0, [&](int i) { return (w.con(i).flags & GB_C_TOI_CAND) ? 1 : 0; }, ids);
    g.sync();
    for (int i = g.rank(); i < nc0; i += g.size())
        if (w.con(i).flags & GB_C_TOI_CAND) cand[ids[i]] = i;
    g.sync();
    return ncand;
}

// The event loop of world.py:612-821; `first_done` means pass 0 already ran
// (in the batch-wide kernel).  Passes scan the candidate list only, and the
// contact lists of the event bodies come from a per-body adjacency built
// once per step.
template <class R, class G> __device__ void toi_loop(const G &g, const WView<R> &w, const StepParams &sp, WShared *sh,
                                                     bool par_first, bool first_done, PhaseClock *pc = nullptr) {
    PhaseClock dummy;
    dummy.acc = nullptr;
    PhaseClock &ck = pc ? *pc : dummy;
    int *proc = w.B.s_proc + w.cb;
    int *ids = w.B.s_pref + w.cb;
    TPlan *plan = w.B.s_plan + (size_t)w.wi * GB_TOI_PLAN_CAP;
    unsigned char *bflag = w.B.s_bvis + w.bb;
    int *cand = w.B.s_cons_of + w.cb;                          // candidate contacts, list order
    int *off = w.B.s_adjoff + w.bb + w.wi;                     // adjacency of dynamic bodies (nb + 1)
    int *adj = reinterpret_cast<int *>(w.B.s_kb + w.cb);       // 2 ccap entries
    const int nc0 = w.H->nc;
    unsigned long long *lhash = w.B.s_hash + 4 * (size_t)w.cb;
    int ncand;
    if (w.H->toi_ready) {   // made by the set-up kernel
        ncand = w.H->toi_ncand;
        if (g.rank() == 0) sh->lhcap = w.H->toi_hcap;
        g.sync();
    } else {
        ncand = toi_setup(g, w, sh);
    }
    if (g.rank() == 0) ck.mark(11);
    for (int pass = 0; pass < (1 << 20); ++pass) {
        const int nc = w.H->nc;
        if (pass == 0 && first_done) {
            // computed by the batch-wide first pass
        } else if (pass == 0 && par_first) {
            for (int k = g.rank(); k < ncand; k += g.size()) proc[cand[k]] = toi_of_contact(w, cand[k]) ? 1 : 0;
        } else {
            // statuses in parallel; the contacts needing a fresh TOI in list order
            int nfresh = group_scan(g, ncand, [&](int k) {
                int i = cand[k];
                int st = toi_status(w, i);
                proc[i] = st != 0 ? 1 : 0;
                return st == 2 ? 1 : 0;
            }, ids);
            g.sync();
            if (g.rank() == 0) { ck.mark(16); if (ck.acc) ck.acc[23] += nfresh; }
            if (nfresh > 0) {
                int *fresh = w.B.s_adj + 2 * (size_t)w.cb;   // free during the TOI loop
                for (int k = g.rank(); k < ncand; k += g.size()) {
                    int i = cand[k];
                    if (proc[i] && !(w.con(i).flags & GB_C_TOI)) fresh[ids[k]] = i;
                }
                g.sync();
                if (nfresh <= GB_TOI_PLAN_CAP) {
                    // the sweep alignment is order dependent and cheap: rank 0 replays
                    // it in list order; the float64 TOIs then run in parallel
                    if (g.rank() == 0)
                        for (int k = 0; k < nfresh; ++k) plan[k].alpha0 = toi_align(w, fresh[k], &plan[k].sa, &plan[k].sb);
                    g.sync();
                    if (g.rank() == 0) ck.mark(17);
                    for (int k = g.rank(); k < nfresh; k += g.size()) toi_compute(w, fresh[k], plan[k].alpha0, plan[k].sa, plan[k].sb);
                    g.sync();
                    if (g.rank() == 0) ck.mark(18);
                } else if (g.rank() == 0) {
                    for (int k = 0; k < nfresh; ++k) {
                        Sweep sa, sb;
                        double a0 = toi_align(w, fresh[k], &sa, &sb);
                        toi_compute(w, fresh[k], a0, sa, sb);
                    }
                }
            }
        }
        g.sync();
        if (g.rank() == 0) ck.mark(11);
        // earliest event: lexicographic minimum of (toi, list position)
        unsigned long long key = ~0ull;
        int mi = GB_INF_IDX;
        for (int k = g.rank(); k < ncand; k += g.size()) {
            int i = cand[k];
            double t = w.con(i).toi;
            if (proc[i] && t < 1.0) {
                unsigned long long kk = dkey(t);
                if (kk < key || (kk == key && i < mi)) { key = kk; mi = i; }
            }
        }
        g.argmin(key, mi);
        const double min_alpha = mi == GB_INF_IDX ? 1.0 : dkey_inv(key);
        if (mi == GB_INF_IDX || (1.0 - (10.0 * GB_EPSILON)) < min_alpha) {
            if (g.rank() == 0) w.H->flags |= GB_W_STEP_COMPLETE;
            g.sync();
            break;
        }
        // contact lists of the event's two bodies (Body._contacts)
        const ContactRec<R> &mc = w.con(mi);
        const int bia = w.fbody(mc.fa), bib = w.fbody(mc.fb);
        int *la = w.B.s_adj + 2 * (size_t)w.cb;
        int *lb = la + w.H->ccap;
        if (g.rank() == 0) {
            ck.mark(12);
            int na = 0, nlb = 0;
            if (w.btype(bia) == GB_BODY_DYNAMIC) body_contacts(w, off, adj, nc0, nc, bia, [&](int i) { la[na++] = i; });
            if (w.btype(bib) == GB_BODY_DYNAMIC) body_contacts(w, off, adj, nc0, nc, bib, [&](int i) { lb[nlb++] = i; });
            sh->nmove = 0;
            const EvCtx ev{sp.events, sp.step_index, GB_EV_PHASE_TOI, sp.record_order ? w.B.rec + w.bb : nullptr};
            toi_event(w, mi, min_alpha, sp.dt, sp.vel_iters, sh, la, na, lb, nlb, &ev, &ck);
            ck.mark(13);
        }
        g.sync();
        // invalidate the TOIs of every contact of a displaced dynamic body and
        // clear the island marks (world.py:804-813)
        const int nisl = sh->nisland;
        const int *isl = w.B.s_stack + w.bb;
        for (int k = g.rank(); k < nisl; k += g.size()) {
            int b = isl[k];
            if (w.btype(b) != GB_BODY_DYNAMIC) continue;
            body_contacts(w, off, adj, nc0, nc, b, [&](int i) { atomicAnd(&w.con(i).flags, ~(GB_C_TOI | GB_C_ISLAND)); });
        }
        g.sync();
        for (int k = g.rank(); k < nisl; k += g.size()) bflag[isl[k]] = 0;
        g.sync();
        toi_find_pairs(g, w, sh, lhash);
        // new contacts join the candidate list (they follow every older one)
        const int nc2 = w.H->nc;
        if (nc2 > nc) {
            int nnew = group_scan(g, nc2 - nc, [&](int k) { return (w.con(nc + k).flags & GB_C_TOI_CAND) ? 1 : 0; }, ids);
            g.sync();
            for (int k = g.rank(); k < nc2 - nc; k += g.size())
                if (w.con(nc + k).flags & GB_C_TOI_CAND) { cand[ncand + ids[k]] = nc + k; proc[nc + k] = 0; }
            ncand += nnew;
            g.sync();
        }
        if (g.rank() == 0) { ck.mark(14); if (ck.acc) ck.acc[15] += 1; }
    }
}

template <class R, class G> __device__ void world_solve_toi(const G &g, const WView<R> &w, const StepParams &sp, WShared *sh) {
    const int nb = w.H->nb;
    // every sweep starts at alpha0 = 0 after a complete step, so the first
    // pass advances no sweep and may run in parallel
    const bool par_first = (w.H->flags & GB_W_STEP_COMPLETE) != 0;
    if (w.H->flags & GB_W_STEP_COMPLETE) {
        for (int b = g.rank(); b < nb; b += g.size()) { w.B.b_alpha0[w.bb + b] = 0.0; w.B.s_bvis[w.bb + b] = 0; }
        for (int i = g.rank(); i < w.H->nc; i += g.size()) toi_reset_contact(w, i);
    }
    g.sync();
    toi_loop(g, w, sp, sh, par_first, false);
}

template <class R, class G> __device__ void world_step(const G &g, const WView<R> &w, StepParams sp, WShared *sh) {
    PhaseClock pc;
    pc.acc = (sp.profile && g.rank() == 0) ? w.B.prof + (size_t)w.wi * GB_NPROF : nullptr;
    pc.start();
    if (sp.record_order)
        for (int b = g.rank(); b < w.H->nb; b += g.size()) { w.B.rec[w.bb + b] = 0; w.B.rec_island[w.bb + b] = -1; }
    if (w.H->flags & GB_W_NEW_FIXTURE) {
        int nf = w.H->nf;
        int n0 = w.H->nmove0;
        if (n0 == 0)
            for (int f = g.rank(); f < nf; f += g.size()) w.B.s_move[w.fb + f] = f;
        g.sync();
        if (g.rank() == 0) { sh->nmove = n0 ? n0 : nf; w.H->nmove0 = 0; }
        g.sync();
        find_new_contacts(g, w, sh);
        if (g.rank() == 0) w.H->flags &= ~GB_W_NEW_FIXTURE;
        g.sync();
    }
    sp.dt_ratio = w.H->inv_dt0 * sp.dt;
    pc.mark(0);
    collide(g, w, sp);
    pc.mark(1);
    if ((w.H->flags & GB_W_STEP_COMPLETE) && sp.dt > 0.0) world_solve(g, w, sp, sh, pc);
    if ((w.H->flags & GB_W_CONTINUOUS) && sp.dt > 0.0) world_solve_toi(g, w, sp, sh);
    g.sync();
    pc.mark(9);
    if (g.rank() == 0 && sp.dt > 0.0) w.H->inv_dt0 = sp.inv_dt;
    if (w.H->flags & GB_W_AUTO_CLEAR_FORCES)
        for (int b = g.rank(); b < w.H->nb; b += g.size()) {
            w.B.b_f[w.bb + b] = mk<R>(0, 0);
            w.B.b_torque[w.bb + b] = (R)0;
        }
    g.sync();
    pc.mark(10);
}

// ---------------------------------------------------------------- kernels
// One CTA per world; worlds[] lists the worlds of this launch (largest
// first, so the longest worlds start first).
template <class R> __global__ void k_step_cta(Batch<R> B, StepParams sp, int n_steps, const int *worlds) {
    __shared__ int sm[96];
    __shared__ WorldHdr H;
    __shared__ WShared sh;
    const int wi = worlds[blockIdx.x];
    if (threadIdx.x == 0) { H = B.hdr[wi]; sh.nmove = 0; }
    __syncthreads();
    GroupCta g{sm};
    WView<R> w{B, &H, H.bbase, H.fbase, H.cbase, wi};
    for (int s = 0; s < n_steps; ++s) {
        StepParams q = sp;
        q.step_index = s;
        world_step(g, w, q, &sh);
    }
    __syncthreads();
    if (threadIdx.x == 0) B.hdr[wi] = H;
}

// One warp per world (worlds_per_cta = blockDim.x / 32).
template <class R> __global__ void k_step_warp(Batch<R> B, StepParams sp, int n_steps, const int *worlds, int n_list) {
    __shared__ int sm[32][8];
    __shared__ WorldHdr H[32];
    __shared__ WShared sh[32];
    const int lw = threadIdx.x >> 5;
    const int li = blockIdx.x * (blockDim.x >> 5) + lw;
    if (li >= n_list) return;
    const int wi = worlds[li];
    if ((threadIdx.x & 31) == 0) { H[lw] = B.hdr[wi]; sh[lw].nmove = 0; }
    __syncwarp();
    GroupWarp g{sm[lw]};
    WView<R> w{B, &H[lw], H[lw].bbase, H[lw].fbase, H[lw].cbase, wi};
    for (int s = 0; s < n_steps; ++s) {
        StepParams q = sp;
        q.step_index = s;
        world_step(g, w, q, &sh[lw]);
    }
    __syncwarp();
    if ((threadIdx.x & 31) == 0) B.hdr[wi] = H[lw];
}

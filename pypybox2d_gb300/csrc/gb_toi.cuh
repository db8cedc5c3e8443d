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

// world.py:617-686 for one contact: its cached or freshly computed TOI.
// Returns false when the contact is skipped (sensor, inactive, no bullet).
template <class R> __device__ bool toi_of_contact(const WView<R> &w, int i, double *alpha_out) {
    ContactRec<R> &c = w.con(i);
    if (c.flags & GB_C_TOI) { *alpha_out = c.toi; return true; }
    if (fx_sensor(w, c.fa) || fx_sensor(w, c.fb)) return false;
    int ba = w.fbody(c.fa), bb = w.fbody(c.fb);
    int ta = w.btype(ba), tb = w.btype(bb);
    bool act_a = w.awake(ba) && ta != GB_BODY_STATIC;
    bool act_b = w.awake(bb) && tb != GB_BODY_STATIC;
    if (!act_a && !act_b) return false;
    bool col_a = (w.B.b_flags[w.bb + ba] & GB_BODY_BULLET) || ta != GB_BODY_DYNAMIC;
    bool col_b = (w.B.b_flags[w.bb + bb] & GB_BODY_BULLET) || tb != GB_BODY_DYNAMIC;
    if (!col_a && !col_b) return false;
    double al_a = w.B.b_alpha0[w.bb + ba], al_b = w.B.b_alpha0[w.bb + bb];
    double alpha0 = al_a;
    if (al_a < al_b) {
        alpha0 = al_b;
        Sweep s = w.sweep(ba); sweep_advance(s, alpha0); w.put_sweep(ba, s);
    } else if (al_b < al_a) {
        Sweep s = w.sweep(bb); sweep_advance(s, alpha0); w.put_sweep(bb, s);
    }
    DProxy pa, pb;
    dproxy_init(pa, w.shape(c.fa));
    dproxy_init(pb, w.shape(c.fb));
    Sweep sa = w.sweep(ba), sb = w.sweep(bb);
    double beta;
    bool lim = false;
    int state = time_of_impact(pa, pb, sa, sb, 1.0, &beta, &lim);
    if (lim) w.H->status |= GB_ST_ITER_LIMIT;
    double alpha = (state == TOI_TOUCHING) ? pymin(alpha0 + (1.0 - alpha0) * beta, 1.0) : 1.0;
    c.toi = alpha;
    c.flags |= GB_C_TOI;
    *alpha_out = alpha;
    return true;
}

// island.py:181-243 Island.solve_toi on rank 0 (island of at most 64
// bodies and 32 contacts).
template <class R> __device__ void island_solve_toi(const WView<R> &w, const int *ib, int nbi, const int *ic, int nci,
                                                    double sub_dt, int vel_iters, int toi_a, int toi_b) {
    vec2<double> pc[2 * GB_MAX_TOI_CONTACTS];
    double pa[2 * GB_MAX_TOI_CONTACTS];
    vec2<R> vv[2 * GB_MAX_TOI_CONTACTS];
    R ww[2 * GB_MAX_TOI_CONTACTS];
    int idx[2 * GB_MAX_TOI_CONTACTS][2];
    Cons<R> *ks = w.B.s_cons + w.cb;
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
    for (int it = 0; it < 20; ++it) {
        double minsep = 0.0;
        for (int k = 0; k < nci; ++k) {
            int la = idx[k][0], lb = idx[k][1];
            minsep = solve_position(ks[k], pc[la], pa[la], pc[lb], pa[lb], minsep, true,
                                    la == toi_a || la == toi_b, lb == toi_a || lb == toi_b);
        }
        if (minsep >= -1.5 * GB_LINEAR_SLOP) break;
    }
    w.B.b_c0[w.bb + ib[toi_a]] = pc[toi_a]; w.B.b_a0[w.bb + ib[toi_a]] = pa[toi_a];
    w.B.b_c0[w.bb + ib[toi_b]] = pc[toi_b]; w.B.b_a0[w.bb + ib[toi_b]] = pa[toi_b];
    for (int k = 0; k < nci; ++k) {
        int la = idx[k][0], lb = idx[k][1];
        init_velocity(ks[k], pc[la], pa[la], pc[lb], pa[lb], vv[la], ww[la], vv[lb], ww[lb]);
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
            w.B.b_c[g] = pc[i] + cvt<double>(dtr * v);
            w.B.b_a[g] = pa[i] + (double)(dtr * om);
            w.B.b_v[g] = v; w.B.b_w[g] = om;
            sync_transform(w, ib[i]);
        }
    }
}

// One TOI event (world.py:693-817) on rank 0.  Appends the re-fattened
// proxies to the move buffer (sh->nmove).
template <class R> __device__ void toi_event(const WView<R> &w, int mi, double min_alpha, double dt, int vel_iters, WShared *sh) {
    ContactRec<R> &mc = w.con(mi);
    unsigned char *bflag = w.B.s_bvis + w.bb;
    int bia = w.fbody(mc.fa), bib = w.fbody(mc.fb);
    Sweep back_a = w.sweep(bia), back_b = w.sweep(bib);
    body_advance(w, bia, min_alpha);
    body_advance(w, bib, min_alpha);
    contact_update(w, mi);
    mc.flags &= ~GB_C_TOI;
    mc.toi_count += 1;
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
    const int nc = w.H->nc;
    for (int di = 0; di < nd; ++di) {
        int bi = dyn[di];
        bool bullet = (w.B.b_flags[w.bb + bi] & GB_BODY_BULLET) != 0;
        for (int ci = 0; ci < nc; ++ci) {   // Body._contacts in contact-list order
            ContactRec<R> &c = w.con(ci);
            int fa = w.fbody(c.fa), fbb = w.fbody(c.fb);
            if (fa != bi && fbb != bi) continue;
            if (nbi == 2 * GB_MAX_TOI_CONTACTS || nci == GB_MAX_TOI_CONTACTS) { w.H->status |= GB_ST_TOI_ISLAND_CAP; break; }
            if (c.flags & GB_C_ISLAND) continue;
            int oi = (fa == bi) ? fbb : fa;
            if (w.btype(oi) == GB_BODY_DYNAMIC && !bullet && !(w.B.b_flags[w.bb + oi] & GB_BODY_BULLET)) continue;
            if (fx_sensor(w, c.fa) || fx_sensor(w, c.fb)) continue;
            Sweep backup = w.sweep(oi);
            if (!bflag[oi]) body_advance(w, oi, min_alpha);
            contact_update(w, ci);
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
    island_solve_toi(w, ib, nbi, ic, nci, sub_dt, vel_iters, 0, 1);
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
    // invalidate the TOIs of every contact of a displaced dynamic body
    for (int ci = 0; ci < nc; ++ci) {
        ContactRec<R> &c = w.con(ci);
        int fa = w.fbody(c.fa), fbb = w.fbody(c.fb);
        bool hit = (bflag[fa] && w.btype(fa) == GB_BODY_DYNAMIC) || (bflag[fbb] && w.btype(fbb) == GB_BODY_DYNAMIC);
        if (hit) c.flags &= ~(GB_C_TOI | GB_C_ISLAND);
    }
    for (int i = 0; i < nbi; ++i) bflag[ib[i]] = 0;
}

template <class R, class G> __device__ void world_solve_toi(const G &g, const WView<R> &w, const StepParams &sp, WShared *sh) {
    const int nb = w.H->nb;
    int *proc = w.B.s_proc + w.cb;
    // every sweep starts at alpha0 = 0 after a complete step, so the first
    // pass advances no sweep and may run in parallel
    const bool par_first = (w.H->flags & GB_W_STEP_COMPLETE) != 0;
    if (w.H->flags & GB_W_STEP_COMPLETE) {
        for (int b = g.rank(); b < nb; b += g.size()) { w.B.b_alpha0[w.bb + b] = 0.0; w.B.s_bvis[w.bb + b] = 0; }
        for (int i = g.rank(); i < w.H->nc; i += g.size()) {
            ContactRec<R> &c = w.con(i);
            c.flags &= ~(GB_C_TOI | GB_C_ISLAND);
            c.toi_count = 0;
            c.toi = 1.0;
        }
    }
    g.sync();
    unsigned long long *red = &sh->red;
    for (int pass = 0; pass < (1 << 20); ++pass) {
        const int nc = w.H->nc;
        if (pass == 0 && par_first) {
            for (int i = g.rank(); i < nc; i += g.size()) {
                const ContactRec<R> &c = w.con(i);
                double a;
                bool ok = (c.flags & GB_C_ENABLED) && c.toi_count <= GB_MAX_SUB_STEPS && toi_of_contact(w, i, &a);
                proc[i] = ok ? 1 : 0;
            }
        } else if (g.rank() == 0) {
            for (int i = 0; i < nc; ++i) {
                const ContactRec<R> &c = w.con(i);
                double a;
                bool ok = (c.flags & GB_C_ENABLED) && c.toi_count <= GB_MAX_SUB_STEPS && toi_of_contact(w, i, &a);
                proc[i] = ok ? 1 : 0;
            }
        }
        if (g.rank() == 0) { red[0] = dkey(1.0); sh->min_contact = GB_INF_IDX; }
        g.sync();
        for (int i = g.rank(); i < nc; i += g.size())
            if (proc[i] && w.con(i).toi < 1.0) atomicMin(&red[0], dkey(w.con(i).toi));
        g.sync();
        double min_alpha = dkey_inv(red[0]);
        for (int i = g.rank(); i < nc; i += g.size())
            if (proc[i] && w.con(i).toi < 1.0 && w.con(i).toi == min_alpha) atomicMin(&sh->min_contact, i);
        g.sync();
        int mi = sh->min_contact;
        if (mi == GB_INF_IDX || (1.0 - (10.0 * GB_EPSILON)) < min_alpha) {
            if (g.rank() == 0) w.H->flags |= GB_W_STEP_COMPLETE;
            g.sync();
            break;
        }
        if (g.rank() == 0) {
            sh->nmove = 0;
            toi_event(w, mi, min_alpha, sp.dt, sp.vel_iters, sh);
        }
        g.sync();
        find_new_contacts(g, w, sh);
    }
}

template <class R, class G> __device__ void world_step(const G &g, const WView<R> &w, StepParams sp, WShared *sh) {
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
    collide(g, w);
    if ((w.H->flags & GB_W_STEP_COMPLETE) && sp.dt > 0.0) world_solve(g, w, sp, sh);
    if ((w.H->flags & GB_W_CONTINUOUS) && sp.dt > 0.0) world_solve_toi(g, w, sp, sh);
    g.sync();
    if (g.rank() == 0 && sp.dt > 0.0) w.H->inv_dt0 = sp.inv_dt;
    if (w.H->flags & GB_W_AUTO_CLEAR_FORCES)
        for (int b = g.rank(); b < w.H->nb; b += g.size()) {
            w.B.b_f[w.bb + b] = mk<R>(0, 0);
            w.B.b_torque[w.bb + b] = (R)0;
        }
    g.sync();
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
    for (int s = 0; s < n_steps; ++s) world_step(g, w, sp, &sh);
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
    for (int s = 0; s < n_steps; ++s) world_step(g, w, sp, &sh[lw]);
    __syncwarp();
    if ((threadIdx.x & 31) == 0) B.hdr[wi] = H[lw];
}

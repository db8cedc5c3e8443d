// gb_phases.cuh -- the batched step as a sequence of phase kernels.
//
// One World.step of every world of the batch is 13 launches (14 with a
// second solver launch; captured once into a CUDA graph and replayed per
// step):
//
//   k_pairs0    per world   pair finding over the pending move buffer (new fixtures)
//   k_pre       per body    collide wake marks, TOI state reset
//   k_collide   per contact narrow phase + warm-start matching of every contact with
//                           an awake non-static body (contact_manager.py:174-223)
//   k_collide2  per world   the same loop for contacts whose bodies were asleep (in
//                           list order, on one thread: wakes propagate forward), wakes,
//                           destruction of non-overlapping contacts
//   k_islands   per world   union-find islands, constraint list, graph colouring
//   k_vinit     per body    velocity integration (island.py:71-95)
//   k_cinit     per constraint  solver set-up (contact.py:375-496)
//   k_solve     per world   warm start, velocity and position iterations, sleep
//   k_pairs     per world   fixture sync and pair finding (world.py:582-592)
//   k_toi1      per contact TOI state reset, candidates of the first pass
//   k_toi1b     per candidate  the first pass's float64 times of impact
//   k_toi_setup per world   the event loop's adjacency, pair hash and candidate list
//   k_toi2      per world   the rest of the event loop (one warp), force clear
//
// "per body / contact / constraint" kernels run one thread per element of
// every world (the 4096-world batch gives ~2.4 M contact threads), "per
// world" kernels one CTA per world.  The order inside each world is the
// monolithic step's, so both give the same doubles.
#pragma once
#include "gb_toi.cuh"

#define P_DEFERRED 1u   // some contact was skipped by k_collide (both bodies asleep)
#define P_WOKE 2u       // k_collide woke a body that was asleep
#define P_DESTROY 4u    // some contact is to be destroyed
#define P_SOLVING 8u    // the island solve runs this step

template <class R> __device__ __forceinline__ WView<R> view_global(const Batch<R> &B, int wi) {
    WorldHdr *H = &B.hdr[wi];
    WView<R> w{B, H, H->bbase, H->fbase, H->cbase, wi};
    return w;
}

template <class R> __global__ void k_pre(Batch<R> B, int n_bodies, StepParams sp) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b == 0) *B.toi_n = 0;
    if (b >= n_bodies) return;
    b += B.body0;
    const WorldHdr *H = &B.hdr[B.b_world[b]];
    uint32_t f = B.b_flags[b];
    B.s_wake[b] = ((f & GB_BODY_AWAKE) && B.b_type[b] != GB_BODY_STATIC) ? -1 : GB_INF_IDX;
    if (sp.record_order) { B.rec[b] = 0; B.rec_island[b] = -1; }
    // world.py:599-602 (alpha0 is read by nothing before the TOI loop)
    if ((H->flags & GB_W_CONTINUOUS) && (H->flags & GB_W_STEP_COMPLETE) && sp.dt > 0.0) B.b_alpha0[b] = 0.0;
}

template <class R, bool EV> __global__ void k_collide(Batch<R> B, int n_slots, StepParams sp) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n_slots) return;
    s += B.slot0;
    int wi = B.c_world[s];
    WView<R> w = view_global(B, wi);
    int i = s - w.cb;
    if (i >= w.H->nc) return;
    int *wake = B.s_wake + w.bb;
    bool woke;
    const EvCtx ev{sp.events, sp.step_index, GB_EV_PHASE_UPDATE};
    int r = collide_one<R, EV>(w, i, wake, &woke, &ev);
    B.s_proc[s] = r;
    if (r == 0) { atomicOr(&w.H->pflags, P_DEFERRED); return; }
    if (r == 2) { atomicOr(&w.H->pflags, P_DESTROY); return; }
    if (woke) {
        const ContactRec<R> &c = w.con(i);
        int oa = atomicMin(&wake[w.fbody(c.fa)], i);
        int ob = atomicMin(&wake[w.fbody(c.fb)], i);
        if (oa == GB_INF_IDX || ob == GB_INF_IDX) atomicOr(&w.H->pflags, P_WOKE);
    }
}

template <class R> __global__ void k_vinit(Batch<R> B, int n_bodies, StepParams sp) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n_bodies) return;
    b += B.body0;
    WView<R> w = view_global(B, B.b_world[b]);
    if (!(w.H->pflags & P_SOLVING)) return;
    integrate_velocity_body(w, b - w.bb, sp.dt);
#if defined(GB_POSE_ROT_F32)
    const rot2<float> q = rot_of_f32(B.b_a[b]);
    const vec2<double> c = B.b_c[b];
    B.s_pose[b] = make_float4((float)c.x, (float)c.y, q.c, q.s);
#endif
}

template <class R> __global__ void k_cinit(Batch<R> B, int n_slots, StepParams sp) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n_slots) return;
    s += B.slot0;
    WView<R> w = view_global(B, B.c_world[s]);
    int k = s - w.cb;
    if (!(w.H->pflags & P_SOLVING) || k >= w.H->last_ncons) return;
#if defined(GB_POSE_ROT_F32)
    init_constraint(w, k, sp, true);   // poses from k_vinit (s_pose)
#else
    init_constraint(w, k, sp);
#endif
}

// First TOI pass, part 1: reset every contact's TOI state (world.py:604-609)
// and list the contacts that need a time of impact.  All sweeps start at
// alpha0 = 0, so the listed computations are independent of each other.
template <class R> __global__ void k_toi1(Batch<R> B, int n_slots, StepParams sp) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n_slots) return;
    s += B.slot0;
    WView<R> w = view_global(B, B.c_world[s]);
    int i = s - w.cb;
    if (i >= w.H->nc) return;
    if (!((w.H->flags & GB_W_CONTINUOUS) && sp.dt > 0.0)) return;
    if (!(w.H->flags & GB_W_STEP_COMPLETE)) return;   // k_toi2 then runs the whole loop in order
    ContactRec<R> &c = w.con(i);
    const uint32_t f = c.flags;
    if (!(f & GB_C_TOI_CAND)) {
        // a contact that cannot take part: the same reset, stored only
        // where it changes (most such contacts are already reset)
        if (f & (GB_C_TOI | GB_C_ISLAND)) c.flags = f & ~(GB_C_TOI | GB_C_ISLAND);
        if (c.toi_count != 0) c.toi_count = 0;
        if (__double_as_longlong(c.toi) != __double_as_longlong(1.0)) c.toi = 1.0;
        B.s_proc[s] = 0;
        return;
    }
    toi_reset_contact(w, i);
    int st = toi_status(w, i);
    B.s_proc[s] = st != 0 ? 1 : 0;
    if (st == 2) B.toi_list[B.slot0 + atomicAdd(B.toi_n, 1)] = s;   // the group's part of the list
}

// First TOI pass, part 2: the float64 times of impact of the listed
// contacts, one per thread (dense warps; the list order does not matter).
template <class R> __global__ void k_toi1b(Batch<R> B) {
    const int n = *B.toi_n;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        int s = B.toi_list[B.slot0 + t];
        WView<R> w = view_global(B, B.c_world[s]);
        int i = s - w.cb;
        const ContactRec<R> &c = w.con(i);
        int ba = w.fbody(c.fa), bb = w.fbody(c.fb);
        toi_compute<R, true>(w, i, 0.0, w.sweep(ba), w.sweep(bb));
        const double toi = c.toi;
        if (toi < 1.0) atomicMin(&B.hdr[w.wi].toimin, dkey(toi));
    }
}

// Per-world phases ---------------------------------------------------------
#define PH_PAIRS0 0
#define PH_COLLIDE2 1
#define PH_ISLANDS 2
#define PH_SOLVE 3
#define PH_PAIRS 4
#define PH_TOI2 5
#define PH_TOI1 6   // the event loop's set-up, a CTA per world ahead of the one-warp loop
#define PH_CTL 7    // controllers, launched ahead of PH_ISLANDS only for batches that have some

template <class R, int PH> __device__ __forceinline__ void world_phase(const Batch<R> &B, const StepParams &sp, const int wi);

template <class R, int PH> __global__ void __launch_bounds__(256) k_world(Batch<R> B, StepParams sp, const int *worlds) {
    world_phase<R, PH>(B, sp, worlds[blockIdx.x]);
}

// The TOI event loop is latency bound (float64, mostly one thread): one warp
// per world with a register cap keeps many worlds in flight per SM.
// (Measured on the uneven batch: 16 or 12 resident warps, with up to 128
// and 168 registers, make the slowest world's event chain 10 % longer.)
template <class R> __global__ void __launch_bounds__(32, 24) k_world_toi2(Batch<R> B, StepParams sp, const int *worlds) {
    world_phase<R, PH_TOI2>(B, sp, worlds[blockIdx.x]);
}

template <class R, int PH, class G> __device__ __forceinline__ void phase_body(const Batch<R> &B, const StepParams &sp, const int wi,
                                                                              const G &g, WorldHdr &H, WShared &sh,
                                                                              unsigned char *dyn) {
    WView<R> w{B, &H, H.bbase, H.fbase, H.cbase, wi};
    const bool solving = (H.flags & GB_W_STEP_COMPLETE) && sp.dt > 0.0;
    if (PH == PH_PAIRS0) {
        if (g.rank() == 0) H.pflags = 0;
        if (H.flags & GB_W_NEW_FIXTURE) {
            int nf = H.nf;
            int n0 = H.nmove0;
            if (n0 == 0)
                for (int f = g.rank(); f < nf; f += g.size()) B.s_move[w.fb + f] = f;
            g.sync();
            if (g.rank() == 0) { sh.nmove = n0 ? n0 : nf; H.nmove0 = 0; }
            g.sync();
            find_new_contacts(g, w, &sh);
            if (g.rank() == 0) H.flags &= ~GB_W_NEW_FIXTURE;
        }
    } else if (PH == PH_COLLIDE2) {
        int *wake = B.s_wake + w.bb;
        int *proc = B.s_proc + w.cb;
        uint32_t pf = H.pflags;
        bool woke_any = (pf & P_WOKE) != 0;
        if ((pf & P_DEFERRED) && (pf & P_WOKE)) {
            // contacts between sleeping bodies, in list order: a body woken at
            // position j makes the contacts after j active (sequential rule);
            // the deferred contacts are listed in parallel first
            int *pos = B.s_pref + w.cb;
            int *dl = B.s_order + w.cb;
            int nd = group_scan(g, H.nc, [&](int i) { return proc[i] == 0 ? 1 : 0; }, pos);
            g.sync();
            for (int i = g.rank(); i < H.nc; i += g.size())
                if (proc[i] == 0) dl[pos[i]] = i;
            g.sync();
            if (g.rank() == 0) {
                for (int k = 0; k < nd; ++k) {
                    const int i = dl[k];
                    bool woke;
                    const EvCtx ev{sp.events, sp.step_index, GB_EV_PHASE_UPDATE};
                    int r = collide_one(w, i, wake, &woke, &ev);
                    proc[i] = r;
                    if (r == 2) H.pflags |= P_DESTROY;
                    if (woke) {
                        const ContactRec<R> &c = w.con(i);
                        int a = w.fbody(c.fa), b = w.fbody(c.fb);
                        if (wake[a] > i) wake[a] = i;
                        if (wake[b] > i) wake[b] = i;
                    }
                }
            }
            g.sync();
        }
        if (woke_any)
            for (int b = g.rank(); b < H.nb; b += g.size())
                if (wake[b] >= 0 && wake[b] != GB_INF_IDX) wake_body(w, b);
        g.sync();
        if (H.pflags & P_DESTROY) compact_contacts(g, w, proc);
    } else if (PH == PH_ISLANDS) {
        if (solving) {
            if (g.rank() == 0) H.pflags |= P_SOLVING;
            islands_group(g, w, sp);
            constraints_group(g, w, sp);
        } else if (g.rank() == 0) {
            H.last_ncons = 0;
            H.last_njcons = 0;
        }
    } else if (PH == PH_CTL) {
        // the controllers open the solve (world.py:476-479): a kernel of their
        // own keeps their registers out of the island kernel
        if (solving && H.nctl) controllers_group(g, w);
    } else if (PH == PH_SOLVE) {
        if (H.pflags & P_SOLVING) {
            PhaseClock pc;
            pc.acc = (sp.profile && g.rank() == 0) ? B.prof + (size_t)wi * GB_NPROF : nullptr;
            pc.start();
            BodyCache cache{(dyn && H.nb <= B.cache_bodies) ? dyn : nullptr, B.pipe_bufs};
            solve_group(g, w, sp, &pc, cache);
            sleep_group(g, w, sp);
            if (g.rank() == 0) pc.mark(7);
        }
    } else if (PH == PH_PAIRS) {
        if (g.rank() == 0) H.toimin = ~0ull;   // k_toi1b lowers it
        if (H.pflags & P_SOLVING) sync_pairs_group(g, w, sp, &sh);
    } else if (PH == PH_TOI1) {
        // the loop's adjacency, pair hash and candidate list with the whole
        // CTA, for the worlds whose loop will run (the test of PH_TOI2)
        const bool par_first = (H.flags & GB_W_STEP_COMPLETE) != 0;
        const bool none = par_first && (H.toimin == ~0ull || (1.0 - (10.0 * GB_EPSILON)) < dkey_inv(H.toimin));
        if ((H.flags & GB_W_CONTINUOUS) && sp.dt > 0.0 && par_first && !none) {
            const int ncand = toi_setup(g, w, &sh);
            if (g.rank() == 0) { H.toi_ncand = ncand; H.toi_hcap = sh.lhcap; H.toi_ready = 1; }
        }
    } else if (PH == PH_TOI2) {
        if ((H.flags & GB_W_CONTINUOUS) && sp.dt > 0.0) {
            const bool par_first = (H.flags & GB_W_STEP_COMPLETE) != 0;
            // the batch-wide first pass found no event: the loop would end at once
            const bool none = par_first && (H.toimin == ~0ull || (1.0 - (10.0 * GB_EPSILON)) < dkey_inv(H.toimin));
            if (!none) {
                if (par_first)   // island flags of the bodies (world.py:600-601)
                    for (int b = g.rank(); b < H.nb; b += g.size()) B.s_bvis[w.bb + b] = 0;
                g.sync();
                PhaseClock pc;
                pc.acc = (sp.profile && g.rank() == 0) ? B.prof + (size_t)wi * GB_NPROF : nullptr;
                pc.start();
                toi_loop(g, w, sp, &sh, par_first, par_first, &pc);
            }
        }
        g.sync();
        if (g.rank() == 0) H.toi_ready = 0;
        if (g.rank() == 0 && sp.dt > 0.0) H.inv_dt0 = sp.inv_dt;
        if (H.flags & GB_W_AUTO_CLEAR_FORCES)
            for (int b = g.rank(); b < H.nb; b += g.size()) {
                B.b_f[w.bb + b] = mk<R>(0, 0);
                B.b_torque[w.bb + b] = (R)0;
            }
    }
}

template <class R, int PH> __device__ __forceinline__ void world_phase(const Batch<R> &B, const StepParams &sp, const int wi) {
    __shared__ int sm[96];
    __shared__ WorldHdr H;
    __shared__ WShared sh;
    extern __shared__ __align__(16) unsigned char gb_dyn_smem[];
    if (threadIdx.x == 0) { H = B.hdr[wi]; sh.nmove = 0; }
    __syncthreads();
    GroupCta g{sm};
    phase_body<R, PH>(B, sp, wi, g, H, sh, gb_dyn_smem);
    __syncthreads();
    if (threadIdx.x == 0) B.hdr[wi] = H;
}

static_assert(sizeof(WShared) <= GB_GRID_SHARED_BYTES, "WShared of grid worlds");

// The largest worlds (GB_HUGE_BODIES bodies or more) are advanced by a whole
// cooperative grid: the same phase code with every group operation grid-wide
// and the world header and scalars in global memory.
template <class R, int PH> __global__ void __launch_bounds__(GB_GRID_THREADS) k_world_grid(Batch<R> B, StepParams sp, int wi) {
    __shared__ __align__(16) int sm[96];   // GroupGrid reads sm + 16 as long longs
    if (threadIdx.x == 0) sm[80] = 0;
    __syncthreads();
    GroupGrid g{sm, B.g_scr};
    WorldHdr &H = B.hdr[wi];
    WShared &sh = *reinterpret_cast<WShared *>(B.g_sh);
    if (g.rank() == 0) sh.nmove = 0;
    g.sync();
    phase_body<R, PH>(B, sp, wi, g, H, sh, nullptr);
}

// gb_kernels.cuh -- host-callable launchers of the step kernel and of the
// body pack/unpack kernels for one precision.  Included by gb_f64.cu
// (GB_REAL = double, compiled without FMA contraction so the float64 path
// reproduces the CPU restatement bit for bit) and gb_f32.cu (GB_REAL = float).
#pragma once
#include <cuda_runtime.h>
#include <type_traits>
#include "gb_phases.cuh"
#include "gb_launch.h"
#include "gb_query.cuh"

// Each precision unit is compiled once per part, in parallel, and a part
// instantiates only its own kernels: 0 batch-wide kernels, record
// (un)packing, queries and the step orchestration; 1 and 8 the one-launch
// step kernels (one CTA, one warp per world); 2-5 the per-world phase
// kernels; 6-7 their cooperative-grid forms.  Without GB_PART every part is
// built.
#ifndef GB_PART
#define GB_PART -1
#endif
#define GB_IN_PART(p) (GB_PART < 0 || GB_PART == (p))

#if GB_IN_PART(0)
namespace {

__global__ void k_unpack_bodies(Batch<GB_REAL> B, const gb_body *src, int b0, int n) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int i = b0 + k;
    const gb_body &s = src[i];
    B.b_type[i] = s.type; B.b_flags[i] = s.flags; B.b_fstart[i] = s.fixture_start; B.b_fcount[i] = s.fixture_count;
    B.b_xp[i] = mk<double>(s.px, s.py);
    rot2<double> q; q.c = s.qc; q.s = s.qs; B.b_xq[i] = q;
    B.b_lc[i] = mk<double>(s.lcx, s.lcy); B.b_c[i] = mk<double>(s.cx, s.cy); B.b_c0[i] = mk<double>(s.c0x, s.c0y);
    B.b_a[i] = s.a; B.b_a0[i] = s.a0; B.b_alpha0[i] = s.alpha0;
    B.b_v[i] = mk<GB_REAL>((GB_REAL)s.vx, (GB_REAL)s.vy); B.b_w[i] = (GB_REAL)s.w;
    B.b_f[i] = mk<GB_REAL>((GB_REAL)s.fx, (GB_REAL)s.fy); B.b_torque[i] = (GB_REAL)s.torque;
    B.b_inv_mass[i] = (GB_REAL)s.inv_mass; B.b_inv_I[i] = (GB_REAL)s.inv_I;
    B.b_ldamp[i] = (GB_REAL)s.linear_damping; B.b_adamp[i] = (GB_REAL)s.angular_damping;
    B.b_gscale[i] = (GB_REAL)s.gravity_scale;
    B.b_mass[i] = s.mass; B.b_I[i] = s.I; B.b_sleep[i] = s.sleep_time;
}

__global__ void k_pack_bodies(Batch<GB_REAL> B, gb_body *dst, int b0, int n) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int i = b0 + k;
    gb_body s;
    s.type = B.b_type[i]; s.flags = B.b_flags[i]; s.fixture_start = B.b_fstart[i]; s.fixture_count = B.b_fcount[i];
    s.px = B.b_xp[i].x; s.py = B.b_xp[i].y; s.qc = B.b_xq[i].c; s.qs = B.b_xq[i].s;
    s.lcx = B.b_lc[i].x; s.lcy = B.b_lc[i].y; s.c0x = B.b_c0[i].x; s.c0y = B.b_c0[i].y;
    s.cx = B.b_c[i].x; s.cy = B.b_c[i].y; s.a0 = B.b_a0[i]; s.a = B.b_a[i]; s.alpha0 = B.b_alpha0[i];
    s.vx = (double)B.b_v[i].x; s.vy = (double)B.b_v[i].y; s.w = (double)B.b_w[i];
    s.fx = (double)B.b_f[i].x; s.fy = (double)B.b_f[i].y; s.torque = (double)B.b_torque[i];
    s.mass = B.b_mass[i]; s.inv_mass = (double)B.b_inv_mass[i]; s.I = B.b_I[i]; s.inv_I = (double)B.b_inv_I[i];
    s.linear_damping = (double)B.b_ldamp[i]; s.angular_damping = (double)B.b_adamp[i];
    s.gravity_scale = (double)B.b_gscale[i]; s.sleep_time = B.b_sleep[i];
    dst[i] = s;
}

__global__ void k_unpack_states(Batch<GB_REAL> B, const gb_body_state *src, int b0, int n) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int i = b0 + k;
    const gb_body_state &s = src[i];
    B.b_flags[i] = s.flags;
    B.b_xp[i] = mk<double>(s.px, s.py);
    rot2<double> q; q.c = s.qc; q.s = s.qs; B.b_xq[i] = q;
    B.b_c[i] = mk<double>(s.cx, s.cy); B.b_c0[i] = mk<double>(s.c0x, s.c0y);
    B.b_a[i] = s.a; B.b_a0[i] = s.a0; B.b_alpha0[i] = s.alpha0;
    B.b_v[i] = mk<GB_REAL>((GB_REAL)s.vx, (GB_REAL)s.vy); B.b_w[i] = (GB_REAL)s.w;
    B.b_f[i] = mk<GB_REAL>((GB_REAL)s.fx, (GB_REAL)s.fy); B.b_torque[i] = (GB_REAL)s.torque;
    B.b_sleep[i] = s.sleep_time;
}

__global__ void k_pack_states(Batch<GB_REAL> B, gb_body_state *dst, int b0, int n) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int i = b0 + k;
    gb_body_state s;
    s.flags = B.b_flags[i]; s._pad0 = 0;
    s.px = B.b_xp[i].x; s.py = B.b_xp[i].y; s.qc = B.b_xq[i].c; s.qs = B.b_xq[i].s;
    s.c0x = B.b_c0[i].x; s.c0y = B.b_c0[i].y; s.cx = B.b_c[i].x; s.cy = B.b_c[i].y;
    s.a0 = B.b_a0[i]; s.a = B.b_a[i]; s.alpha0 = B.b_alpha0[i];
    s.vx = (double)B.b_v[i].x; s.vy = (double)B.b_v[i].y; s.w = (double)B.b_w[i];
    s.fx = (double)B.b_f[i].x; s.fy = (double)B.b_f[i].y; s.torque = (double)B.b_torque[i];
    s.sleep_time = B.b_sleep[i];
    dst[i] = s;
}

__global__ void k_unpack_fixtures(Batch<GB_REAL> B, const gb_fixture *src, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const gb_fixture &f = src[i];
    B.f_body[i] = f.body; B.f_type[i] = f.shape_type; B.f_count[i] = f.vertex_count; B.f_flags[i] = f.flags;
    B.f_radius[i] = (GB_REAL)f.radius; B.f_friction[i] = (GB_REAL)f.friction;
    B.f_restitution[i] = (GB_REAL)f.restitution; B.f_density[i] = f.density;
    B.f_cat[i] = f.category_bits; B.f_mask[i] = f.mask_bits; B.f_group[i] = f.group_index;
    for (int k = 0; k < GB_MAX_POLY_VERTS; ++k) {
        B.f_v[(size_t)i * GB_MAX_POLY_VERTS + k] = mk<GB_REAL>((GB_REAL)f.vx[k], (GB_REAL)f.vy[k]);
        B.f_n[(size_t)i * GB_MAX_POLY_VERTS + k] = mk<GB_REAL>((GB_REAL)f.nx[k], (GB_REAL)f.ny[k]);
    }
    B.f_aabb[i] = mkbox(f.aabb[0], f.aabb[1], f.aabb[2], f.aabb[3]);
    B.f_aabbf[i] = boxf_of(B.f_aabb[i]);
}

// contacts: host records (one world per launch range) <-> device ContactRec
__global__ void k_unpack_contacts(Batch<GB_REAL> B, const gb_contact *src, const int *dst_slot, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const gb_contact &g = src[i];
    ContactRec<GB_REAL> c;
    c.fa = g.fixture_a; c.fb = g.fixture_b; c.flags = g.flags & ~GB_C_TOI_CAND; c.toi_count = g.toi_count; c.toi = g.toi;
    c.friction = (GB_REAL)g.friction; c.restitution = (GB_REAL)g.restitution;
    c.m.type = g.m_type; c.m.count = g.m_point_count;
    c.m.ln = mk<GB_REAL>((GB_REAL)g.m_lnx, (GB_REAL)g.m_lny); c.m.lp = mk<GB_REAL>((GB_REAL)g.m_lpx, (GB_REAL)g.m_lpy);
    for (int k = 0; k < 2; ++k) {
        c.m.plp[k] = mk<GB_REAL>((GB_REAL)g.p_lx[k], (GB_REAL)g.p_ly[k]);
        c.m.ni[k] = (GB_REAL)g.p_ni[k]; c.m.ti[k] = (GB_REAL)g.p_ti[k]; c.m.id[k] = g.p_id[k];
    }
    B.c[dst_slot[i]] = c;
}

__global__ void k_pack_contacts(Batch<GB_REAL> B, gb_contact *dst, int base, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const ContactRec<GB_REAL> &c = B.c[base + i];
    gb_contact g;
    g.fixture_a = c.fa; g.fixture_b = c.fb; g.child_a = 0; g.child_b = 0;
    g.flags = c.flags & ~GB_C_TOI_CAND; g.toi_count = c.toi_count; g.toi = c.toi;
    g.friction = (double)c.friction; g.restitution = (double)c.restitution;
    g.m_type = c.m.type; g.m_point_count = c.m.count;
    g.m_lnx = (double)c.m.ln.x; g.m_lny = (double)c.m.ln.y; g.m_lpx = (double)c.m.lp.x; g.m_lpy = (double)c.m.lp.y;
    for (int k = 0; k < 2; ++k) {
        g.p_lx[k] = (double)c.m.plp[k].x; g.p_ly[k] = (double)c.m.plp[k].y;
        g.p_ni[k] = (double)c.m.ni[k]; g.p_ti[k] = (double)c.m.ti[k]; g.p_id[k] = c.m.id[k];
    }
    dst[i] = g;
}

__global__ void k_refresh_toi_cand(Batch<GB_REAL> B, int s0, int n_slots) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_slots) return;
    const int s = s0 + k;
    WView<GB_REAL> w = view_global(B, B.c_world[s]);
    int i = s - w.cb;
    if (i >= w.H->nc) return;
    ContactRec<GB_REAL> &c = w.con(i);
    c.flags = (c.flags & ~GB_C_TOI_CAND) | (toi_candidate(w, i) ? GB_C_TOI_CAND : 0u);
}

}  // namespace
#endif  // GB_IN_PART(0)

// Launchers of the kernels that live in the other parts (declared here,
// defined by the part that instantiates the kernel).
template <int PH> cudaError_t gb_world_launch(int blocks, int threads, size_t smem, cudaStream_t st, const Batch<GB_REAL> &B,
                                              const StepParams &sp, const int *worlds);
template <int PH> cudaError_t gb_grid_launch(const Batch<GB_REAL> &B, const StepParams &sp, int wi, cudaStream_t st);
#define GB_DECL_PHASE_LAUNCHERS(PH)                                                                                        \
    template <> cudaError_t gb_world_launch<PH>(int, int, size_t, cudaStream_t, const Batch<GB_REAL> &, const StepParams &, \
                                                const int *);                                                              \
    template <> cudaError_t gb_grid_launch<PH>(const Batch<GB_REAL> &, const StepParams &, int, cudaStream_t);
GB_DECL_PHASE_LAUNCHERS(PH_PAIRS0)
GB_DECL_PHASE_LAUNCHERS(PH_COLLIDE2)
GB_DECL_PHASE_LAUNCHERS(PH_ISLANDS)
GB_DECL_PHASE_LAUNCHERS(PH_SOLVE)
GB_DECL_PHASE_LAUNCHERS(PH_PAIRS)
GB_DECL_PHASE_LAUNCHERS(PH_TOI2)
GB_DECL_PHASE_LAUNCHERS(PH_CTL)
#undef GB_DECL_PHASE_LAUNCHERS
template <> cudaError_t gb_world_launch<PH_TOI1>(int, int, size_t, cudaStream_t, const Batch<GB_REAL> &, const StepParams &,
                                                 const int *);
cudaError_t gb_cta_step_launch(const Batch<GB_REAL> &B, const StepParams &sp, int n_steps, const int *worlds, int n_list,
                               int threads, cudaStream_t st);
cudaError_t gb_warp_step_launch(const Batch<GB_REAL> &B, const StepParams &sp, int n_steps, const int *worlds, int n_list,
                                int threads, cudaStream_t st);

#if GB_IN_PART(1)
cudaError_t gb_cta_step_launch(const Batch<GB_REAL> &B, const StepParams &sp, int n_steps, const int *worlds, int n_list,
                               int threads, cudaStream_t st) {
    k_step_cta<GB_REAL><<<n_list, threads, 0, st>>>(B, sp, n_steps, worlds);
    return cudaGetLastError();
}
#endif
#if GB_IN_PART(8)
cudaError_t gb_warp_step_launch(const Batch<GB_REAL> &B, const StepParams &sp, int n_steps, const int *worlds, int n_list,
                                int threads, cudaStream_t st) {
    int wpc = threads / 32;
    if (wpc < 1) wpc = 1;
    const int blocks = (n_list + wpc - 1) / wpc;
    k_step_warp<GB_REAL><<<blocks, wpc * 32, 0, st>>>(B, sp, n_steps, worlds, n_list);
    return cudaGetLastError();
}
#endif

// Per-world phase kernels: one CTA per listed world (the TOI event loop one
// warp per world).  The solver's dynamic shared memory above the default
// 48 KB is opted into once per size.
#define GB_DEF_WORLD_LAUNCH(PH)                                                                                              \
    template <> cudaError_t gb_world_launch<PH>(int blocks, int threads, size_t smem, cudaStream_t st, const Batch<GB_REAL> &B, \
                                                const StepParams &sp, const int *worlds) {                                    \
        if (blocks <= 0) return cudaSuccess;                                                                                 \
        if constexpr (PH == PH_TOI2) {                                                                                       \
            k_world_toi2<GB_REAL><<<blocks, 32, 0, st>>>(B, sp, worlds);                                                     \
        } else {                                                                                                             \
            if (smem > 48 * 1024) {                                                                                          \
                static size_t opted = 0;                                                                                     \
                if (smem > opted) {                                                                                          \
                    cudaError_t e = cudaFuncSetAttribute(k_world<GB_REAL, PH>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                                         (int)smem);                                                         \
                    if (e != cudaSuccess) return e;                                                                          \
                    opted = smem;                                                                                            \
                }                                                                                                            \
            }                                                                                                                \
            k_world<GB_REAL, PH><<<blocks, threads, smem, st>>>(B, sp, worlds);                                              \
        }                                                                                                                    \
        return cudaGetLastError();                                                                                           \
    }
// Cooperative grid over one world (GB_HUGE_BODIES bodies or more): as many
// CTAs as are resident at once.
#define GB_DEF_GRID_LAUNCH(PH)                                                                                               \
    template <> cudaError_t gb_grid_launch<PH>(const Batch<GB_REAL> &B, const StepParams &sp, int wi, cudaStream_t st) {     \
        static int n = 0;                                                                                                    \
        if (n == 0) {                                                                                                        \
            int dev = 0, sms = 0, per_sm = 0;                                                                                \
            cudaGetDevice(&dev);                                                                                             \
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);                                               \
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_world_grid<GB_REAL, PH>, GB_GRID_THREADS, 0);           \
            n = sms * (per_sm > 0 ? per_sm : 1);                                                                             \
            if (n > GB_GRID_MAX_CTAS) n = GB_GRID_MAX_CTAS;                                                                  \
        }                                                                                                                    \
        Batch<GB_REAL> b = B;                                                                                                \
        StepParams p = sp;                                                                                                   \
        int w = wi;                                                                                                          \
        void *args[] = {&b, &p, &w};                                                                                         \
        return cudaLaunchCooperativeKernel((const void *)k_world_grid<GB_REAL, PH>, dim3(n), dim3(GB_GRID_THREADS), args, 0, \
                                           st);                                                                              \
    }
#if GB_IN_PART(2)
GB_DEF_WORLD_LAUNCH(PH_PAIRS0)
GB_DEF_WORLD_LAUNCH(PH_PAIRS)
#endif
#if GB_IN_PART(3)
GB_DEF_WORLD_LAUNCH(PH_COLLIDE2)
GB_DEF_WORLD_LAUNCH(PH_ISLANDS)
#endif
#if GB_IN_PART(4)
GB_DEF_WORLD_LAUNCH(PH_SOLVE)
GB_DEF_WORLD_LAUNCH(PH_CTL)
#endif
#if GB_IN_PART(5)
GB_DEF_WORLD_LAUNCH(PH_TOI2)
GB_DEF_WORLD_LAUNCH(PH_TOI1)
#endif
#if GB_IN_PART(6)
GB_DEF_GRID_LAUNCH(PH_PAIRS0)
GB_DEF_GRID_LAUNCH(PH_PAIRS)
GB_DEF_GRID_LAUNCH(PH_COLLIDE2)
#endif
#if GB_IN_PART(7)
GB_DEF_GRID_LAUNCH(PH_CTL)
GB_DEF_GRID_LAUNCH(PH_ISLANDS)
GB_DEF_GRID_LAUNCH(PH_SOLVE)
GB_DEF_GRID_LAUNCH(PH_TOI2)
#endif
#undef GB_DEF_WORLD_LAUNCH
#undef GB_DEF_GRID_LAUNCH

#if GB_IN_PART(0)
template <> int gb_launch_step<GB_REAL>(const Batch<GB_REAL> &B, const StepParams &sp, int n_steps, const int *d_worlds,
                                        int n_list, int mode, int threads, cudaStream_t st, KernelTimer *kt,
                                        const SideStream *side) {
    if (n_list <= 0) return 0;
    // the step kernels use ~220 registers per thread: at most 256 threads per CTA
    if (threads > 256) threads = 256;
    if (mode == 2) return (int)gb_warp_step_launch(B, sp, n_steps, d_worlds, n_list, threads, st);
    if (mode != 3) return (int)gb_cta_step_launch(B, sp, n_steps, d_worlds, n_list, threads, st);
    // phased: batch-wide kernels for the per-element work, per-world CTAs
    // for the ordered parts (see gb_phases.cuh)
    const int nb = B.n_bodies, ns = B.n_slots, T = 256;
    const int gb = (nb + T - 1) / T, gs = (ns + T - 1) / T;
    // the solve kernel stages each world's bodies in shared memory and
    // streams its constraint records through chunk buffers; the largest
    // worlds (first in the list) get a wider launch of their own
    const int nhuge = B.n_huge < n_list ? B.n_huge : n_list;
    const int nbig = B.n_big < n_list ? B.n_big : n_list;
    const int n_norm = n_list - nhuge;
    const int *w_norm = d_worlds + nhuge;
    const int tbig = GB_SOLVE_BIG_THREADS;
    // per-phase CTA widths: the island and pair phases run more threads
    // a world than the solver (measured on the uneven 8192-world batch:
    // islands 2.6 -> 1.3 ms at 4x, pair phases best at 2x)
    const int t_isl = threads * 4 < 256 ? threads * 4 : 256;
    const int t_pair = threads * 2 < 256 ? threads * 2 : 256;
    Batch<GB_REAL> Bb = B, Bs = B;
    Bb.cache_bodies = B.cache_big;
    Bs.cache_bodies = B.cache_small;
    const size_t smem_big = Bb.cache_bodies > 0 ? solve_smem_bytes<GB_REAL>(Bb.cache_bodies, tbig, B.pipe_bufs) : 0;
    const size_t smem_small = Bs.cache_bodies > 0 ? solve_smem_bytes<GB_REAL>(Bs.cache_bodies, threads, B.pipe_bufs) : 0;
    // kt: an event after every launch, the host accumulates the gaps
    // (one host synchronisation per step, measurement only)
    auto mark = [&](int k) { if (kt) cudaEventRecord(kt->ev[k], st); };
    cudaError_t e = cudaSuccess;
#define GB_CK(call) do { if ((e = (call)) != cudaSuccess) return (int)e; } while (0)
#define GB_GRID(PHX) for (int h = 0; h < nhuge; ++h) GB_CK(gb_grid_launch<PHX>(B, sp, B.huge_ids[h], st))
    const StepParams sp1 = sp;
    for (int s = 0; s < n_steps; ++s) {
        const StepParams sp = [&] { StepParams q = sp1; q.step_index = s; return q; }();
        mark(0);
        GB_GRID(PH_PAIRS0);
        GB_CK(gb_world_launch<PH_PAIRS0>(n_norm, threads, 0, st, B, sp, w_norm));
        mark(1);
        if (nb) k_pre<GB_REAL><<<gb, T, 0, st>>>(B, nb, sp);
        mark(2);
        if (ns) {
            if (sp.events) k_collide<GB_REAL, true><<<gs, T, 0, st>>>(B, ns, sp);
            else k_collide<GB_REAL, false><<<gs, T, 0, st>>>(B, ns, sp);
        }
        GB_CK(cudaGetLastError());
        mark(3);
        GB_GRID(PH_COLLIDE2);
        GB_CK(gb_world_launch<PH_COLLIDE2>(n_norm, t_pair, 0, st, B, sp, w_norm));
        mark(4);
        if (B.n_ctl) {   // controllers (timed with the islands)
            GB_GRID(PH_CTL);
            GB_CK(gb_world_launch<PH_CTL>(n_norm, t_isl, 0, st, B, sp, w_norm));
        }
        GB_GRID(PH_ISLANDS);
        GB_CK(gb_world_launch<PH_ISLANDS>(n_norm, t_isl, 0, st, B, sp, w_norm));
        mark(5);
        if (nb) k_vinit<GB_REAL><<<gb, T, 0, st>>>(B, nb, sp);
        mark(6);
        if (ns) k_cinit<GB_REAL><<<gs, T, 0, st>>>(B, ns, sp);
        GB_CK(cudaGetLastError());
        mark(7);
        GB_GRID(PH_SOLVE);
        if (side && nbig > nhuge && n_list > nbig) {
            // the larger worlds first on the caller's stream; the smaller
            // ones beside them on the low-priority side stream, filling
            // the shared memory the wide launch leaves free on each SM
            GB_CK(cudaEventRecord(side->fork, st));
            GB_CK(cudaStreamWaitEvent(side->s, side->fork, 0));
            GB_CK(gb_world_launch<PH_SOLVE>(nbig - nhuge, tbig, smem_big, st, Bb, sp, w_norm));
            GB_CK(gb_world_launch<PH_SOLVE>(n_list - nbig, threads, smem_small, side->s, Bs, sp, d_worlds + nbig));
            GB_CK(cudaEventRecord(side->join, side->s));
            GB_CK(cudaStreamWaitEvent(st, side->join, 0));
        } else {
            if (nbig > nhuge) GB_CK(gb_world_launch<PH_SOLVE>(nbig - nhuge, tbig, smem_big, st, Bb, sp, w_norm));
            if (n_list > nbig) GB_CK(gb_world_launch<PH_SOLVE>(n_list - nbig, threads, smem_small, st, Bs, sp, d_worlds + nbig));
        }
        mark(8);
        GB_GRID(PH_PAIRS);
        GB_CK(gb_world_launch<PH_PAIRS>(n_norm, t_pair, 0, st, B, sp, w_norm));
        mark(9);
        if (ns) k_toi1<GB_REAL><<<gs, T, 0, st>>>(B, ns, sp);
        mark(10);
        if (ns) k_toi1b<GB_REAL><<<152 * 4, 128, 0, st>>>(B);
        GB_CK(cudaGetLastError());
        mark(11);
        GB_CK(gb_world_launch<PH_TOI1>(n_norm, t_isl, 0, st, B, sp, w_norm));
        mark(12);
        GB_GRID(PH_TOI2);
        GB_CK(gb_world_launch<PH_TOI2>(n_norm, 32, 0, st, B, sp, w_norm));
        mark(13);
        if (kt) {
            GB_CK(cudaEventSynchronize(kt->ev[GB_NKTIME]));
            for (int k = 0; k < GB_NKTIME; ++k) {
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, kt->ev[k], kt->ev[k + 1]);
                kt->total_ms[k] += ms;
            }
            kt->steps += 1;
        }
    }
#undef GB_GRID
#undef GB_CK
    return (int)cudaGetLastError();
}

template <> void gb_launch_unpack_bodies<GB_REAL>(const Batch<GB_REAL> &B, const gb_body *d, int b0, int n, cudaStream_t st) {
    if (n > 0) k_unpack_bodies<<<(n + 255) / 256, 256, 0, st>>>(B, d, b0, n);
}
template <> void gb_launch_pack_bodies<GB_REAL>(const Batch<GB_REAL> &B, gb_body *d, int b0, int n, cudaStream_t st) {
    if (n > 0) k_pack_bodies<<<(n + 255) / 256, 256, 0, st>>>(B, d, b0, n);
}
template <> void gb_launch_unpack_states<GB_REAL>(const Batch<GB_REAL> &B, const gb_body_state *d, int b0, int n, cudaStream_t st) {
    if (n > 0) k_unpack_states<<<(n + 255) / 256, 256, 0, st>>>(B, d, b0, n);
}
template <> void gb_launch_pack_states<GB_REAL>(const Batch<GB_REAL> &B, gb_body_state *d, int b0, int n, cudaStream_t st) {
    if (n > 0) k_pack_states<<<(n + 255) / 256, 256, 0, st>>>(B, d, b0, n);
}
template <> void gb_launch_unpack_fixtures<GB_REAL>(const Batch<GB_REAL> &B, const gb_fixture *d, int n, cudaStream_t st) {
    if (n > 0) k_unpack_fixtures<<<(n + 255) / 256, 256, 0, st>>>(B, d, n);
}
template <> void gb_launch_unpack_contacts<GB_REAL>(const Batch<GB_REAL> &B, const gb_contact *d, const int *slots, int n, cudaStream_t st) {
    if (n > 0) k_unpack_contacts<<<(n + 255) / 256, 256, 0, st>>>(B, d, slots, n);
}
template <> void gb_launch_pack_contacts<GB_REAL>(const Batch<GB_REAL> &B, gb_contact *d, int base, int n, cudaStream_t st) {
    if (n > 0) k_pack_contacts<<<(n + 255) / 256, 256, 0, st>>>(B, d, base, n);
}
template <> void gb_launch_refresh_toi_cand<GB_REAL>(const Batch<GB_REAL> &B, int s0, int n, cudaStream_t st) {
    if (n > 0) k_refresh_toi_cand<<<(n + 255) / 256, 256, 0, st>>>(B, s0, n);
}
static_assert(GB_CFG_MAX_PIPE_BUFS <= GB_MAX_PIPE_BUFS, "launch configurations may ask for more chunk buffers than the solver has barriers");
template <> size_t gb_solve_smem<GB_REAL>(int cache_bodies, int threads, int nbuf) {
    return solve_smem_bytes<GB_REAL>(cache_bodies, threads, nbuf);
}
template <> void gb_launch_ray_cast<GB_REAL>(const Batch<GB_REAL> &B, const gb_ray *rays, int n, gb_ray_hit *hits, cudaStream_t st) {
    if (n > 0) k_ray_cast<GB_REAL><<<(n + 7) / 8, 256, 0, st>>>(B, rays, n, hits);
}
template <> void gb_launch_query_aabb<GB_REAL>(const Batch<GB_REAL> &B, const gb_aabb_query *qs, int n, int *out, int cap,
                                               int *counts, cudaStream_t st) {
    if (n > 0) k_query_aabb<GB_REAL><<<(n + 7) / 8, 256, 0, st>>>(B, qs, n, out, cap, counts);
}
template <> void gb_launch_ray_cast_all<GB_REAL>(const Batch<GB_REAL> &B, const gb_ray *rays, int n, gb_ray_hit *hits, int cap,
                                                 int *counts, cudaStream_t st) {
    if (n > 0) k_ray_cast_all<GB_REAL><<<(n + 7) / 8, 256, 0, st>>>(B, rays, n, hits, cap, counts);
}
#endif  // GB_IN_PART(0)

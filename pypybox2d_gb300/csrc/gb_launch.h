// gb_launch.h -- launchers shared by the precision translation units
// (gb_f64.cu, gb_f32.cu) and the C ABI (gb_api.cu).
#pragma once
#include <cuda_runtime.h>
#include "gb_world.cuh"

// Phased-step kernel timing: GB_NKTIME launch slots, GB_NKTIME + 1 events.
#define GB_NKTIME 13
struct KernelTimer {
    cudaEvent_t ev[GB_NKTIME + 1];
    double total_ms[GB_NKTIME];
    long long steps;
};
// A second stream of the batch (lowest priority) for the solver launch of
// the smaller worlds, which then runs beside the launch of the larger ones;
// fork and join are events on the caller's stream.
struct SideStream {
    cudaStream_t s;
    cudaEvent_t fork, join;
};
template <class R> int gb_launch_step(const Batch<R> &B, const StepParams &sp, int n_steps, const int *d_worlds, int n_list,
                                      int mode, int threads, cudaStream_t st, KernelTimer *kt = nullptr,
                                      const SideStream *side = nullptr);
template <class R> void gb_launch_unpack_bodies(const Batch<R> &B, const gb_body *d, int b0, int n, cudaStream_t st);
template <class R> void gb_launch_pack_bodies(const Batch<R> &B, gb_body *d, int b0, int n, cudaStream_t st);
template <class R> void gb_launch_unpack_states(const Batch<R> &B, const gb_body_state *d, int b0, int n, cudaStream_t st);
template <class R> void gb_launch_pack_states(const Batch<R> &B, gb_body_state *d, int b0, int n, cudaStream_t st);
template <class R> void gb_launch_unpack_fixtures(const Batch<R> &B, const gb_fixture *d, int n, cudaStream_t st);
template <class R> void gb_launch_unpack_contacts(const Batch<R> &B, const gb_contact *d, const int *slots, int n, cudaStream_t st);
template <class R> void gb_launch_pack_contacts(const Batch<R> &B, gb_contact *d, int base, int n, cudaStream_t st);
// shared memory of the phased solver launch: body cache of `cache_bodies`
// bodies plus `nbuf` constraint-chunk buffers for `threads` threads
template <class R> size_t gb_solve_smem(int cache_bodies, int threads, int nbuf);
#define GB_CFG_MAX_PIPE_BUFS 4
// world queries (gb_query.cuh): device arrays in and out
template <class R> void gb_launch_ray_cast(const Batch<R> &B, const gb_ray *rays, int n, gb_ray_hit *hits, cudaStream_t st);
template <class R> void gb_launch_query_aabb(const Batch<R> &B, const gb_aabb_query *qs, int n, int *out, int cap, int *counts,
                                             cudaStream_t st);
template <class R> void gb_launch_ray_cast_all(const Batch<R> &B, const gb_ray *rays, int n, gb_ray_hit *hits, int cap,
                                               int *counts, cudaStream_t st);
// recompute the device-only TOI candidate flag of every contact (after an upload)
template <class R> void gb_launch_refresh_toi_cand(const Batch<R> &B, int s0, int n, cudaStream_t st);

template <> int gb_launch_step<double>(const Batch<double> &, const StepParams &, int, const int *, int, int, int, cudaStream_t,
                                       KernelTimer *, const SideStream *);
template <> int gb_launch_step<float>(const Batch<float> &, const StepParams &, int, const int *, int, int, int, cudaStream_t,
                                      KernelTimer *, const SideStream *);
template <> void gb_launch_unpack_bodies<double>(const Batch<double> &, const gb_body *, int, int, cudaStream_t);
template <> void gb_launch_unpack_bodies<float>(const Batch<float> &, const gb_body *, int, int, cudaStream_t);
template <> void gb_launch_pack_bodies<double>(const Batch<double> &, gb_body *, int, int, cudaStream_t);
template <> void gb_launch_unpack_states<double>(const Batch<double> &, const gb_body_state *, int, int, cudaStream_t);
template <> void gb_launch_pack_states<double>(const Batch<double> &, gb_body_state *, int, int, cudaStream_t);
template <> void gb_launch_pack_bodies<float>(const Batch<float> &, gb_body *, int, int, cudaStream_t);
template <> void gb_launch_unpack_states<float>(const Batch<float> &, const gb_body_state *, int, int, cudaStream_t);
template <> void gb_launch_pack_states<float>(const Batch<float> &, gb_body_state *, int, int, cudaStream_t);
template <> void gb_launch_unpack_fixtures<double>(const Batch<double> &, const gb_fixture *, int, cudaStream_t);
template <> void gb_launch_unpack_fixtures<float>(const Batch<float> &, const gb_fixture *, int, cudaStream_t);
template <> void gb_launch_unpack_contacts<double>(const Batch<double> &, const gb_contact *, const int *, int, cudaStream_t);
template <> void gb_launch_unpack_contacts<float>(const Batch<float> &, const gb_contact *, const int *, int, cudaStream_t);
template <> void gb_launch_pack_contacts<double>(const Batch<double> &, gb_contact *, int, int, cudaStream_t);
template <> void gb_launch_pack_contacts<float>(const Batch<float> &, gb_contact *, int, int, cudaStream_t);
template <> void gb_launch_refresh_toi_cand<double>(const Batch<double> &, int, int, cudaStream_t);
template <> size_t gb_solve_smem<double>(int, int, int);
template <> size_t gb_solve_smem<float>(int, int, int);
template <> void gb_launch_refresh_toi_cand<float>(const Batch<float> &, int, int, cudaStream_t);
template <> void gb_launch_ray_cast<double>(const Batch<double> &, const gb_ray *, int, gb_ray_hit *, cudaStream_t);
template <> void gb_launch_ray_cast<float>(const Batch<float> &, const gb_ray *, int, gb_ray_hit *, cudaStream_t);
template <> void gb_launch_query_aabb<double>(const Batch<double> &, const gb_aabb_query *, int, int *, int, int *, cudaStream_t);
template <> void gb_launch_query_aabb<float>(const Batch<float> &, const gb_aabb_query *, int, int *, int, int *, cudaStream_t);
template <> void gb_launch_ray_cast_all<double>(const Batch<double> &, const gb_ray *, int, gb_ray_hit *, int, int *, cudaStream_t);
template <> void gb_launch_ray_cast_all<float>(const Batch<float> &, const gb_ray *, int, gb_ray_hit *, int, int *, cudaStream_t);

// gb_world.cuh -- device layout of a batch of worlds and the "group"
// abstraction the step is written against.
//
// A world is advanced by one group of threads: a whole CTA (launch mode 1)
// or one warp (launch mode 2).  Every phase of World.step is a loop over the
// world's bodies / fixtures / contacts / constraints strided by the group
// size, separated by group barriers; the few phases whose result depends on
// the reference's sequential order (the time-of-impact event loop, the
// island depth-first search that picks which body may sleep) run on the
// group's rank 0.  All group algorithms (scans, union-find, colouring) give
// results independent of the group size, so the CTA and warp mappings are
// bit-identical.
#pragma once
#include <cooperative_groups.h>
#include "gb_collide.cuh"

// ---------------------------------------------------------------- layout
// Batch-global structure of arrays.  Body / fixture arrays are indexed by
// the batch-global index (world base + world-local index); contact slots by
// world contact base + list position (contacts are kept dense, in creation
// order = ContactManager.contacts order).
template <class R> struct ContactRec {
    int fa, fb;          // world-local fixtures, fa is the primary shape
    uint32_t flags;      // GB_C_*
    int toi_count;
    double toi;
    R friction, restitution;
    Manifold<R> m;
};

template <class R> struct Cons {
    int cidx;            // contact list position
    int ia, ib;          // world-local bodies
    int root;            // island (union-find root, world-local body)
    R ma, mb, iA, iB;
    vec2<R> lca, lcb;
    R ra, rb, friction, restitution;
    int npts, mcount, mtype;
    vec2<R> normal;
    vec2<R> rA[2], rB[2];
    R ni[2], ti[2], nm[2], tm[2], bias[2];
    R k11, k12, k22, nm11, nm12, nm21, nm22;
    vec2<R> ln, lp, lpts[2];
    int dec;             // set-up decisions: restitution bias of point 0/1 (bits 0/1), block dropped to one point (bit 2)
};

// The solver's constraint records, stored colour-major.  ConsVel holds what
// the warm start and the velocity iterations read (the impulses first: the
// only fields they write back); ConsPos what the position iterations and
// the impulse store read.  The inverse masses come from the bodies.  Both
// are multiples of 16 bytes so a run of records moves as one bulk copy.
template <class R> struct __align__(16) ConsVel {
    R ni[2], ti[2];
    int ia, ib, npts, _pad;
    vec2<R> normal;
    vec2<R> rA[2], rB[2];
    R nm[2], tm[2], bias[2];
    R friction, k11, k12, k22, nm11, nm12, nm22;   // inverse K is symmetric: nm21 = nm12
};
template <class R> struct __align__(16) ConsPos {
    int cidx, ia, ib, root;
    int mcount, mtype, _pad0, _pad1;
    vec2<R> lca, lcb, ln, lp, lpts[2];
    R ra, rb;
};

// One joint's set-up for a step (float64 in both units): the attributes a
// joint's _init_velocity_constraints leaves for the passes (pypybox2d/joints).
struct d3 { double x, y, z; };
struct m33d { d3 c1, c2, c3; };   // Mat33, column-major (common.py:533-612)
struct __align__(16) JCons {
    int j, ia, ib, root;        // world-local joint and bodies, island (union-find root)
    double ma, mb, iA, iB;
    vec2<double> lca, lcb, ra, rb;
    m33d m;                     // revolute/weld _mass, prismatic _k
    double motor_mass;
    vec2<double> u;             // distance
    double dmass;
    vec2<double> axis, perp;    // prismatic
    double s1, s2, a1, a2;
};

struct WorldHdr {              // per-world scalars (device)
    int nb, nf, nc, ccap;      // counts, contact capacity
    int bbase, fbase, cbase;   // batch bases
    int pcap;                  // move-buffer capacity (fixtures)
    uint32_t flags;            // GB_W_*
    uint32_t status;           // GB_ST_*
    double gx, gy, inv_dt0;
    int last_ncons, last_ncolours;
    int nmove0;                // pending move buffer given at creation (in s_move)
    int all_allow;             // every body allows sleep (island.py:168 reads one body's flag)
    uint32_t pflags;           // phase flags of the current step (P_*)
    int nj;                    // joints of the world
    unsigned long long toimin; // dkey of the earliest first-pass time of impact below 1 (~0: none)
    int jbase;                 // batch index of its first joint
    int last_njcons, last_njcolours;   // joint constraints and their colours in the current step
    int toi_ncand, toi_hcap;   // TOI loop set-up made by the set-up kernel: candidates, pair-hash slots
    int toi_ready;             // that set-up is there for this step's loop
    int nctl;                  // controllers of the world
    int ctlbase;               // batch index of its first controller
    int _pad2;
};

#define GB_HUGE_BODIES 16384       // worlds this large run as one cooperative grid per phase
#define GB_MAX_HUGE 8
#define GB_GRID_THREADS 256
#define GB_GRID_MAX_CTAS 1024
#define GB_GRID_SHARED_BYTES 1024   // global room for the WShared of a grid world

template <class R> struct Batch {
    int n_worlds, n_bodies, n_slots;
    // the bodies [body0, body0 + n_bodies) and contact slots [slot0, slot0 +
    // n_slots) the batch-wide kernels of a launch cover: the whole batch, or
    // one world group (a run of worlds stepped on a stream of its own)
    int body0, slot0;
    int cache_bodies;         // worlds of at most this many bodies are solved from shared memory
    int pipe_bufs;            // solver: constraint chunk buffers in shared memory (0: read global memory)
    int n_big;                // worlds solved by the wide launch (the first n_big of the size-sorted list)
    int cache_big, cache_small;   // body capacity of the solver's shared memory in the two launches
    int wait_polls;           // poll limit of the solver's waits for its bulk copies (GB_WAIT_POLLS; a test may lower it)
    WorldHdr *hdr;
    int *b_world;             // world of each body
    int *c_world;             // world of each contact slot
    // bodies
    int *b_type; uint32_t *b_flags; int *b_fstart; int *b_fcount;
    vec2<double> *b_xp; rot2<double> *b_xq;
    vec2<double> *b_lc, *b_c, *b_c0; double *b_a, *b_a0, *b_alpha0;
    vec2<R> *b_v; R *b_w; vec2<R> *b_f; R *b_torque;
    R *b_inv_mass, *b_inv_I, *b_ldamp, *b_adamp, *b_gscale;
    double *b_mass, *b_I, *b_sleep;
    // fixtures
    int *f_body, *f_type, *f_count; uint32_t *f_flags;
    R *f_radius, *f_friction, *f_restitution; double *f_density;
    uint32_t *f_cat, *f_mask; int *f_group;
    vec2<R> *f_v, *f_n;       // 8 slots per fixture
    dbox *f_aabb;          // fat AABB
    float4 *f_aabbf;       // its float32 copy (rounded to nearest), read by the pair-finding grid
    // contacts
    ContactRec<R> *c;
    // scratch (body-indexed)
    int *s_parent, *s_wake, *s_seed, *s_stack, *s_adjoff;
    uint32_t *s_root;         // per-root bits
    unsigned long long *s_claim, *s_minsep, *s_minsleep;
    unsigned char *s_bvis;
    float4 *s_pose;              // float32 unit: each body's float32 centre and rotation at the solver set-up
    // scratch (fixture-indexed)
    int *s_move, *s_first, *s_cnt;
    int *s_grid;              // pair-finding grid: 12 nf + 2 ints per world (cell ends, listed and big proxies)
    // scratch (contact-slot-indexed)
    int *s_proc, *s_pref, *s_adj, *s_colour, *s_order, *s_cons_of;
    int2 *s_kb;
    unsigned char *s_cvis;
    Cons<R> *s_cons;             // GB_MAX_TOI_CONTACTS per world: the TOI sub-island solver
    ConsVel<R> *s_cv;            // colour-major solver records (contact capacity per world)
    ConsPos<R> *s_cp;
    unsigned long long *s_hash;  // 4 * ccap slots per world (a power of two >= 2*ccap fits)
    int *order_out;              // recorded solver order (contact positions), ccap per world
    long long *prof;             // per-world phase clocks (GB_NPROF per world), when profiling
    struct TPlan *s_plan;        // GB_TOI_PLAN_CAP planned TOI sweeps per world
    int *toi_list;               // contact slots needing a first-pass TOI (batch-wide)
    int *toi_n;                  // their count (one counter per world group)
    int *rec;                    // per body: the step record of the last record_order step
    int *rec_island;             // per body: its island in that step's solve (world-local union-find root, -1: none)
    gb_event *ev;                // contact events: 3 ccap + 64 per world, from 3 cbase + 64 world
    int *ev_n;                   // events recorded per world
    // joints (float64 records in both units, batch order = world order, then World.joints order)
    int n_joints;
    gb_joint *j;
    int *b_joff;                 // each body's joint list: world-local offsets, nb + 1 per world (from bbase + world)
    int *b_jadj;                 // world-local joint indices of the lists (2 per joint, from 2 jbase)
    JCons *s_jc;                 // the step's joint set-up, colour-major (per joint slot)
    int *s_jkj;                  // joint of each joint constraint (constraint order = World.joints order)
    int2 *s_jkb;                 // its non-static bodies (-1: static)
    int *s_jcol;                 // its colour
    int *s_jpref;                // scan / colour-compaction scratch (per joint slot)
    int *s_joff;                 // colour offsets of the colour-major layout: nj + 1 per world (from jbase + world)
    unsigned char *s_jvis;       // depth-first search marks (Joint._island_flag)
    int *jorder_out;
    // controllers (sorted by world) and their body lists (world-local bodies)
    int n_ctl;
    gb_controller *ctl;
    int *ctl_bodies;             // recorded joint order of the last record_order step (per joint slot)
    // custom contact filters (gb_batch_set_pair_filter): per world the offset
    // of its accept table in pf_accept (nf x nf bytes), -1 for the default rule
    const long long *pf_off;
    const unsigned char *pf_accept;
    // worlds advanced by a cooperative grid (the first n_huge of the size-sorted list)
    int n_huge;
    int huge_ids[GB_MAX_HUGE];
    long long *g_scr;            // their group scratch (2 x grid + 8)
    void *g_sh;                  // their WShared
};
#define GB_NPROF 24
#define GB_MAX_GROUPS 8            // world groups of a batch (streams stepping runs of worlds concurrently)
#define GB_WAIT_POLLS (1 << 18)    // default poll limit of the solver's waits for its bulk copies
// finite float64 / float32 value (integer test of the exponent bits)
static __device__ __forceinline__ bool finite_bits(double x) {
    return ((unsigned long long)__double_as_longlong(x) & 0x7ff0000000000000ull) != 0x7ff0000000000000ull;
}
static __device__ __forceinline__ bool finite_bits(float x) { return (__float_as_uint(x) & 0x7f800000u) != 0x7f800000u; }
#define GB_SOLVE_BIG_BODIES 512    // worlds this large are solved by the wide launch
#define GB_SOLVE_BIG_THREADS 128
#define GB_SOLVE_PIPE_BUFS 2       // constraint chunk buffers of the solver
#define GB_MAX_TOI_CONTACTS 32     // contacts of one TOI sub-island
// contact flag kept on the device only (cleared in exported records): the
// contact can take part in the TOI loop (toi_candidate)
#define GB_C_TOI_CAND 0x80000000u
#define GB_TOI_PLAN_CAP 64
// A TOI computation prepared by the order-dependent sweep alignment.
struct TPlan { double alpha0; Sweep sa, sb; };

struct StepParams {
    double dt, inv_dt, dt_ratio;
    int vel_iters, pos_iters;
    int record_order;
    int profile;
    int events;       // record contact events
    int step_index;   // step of the current call (event keys)
};

// Contact-event recording (listeners replayed on the host after the step).
#define GB_EV_PHASE_UPDATE 0
#define GB_EV_PHASE_SOLVE 1
#define GB_EV_PHASE_TOI 2
struct EvCtx {
    int on, step, phase;
    int *rec;         // the world's step record (record_order steps), else null
};

// Step record of a body (record_order steps; gb_batch_get_step_record):
// decisions of the step that its final state does not show.
#define GB_REC_TOI_ITERS_SHIFT 8    // TOI position-pass iterations, summed over its events (contact.py:866-933)
#define GB_REC_TOI_EVENTS_SHIFT 16  // TOI events it took part in (world.py:693-817)
#define GB_REC_SETUP_SHIFT 24       // parity of its constraints' restitution-bias points (bit 24) and block-solver
                                    // drops (bit 25) in the island solve; bits 26/27 the same in TOI sub-steps
                                    // (contact.py:470-496); bits 0-7: position iterations of its island
static __device__ __forceinline__ void rec_add_byte(int *x, int shift, int v) {
    int cur = (*x >> shift) & 0xff;
    int nv = cur + v > 255 ? 255 : cur + v;
    *x = (*x & ~(0xff << shift)) | (nv << shift);
}
// the parity bits of one constraint's set-up decisions (Cons::dec) at `shift`
static __device__ __forceinline__ int rec_setup_bits(int dec, int shift) {
    return ((((dec & 1) + ((dec >> 1) & 1)) & 1) << shift) | (((dec >> 2) & 1) << (shift + 1));
}

// Phase clocks: rank 0 adds the SM clock delta since the last mark.
struct PhaseClock {
    long long *acc;
    long long t;
    __device__ __forceinline__ void start() { if (acc) t = clock64(); }
    __device__ __forceinline__ void mark(int k) {
        if (acc) { long long n = clock64(); acc[k] += n - t; t = n; }
    }
};

// ---------------------------------------------------------------- groups
struct GroupCta {
    int *sm;   // >= 64 ints of shared memory owned by the group
    __device__ __forceinline__ int rank() const { return threadIdx.x; }
    __device__ __forceinline__ int size() const { return blockDim.x; }
    __device__ __forceinline__ void sync() const { __syncthreads(); }
    __device__ __forceinline__ bool any(bool p) const { return __syncthreads_or(p) != 0; }
    // exclusive scan of v over the group; *total = sum.  Contains barriers.
    __device__ int exscan(int v, int *total) const {
        int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
        int x = v;
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) sm[warp] = x;
        __syncthreads();
        if (warp == 0) {
            int s = (lane < nw) ? sm[lane] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                int y = __shfl_up_sync(0xffffffffu, s, o);
                if (lane >= o) s += y;
            }
            if (lane < nw) sm[32 + lane] = s;
        }
        __syncthreads();
        int base = warp ? sm[32 + warp - 1] : 0;
        *total = sm[32 + nw - 1];
        __syncthreads();
        return base + x - v;
    }
    // lexicographic minimum of (key, idx) over the group, returned to every
    // thread (uses sm[0..3 * warps)).  Contains barriers.
    __device__ void argmin(unsigned long long &key, int &idx) const {
        int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
        for (int o = 16; o > 0; o >>= 1) {
            unsigned long long k2 = __shfl_xor_sync(0xffffffffu, key, o);
            int i2 = __shfl_xor_sync(0xffffffffu, idx, o);
            if (k2 < key || (k2 == key && i2 < idx)) { key = k2; idx = i2; }
        }
        if (lane == 0) {
            sm[3 * warp] = (int)(unsigned)(key & 0xffffffffull);
            sm[3 * warp + 1] = (int)(unsigned)(key >> 32);
            sm[3 * warp + 2] = idx;
        }
        __syncthreads();
        for (int k = 0; k < nw; ++k) {
            unsigned long long k2 = ((unsigned long long)(unsigned)sm[3 * k + 1] << 32) | (unsigned)sm[3 * k];
            int i2 = sm[3 * k + 2];
            if (k2 < key || (k2 == key && i2 < idx)) { key = k2; idx = i2; }
        }
        __syncthreads();
    }
};

struct GroupWarp {
    int *sm;
    __device__ __forceinline__ int rank() const { return threadIdx.x & 31; }
    __device__ __forceinline__ int size() const { return 32; }
    __device__ __forceinline__ void sync() const { __syncwarp(); }
    __device__ __forceinline__ bool any(bool p) const { __syncwarp(); return __any_sync(0xffffffffu, p) != 0; }
    __device__ int exscan(int v, int *total) const {
        int lane = threadIdx.x & 31;
        int x = v;
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        *total = __shfl_sync(0xffffffffu, x, 31);
        __syncwarp();
        return x - v;
    }
    __device__ void argmin(unsigned long long &key, int &idx) const {
        for (int o = 16; o > 0; o >>= 1) {
            unsigned long long k2 = __shfl_xor_sync(0xffffffffu, key, o);
            int i2 = __shfl_xor_sync(0xffffffffu, idx, o);
            if (k2 < key || (k2 == key && i2 < idx)) { key = k2; idx = i2; }
        }
        __syncwarp();
    }
};

// A whole cooperative grid working on one world: grid-wide ranks, barriers
// (grid.sync) and reductions.  A reduction writes one partial per CTA to a
// global scratch, syncs the grid once, and every CTA then reduces the
// partials with all its threads.  Consecutive reductions alternate between
// two halves of the scratch, so a CTA may start the next one while others
// still read the previous.  Scratch: 4 x gridDim longs.
struct GroupGrid {
    int *sm;               // this CTA's shared scratch (>= 96 ints; [80] counts reductions)
    long long *gs;         // global scratch
    __device__ __forceinline__ int rank() const { return blockIdx.x * blockDim.x + threadIdx.x; }
    __device__ __forceinline__ int size() const { return gridDim.x * blockDim.x; }
    __device__ __forceinline__ void sync() const { cooperative_groups::this_grid().sync(); }
    // this reduction's half of the scratch (2 x gridDim longs)
    __device__ __forceinline__ long long *half() const {
        long long *h = gs + ((sm[80] & 1) ? 2 * (size_t)gridDim.x : 0);
        return h;
    }
    __device__ __forceinline__ void next() const {
        __syncthreads();
        if (threadIdx.x == 0) sm[80] += 1;
        __syncthreads();
    }
    // sums over the CTA of (a, b); every thread gets them
    __device__ void cta_sum2(long long &a, long long &b) const {
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, o);
            b += __shfl_xor_sync(0xffffffffu, b, o);
        }
        long long *s64 = reinterpret_cast<long long *>(sm + 16);   // sm[16..47]: 8 warps x 2 longs
        int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
        if (lane == 0) { s64[2 * warp] = a; s64[2 * warp + 1] = b; }
        __syncthreads();
        a = 0; b = 0;
        for (int k = 0; k < nw; ++k) { a += s64[2 * k]; b += s64[2 * k + 1]; }
        __syncthreads();
    }
    __device__ bool any(bool p) const {
        int bflag = __syncthreads_or(p);
        long long *h = half();
        if (threadIdx.x == 0) h[blockIdx.x] = bflag;
        sync();
        long long a = 0, b = 0;
        for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) a |= h[k];
        cta_sum2(a, b);
        next();
        return a != 0;
    }
    __device__ int exscan(int v, int *total) const {
        GroupCta c{sm};
        int ctot;
        int ex = c.exscan(v, &ctot);
        long long *h = half();
        if (threadIdx.x == 0) h[blockIdx.x] = ctot;
        sync();
        long long base = 0, tot = 0;
        for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) {
            long long x = h[k];
            if (k < (int)blockIdx.x) base += x;
            tot += x;
        }
        cta_sum2(base, tot);
        *total = (int)tot;
        next();
        return (int)base + ex;
    }
    __device__ void argmin(unsigned long long &key, int &idx) const {
        GroupCta c{sm};
        c.argmin(key, idx);
        long long *h = half();
        if (threadIdx.x == 0) { h[2 * blockIdx.x] = (long long)key; h[2 * blockIdx.x + 1] = idx; }
        sync();
        unsigned long long bk = ~0ull;
        int bi = 0x7fffffff;
        for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) {
            unsigned long long k2 = (unsigned long long)h[2 * k];
            int i2 = (int)h[2 * k + 1];
            if (k2 < bk || (k2 == bk && i2 < bi)) { bk = k2; bi = i2; }
        }
        c.argmin(bk, bi);
        key = bk;
        idx = bi;
        next();
    }
};

// Number of i < n with pred(i) over the group (contains barriers).
template <class G, class F> __device__ int group_count(const G &g, int n, F pred) {
    int local = 0;
    for (int i = g.rank(); i < n; i += g.size()) local += pred(i);
    int tot;
    g.exscan(local, &tot);
    return tot;
}

// Chunked exclusive scan of flag(i) for i < n into out[i]; returns the total.
template <class G, class F> __device__ int group_scan(const G &g, int n, F flag, int *out) {
    int carry = 0;
    for (int base = 0; base < n; base += g.size()) {
        int i = base + g.rank();
        int v = (i < n) ? flag(i) : 0;
        int tot;
        int ex = g.exscan(v, &tot);
        if (i < n) out[i] = carry + ex;
        carry += tot;
    }
    return carry;
}

// Per-world view: world-local indexing helpers over the batch arrays.
template <class R> struct WView {
    Batch<R> B;
    WorldHdr *H;   // group-shared copy
    int bb, fb, cb, wi;
    __device__ __forceinline__ Shape<R> shape(int f) const {
        int gf = fb + f;
        Shape<R> s;
        s.type = B.f_type[gf]; s.count = B.f_count[gf]; s.flags = B.f_flags[gf]; s.radius = B.f_radius[gf];
        s.v = B.f_v + (size_t)gf * GB_MAX_POLY_VERTS;
        s.n = B.f_n + (size_t)gf * GB_MAX_POLY_VERTS;
        return s;
    }
    __device__ __forceinline__ int fbody(int f) const { return B.f_body[fb + f]; }
    __device__ __forceinline__ xform2<R> xf(int b) const {
        xform2<R> x;
        vec2<double> p = B.b_xp[bb + b];
        rot2<double> q = B.b_xq[bb + b];
        x.p = mk<R>((R)p.x, (R)p.y);
        x.q.c = (R)q.c; x.q.s = (R)q.s;
        return x;
    }
    __device__ __forceinline__ xform2<double> xfd(int b) const {
        xform2<double> x;
        x.p = B.b_xp[bb + b];
        x.q = B.b_xq[bb + b];
        return x;
    }
    __device__ __forceinline__ bool awake(int b) const { return (B.b_flags[bb + b] & GB_BODY_AWAKE) != 0; }
    __device__ __forceinline__ int btype(int b) const { return B.b_type[bb + b]; }
    __device__ __forceinline__ ContactRec<R> &con(int i) const { return B.c[cb + i]; }
    __device__ __forceinline__ Sweep sweep(int b) const {
        Sweep s;
        s.lc = B.b_lc[bb + b]; s.c0 = B.b_c0[bb + b]; s.c = B.b_c[bb + b];
        s.a0 = B.b_a0[bb + b]; s.a = B.b_a[bb + b]; s.alpha0 = B.b_alpha0[bb + b];
        return s;
    }
    __device__ __forceinline__ void put_sweep(int b, const Sweep &s) const {
        B.b_lc[bb + b] = s.lc; B.b_c0[bb + b] = s.c0; B.b_c[bb + b] = s.c;
        B.b_a0[bb + b] = s.a0; B.b_a[bb + b] = s.a; B.b_alpha0[bb + b] = s.alpha0;
    }
};

// gb_api.cu -- the C ABI of libgb2d.so (include/gb2d.h).
//
// A gb_batch owns one device arena holding every world of the batch in the
// structure-of-arrays layout of gb_world.cuh plus the per-world scratch of
// the step.  Host records (gb_body, gb_fixture, gb_contact) cross the bus in
// their AoS form and are (un)packed on the device.  Errors are reported as
// negative status codes with a thread-local message; no call falls back to
// the CPU.
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "gb_launch.h"

namespace {
thread_local std::string g_err = "ok";

int fail(int code, const std::string &msg) {
    g_err = msg;
    return code;
}
int cuda_fail(cudaError_t e, const char *where) {
    g_err = std::string(where) + ": " + cudaGetErrorString(e);
    return GB_E_CUDA;
}
#define CK(call)                                             \
    do {                                                     \
        cudaError_t e_ = (call);                             \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);  \
    } while (0)

// Bump allocator over one cudaMalloc'ed arena.
struct Arena {
    size_t off = 0;
    char *base = nullptr;
    template <class T> T *take(size_t n) {
        off = (off + 255) & ~size_t(255);
        T *p = base ? reinterpret_cast<T *>(base + off) : nullptr;
        off += sizeof(T) * (n ? n : 1);
        return p;
    }
};

template <class R> void carve(Arena &a, Batch<R> &B, int nw, int nb, int nf, int ncap, int nj, int nctl, int nctlb) {
    B.n_worlds = nw;
    B.n_bodies = nb;
    B.n_slots = ncap;
    B.hdr = a.take<WorldHdr>(nw);
    B.b_world = a.take<int>(nb);
    B.c_world = a.take<int>(ncap);
    B.b_type = a.take<int>(nb); B.b_flags = a.take<uint32_t>(nb); B.b_fstart = a.take<int>(nb); B.b_fcount = a.take<int>(nb);
    B.b_xp = a.take<vec2<double>>(nb); B.b_xq = a.take<rot2<double>>(nb);
    B.b_lc = a.take<vec2<double>>(nb); B.b_c = a.take<vec2<double>>(nb); B.b_c0 = a.take<vec2<double>>(nb);
    B.b_a = a.take<double>(nb); B.b_a0 = a.take<double>(nb); B.b_alpha0 = a.take<double>(nb);
    B.b_v = a.take<vec2<R>>(nb); B.b_w = a.take<R>(nb); B.b_f = a.take<vec2<R>>(nb); B.b_torque = a.take<R>(nb);
    B.b_inv_mass = a.take<R>(nb); B.b_inv_I = a.take<R>(nb); B.b_ldamp = a.take<R>(nb); B.b_adamp = a.take<R>(nb);
    B.b_gscale = a.take<R>(nb);
    B.b_mass = a.take<double>(nb); B.b_I = a.take<double>(nb); B.b_sleep = a.take<double>(nb);
    B.f_body = a.take<int>(nf); B.f_type = a.take<int>(nf); B.f_count = a.take<int>(nf); B.f_flags = a.take<uint32_t>(nf);
    B.f_radius = a.take<R>(nf); B.f_friction = a.take<R>(nf); B.f_restitution = a.take<R>(nf); B.f_density = a.take<double>(nf);
    B.f_cat = a.take<uint32_t>(nf); B.f_mask = a.take<uint32_t>(nf); B.f_group = a.take<int>(nf);
    B.f_v = a.take<vec2<R>>((size_t)nf * GB_MAX_POLY_VERTS); B.f_n = a.take<vec2<R>>((size_t)nf * GB_MAX_POLY_VERTS);
    B.f_aabb = a.take<dbox>(nf);
    B.f_aabbf = a.take<float4>(nf);
    B.c = a.take<ContactRec<R>>(ncap);
    B.s_parent = a.take<int>(nb); B.s_wake = a.take<int>(nb); B.s_seed = a.take<int>(nb); B.s_stack = a.take<int>(nb);
    B.s_adjoff = a.take<int>(nb + nw);
    B.s_root = a.take<uint32_t>(nb);
    B.s_claim = a.take<unsigned long long>(nb); B.s_minsep = a.take<unsigned long long>(nb);
    B.s_minsleep = a.take<unsigned long long>(nb);
    B.s_bvis = a.take<unsigned char>(nb);
    B.s_pose = a.take<float4>(nb);
    B.s_move = a.take<int>(nf); B.s_first = a.take<int>(nf); B.s_cnt = a.take<int>(nf);
    B.s_grid = a.take<int>(12 * (size_t)nf + 2 * (size_t)nw);
    B.s_proc = a.take<int>(ncap); B.s_pref = a.take<int>(ncap); B.s_adj = a.take<int>(2 * (size_t)ncap);
    B.s_colour = a.take<int>(ncap); B.s_order = a.take<int>(ncap); B.s_cons_of = a.take<int>(ncap);
    B.s_cvis = a.take<unsigned char>(ncap);
    B.s_kb = a.take<int2>(ncap);
    B.s_cons = a.take<Cons<R>>((size_t)nw * GB_MAX_TOI_CONTACTS);
    B.s_cv = a.take<ConsVel<R>>(ncap);
    B.s_cp = a.take<ConsPos<R>>(ncap);
    B.s_hash = a.take<unsigned long long>(4 * (size_t)ncap);
    B.order_out = a.take<int>(ncap);
    B.rec = a.take<int>(nb);
    B.rec_island = a.take<int>(nb);
    B.prof = a.take<long long>((size_t)nw * GB_NPROF);
    B.s_plan = a.take<TPlan>((size_t)nw * GB_TOI_PLAN_CAP);
    B.toi_list = a.take<int>(ncap);
    B.toi_n = a.take<int>(GB_MAX_GROUPS);
    B.g_scr = a.take<long long>(4 * (size_t)GB_GRID_MAX_CTAS + 8);
    B.g_sh = a.take<unsigned char>(GB_GRID_SHARED_BYTES);
    B.n_joints = nj;
    B.j = a.take<gb_joint>(nj);
    B.b_joff = a.take<int>(nb + nw);
    B.b_jadj = a.take<int>(2 * (size_t)nj);
    B.s_jc = a.take<JCons>(nj);
    B.s_jkj = a.take<int>(nj);
    B.s_jkb = a.take<int2>(nj);
    B.s_jcol = a.take<int>(nj);
    B.s_jpref = a.take<int>(nj);
    B.s_joff = a.take<int>(nj + nw);
    B.s_jvis = a.take<unsigned char>(nj);
    B.jorder_out = a.take<int>(nj);
    B.n_ctl = nctl;
    B.ctl = a.take<gb_controller>(nctl);
    B.ctl_bodies = a.take<int>(nctlb);
}
// Re-points the per-step scratch arrays of a batch into one region laid out
// by `a` (a.base == nullptr only measures it).  The state that outlives a step
// stays in the batch arena: the pending move buffer (s_move, read by the
// first step), the recorded solver order and the phase clocks.
template <class R> void carve_step_scratch(Arena &a, Batch<R> &B, int nw, int nb, int nf, int ncap, int nj) {
    B.s_parent = a.take<int>(nb); B.s_wake = a.take<int>(nb); B.s_seed = a.take<int>(nb); B.s_stack = a.take<int>(nb);
    B.s_adjoff = a.take<int>(nb + nw);
    B.s_root = a.take<uint32_t>(nb);
    B.s_claim = a.take<unsigned long long>(nb); B.s_minsep = a.take<unsigned long long>(nb);
    B.s_minsleep = a.take<unsigned long long>(nb);
    B.s_bvis = a.take<unsigned char>(nb);
    B.s_pose = a.take<float4>(nb);
    B.s_first = a.take<int>(nf); B.s_cnt = a.take<int>(nf);
    B.s_grid = a.take<int>(12 * (size_t)nf + 2 * (size_t)nw);
    B.s_proc = a.take<int>(ncap); B.s_pref = a.take<int>(ncap); B.s_adj = a.take<int>(2 * (size_t)ncap);
    B.s_colour = a.take<int>(ncap); B.s_order = a.take<int>(ncap); B.s_cons_of = a.take<int>(ncap);
    B.s_cvis = a.take<unsigned char>(ncap);
    B.s_kb = a.take<int2>(ncap);
    B.s_cons = a.take<Cons<R>>((size_t)nw * GB_MAX_TOI_CONTACTS);
    B.s_cv = a.take<ConsVel<R>>(ncap);
    B.s_cp = a.take<ConsPos<R>>(ncap);
    B.s_hash = a.take<unsigned long long>(4 * (size_t)ncap);
    B.s_plan = a.take<TPlan>((size_t)nw * GB_TOI_PLAN_CAP);
    B.toi_list = a.take<int>(ncap);
    B.toi_n = a.take<int>(GB_MAX_GROUPS);
    B.s_jc = a.take<JCons>(nj);
    B.s_jkj = a.take<int>(nj);
    B.s_jkb = a.take<int2>(nj);
    B.s_jcol = a.take<int>(nj);
    B.s_jpref = a.take<int>(nj);
    B.s_joff = a.take<int>(nj + nw);
    B.s_jvis = a.take<unsigned char>(nj);
}
}  // namespace

// A world group: a run of consecutive worlds stepped on a stream of its own
// (gb_launch_config.groups), so that the latency-bound tail of one group's
// per-world phases overlaps the other groups' kernels.
struct WorldGroup {
    int w0 = 0, w1 = 0;              // worlds [w0, w1)
    int b0 = 0, nb = 0, s0 = 0, ns = 0;   // their bodies and contact slots
    int *d_worlds = nullptr;         // their list, largest first (device)
    int n_list = 0, nbig = 0;        // list length, worlds of the wide solver launch
    cudaStream_t st = nullptr;
    cudaEvent_t done = nullptr;
};

struct gb_batch {
    int prec = GB_PREC_F64;
    int nw = 0, nb = 0, nf = 0, ncap = 0, nj = 0;
    int nctl = 0, nctlb = 0;       // controllers and the entries of their body lists
    std::vector<gb_controller> controllers;   // at creation (world, kind and body lists are fixed for the batch)
    std::vector<WorldHdr> hdr;     // host copy of the headers at creation
    std::vector<gb_joint> joints;  // the joints at creation (world, type and bodies are fixed for the batch)
    std::vector<int> launch_order; // worlds sorted by body count, largest first
    char *arena = nullptr;
    size_t arena_bytes = 0;
    Batch<double> bd{};
    Batch<float> bf{};
    int *d_worlds = nullptr;
    gb_body *d_bstage = nullptr;
    gb_contact *d_cstage = nullptr;
    int cstage_cap = 0;
    long long counters[3] = {0, 0, 0};
    KernelTimer *ktimer = nullptr;   // created by the first timed step
    gb_event *d_ev = nullptr;        // contact events, allocated by the first step that records them
    int *d_ev_n = nullptr;
    SideStream side{};               // the solver's second stream (gb_launch.h)
    bool has_side = false;
    gb_launch_config cfg{3, 128, GB_SOLVE_PIPE_BUFS, GB_SOLVE_BIG_BODIES, 1, 0, 0.0};   // launch_mode 0 steps
    std::vector<WorldGroup> groups;  // world groups of cfg.groups > 1
    std::vector<WorldGroup> chunks;  // gb_batch_step_host's chunks while cfg.groups is 1
    int chunks_big = -1;             // the wide-launch threshold the chunks were made with
    cudaEvent_t fork = nullptr;      // the caller's stream -> the groups' streams
    std::vector<gb_graph *> graphs;  // captured rollouts, disarmed when the batch is destroyed
    char *d_query = nullptr;         // staging of query inputs and outputs, grown on demand
    size_t query_bytes = 0;
    std::vector<std::vector<unsigned char>> pf;   // custom contact filters' accept tables per world (empty: default)
    long long *d_pf_off = nullptr;   // their offsets on the device (-1: default rule)
    unsigned char *d_pf = nullptr;   // the tables
};

namespace {
template <class R> int run_steps(gb_batch *b, const Batch<R> &B, const StepParams &sp, int n_steps, int mode, int threads,
                                 cudaStream_t st, KernelTimer *kt);
void free_groups(std::vector<WorldGroup> &groups);
}

// A captured rollout (gb_graph_capture).  `b` is null once its batch is gone.
struct gb_graph {
    gb_batch *b = nullptr;
    cudaGraphExec_t exec = nullptr;
    int n_steps = 0;
};

namespace {
// launch mode and CTA width of a step call: launch_mode 0 takes the batch's
// launch configuration
void resolve_mapping(const gb_batch *b, const gb_step_opts *o, int *mode, int *threads) {
    if (o->launch_mode == 0) *mode = b->cfg.launch_mode;
    else *mode = (o->launch_mode == 2 || o->launch_mode == 3) ? o->launch_mode : 1;
    *threads = o->block_threads > 0 ? o->block_threads : (o->launch_mode == 0 ? b->cfg.block_threads : 128);
}
// contact-event buffers, allocated by the first step that records events
int ensure_event_buffers(gb_batch *b) {
    if (!b->d_ev) {
        CK(cudaMalloc((void **)&b->d_ev, sizeof(gb_event) * (3 * (size_t)b->ncap + 64 * (size_t)b->nw)));
        CK(cudaMalloc((void **)&b->d_ev_n, sizeof(int) * b->nw));
        b->bd.ev = b->bf.ev = b->d_ev;
        b->bd.ev_n = b->bf.ev_n = b->d_ev_n;
    }
    return 0;
}
}  // namespace

extern "C" {

const char *gb_version(void) { return "gb2d 0.1 sm_103a"; }
const char *gb_last_error(void) { return g_err.c_str(); }
int gb_joint_size(void) { return (int)sizeof(gb_joint); }
int gb_controller_size(void) { return (int)sizeof(gb_controller); }
int gb_body_state_size(void) { return (int)sizeof(gb_body_state); }

int gb_struct_sizes(int32_t *sizes) {
    if (!sizes) return fail(GB_E_ARG, "sizes is NULL");
    sizes[0] = (int32_t)sizeof(gb_body);
    sizes[1] = (int32_t)sizeof(gb_fixture);
    sizes[2] = (int32_t)sizeof(gb_contact);
    sizes[3] = (int32_t)sizeof(gb_world_desc);
    sizes[4] = (int32_t)sizeof(gb_scene);
    sizes[5] = (int32_t)sizeof(gb_step_opts);
    return 0;
}

int gb_batch_create(const gb_scene *scene, int32_t precision, gb_batch **out) {
    if (!scene || !out) return fail(GB_E_ARG, "scene or out is NULL");
    if (precision != GB_PREC_F64 && precision != GB_PREC_F32) return fail(GB_E_ARG, "precision must be GB_PREC_F64 or GB_PREC_F32");
    if (scene->n_worlds <= 0) return fail(GB_E_ARG, "scene has no worlds");
    gb_batch *b = new gb_batch();
    b->prec = precision;
    b->nw = scene->n_worlds;
    b->nb = scene->n_bodies;
    b->nf = scene->n_fixtures;
    b->hdr.resize(b->nw);
    int cbase = 0;
    for (int i = 0; i < b->nw; ++i) {
        const gb_world_desc &d = scene->worlds[i];
        if (i > 0) {   // worlds lie in order, without overlap (per-world scratch is laid out the same way)
            const gb_world_desc &p = scene->worlds[i - 1];
            if (d.body_start < p.body_start + p.body_count || d.fixture_start < p.fixture_start + p.fixture_count) {
                delete b;
                return fail(GB_E_ARG, "world " + std::to_string(i) + ": body/fixture ranges must follow the previous world's");
            }
        }
        if (d.body_start < 0 || d.body_count < 0 || d.body_start + d.body_count > scene->n_bodies ||
            d.fixture_start < 0 || d.fixture_count < 0 || d.fixture_start + d.fixture_count > scene->n_fixtures ||
            d.contact_count < 0 || (d.contact_count > 0 && (!scene->contacts || d.contact_start < 0 ||
                                                            d.contact_start + d.contact_count > scene->n_contacts))) {
            delete b;
            return fail(GB_E_ARG, "world " + std::to_string(i) + ": ranges outside the scene arrays");
        }
        for (int k = 0; k < d.fixture_count; ++k) {
            const gb_fixture &f = scene->fixtures[d.fixture_start + k];
            if (f.body < 0 || f.body >= d.body_count || f.vertex_count < 1 || f.vertex_count > GB_MAX_POLY_VERTS ||
                f.shape_type == GB_SHAPE_LOOP || f.shape_type < 0 || f.shape_type > GB_SHAPE_EDGE ||
                ((f.flags & GB_FIX_LOOP_CHILD) && f.shape_type != GB_SHAPE_EDGE)) {
                delete b;
                return fail(GB_E_UNSUPPORTED, "world " + std::to_string(i) + " fixture " + std::to_string(k) +
                                                  ": unsupported shape or bad body index");
            }
        }
        if (d.move_count < 0 || d.move_count > d.fixture_count ||
            (d.move_count > 0 && (!scene->moves || d.move_start < 0 || d.move_start + d.move_count > scene->n_moves))) {
            delete b;
            return fail(GB_E_ARG, "world " + std::to_string(i) + ": bad move buffer range");
        }
        for (int k = 0; k < d.move_count; ++k) {
            int m = scene->moves[d.move_start + k];
            if (m < 0 || m >= d.fixture_count) {
                delete b;
                return fail(GB_E_ARG, "world " + std::to_string(i) + ": move buffer entry outside the world");
            }
        }
        // default slots: 6 per fixture; 10 for worlds run as a cooperative grid,
        // whose dense piles hold more fat-AABB pairs per fixture
        int per = d.body_count >= GB_HUGE_BODIES ? 10 : 6;
        int cap = d.contact_capacity > 0 ? d.contact_capacity : per * d.fixture_count;
        cap = std::max(std::max(cap, 64), d.contact_count + 16);
        WorldHdr &h = b->hdr[i];
        memset(&h, 0, sizeof(h));
        h.nb = d.body_count; h.nf = d.fixture_count; h.nc = d.contact_count; h.ccap = cap;
        h.bbase = d.body_start; h.fbase = d.fixture_start; h.cbase = cbase; h.pcap = d.fixture_count;
        h.flags = d.flags; h.status = 0;
        h.gx = d.gx; h.gy = d.gy; h.inv_dt0 = d.inv_dt0;
        h.nmove0 = d.move_count;
        cbase += cap;
    }
    b->ncap = cbase;
    // joints: sorted by world, bodies inside their world, known kinds
    if (scene->n_joints < 0 || (scene->n_joints > 0 && !scene->joints)) {
        delete b;
        return fail(GB_E_ARG, "bad joint array");
    }
    b->nj = scene->n_joints;
    b->joints.assign(scene->joints, scene->joints + b->nj);
    for (int i = 0; i < b->nj; ++i) {
        const gb_joint &J = b->joints[i];
        const bool ok = J.world >= 0 && J.world < b->nw && (i == 0 || J.world >= b->joints[i - 1].world) &&
                        J.body_a >= 0 && J.body_a < b->hdr[J.world].nb && J.body_b >= 0 && J.body_b < b->hdr[J.world].nb &&
                        (J.type == GB_JOINT_MOUSE ? J.body_a == J.body_b : J.body_a != J.body_b) &&
                        J.type >= GB_JOINT_REVOLUTE && J.type <= GB_JOINT_MOUSE;
        if (!ok) {
            delete b;
            return fail(J.type < GB_JOINT_REVOLUTE || J.type > GB_JOINT_MOUSE ? GB_E_UNSUPPORTED : GB_E_ARG,
                        "joint " + std::to_string(i) + ": world out of order, body outside its world or unknown type");
        }
        if (b->hdr[J.world].nj == 0) b->hdr[J.world].jbase = i;
        b->hdr[J.world].nj += 1;
    }
    // controllers: sorted by world, known kinds, body lists inside the scene
    // array and their bodies inside their world
    if (scene->n_controllers < 0 || scene->n_controller_bodies < 0 ||
        (scene->n_controllers > 0 && (!scene->controllers || (scene->n_controller_bodies > 0 && !scene->controller_bodies)))) {
        delete b;
        return fail(GB_E_ARG, "bad controller arrays");
    }
    b->nctl = scene->n_controllers;
    b->nctlb = scene->n_controllers > 0 ? scene->n_controller_bodies : 0;
    b->controllers.assign(scene->controllers, scene->controllers + b->nctl);
    for (int i = 0; i < b->nctl; ++i) {
        const gb_controller &C = b->controllers[i];
        bool ok = C.world >= 0 && C.world < b->nw && (i == 0 || C.world >= b->controllers[i - 1].world) &&
                  C.type >= GB_CONTROLLER_BUOYANCY && C.type <= GB_CONTROLLER_GRAVITY && C.body_start >= 0 &&
                  C.body_count >= 0 && C.body_start + C.body_count <= b->nctlb;
        for (int k = 0; ok && k < C.body_count; ++k) {
            const int bi = scene->controller_bodies[C.body_start + k];
            ok = bi >= 0 && bi < b->hdr[C.world].nb;
        }
        if (!ok) {
            delete b;
            return fail(C.type < GB_CONTROLLER_BUOYANCY || C.type > GB_CONTROLLER_GRAVITY ? GB_E_UNSUPPORTED : GB_E_ARG,
                        "controller " + std::to_string(i) + ": world out of order, unknown kind or body outside its world");
        }
        if (b->hdr[C.world].nctl == 0) b->hdr[C.world].ctlbase = i;
        b->hdr[C.world].nctl += 1;
    }
    b->launch_order.resize(b->nw);
    for (int i = 0; i < b->nw; ++i) b->launch_order[i] = i;
    std::stable_sort(b->launch_order.begin(), b->launch_order.end(),
                     [&](int x, int y) { return b->hdr[x].nb > b->hdr[y].nb; });
    Arena a;
    if (precision == GB_PREC_F64) carve(a, b->bd, b->nw, b->nb, b->nf, b->ncap, b->nj, b->nctl, b->nctlb);
    else carve(a, b->bf, b->nw, b->nb, b->nf, b->ncap, b->nj, b->nctl, b->nctlb);
    size_t bytes = a.off + 256;
    cudaError_t e = cudaMalloc((void **)&b->arena, bytes);
    if (e != cudaSuccess) { delete b; return cuda_fail(e, "cudaMalloc(arena)"); }
    b->arena_bytes = bytes;
    CK(cudaMemset(b->arena, 0, bytes));
    Arena a2;
    a2.base = b->arena;
    if (precision == GB_PREC_F64) carve(a2, b->bd, b->nw, b->nb, b->nf, b->ncap, b->nj, b->nctl, b->nctlb);
    else carve(a2, b->bf, b->nw, b->nb, b->nf, b->ncap, b->nj, b->nctl, b->nctlb);
    {
        std::vector<int> bw(std::max(1, b->nb), 0), cw(std::max(1, b->ncap), 0);
        for (int i = 0; i < b->nw; ++i) {
            for (int k = 0; k < b->hdr[i].nb; ++k) bw[b->hdr[i].bbase + k] = i;
            for (int k = 0; k < b->hdr[i].ccap; ++k) cw[b->hdr[i].cbase + k] = i;
        }
        // bodies outside every world keep world 0 but are never stepped
        int *d_bw = precision == GB_PREC_F64 ? b->bd.b_world : b->bf.b_world;
        int *d_cw = precision == GB_PREC_F64 ? b->bd.c_world : b->bf.c_world;
        if (b->nb > 0) CK(cudaMemcpy(d_bw, bw.data(), sizeof(int) * b->nb, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(d_cw, cw.data(), sizeof(int) * b->ncap, cudaMemcpyHostToDevice));
    }
    {
        // solver launches: worlds of GB_SOLVE_BIG_BODIES bodies or more (the
        // front of the size-sorted list) run in the wide launch; each launch's
        // shared-memory body cache fits its largest world, up to 2048 bodies
        int nbig = 0, max_big = 0, max_small = 0;
        for (int i : b->launch_order) {
            int n = b->hdr[i].nb;
            if (n >= GB_SOLVE_BIG_BODIES) { ++nbig; max_big = std::max(max_big, n); }
            else max_small = std::max(max_small, n);
        }
        for (auto *B : {&b->bd.cache_bodies, &b->bf.cache_bodies}) *B = 0;
        b->bd.n_big = b->bf.n_big = nbig;
        b->bd.cache_big = b->bf.cache_big = max_big <= 2048 ? max_big : 0;
        b->bd.cache_small = b->bf.cache_small = max_small;
        b->bd.pipe_bufs = b->bf.pipe_bufs = GB_SOLVE_PIPE_BUFS;
        b->bd.wait_polls = b->bf.wait_polls = GB_WAIT_POLLS;
        // the largest worlds run each phase as one cooperative grid
        int nh = 0;
        for (int i : b->launch_order)
            if (b->hdr[i].nb >= GB_HUGE_BODIES && nh < GB_MAX_HUGE) { b->bd.huge_ids[nh] = b->bf.huge_ids[nh] = i; ++nh; }
            else break;
        b->bd.n_huge = b->bf.n_huge = nh;
    }
    if (b->nj > 0) {
        // the joints and each body's joint list (Body.joints: World.joints order)
        std::vector<int> joff((size_t)b->nb + b->nw, 0), jadj(2 * (size_t)b->nj, 0);
        for (int w = 0; w < b->nw; ++w) {
            const WorldHdr &h = b->hdr[w];
            int *off = joff.data() + h.bbase + w;
            for (int k = 0; k < h.nj; ++k) {
                const gb_joint &J = b->joints[h.jbase + k];
                off[J.body_a + 1] += 1;
                if (J.body_b != J.body_a) off[J.body_b + 1] += 1;   // a mouse joint's one body lists it once
            }
            for (int k = 0; k < h.nb; ++k) off[k + 1] += off[k];
            std::vector<int> cur(off, off + h.nb);
            int *adj = jadj.data() + 2 * (size_t)h.jbase;
            for (int k = 0; k < h.nj; ++k) {
                const gb_joint &J = b->joints[h.jbase + k];
                adj[cur[J.body_a]++] = k;
                if (J.body_b != J.body_a) adj[cur[J.body_b]++] = k;
            }
        }
        const bool f64 = precision == GB_PREC_F64;
        CK(cudaMemcpy(f64 ? b->bd.j : b->bf.j, b->joints.data(), sizeof(gb_joint) * b->nj, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(f64 ? b->bd.b_joff : b->bf.b_joff, joff.data(), sizeof(int) * joff.size(), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(f64 ? b->bd.b_jadj : b->bf.b_jadj, jadj.data(), sizeof(int) * jadj.size(), cudaMemcpyHostToDevice));
    }
    if (b->nctl > 0) {
        const bool f64 = precision == GB_PREC_F64;
        CK(cudaMemcpy(f64 ? b->bd.ctl : b->bf.ctl, b->controllers.data(), sizeof(gb_controller) * b->nctl,
                      cudaMemcpyHostToDevice));
        if (b->nctlb > 0)
            CK(cudaMemcpy(f64 ? b->bd.ctl_bodies : b->bf.ctl_bodies, scene->controller_bodies, sizeof(int) * b->nctlb,
                          cudaMemcpyHostToDevice));
    }
    CK(cudaMalloc((void **)&b->d_worlds, sizeof(int) * b->nw));
    CK(cudaMemcpy(b->d_worlds, b->launch_order.data(), sizeof(int) * b->nw, cudaMemcpyHostToDevice));
    CK(cudaMalloc((void **)&b->d_bstage, sizeof(gb_body) * std::max(1, b->nb)));
    WorldHdr *d_hdr = precision == GB_PREC_F64 ? b->bd.hdr : b->bf.hdr;
    CK(cudaMemcpy(d_hdr, b->hdr.data(), sizeof(WorldHdr) * b->nw, cudaMemcpyHostToDevice));
    if (b->nb > 0) CK(cudaMemcpy(b->d_bstage, scene->bodies, sizeof(gb_body) * b->nb, cudaMemcpyHostToDevice));
    gb_fixture *d_fst = nullptr;
    CK(cudaMalloc((void **)&d_fst, sizeof(gb_fixture) * std::max(1, b->nf)));
    if (b->nf > 0) CK(cudaMemcpy(d_fst, scene->fixtures, sizeof(gb_fixture) * b->nf, cudaMemcpyHostToDevice));
    if (precision == GB_PREC_F64) {
        gb_launch_unpack_bodies<double>(b->bd, b->d_bstage, 0, b->nb, 0);
        gb_launch_unpack_fixtures<double>(b->bd, d_fst, b->nf, 0);
    } else {
        gb_launch_unpack_bodies<float>(b->bf, b->d_bstage, 0, b->nb, 0);
        gb_launch_unpack_fixtures<float>(b->bf, d_fst, b->nf, 0);
    }
    {
        // pending move buffers go to the front of each world's s_move slice
        std::vector<int> mv(std::max(1, b->nf), 0);
        bool any = false;
        for (int i = 0; i < b->nw; ++i) {
            const gb_world_desc &d = scene->worlds[i];
            for (int k = 0; k < d.move_count; ++k) { mv[d.fixture_start + k] = scene->moves[d.move_start + k]; any = true; }
        }
        int *d_move = precision == GB_PREC_F64 ? b->bd.s_move : b->bf.s_move;
        if (any) CK(cudaMemcpy(d_move, mv.data(), sizeof(int) * b->nf, cudaMemcpyHostToDevice));
    }
    if (scene->n_contacts > 0 && scene->contacts) {
        std::vector<gb_contact> hc;
        std::vector<int> slots;
        for (int i = 0; i < b->nw; ++i) {
            const gb_world_desc &d = scene->worlds[i];
            for (int k = 0; k < d.contact_count; ++k) {
                hc.push_back(scene->contacts[d.contact_start + k]);
                slots.push_back(b->hdr[i].cbase + k);
            }
        }
        if (!hc.empty()) {
            gb_contact *d_c = nullptr;
            int *d_s = nullptr;
            CK(cudaMalloc((void **)&d_c, sizeof(gb_contact) * hc.size()));
            CK(cudaMalloc((void **)&d_s, sizeof(int) * slots.size()));
            CK(cudaMemcpy(d_c, hc.data(), sizeof(gb_contact) * hc.size(), cudaMemcpyHostToDevice));
            CK(cudaMemcpy(d_s, slots.data(), sizeof(int) * slots.size(), cudaMemcpyHostToDevice));
            if (precision == GB_PREC_F64) {
                gb_launch_unpack_contacts<double>(b->bd, d_c, d_s, (int)hc.size(), 0);
                gb_launch_refresh_toi_cand<double>(b->bd, 0, b->bd.n_slots, 0);
            } else {
                gb_launch_unpack_contacts<float>(b->bf, d_c, d_s, (int)hc.size(), 0);
                gb_launch_refresh_toi_cand<float>(b->bf, 0, b->bf.n_slots, 0);
            }
            CK(cudaDeviceSynchronize());
            cudaFree(d_c);
            cudaFree(d_s);
        }
    }
    CK(cudaDeviceSynchronize());
    cudaFree(d_fst);
    {
        // the solver's side stream, at the lowest priority so the wide launch
        // on the caller's stream keeps first claim on freed SM resources
        int least = 0, greatest = 0;
        cudaDeviceGetStreamPriorityRange(&least, &greatest);
        if (cudaStreamCreateWithPriority(&b->side.s, cudaStreamNonBlocking, least) == cudaSuccess) {
            if (cudaEventCreateWithFlags(&b->side.fork, cudaEventDisableTiming) == cudaSuccess &&
                cudaEventCreateWithFlags(&b->side.join, cudaEventDisableTiming) == cudaSuccess)
                b->has_side = true;
        }
        (void)cudaGetLastError();   // without a side stream both solver launches share the caller's
    }
    *out = b;
    return 0;
}

int gb_batch_destroy(gb_batch *b) {
    if (!b) return 0;
    for (gb_graph *g : b->graphs) {
        if (g->exec) cudaGraphExecDestroy(g->exec);
        g->exec = nullptr;
        g->b = nullptr;
    }
    cudaFree(b->arena);
    cudaFree(b->d_worlds);
    cudaFree(b->d_bstage);
    cudaFree(b->d_cstage);
    if (b->ktimer) {
        for (int k = 0; k <= GB_NKTIME; ++k) cudaEventDestroy(b->ktimer->ev[k]);
        delete b->ktimer;
    }
    cudaFree(b->d_ev);
    cudaFree(b->d_ev_n);
    cudaFree(b->d_query);
    cudaFree(b->d_pf_off);
    cudaFree(b->d_pf);
    free_groups(b->groups);
    free_groups(b->chunks);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->has_side) {
        cudaEventDestroy(b->side.fork);
        cudaEventDestroy(b->side.join);
        cudaStreamDestroy(b->side.s);
    }
    delete b;
    return 0;
}

int gb_batch_step(gb_batch *b, const gb_step_opts *o, void *stream) {
    if (!b || !o) return fail(GB_E_ARG, "batch or opts is NULL");
    if (o->n_steps < 0 || o->vel_iters < 0 || o->pos_iters < 0) return fail(GB_E_ARG, "negative step count or iterations");
    cudaStream_t st = (cudaStream_t)stream;
    StepParams sp;
    sp.dt = o->dt;
    sp.inv_dt = o->dt > 0.0 ? 1.0 / o->dt : 0.0;
    sp.dt_ratio = 0.0;
    sp.vel_iters = o->vel_iters;
    sp.pos_iters = o->pos_iters;
    sp.record_order = o->record_order & 1;
    sp.profile = (o->record_order >> 1) & 1;
    sp.events = (o->record_order & GB_OPT_EVENTS) ? 1 : 0;
    sp.step_index = 0;
    int mode = 0, threads = 0;
    resolve_mapping(b, o, &mode, &threads);
    if (sp.events) {
        int rc = ensure_event_buffers(b);
        if (rc) return rc;
        CK(cudaMemsetAsync(b->d_ev_n, 0, sizeof(int) * b->nw, st));
    }
    if (threads % 32 || threads > 1024) return fail(GB_E_ARG, "block_threads must be a multiple of 32 up to 1024");
    KernelTimer *kt = nullptr;
    if ((o->record_order & GB_OPT_KERNEL_TIMES) && mode == 3) {
        if (!b->ktimer) {
            b->ktimer = new KernelTimer();
            memset(b->ktimer, 0, sizeof(KernelTimer));
            for (int k = 0; k <= GB_NKTIME; ++k) CK(cudaEventCreate(&b->ktimer->ev[k]));
        }
        kt = b->ktimer;
    }
    int rc = b->prec == GB_PREC_F64 ? run_steps<double>(b, b->bd, sp, o->n_steps, mode, threads, st, kt)
                                    : run_steps<float>(b, b->bf, sp, o->n_steps, mode, threads, st, kt);
    if (rc) return cuda_fail((cudaError_t)rc, "step launch");
    b->counters[0] += 1;
    b->counters[2] += o->n_steps;
    return 0;
}

int gb_batch_set_bodies(gb_batch *b, const gb_body *bodies, int32_t n, void *stream) {
    if (!b || !bodies) return fail(GB_E_ARG, "batch or bodies is NULL");
    if (n != b->nb) return fail(GB_E_ARG, "body count mismatch");
    cudaStream_t st = (cudaStream_t)stream;
    CK(cudaMemcpyAsync(b->d_bstage, bodies, sizeof(gb_body) * n, cudaMemcpyHostToDevice, st));
    // body types and bullet flags decide which contacts can take part in the TOI loop
    if (b->prec == GB_PREC_F64) {
        gb_launch_unpack_bodies<double>(b->bd, b->d_bstage, 0, n, st);
        gb_launch_refresh_toi_cand<double>(b->bd, 0, b->bd.n_slots, st);
    } else {
        gb_launch_unpack_bodies<float>(b->bf, b->d_bstage, 0, n, st);
        gb_launch_refresh_toi_cand<float>(b->bf, 0, b->bf.n_slots, st);
    }
    CK(cudaGetLastError());
    return 0;
}

int gb_batch_get_bodies(gb_batch *b, gb_body *bodies, int32_t n, void *stream) {
    if (!b || !bodies) return fail(GB_E_ARG, "batch or bodies is NULL");
    if (n != b->nb) return fail(GB_E_ARG, "body count mismatch");
    cudaStream_t st = (cudaStream_t)stream;
    if (b->prec == GB_PREC_F64) gb_launch_pack_bodies<double>(b->bd, b->d_bstage, 0, n, st);
    else gb_launch_pack_bodies<float>(b->bf, b->d_bstage, 0, n, st);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(bodies, b->d_bstage, sizeof(gb_body) * n, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return 0;
}

int gb_batch_get_proxies(gb_batch *b, double *aabbs, int32_t n, void *stream) {
    if (!b || !aabbs) return fail(GB_E_ARG, "batch or aabbs is NULL");
    if (n != b->nf) return fail(GB_E_ARG, "fixture count mismatch");
    cudaStream_t st = (cudaStream_t)stream;
    const dbox *src = b->prec == GB_PREC_F64 ? b->bd.f_aabb : b->bf.f_aabb;
    CK(cudaMemcpyAsync(aabbs, src, sizeof(dbox) * n, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return 0;
}

static int read_headers(gb_batch *b, std::vector<WorldHdr> &h, cudaStream_t st) {
    h.resize(b->nw);
    const WorldHdr *src = b->prec == GB_PREC_F64 ? b->bd.hdr : b->bf.hdr;
    CK(cudaMemcpyAsync(h.data(), src, sizeof(WorldHdr) * b->nw, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return 0;
}

int gb_batch_get_contact_counts(gb_batch *b, int32_t *counts, void *stream) {
    if (!b || !counts) return fail(GB_E_ARG, "batch or counts is NULL");
    std::vector<WorldHdr> h;
    int rc = read_headers(b, h, (cudaStream_t)stream);
    if (rc) return rc;
    for (int i = 0; i < b->nw; ++i) counts[i] = h[i].nc;
    return 0;
}

int gb_batch_get_contacts(gb_batch *b, int32_t world, gb_contact *out, int32_t capacity, int32_t *n_out, void *stream) {
    if (!b || !out || !n_out) return fail(GB_E_ARG, "NULL argument");
    if (world < 0 || world >= b->nw) return fail(GB_E_ARG, "world index out of range");
    cudaStream_t st = (cudaStream_t)stream;
    std::vector<WorldHdr> h;
    int rc = read_headers(b, h, st);
    if (rc) return rc;
    int n = h[world].nc;
    *n_out = n;
    if (n > capacity) return fail(GB_E_ARG, "capacity too small for the world's contacts");
    if (n == 0) return 0;
    if (b->cstage_cap < n) {
        cudaFree(b->d_cstage);
        b->d_cstage = nullptr;
        CK(cudaMalloc((void **)&b->d_cstage, sizeof(gb_contact) * n));
        b->cstage_cap = n;
    }
    if (b->prec == GB_PREC_F64) gb_launch_pack_contacts<double>(b->bd, b->d_cstage, h[world].cbase, n, st);
    else gb_launch_pack_contacts<float>(b->bf, b->d_cstage, h[world].cbase, n, st);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, b->d_cstage, sizeof(gb_contact) * n, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return 0;
}

int gb_batch_get_solver_order(gb_batch *b, int32_t world, int32_t *order, int32_t capacity, int32_t *n_out, void *stream) {
    if (!b || !order || !n_out) return fail(GB_E_ARG, "NULL argument");
    if (world < 0 || world >= b->nw) return fail(GB_E_ARG, "world index out of range");
    cudaStream_t st = (cudaStream_t)stream;
    std::vector<WorldHdr> h;
    int rc = read_headers(b, h, st);
    if (rc) return rc;
    int n = h[world].last_ncons;
    *n_out = n;
    if (n > capacity) return fail(GB_E_ARG, "capacity too small");
    const int *src = (b->prec == GB_PREC_F64 ? b->bd.order_out : b->bf.order_out) + h[world].cbase;
    if (n > 0) CK(cudaMemcpyAsync(order, src, sizeof(int) * n, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return 0;
}

int gb_batch_get_joint_order(gb_batch *b, int32_t world, int32_t *order, int32_t capacity, int32_t *n_out, void *stream) {
    if (!b || !order || !n_out) return fail(GB_E_ARG, "NULL argument");
    if (world < 0 || world >= b->nw) return fail(GB_E_ARG, "world out of range");
    cudaStream_t st = (cudaStream_t)stream;
    std::vector<WorldHdr> h;
    int rc = read_headers(b, h, st);
    if (rc) return rc;
    const int n = h[world].nj > 0 ? h[world].last_njcons : 0;
    *n_out = n;
    if (n > capacity) return fail(GB_E_ARG, "capacity too small");
    const int *src = (b->prec == GB_PREC_F64 ? b->bd.jorder_out : b->bf.jorder_out) + h[world].jbase;
    if (n > 0) CK(cudaMemcpyAsync(order, src, sizeof(int) * n, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return 0;
}

int gb_batch_get_joints(gb_batch *b, gb_joint *joints, int32_t n, void *stream) {
    if (!b || (!joints && n > 0)) return fail(GB_E_ARG, "NULL argument");
    if (n != b->nj) return fail(GB_E_ARG, "n_joints must equal the batch's joint count");
    cudaStream_t st = (cudaStream_t)stream;
    if (n > 0)
        CK(cudaMemcpyAsync(joints, b->prec == GB_PREC_F64 ? b->bd.j : b->bf.j, sizeof(gb_joint) * n, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return 0;
}

int gb_batch_set_joints(gb_batch *b, const gb_joint *joints, int32_t n, void *stream) {
    if (!b || (!joints && n > 0)) return fail(GB_E_ARG, "NULL argument");
    if (n != b->nj) return fail(GB_E_ARG, "n_joints must equal the batch's joint count");
    for (int i = 0; i < n; ++i) {
        const gb_joint &J = joints[i], &K = b->joints[i];
        if (J.world != K.world || J.type != K.type || J.body_a != K.body_a || J.body_b != K.body_b)
            return fail(GB_E_ARG, "joint " + std::to_string(i) + ": world, type and bodies are fixed for the batch");
    }
    cudaStream_t st = (cudaStream_t)stream;
    if (n > 0)
        CK(cudaMemcpyAsync(b->prec == GB_PREC_F64 ? b->bd.j : b->bf.j, joints, sizeof(gb_joint) * n, cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));
    return 0;
}

int gb_batch_set_controllers(gb_batch *b, const gb_controller *controllers, int32_t n, void *stream) {
    if (!b || (!controllers && n > 0)) return fail(GB_E_ARG, "NULL argument");
    if (n != b->nctl) return fail(GB_E_ARG, "n_controllers must equal the batch's controller count");
    for (int i = 0; i < n; ++i) {
        const gb_controller &C = controllers[i], &K = b->controllers[i];
        if (C.world != K.world || C.type != K.type || C.body_start != K.body_start || C.body_count != K.body_count)
            return fail(GB_E_ARG, "controller " + std::to_string(i) + ": world, kind and body list are fixed for the batch");
    }
    cudaStream_t st = (cudaStream_t)stream;
    if (n > 0)
        CK(cudaMemcpyAsync(b->prec == GB_PREC_F64 ? b->bd.ctl : b->bf.ctl, controllers, sizeof(gb_controller) * n,
                           cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));
    for (int i = 0; i < n; ++i) b->controllers[i] = controllers[i];
    return 0;
}

int gb_batch_set_pair_filter(gb_batch *b, int32_t world, const uint8_t *accept, int32_t n_fixtures, void *stream) {
    if (!b) return fail(GB_E_ARG, "batch is NULL");
    if (world < 0 || world >= b->nw) return fail(GB_E_ARG, "world index out of range");
    if (accept && n_fixtures != b->hdr[world].nf)
        return fail(GB_E_ARG, "n_fixtures must equal the world's fixture record count");
    if (accept && n_fixtures > GB_PAIR_FILTER_MAX_FIXTURES)
        return fail(GB_E_ARG, "a contact filter table holds at most GB_PAIR_FILTER_MAX_FIXTURES fixture records");
    if (!b->graphs.empty())
        return fail(GB_E_UNSUPPORTED, "captured rollouts keep the batch's contact filter tables: destroy them first");
    cudaStream_t st = (cudaStream_t)stream;
    if (b->pf.empty()) b->pf.resize(b->nw);
    if (accept) b->pf[world].assign(accept, accept + (size_t)n_fixtures * (size_t)n_fixtures);
    else b->pf[world].clear();
    std::vector<long long> off(b->nw, -1);
    size_t total = 0;
    for (int i = 0; i < b->nw; ++i)
        if (!b->pf[i].empty()) { off[i] = (long long)total; total += b->pf[i].size(); }
    CK(cudaStreamSynchronize(st));
    CK(cudaDeviceSynchronize());   // steps on other streams may still read the old tables
    cudaFree(b->d_pf);
    b->d_pf = nullptr;
    if (!b->d_pf_off) CK(cudaMalloc((void **)&b->d_pf_off, sizeof(long long) * b->nw));
    if (total) {
        CK(cudaMalloc((void **)&b->d_pf, total));
        for (int i = 0; i < b->nw; ++i)
            if (!b->pf[i].empty()) CK(cudaMemcpy(b->d_pf + off[i], b->pf[i].data(), b->pf[i].size(), cudaMemcpyHostToDevice));
    }
    CK(cudaMemcpy(b->d_pf_off, off.data(), sizeof(long long) * b->nw, cudaMemcpyHostToDevice));
    const long long *po = total ? b->d_pf_off : nullptr;
    b->bd.pf_off = b->bf.pf_off = po;
    b->bd.pf_accept = b->bf.pf_accept = b->d_pf;
    return 0;
}

int gb_batch_get_step_record(gb_batch *b, int32_t world, int32_t *out, int32_t capacity, int32_t *n_out, void *stream) {
    if (!b || !out || !n_out) return fail(GB_E_ARG, "NULL argument");
    if (world < 0 || world >= b->nw) return fail(GB_E_ARG, "world index out of range");
    const WorldHdr &h = b->hdr[world];
    *n_out = h.nb;
    if (2 * h.nb > capacity) return fail(GB_E_ARG, "capacity too small: 2 ints per body of the world");
    cudaStream_t st = (cudaStream_t)stream;
    const int *src = (b->prec == GB_PREC_F64 ? b->bd.rec : b->bf.rec) + h.bbase;
    const int *isl = (b->prec == GB_PREC_F64 ? b->bd.rec_island : b->bf.rec_island) + h.bbase;
    if (h.nb > 0) CK(cudaMemcpyAsync(out, src, sizeof(int) * h.nb, cudaMemcpyDeviceToHost, st));
    if (h.nb > 0) CK(cudaMemcpyAsync(out + h.nb, isl, sizeof(int) * h.nb, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return 0;
}

int gb_batch_set_wait_polls(gb_batch *b, int32_t polls) {
    if (!b) return fail(GB_E_ARG, "batch is NULL");
    if (polls < 0) return fail(GB_E_ARG, "polls must be >= 0");
    b->bd.wait_polls = b->bf.wait_polls = polls;
    return 0;
}

int gb_batch_clear_status(gb_batch *b, void *stream) {
    if (!b) return fail(GB_E_ARG, "batch is NULL");
    WorldHdr *d = b->prec == GB_PREC_F64 ? b->bd.hdr : b->bf.hdr;
    cudaStream_t st = (cudaStream_t)stream;
    // status is a 32-bit field of every header: clear it in place
    for (int i = 0; i < b->nw; ++i)
        CK(cudaMemsetAsync(reinterpret_cast<char *>(d + i) + offsetof(WorldHdr, status), 0, sizeof(uint32_t), st));
    CK(cudaStreamSynchronize(st));
    return 0;
}

int gb_batch_status(gb_batch *b, uint32_t *status, void *stream) {
    if (!b || !status) return fail(GB_E_ARG, "NULL argument");
    std::vector<WorldHdr> h;
    int rc = read_headers(b, h, (cudaStream_t)stream);
    if (rc) return rc;
    for (int i = 0; i < b->nw; ++i) status[i] = h[i].status;
    return 0;
}

int gb_batch_phase_clocks(gb_batch *b, int64_t *clocks, void *stream) {
    if (!b || !clocks) return fail(GB_E_ARG, "NULL argument");
    const long long *src = b->prec == GB_PREC_F64 ? b->bd.prof : b->bf.prof;
    CK(cudaMemcpyAsync(clocks, src, sizeof(long long) * (size_t)b->nw * GB_NPROF, cudaMemcpyDeviceToHost, (cudaStream_t)stream));
    CK(cudaStreamSynchronize((cudaStream_t)stream));
    return 0;
}

int gb_batch_get_events(gb_batch *b, int32_t world, gb_event *out, int32_t capacity, int32_t *n_out, void *stream) {
    if (!b || !out || !n_out) return fail(GB_E_ARG, "NULL argument");
    if (world < 0 || world >= b->nw) return fail(GB_E_ARG, "world index out of range");
    *n_out = 0;
    if (!b->d_ev) return 0;
    cudaStream_t st = (cudaStream_t)stream;
    int n = 0;
    CK(cudaMemcpyAsync(&n, b->d_ev_n + world, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    const WorldHdr &h = b->hdr[world];
    n = std::min(n, 3 * h.ccap + 64);
    *n_out = n;
    if (n > capacity) return fail(GB_E_ARG, "capacity too small for the world's events");
    if (n > 0) {
        CK(cudaMemcpyAsync(out, b->d_ev + 3 * (size_t)h.cbase + 64 * (size_t)world, sizeof(gb_event) * n,
                           cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
    }
    return 0;
}

int gb_batch_kernel_times(gb_batch *b, double *total_ms, int32_t capacity, int32_t *n_slots, int64_t *n_steps) {
    if (!b || !total_ms || !n_slots || !n_steps) return fail(GB_E_ARG, "NULL argument");
    *n_slots = GB_NKTIME;
    *n_steps = b->ktimer ? b->ktimer->steps : 0;
    for (int k = 0; k < GB_NKTIME && k < capacity; ++k) total_ms[k] = b->ktimer ? b->ktimer->total_ms[k] : 0.0;
    return 0;
}

int gb_batch_counters(gb_batch *b, int64_t *c) {
    if (!b || !c) return fail(GB_E_ARG, "NULL argument");
    c[0] = b->counters[0];
    c[1] = (int64_t)b->arena_bytes;
    c[2] = b->counters[2];
    return 0;
}

}  // extern "C"

// ------------------------------------------------------------------------
// Launch configurations, the autotuner and captured rollouts.
static_assert(sizeof(gb_launch_config) == GB_LAUNCH_CONFIG_BYTES, "gb_launch_config layout");
namespace {
StepParams params_of(const gb_step_opts *o) {
    StepParams sp;
    sp.dt = o->dt;
    sp.inv_dt = o->dt > 0.0 ? 1.0 / o->dt : 0.0;
    sp.dt_ratio = 0.0;
    sp.vel_iters = o->vel_iters;
    sp.pos_iters = o->pos_iters;
    sp.record_order = o->record_order & 1;
    sp.profile = (o->record_order >> 1) & 1;
    sp.events = (o->record_order & GB_OPT_EVENTS) ? 1 : 0;
    sp.step_index = 0;
    return sp;
}

// The batch as group k's launch sequence sees it: its bodies and contact
// slots, its first-pass TOI list counter, its wide-launch worlds.
template <class R> Batch<R> group_view(const Batch<R> &B, const WorldGroup &g, int k) {
    Batch<R> G = B;
    G.n_bodies = g.nb; G.body0 = g.b0;
    G.n_slots = g.ns; G.slot0 = g.s0;
    G.toi_n = B.toi_n + k;
    G.n_big = g.nbig;
    G.n_huge = 0;
    return G;
}

// n_steps steps of every world on `st`: one launch sequence over the whole
// batch, or (phased launch, world groups) one per group, each on the group's
// stream, forked from and joined back into `st` (also under stream capture).
template <class R> int run_steps(gb_batch *b, const Batch<R> &B, const StepParams &sp, int n_steps, int mode, int threads,
                                 cudaStream_t st, KernelTimer *kt) {
    if (mode != 3 || kt || b->groups.size() < 2) {
        const SideStream *side = b->has_side ? &b->side : nullptr;
        return gb_launch_step<R>(B, sp, n_steps, b->d_worlds, b->nw, mode, threads, st, kt, side);
    }
    cudaError_t e = cudaEventRecord(b->fork, st);
    for (size_t k = 0; k < b->groups.size() && e == cudaSuccess; ++k) {
        const WorldGroup &g = b->groups[k];
        e = cudaStreamWaitEvent(g.st, b->fork, 0);
        if (e != cudaSuccess) break;
        const int rc = gb_launch_step<R>(group_view(B, g, (int)k), sp, n_steps, g.d_worlds, g.n_list, mode, threads, g.st,
                                         nullptr, nullptr);
        if (rc) return rc;
        e = cudaEventRecord(g.done, g.st);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(st, g.done, 0);
    }
    return (int)e;
}

int launch_steps(gb_batch *b, const StepParams &sp, int n_steps, int mode, int threads, cudaStream_t st) {
    return b->prec == GB_PREC_F64 ? run_steps<double>(b, b->bd, sp, n_steps, mode, threads, st, nullptr)
                                  : run_steps<float>(b, b->bf, sp, n_steps, mode, threads, st, nullptr);
}

void free_groups(std::vector<WorldGroup> &groups) {
    for (WorldGroup &g : groups) {
        cudaFree(g.d_worlds);
        if (g.done) cudaEventDestroy(g.done);
        if (g.st) cudaStreamDestroy(g.st);
    }
    groups.clear();
}

// Split the worlds into n runs of about equal body counts (n = 1: none).
int build_groups(gb_batch *b, int n, int big_from, std::vector<WorldGroup> &groups) {
    free_groups(groups);
    n = std::min(n, b->nw);
    if (n < 2) return 0;
    if (!b->fork) CK(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
    long long total = 0;
    for (int i = 0; i < b->nw; ++i) total += b->hdr[i].nb;
    int w = 0;
    long long acc = 0;
    for (int k = 0; k < n; ++k) {
        WorldGroup g;
        g.w0 = w;
        const long long target = total * (k + 1) / n;
        const int last = b->nw - (n - 1 - k);   // leave a world for each later group
        do { acc += b->hdr[w].nb; ++w; } while (w < last && acc < target);
        if (k == n - 1) w = b->nw;
        g.w1 = w;
        const WorldHdr &f = b->hdr[g.w0], &l = b->hdr[g.w1 - 1];
        g.b0 = f.bbase; g.nb = l.bbase + l.nb - f.bbase;
        g.s0 = f.cbase; g.ns = l.cbase + l.ccap - f.cbase;
        std::vector<int> list;
        for (int i : b->launch_order)
            if (i >= g.w0 && i < g.w1) list.push_back(i);
        g.n_list = (int)list.size();
        for (int i : list) g.nbig += b->hdr[i].nb >= big_from ? 1 : 0;
        CK(cudaMalloc((void **)&g.d_worlds, sizeof(int) * list.size()));
        CK(cudaMemcpy(g.d_worlds, list.data(), sizeof(int) * list.size(), cudaMemcpyHostToDevice));
        CK(cudaStreamCreateWithFlags(&g.st, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&g.done, cudaEventDisableTiming));
        groups.push_back(g);
    }
    return 0;
}

int make_groups(gb_batch *b, int n, int big_from) { return build_groups(b, n, big_from, b->groups); }

bool has_grid_worlds(const gb_batch *b) { return (b->prec == GB_PREC_F64 ? b->bd.n_huge : b->bf.n_huge) > 0; }

// Check a launch configuration against the batch and, with `apply`, make it
// the batch's: the wide solver launch takes the worlds of big_bodies bodies
// or more (the front of the size-sorted list), and each solver launch's
// shared-memory body cache fits its largest world up to 2048 bodies.
int apply_config(gb_batch *b, const gb_launch_config &c, bool apply) {
    if (c.launch_mode < 1 || c.launch_mode > 3) return fail(GB_E_ARG, "launch_mode must be 1, 2 or 3");
    if (c.block_threads < 32 || c.block_threads > 1024 || c.block_threads % 32)
        return fail(GB_E_ARG, "block_threads must be a multiple of 32 from 32 to 1024");
    if (c.pipe_bufs < 0 || c.pipe_bufs > GB_CFG_MAX_PIPE_BUFS) return fail(GB_E_ARG, "pipe_bufs must be 0 to 4");
    if (c.big_bodies < 1) return fail(GB_E_ARG, "big_bodies must be positive");
    if (c.groups < 1 || c.groups > GB_MAX_GROUPS) return fail(GB_E_ARG, "groups must be 1 to 8");
    if (c.groups > 1 && (c.launch_mode != 3 || has_grid_worlds(b)))
        return fail(GB_E_UNSUPPORTED, "world groups run the phased launch (mode 3) of batches without cooperative-grid worlds");
    if (c.launch_mode != 3 && has_grid_worlds(b))
        return fail(GB_E_UNSUPPORTED, "worlds of 16384 bodies or more run only in the phased launch (mode 3)");
    // worlds run as a cooperative grid (the front of the list) always count
    // as big, so the per-world solver launches never take them
    const int big_from = std::min(c.big_bodies, (int)GB_HUGE_BODIES);
    int nbig = 0, max_big = 0, max_small = 0;
    for (int i : b->launch_order) {
        int n = b->hdr[i].nb;
        if (n >= big_from) { ++nbig; max_big = std::max(max_big, n); }
        else max_small = std::max(max_small, n);
    }
    const int cache_big = max_big <= 2048 ? max_big : 0, cache_small = max_small <= 2048 ? max_small : 0;
    if (c.launch_mode == 3) {
        int dev = 0, optin = 0;
        CK(cudaGetDevice(&dev));
        CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
        const int t_small = std::min(c.block_threads, 256);
        auto smem = [&](int cache, int threads) -> size_t {
            if (cache <= 0) return 0;
            return b->prec == GB_PREC_F64 ? gb_solve_smem<double>(cache, threads, c.pipe_bufs)
                                          : gb_solve_smem<float>(cache, threads, c.pipe_bufs);
        };
        const size_t need = std::max(smem(cache_big, GB_SOLVE_BIG_THREADS), smem(cache_small, t_small));
        if (need > (size_t)optin)
            return fail(GB_E_ARG, "configuration needs " + std::to_string(need) + " bytes of shared memory per CTA; the device allows " +
                                      std::to_string(optin));
    }
    if (!apply) return 0;
    const int grc = make_groups(b, c.groups, big_from);
    if (grc) return grc;
    for (Batch<double> *B : {&b->bd}) { B->n_big = nbig; B->cache_big = cache_big; B->cache_small = cache_small; B->pipe_bufs = c.pipe_bufs; }
    for (Batch<float> *B : {&b->bf}) { B->n_big = nbig; B->cache_big = cache_big; B->cache_small = cache_small; B->pipe_bufs = c.pipe_bufs; }
    b->cfg = c;
    return 0;
}
}  // namespace

extern "C" {

int gb_batch_set_launch_config(gb_batch *b, const gb_launch_config *cfg) {
    if (!b || !cfg) return fail(GB_E_ARG, "batch or cfg is NULL");
    gb_launch_config c = *cfg;
    c.ms_per_step = 0.0;
    return apply_config(b, c, true);
}

int gb_batch_get_launch_config(gb_batch *b, gb_launch_config *cfg) {
    if (!b || !cfg) return fail(GB_E_ARG, "batch or cfg is NULL");
    *cfg = b->cfg;
    return 0;
}

int gb_batch_autotune(gb_batch *b, const gb_step_opts *o, gb_launch_config *trials, int32_t capacity, int32_t *n_out,
                      gb_launch_config *best, void *stream) {
    if (!b || !o) return fail(GB_E_ARG, "batch or opts is NULL");
    if (o->n_steps < 1 || o->vel_iters < 0 || o->pos_iters < 0)
        return fail(GB_E_ARG, "autotune needs n_steps >= 1 and non-negative iterations");
    if (o->record_order != 0) return fail(GB_E_ARG, "autotune steps record nothing: record_order must be 0");
    if (capacity < 0 || (capacity > 0 && !trials)) return fail(GB_E_ARG, "trials is NULL");
    cudaStream_t st = (cudaStream_t)stream;
    const StepParams sp = params_of(o);
    const gb_launch_config start = b->cfg;
    char *snap = nullptr;
    CK(cudaMalloc((void **)&snap, b->arena_bytes));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        if (e0) cudaEventDestroy(e0);
        cudaFree(snap);
        return fail(GB_E_CUDA, "cudaEventCreate");
    }
    int err = 0;
    cudaError_t ce = cudaMemcpyAsync(snap, b->arena, b->arena_bytes, cudaMemcpyDeviceToDevice, st);
    if (ce != cudaSuccess) err = cuda_fail(ce, "autotune: copy of the arena");
    std::vector<gb_launch_config> log;
    gb_launch_config best_c = start;
    best_c.ms_per_step = -1.0;
    // the status words the trials start from (they are part of the saved state)
    std::vector<WorldHdr> h0, h1;
    if (!err) err = read_headers(b, h0, st);
    // one trial: from the saved state, an untimed run (first launches load
    // their kernels), then the timed run from the saved state again
    auto trial = [&](gb_launch_config c) {
        c.ms_per_step = -1.0;
        if (err) return;
        if (apply_config(b, c, true) == 0) {
            float ms = 0.0f;
            int rc = 0;
            for (int pass = 0; pass < 2 && rc == 0; ++pass) {
                rc = (int)cudaMemcpyAsync(b->arena, snap, b->arena_bytes, cudaMemcpyDeviceToDevice, st);
                if (rc == 0) rc = (int)cudaEventRecord(e0, st);
                if (rc == 0) rc = launch_steps(b, sp, o->n_steps, c.launch_mode, c.block_threads, st);
                if (rc == 0) rc = (int)cudaEventRecord(e1, st);
                if (rc == 0) rc = (int)cudaEventSynchronize(e1);
                if (rc == 0) rc = (int)cudaEventElapsedTime(&ms, e0, e1);
            }
            if (rc != 0) err = cuda_fail((cudaError_t)rc, "autotune trial");
            else c.ms_per_step = (double)ms / o->n_steps;
            // a trial whose steps raised a status bit (a wait that gave up
            // ends its solve early, an overflow drops work) is not a candidate
            if (!err && (err = read_headers(b, h1, st)) == 0)
                for (int i = 0; i < b->nw; ++i)
                    if (h1[i].status != h0[i].status) { c.ms_per_step = -2.0; break; }
        }
        log.push_back(c);
        if (c.ms_per_step >= 0.0 && (best_c.ms_per_step < 0.0 || c.ms_per_step < best_c.ms_per_step)) best_c = c;
    };
    // stage 1: world-to-thread mapping
    {
        std::vector<std::pair<int, int>> maps = {{3, 32}, {3, 64}, {3, 128}};
        if (!has_grid_worlds(b)) {
            maps.push_back({1, 128}); maps.push_back({1, 256});
            maps.push_back({2, 64}); maps.push_back({2, 128});
        }
        for (auto &m : maps) {
            gb_launch_config c = start;
            c.launch_mode = m.first;
            c.block_threads = m.second;
            if (c.launch_mode != 3) c.groups = 1;
            trial(c);
        }
    }
    // stages 2 and 3 (phased launch): wide-launch threshold, then chunk buffers
    if (!err && best_c.ms_per_step >= 0.0 && best_c.launch_mode == 3) {
        const gb_launch_config base = best_c;
        for (int bb : {256, 512, 1024, 2048, 1 << 30})
            if (bb != base.big_bodies) { gb_launch_config c = base; c.big_bodies = bb; trial(c); }
    }
    if (!err && best_c.ms_per_step >= 0.0 && best_c.launch_mode == 3) {
        const gb_launch_config base = best_c;
        for (int pb = 0; pb <= GB_CFG_MAX_PIPE_BUFS; ++pb)
            if (pb != base.pipe_bufs) { gb_launch_config c = base; c.pipe_bufs = pb; trial(c); }
    }
    // stage 4 (phased launch without cooperative-grid worlds): world groups
    if (!err && best_c.ms_per_step >= 0.0 && best_c.launch_mode == 3 && !has_grid_worlds(b)) {
        const gb_launch_config base = best_c;
        for (int ng : {1, 2, 3, 4})
            if (ng != base.groups && ng <= b->nw) { gb_launch_config c = base; c.groups = ng; trial(c); }
    }
    // the best configuration stays; the state goes back to the saved one
    const bool found = !err && best_c.ms_per_step >= 0.0;
    apply_config(b, found ? best_c : start, true);
    if (found) b->cfg.ms_per_step = best_c.ms_per_step;
    ce = cudaMemcpyAsync(b->arena, snap, b->arena_bytes, cudaMemcpyDeviceToDevice, st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(snap);
    if (err) return err;
    if (ce != cudaSuccess) return cuda_fail(ce, "autotune: restoring the arena");
    if (!found) return fail(GB_E_ARG, "autotune: no candidate configuration could run on this batch");
    if (n_out) *n_out = (int32_t)log.size();
    for (int k = 0; k < capacity && k < (int)log.size(); ++k) trials[k] = log[k];
    if (best) *best = b->cfg;
    return 0;
}

int gb_graph_capture(gb_batch *b, const gb_step_opts *o, gb_graph **out) {
    if (!b || !o || !out) return fail(GB_E_ARG, "batch, opts or out is NULL");
    *out = nullptr;
    if (o->n_steps < 1 || o->vel_iters < 0 || o->pos_iters < 0)
        return fail(GB_E_ARG, "graph capture needs n_steps >= 1 and non-negative iterations");
    if (o->record_order & GB_OPT_KERNEL_TIMES) return fail(GB_E_UNSUPPORTED, "per-launch timing waits on the host and is not captured");
    int mode = 0, threads = 0;
    resolve_mapping(b, o, &mode, &threads);
    if (mode != 3) return fail(GB_E_UNSUPPORTED, "only the phased launch (mode 3) is captured");
    if (has_grid_worlds(b)) return fail(GB_E_UNSUPPORTED, "worlds of 16384 bodies or more (cooperative launches) are not captured");
    if (threads % 32 || threads > 1024) return fail(GB_E_ARG, "block_threads must be a multiple of 32 up to 1024");
    const StepParams sp = params_of(o);
    if (sp.events) {
        int rc = ensure_event_buffers(b);
        if (rc) return rc;
    }
    cudaStream_t cs = nullptr;
    CK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) { cudaStreamDestroy(cs); return cuda_fail(e, "cudaStreamBeginCapture"); }
    int rc = 0;
    if (sp.events) rc = (int)cudaMemsetAsync(b->d_ev_n, 0, sizeof(int) * b->nw, cs);
    if (rc == 0) rc = launch_steps(b, sp, o->n_steps, mode, threads, cs);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(cs, &g);
    cudaStreamDestroy(cs);
    if (rc != 0 || e != cudaSuccess || !g) {
        if (g) cudaGraphDestroy(g);
        (void)cudaGetLastError();
        return cuda_fail(rc != 0 ? (cudaError_t)rc : (e != cudaSuccess ? e : cudaErrorStreamCaptureInvalidated), "graph capture");
    }
    cudaGraphExec_t ex = nullptr;
    e = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
    gb_graph *gr = new gb_graph;
    gr->b = b;
    gr->exec = ex;
    gr->n_steps = o->n_steps;
    b->graphs.push_back(gr);
    *out = gr;
    return 0;
}

int gb_graph_launch(gb_graph *g, void *stream) {
    if (!g) return fail(GB_E_ARG, "graph is NULL");
    if (!g->b || !g->exec) return fail(GB_E_ARG, "the graph's batch was destroyed");
    CK(cudaGraphLaunch(g->exec, (cudaStream_t)stream));
    g->b->counters[0] += 1;
    g->b->counters[2] += g->n_steps;
    return 0;
}

}  // extern "C"

namespace {
// device staging of at least `bytes` for the query entry points
int query_staging(gb_batch *b, size_t bytes, cudaStream_t st) {
    if (bytes <= b->query_bytes) return 0;
    CK(cudaStreamSynchronize(st));
    cudaFree(b->d_query);
    b->d_query = nullptr;
    b->query_bytes = 0;
    bytes = std::max(bytes, (size_t)1 << 20);
    CK(cudaMalloc((void **)&b->d_query, bytes));
    b->query_bytes = bytes;
    return 0;
}
size_t up256(size_t x) { return (x + 255) & ~(size_t)255; }
// rays name a world of the batch and have a length (dynamictree.py:222-224 raises otherwise)
int check_rays(const gb_batch *b, const gb_ray *rays, int n) {
    for (int i = 0; i < n; ++i) {
        const gb_ray &r = rays[i];
        if (r.world < 0 || r.world >= b->nw) return fail(GB_E_ARG, "ray " + std::to_string(i) + ": world out of range");
        const double dx = r.p2x - r.p1x, dy = r.p2y - r.p1y;
        if (!(dx * dx + dy * dy > 0.0)) return fail(GB_E_ARG, "ray " + std::to_string(i) + ": p2 - p1 has no length");
    }
    return 0;
}
}  // namespace

extern "C" {

int gb_batch_ray_cast(gb_batch *b, const gb_ray *rays, int32_t n, gb_ray_hit *hits, void *stream) {
    if (!b) return fail(GB_E_ARG, "batch is NULL");
    if (n < 0) return fail(GB_E_ARG, "negative ray count");
    if (n == 0) return 0;
    if (!rays || !hits) return fail(GB_E_ARG, "rays or hits is NULL");
    int rc = check_rays(b, rays, n);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const size_t in_b = up256(sizeof(gb_ray) * (size_t)n), out_b = sizeof(gb_ray_hit) * (size_t)n;
    rc = query_staging(b, in_b + out_b, st);
    if (rc) return rc;
    gb_ray *d_rays = reinterpret_cast<gb_ray *>(b->d_query);
    gb_ray_hit *d_hits = reinterpret_cast<gb_ray_hit *>(b->d_query + in_b);
    CK(cudaMemcpyAsync(d_rays, rays, sizeof(gb_ray) * (size_t)n, cudaMemcpyHostToDevice, st));
    if (b->prec == GB_PREC_F64) gb_launch_ray_cast<double>(b->bd, d_rays, n, d_hits, st);
    else gb_launch_ray_cast<float>(b->bf, d_rays, n, d_hits, st);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(hits, d_hits, out_b, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return 0;
}

int gb_batch_ray_cast_all(gb_batch *b, const gb_ray *rays, int32_t n, gb_ray_hit *hits, int32_t cap, int32_t *counts,
                          void *stream) {
    if (!b) return fail(GB_E_ARG, "batch is NULL");
    if (n < 0 || cap < 0) return fail(GB_E_ARG, "negative ray count or capacity");
    if (n == 0) return 0;
    if (!rays || !counts || (cap > 0 && !hits)) return fail(GB_E_ARG, "rays, hits or counts is NULL");
    int rc = check_rays(b, rays, n);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const size_t in_b = up256(sizeof(gb_ray) * (size_t)n), cnt_b = up256(sizeof(int) * (size_t)n);
    const size_t out_b = sizeof(gb_ray_hit) * (size_t)n * (size_t)cap;
    rc = query_staging(b, in_b + cnt_b + out_b, st);
    if (rc) return rc;
    gb_ray *d_rays = reinterpret_cast<gb_ray *>(b->d_query);
    int *d_cnt = reinterpret_cast<int *>(b->d_query + in_b);
    gb_ray_hit *d_hits = reinterpret_cast<gb_ray_hit *>(b->d_query + in_b + cnt_b);
    CK(cudaMemcpyAsync(d_rays, rays, sizeof(gb_ray) * (size_t)n, cudaMemcpyHostToDevice, st));
    if (b->prec == GB_PREC_F64) gb_launch_ray_cast_all<double>(b->bd, d_rays, n, d_hits, cap, d_cnt, st);
    else gb_launch_ray_cast_all<float>(b->bf, d_rays, n, d_hits, cap, d_cnt, st);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(counts, d_cnt, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost, st));
    if (out_b) CK(cudaMemcpyAsync(hits, d_hits, out_b, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return 0;
}

int gb_batch_query_aabb(gb_batch *b, const gb_aabb_query *qs, int32_t n, int32_t *fixtures, int32_t cap, int32_t *counts,
                        void *stream) {
    if (!b) return fail(GB_E_ARG, "batch is NULL");
    if (n < 0 || cap < 0) return fail(GB_E_ARG, "negative query count or capacity");
    if (n == 0) return 0;
    if (!qs || !counts || (cap > 0 && !fixtures)) return fail(GB_E_ARG, "queries, fixtures or counts is NULL");
    for (int i = 0; i < n; ++i)
        if (qs[i].world < 0 || qs[i].world >= b->nw) return fail(GB_E_ARG, "query " + std::to_string(i) + ": world out of range");
    cudaStream_t st = (cudaStream_t)stream;
    const size_t in_b = up256(sizeof(gb_aabb_query) * (size_t)n), cnt_b = up256(sizeof(int) * (size_t)n);
    const size_t out_b = sizeof(int) * (size_t)n * (size_t)cap;
    int rc = query_staging(b, in_b + cnt_b + out_b, st);
    if (rc) return rc;
    gb_aabb_query *d_q = reinterpret_cast<gb_aabb_query *>(b->d_query);
    int *d_cnt = reinterpret_cast<int *>(b->d_query + in_b);
    int *d_out = reinterpret_cast<int *>(b->d_query + in_b + cnt_b);
    CK(cudaMemcpyAsync(d_q, qs, sizeof(gb_aabb_query) * (size_t)n, cudaMemcpyHostToDevice, st));
    if (b->prec == GB_PREC_F64) gb_launch_query_aabb<double>(b->bd, d_q, n, d_out, cap, d_cnt, st);
    else gb_launch_query_aabb<float>(b->bf, d_q, n, d_out, cap, d_cnt, st);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(counts, d_cnt, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost, st));
    if (out_b) CK(cudaMemcpyAsync(fixtures, d_out, out_b, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return 0;
}

// ------------------------------------------------------------------------
// Snapshots: a 64-byte header naming the layout, then the arena.
namespace {
struct SnapHeader {
    char magic[8];
    int32_t precision, n_worlds, n_bodies, n_fixtures, n_slots, _pad;
    uint64_t arena_bytes;
    char _rest[GB_SNAPSHOT_HEADER_BYTES - 8 - 6 * 4 - 8];
};
static_assert(sizeof(SnapHeader) == GB_SNAPSHOT_HEADER_BYTES, "snapshot header layout");
SnapHeader snap_header(const gb_batch *b) {
    SnapHeader h;
    memset(&h, 0, sizeof(h));
    memcpy(h.magic, "GB2DSNP1", 8);
    h.precision = b->prec; h.n_worlds = b->nw; h.n_bodies = b->nb; h.n_fixtures = b->nf; h.n_slots = b->ncap;
    h.arena_bytes = b->arena_bytes;
    return h;
}
}  // namespace

int gb_batch_snapshot_bytes(gb_batch *b, uint64_t *bytes) {
    if (!b || !bytes) return fail(GB_E_ARG, "batch or bytes is NULL");
    *bytes = GB_SNAPSHOT_HEADER_BYTES + (uint64_t)b->arena_bytes;
    return 0;
}

int gb_batch_snapshot(gb_batch *b, void *dst, uint64_t bytes, void *stream) {
    if (!b || !dst) return fail(GB_E_ARG, "batch or dst is NULL");
    if (bytes < GB_SNAPSHOT_HEADER_BYTES + (uint64_t)b->arena_bytes)
        return fail(GB_E_ARG, "snapshot buffer too small (see gb_batch_snapshot_bytes)");
    cudaStream_t st = (cudaStream_t)stream;
    const SnapHeader h = snap_header(b);
    char *d = static_cast<char *>(dst);
    CK(cudaMemcpyAsync(d, &h, sizeof(h), cudaMemcpyDefault, st));
    CK(cudaMemcpyAsync(d + GB_SNAPSHOT_HEADER_BYTES, b->arena, b->arena_bytes, cudaMemcpyDefault, st));
    CK(cudaStreamSynchronize(st));   // `h` lives on this stack frame
    return 0;
}

int gb_batch_restore(gb_batch *b, const void *src, uint64_t bytes, void *stream) {
    if (!b || !src) return fail(GB_E_ARG, "batch or src is NULL");
    if (bytes < GB_SNAPSHOT_HEADER_BYTES + (uint64_t)b->arena_bytes)
        return fail(GB_E_ARG, "snapshot too small for this batch");
    cudaStream_t st = (cudaStream_t)stream;
    SnapHeader h;
    CK(cudaMemcpyAsync(&h, src, sizeof(h), cudaMemcpyDefault, st));
    CK(cudaStreamSynchronize(st));
    const SnapHeader want = snap_header(b);
    if (memcmp(&h, &want, sizeof(h)) != 0)
        return fail(GB_E_ARG, "snapshot was taken from a batch of another layout (precision or record counts differ)");
    CK(cudaMemcpyAsync(b->arena, static_cast<const char *>(src) + GB_SNAPSHOT_HEADER_BYTES, b->arena_bytes,
                       cudaMemcpyDefault, st));
    CK(cudaStreamSynchronize(st));
    return 0;
}

int gb_graph_destroy(gb_graph *g) {
    if (!g) return 0;
    if (g->b) {
        auto &v = g->b->graphs;
        v.erase(std::remove(v.begin(), v.end(), g), v.end());
    }
    if (g->exec) cudaGraphExecDestroy(g->exec);
    delete g;
    return 0;
}

}  // extern "C"

// Step scratch in static device memory, for gb_batch_step_static_scratch:
// the call itself allocates no device memory.  Every call on a device shares
// this one region, so calls whose launches may overlap (other streams, other
// host threads) race on it.
static __device__ __align__(256) unsigned char g_step_scratch[GB_STATIC_SCRATCH_BYTES];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void *g_scratch_ptr[kMaxDevices] = {};

// Device address of g_step_scratch on the current device, looked up once per
// device (the lookup loads the module; a later call only reads the table).
int static_scratch_base(void **out) {
    int dev = 0;
    CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(GB_E_ARG, "device ordinal beyond the static scratch table");
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_step_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_step_scratch)");
        if (!p) return fail(GB_E_CUDA, "cudaGetSymbolAddress(g_step_scratch) returned NULL");
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return 0;
}

template <class R> int step_static(gb_batch *b, const Batch<R> &arena_view, const StepParams &sp, int n_steps, int mode,
                                   int threads, cudaStream_t st) {
    Batch<R> B = arena_view;
    Arena need;
    carve_step_scratch(need, B, b->nw, b->nb, b->nf, b->ncap, b->nj);
    if (need.off > (size_t)GB_STATIC_SCRATCH_BYTES)
        return fail(GB_E_SCRATCH, "batch needs " + std::to_string(need.off) + " bytes of step scratch; the static scratch holds " +
                                      std::to_string((size_t)GB_STATIC_SCRATCH_BYTES) + " (use gb_batch_step)");
    void *base = nullptr;
    int rc = static_scratch_base(&base);
    if (rc) return rc;
    Arena a;
    a.base = static_cast<char *>(base);
    carve_step_scratch(a, B, b->nw, b->nb, b->nf, b->ncap, b->nj);
    // every scratch array is written before it is read inside a step, except
    // the first-pass TOI list counter
    CK(cudaMemsetAsync(B.toi_n, 0, sizeof(int) * GB_MAX_GROUPS, st));
    rc = run_steps<R>(b, B, sp, n_steps, mode, threads, st, nullptr);
    if (rc) return cuda_fail((cudaError_t)rc, "step launch (static scratch)");
    return 0;
}
}  // namespace

extern "C" int gb_batch_step_static_scratch(gb_batch *b, const gb_step_opts *o, void *stream) {
    if (!b || !o) return fail(GB_E_ARG, "batch or opts is NULL");
    if (o->n_steps < 0 || o->vel_iters < 0 || o->pos_iters < 0) return fail(GB_E_ARG, "negative step count or iterations");
    // contact events and per-launch timing need buffers and host waits that
    // this entry point does not have: refuse them rather than drop them
    if (o->record_order & (GB_OPT_EVENTS | GB_OPT_KERNEL_TIMES))
        return fail(GB_E_UNSUPPORTED, "gb_batch_step_static_scratch records no contact events and no launch times "
                                      "(GB_OPT_EVENTS, GB_OPT_KERNEL_TIMES): use gb_batch_step");
    const StepParams sp = params_of(o);
    int mode = 0, threads = 0;
    resolve_mapping(b, o, &mode, &threads);   // launch_mode 0: the batch's launch configuration, as gb_batch_step
    if (threads % 32 || threads > 1024) return fail(GB_E_ARG, "block_threads must be a multiple of 32 up to 1024");
    cudaStream_t st = (cudaStream_t)stream;
    int rc = b->prec == GB_PREC_F64 ? step_static<double>(b, b->bd, sp, o->n_steps, mode, threads, st)
                                    : step_static<float>(b, b->bf, sp, o->n_steps, mode, threads, st);
    if (rc) return rc;
    b->counters[0] += 1;
    b->counters[2] += o->n_steps;
    return 0;
}

// Chunks of gb_batch_step_host when the launch configuration has one world
// group: enough that the last chunk's download is short, few enough that
// each chunk's launches still fill the GPU.
static constexpr int kHostChunks = 4;

namespace {
template <class R> void unpack_range(const Batch<R> &B, const gb_body *d, int b0, int n, cudaStream_t st) {
    gb_launch_unpack_bodies<R>(B, d, b0, n, st);
}
template <class R> void unpack_range(const Batch<R> &B, const gb_body_state *d, int b0, int n, cudaStream_t st) {
    gb_launch_unpack_states<R>(B, d, b0, n, st);
}
template <class R> void pack_range(const Batch<R> &B, gb_body *d, int b0, int n, cudaStream_t st) {
    gb_launch_pack_bodies<R>(B, d, b0, n, st);
}
template <class R> void pack_range(const Batch<R> &B, gb_body_state *d, int b0, int n, cudaStream_t st) {
    gb_launch_pack_states<R>(B, d, b0, n, st);
}

// Bodies [b0, b0 + nb) up from the host and into the batch, with the TOI
// candidate flags of contact slots [s0, s0 + ns) (body types and bullet
// flags decide them); the stage holds either record kind.
template <class R, class Rec> cudaError_t upload_range(gb_batch *b, const Batch<R> &B, const Rec *in, int b0, int nb, int s0,
                                                       int ns, cudaStream_t st) {
    Rec *stage = reinterpret_cast<Rec *>(b->d_bstage);
    cudaError_t e = cudaMemcpyAsync(stage + b0, in + b0, sizeof(Rec) * nb, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return e;
    unpack_range<R>(B, stage, b0, nb, st);
    gb_launch_refresh_toi_cand<R>(B, s0, ns, st);
    return cudaGetLastError();
}

template <class R, class Rec> cudaError_t download_range(gb_batch *b, const Batch<R> &B, Rec *out, int b0, int nb, cudaStream_t st) {
    Rec *stage = reinterpret_cast<Rec *>(b->d_bstage);
    pack_range<R>(B, stage, b0, nb, st);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(out + b0, stage + b0, sizeof(Rec) * nb, cudaMemcpyDeviceToHost, st);
    return e;
}

// Each chunk on its own stream: upload of its bodies, the refresh of its
// contacts' TOI candidate flags, its steps, download.  Chunk k's copies
// overlap the other chunks' kernels (the copy engines run beside the SMs).
template <class R, class Rec> int step_host_chunks(gb_batch *b, const Batch<R> &B, const std::vector<WorldGroup> &chunks,
                                                   const Rec *in, Rec *out, const StepParams &sp, int n_steps, int mode,
                                                   int threads, cudaStream_t st) {
    cudaError_t e = cudaEventRecord(b->fork, st);
    for (size_t k = 0; k < chunks.size() && e == cudaSuccess; ++k) {
        const WorldGroup &g = chunks[k];
        e = cudaStreamWaitEvent(g.st, b->fork, 0);
        if (e == cudaSuccess) e = upload_range<R>(b, B, in, g.b0, g.nb, g.s0, g.ns, g.st);
        if (e != cudaSuccess) break;
        const int rc = gb_launch_step<R>(group_view(B, g, (int)k), sp, n_steps, g.d_worlds, g.n_list, mode, threads, g.st,
                                         nullptr, nullptr);
        if (rc) return rc;
        e = download_range<R>(b, B, out, g.b0, g.nb, g.st);
        if (e == cudaSuccess) e = cudaEventRecord(g.done, g.st);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(st, g.done, 0);
    }
    return (int)e;
}

template <class Rec> int step_host(gb_batch *b, const Rec *in, Rec *out, int32_t n, const gb_step_opts *o, void *stream) {
    if (!b || !o || !in || !out) return fail(GB_E_ARG, "batch, bodies or opts is NULL");
    if (n != b->nb) return fail(GB_E_ARG, "body count mismatch");
    if (o->n_steps < 0 || o->vel_iters < 0 || o->pos_iters < 0) return fail(GB_E_ARG, "negative step count or iterations");
    int mode = 0, threads = 0;
    resolve_mapping(b, o, &mode, &threads);
    if (threads % 32 || threads > 1024) return fail(GB_E_ARG, "block_threads must be a multiple of 32 up to 1024");
    cudaStream_t st = (cudaStream_t)stream;
    const bool chunked = mode == 3 && !has_grid_worlds(b) && !(o->record_order & (GB_OPT_EVENTS | GB_OPT_KERNEL_TIMES));
    const std::vector<WorldGroup> *chunks = &b->groups;
    if (chunked && b->groups.size() < 2) {
        const int big_from = std::min(b->cfg.big_bodies, (int)GB_HUGE_BODIES);
        if (b->chunks_big != big_from) {
            const int rc = build_groups(b, kHostChunks, big_from, b->chunks);
            if (rc) return rc;
            b->chunks_big = big_from;
        }
        chunks = &b->chunks;
    }
    if (!chunked || chunks->size() < 2) {
        // other mappings, contact events, launch timing, batches of one
        // world: upload, gb_batch_step and download on the caller's stream
        cudaError_t e = b->prec == GB_PREC_F64 ? upload_range<double>(b, b->bd, in, 0, b->nb, 0, b->bd.n_slots, st)
                                               : upload_range<float>(b, b->bf, in, 0, b->nb, 0, b->bf.n_slots, st);
        if (e != cudaSuccess) return cuda_fail(e, "body upload");
        const int rc = gb_batch_step(b, o, stream);
        if (rc) return rc;
        e = b->prec == GB_PREC_F64 ? download_range<double>(b, b->bd, out, 0, b->nb, st)
                                   : download_range<float>(b, b->bf, out, 0, b->nb, st);
        if (e != cudaSuccess) return cuda_fail(e, "body download");
        CK(cudaStreamSynchronize(st));
        return 0;
    }
    const StepParams sp = params_of(o);
    const int rc = b->prec == GB_PREC_F64 ? step_host_chunks<double>(b, b->bd, *chunks, in, out, sp, o->n_steps, mode, threads, st)
                                          : step_host_chunks<float>(b, b->bf, *chunks, in, out, sp, o->n_steps, mode, threads, st);
    if (rc) return cuda_fail((cudaError_t)rc, "chunked host step");
    CK(cudaStreamSynchronize(st));
    b->counters[0] += 1;
    b->counters[2] += o->n_steps;
    return 0;
}
}  // namespace

extern "C" int gb_batch_step_host(gb_batch *b, const gb_body *in, gb_body *out, int32_t n, const gb_step_opts *o,
                                  void *stream) {
    return step_host<gb_body>(b, in, out, n, o, stream);
}

extern "C" int gb_batch_step_host_state(gb_batch *b, const gb_body_state *in, gb_body_state *out, int32_t n,
                                        const gb_step_opts *o, void *stream) {
    return step_host<gb_body_state>(b, in, out, n, o, stream);
}

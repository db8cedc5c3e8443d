/*
 * gb2d.h -- C ABI of the GB300 world-step library (libgb2d.so).
 *
 * The library replaces the body of pypybox2d's World.step(dt, vel_iters,
 * pos_iters) (pypybox2d/world.py:307-354) for one world or for a batch of
 * independent worlds.  Everything that step touches -- contact update
 * (contact_manager.py:174-223), island solve (world.py:475-592,
 * island.py:65-179), fixture synchronisation and pair finding
 * (body.py:879-885, fixture.py:287-298, broadphase.py:83-109,
 * contact_manager.py:102-158) and continuous collision (world.py:594-821) --
 * runs in sm_103a kernels.  The host side (Python, pypybox2d_gb300) keeps the
 * reference's World/Body/Fixture API and talks to the library only through
 * the plain structs and functions below: no PyTorch types, host pointers and
 * sizes only.
 *
 * Conventions
 *   - every function returns 0 on success, a negative GB_E* code on error;
 *     gb_last_error() returns a message for the calling thread's last error.
 *   - all indices inside a world are world-local (body 0 is the first body
 *     of that world).  Fixtures of one body are contiguous and ordered as the
 *     body's fixture list; the fixture index is also the broad-phase proxy id.
 *   - host master copies are float64; GB_PREC_F64 keeps every device
 *     quantity in float64 (bit-exact with the CPU restatement),
 *     GB_PREC_F32 keeps body position/angle, sweep, sleep timers and the
 *     GJK/TOI iteration in float64 and the rest in float32.
 */
#ifndef GB2D_H
#define GB2D_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* shape type ids, as pypybox2d/shapes.py:884-890 */
#define GB_SHAPE_CIRCLE 0
#define GB_SHAPE_POLYGON 1
#define GB_SHAPE_LOOP 2
#define GB_SHAPE_EDGE 3
#define GB_MAX_POLY_VERTS 8

/* body types, as pypybox2d/body.py:17-19 */
#define GB_BODY_STATIC 0
#define GB_BODY_DYNAMIC 1
#define GB_BODY_KINEMATIC 2

/* gb_body.flags */
#define GB_BODY_AWAKE 1u
#define GB_BODY_ALLOW_SLEEP 2u
#define GB_BODY_BULLET 4u
#define GB_BODY_FIXED_ROTATION 8u
#define GB_BODY_ACTIVE 16u

/* gb_fixture.flags */
#define GB_FIX_SENSOR 1u
#define GB_FIX_EDGE_HAS_V0 2u /* edge vertex0 present (vx[2],vy[2]) */
#define GB_FIX_EDGE_HAS_V3 4u /* edge vertex3 present (vx[3],vy[3]) */
#define GB_FIX_LOOP_CHILD 8u  /* an edge that is one child of a loop: its fat box has no radius margin
                                 (shapes.py:822-837); a loop fixture of n vertices is n consecutive edge
                                 records, child i from vertex i to i+1 with vertices i-1 and i+2 as
                                 vertex0/vertex3 (shapes.py:851-863) */
#define GB_FIX_LOOP_FIRST 16u /* the first child record of a loop fixture: a buoyancy controller sums a
                                 loop's children before it adds them to the body (shapes.py:866-882) */

/* gb_contact.flags, as the Contact._*_flag attributes of contact.py:75-87 */
#define GB_C_TOUCHING 1u
#define GB_C_ENABLED 2u
#define GB_C_FILTER 4u
#define GB_C_ISLAND 8u
#define GB_C_TOI 16u
#define GB_C_BULLET_HIT 32u

/* manifold types, as contact_util.py:140-142 */
#define GB_M_CIRCLES 0
#define GB_M_FACE_A 1
#define GB_M_FACE_B 2

/* gb_world_desc.flags, as World attributes of world.py:65-86 */
#define GB_W_ALLOW_SLEEP 1u
#define GB_W_WARM_STARTING 2u
#define GB_W_CONTINUOUS 4u
#define GB_W_AUTO_CLEAR_FORCES 8u
#define GB_W_NEW_FIXTURE 16u   /* pair finding over every proxy before the next step */
#define GB_W_STEP_COMPLETE 32u

/* precision modes */
#define GB_PREC_F64 0
#define GB_PREC_F32 1

#define GB_OPT_KERNEL_TIMES 4u   /* gb_step_opts.record_order bit: time each phased-step launch */
#define GB_OPT_EVENTS 8u         /* gb_step_opts.record_order bit: record contact events (gb_batch_get_events) */

/* contact events (gb_event.type) */
#define GB_EV_BEGIN 1            /* two fixtures began to touch (contact.py:263-264) */
#define GB_EV_END 2              /* they ceased to touch, or a touching contact was destroyed (contact.py:265-266, contact_manager.py:167-168) */
#define GB_EV_POST_SOLVE 3       /* impulses of a solved contact (island.py:245-252) */

/* error codes (also OR-ed into the per-world device status word) */
#define GB_OK 0
#define GB_E_ARG (-1)
#define GB_E_CUDA (-2)
#define GB_E_CONTACT_OVERFLOW (-3)
#define GB_E_UNSUPPORTED (-4)
#define GB_E_NONFINITE (-5)
#define GB_E_ITER_LIMIT (-6)
#define GB_E_SCRATCH (-7)

/* world status bits reported by gb_batch_status */
#define GB_ST_CONTACT_OVERFLOW 1u
#define GB_ST_NONFINITE 2u
#define GB_ST_ITER_LIMIT 4u
#define GB_ST_PAIR_OVERFLOW 8u
#define GB_ST_TOI_ISLAND_CAP 16u
#define GB_ST_WAIT_TIMEOUT 32u   /* a bounded wait for an in-kernel copy gave up */
#define GB_ST_EVENT_OVERFLOW 64u /* more contact events than the world's event slots */

/* One rigid body: the state of pypybox2d.Body (body.py:46-84). */
typedef struct gb_body {
    int32_t type;            /* GB_BODY_* */
    uint32_t flags;          /* GB_BODY_* flags */
    int32_t fixture_start;   /* world-local index of the first fixture */
    int32_t fixture_count;
    double px, py;           /* _xf.position */
    double qc, qs;           /* _xf rotation: col1 = (qc, qs), col2 = (-qs, qc) */
    double lcx, lcy;         /* _sweep.local_center */
    double c0x, c0y, cx, cy; /* _sweep.c0, _sweep.c */
    double a0, a, alpha0;    /* _sweep.a0, _sweep.a, _sweep.alpha0 */
    double vx, vy, w;        /* _linear_velocity, _angular_velocity */
    double fx, fy, torque;   /* _force, _torque */
    double mass, inv_mass, I, inv_I;
    double linear_damping, angular_damping, gravity_scale;
    double sleep_time;
} gb_body;

/* The fields of a gb_body that World.step (world.py:307-354) reads and
 * writes: transform, sweep, velocity, accumulated force and torque, sleep
 * time and flags.  The others (type, fixtures, local centre, mass and
 * inertia, damping, gravity scale) are inputs the step only reads; they stay
 * as gb_batch_create or the last gb_batch_set_bodies left them.  152 bytes
 * against gb_body's 232. */
typedef struct gb_body_state {
    uint32_t flags;          /* GB_BODY_* flags */
    uint32_t _pad0;
    double px, py, qc, qs;   /* _xf */
    double c0x, c0y, cx, cy; /* _sweep.c0, _sweep.c */
    double a0, a, alpha0;    /* _sweep.a0, _sweep.a, _sweep.alpha0 */
    double vx, vy, w;        /* _linear_velocity, _angular_velocity */
    double fx, fy, torque;   /* _force, _torque */
    double sleep_time;
} gb_body_state;

/* One fixture with its shape and its single broad-phase proxy
 * (fixture.py:42-71, shapes.py).  Polygons store vertices and the unit edge
 * normals computed by the Polygon vertex setter (shapes.py:442-482); a circle
 * stores its centre in (vx[0], vy[0]); an edge stores vertex1/vertex2 in
 * slots 0/1 and the optional vertex0/vertex3 in slots 2/3. */
typedef struct gb_fixture {
    int32_t body;            /* world-local body index */
    int32_t shape_type;      /* GB_SHAPE_* */
    int32_t vertex_count;
    uint32_t flags;          /* GB_FIX_* */
    double radius;
    double friction, restitution, density;
    uint32_t category_bits, mask_bits;
    int32_t group_index, _pad0;
    double vx[GB_MAX_POLY_VERTS], vy[GB_MAX_POLY_VERTS];
    double nx[GB_MAX_POLY_VERTS], ny[GB_MAX_POLY_VERTS];
    double aabb[4];          /* fat AABB of the proxy: lower x, lower y, upper x, upper y */
} gb_fixture;

/* One contact (contact.py:55-87) with its manifold (contact_util.py:120-155).
 * Contacts of a world are kept in creation order, which is the order of
 * ContactManager.contacts. */
typedef struct gb_contact {
    int32_t fixture_a, fixture_b; /* world-local; A is the primary shape of the pair */
    int32_t child_a, child_b;     /* 0: each child of a loop is a record of its own (GB_FIX_LOOP_CHILD) */
    uint32_t flags;               /* GB_C_* */
    int32_t toi_count;
    double toi;
    double friction, restitution;
    int32_t m_type, m_point_count;
    double m_lnx, m_lny;          /* manifold.local_normal */
    double m_lpx, m_lpy;          /* manifold.local_point */
    double p_lx[2], p_ly[2];      /* points[i].local_point */
    double p_ni[2], p_ti[2];      /* points[i].normal_impulse, tangent_impulse */
    uint32_t p_id[2];             /* index_a | index_b<<8 | type_a<<16 | type_b<<24 */
} gb_contact;

/* joint types (pypybox2d/joints/: revolute.py, prismatic.py, distance.py, weld.py,
 * friction.py, rope.py, wheel.py, pulley.py, mouse.py) */
#define GB_JOINT_REVOLUTE 1
#define GB_JOINT_PRISMATIC 2
#define GB_JOINT_DISTANCE 3
#define GB_JOINT_WELD 4
#define GB_JOINT_FRICTION 5
#define GB_JOINT_ROPE 6
#define GB_JOINT_WHEEL 7
#define GB_JOINT_PULLEY 8
#define GB_JOINT_MOUSE 9   /* one body: the reference's body_a is None; the record gives body_a = body_b */

/* gb_joint.flags */
#define GB_J_COLLIDE_CONNECTED 1u /* Joint._collide_connected */
#define GB_J_LIMIT 2u             /* _limit_enabled (revolute, prismatic) */
#define GB_J_MOTOR 4u             /* _motor_enabled (revolute, prismatic, wheel) */

/* gb_joint.limit_state, as joints/joint.py:35 */
#define GB_LIMIT_INACTIVE 0
#define GB_LIMIT_LOWER 1
#define GB_LIMIT_UPPER 2
#define GB_LIMIT_EQUAL 3

/* One joint: its definition and the state it carries between steps
 * (joints/joint.py:41-59 and the kind's __init__).  Joints of a batch are
 * sorted by world; within a world they are in World.joints order (creation
 * order), which is also the order of every body's joint list.  Anchors and
 * the prismatic axis are the local values the reference computes at
 * creation (body.get_local_point / get_local_vector; the axis is not
 * normalised, prismatic.py:82-85). */
typedef struct gb_joint {
    int32_t world;                 /* world of the batch */
    int32_t type;                  /* GB_JOINT_* */
    int32_t body_a, body_b;        /* world-local bodies */
    uint32_t flags;                /* GB_J_* */
    int32_t limit_state;           /* GB_LIMIT_* (revolute, prismatic) */
    double la_x, la_y, lb_x, lb_y; /* _local_anchor_a, _local_anchor_b */
    double ref_angle;              /* _reference_angle (revolute, prismatic, weld) */
    double ax_x, ax_y;             /* prismatic _local_x_axis */
    double lower, upper;           /* revolute _lower_angle/_upper_angle, prismatic _lower_limit/_upper_limit */
    double max_motor;              /* revolute _max_motor_torque, prismatic _max_motor_force */
    double motor_speed;
    double length, frequency, damping_ratio; /* distance */
    double impulse[3];             /* _impulse (distance: impulse[0]) */
    double motor_impulse;          /* _motor_impulse */
    double gamma, bias;            /* distance: kept from the last set-up with frequency > 0 (distance.py:246-266) */
    double ux, uy;                 /* last set-up: distance _u, prismatic _axis (for the reaction force),
                                      rope _u (the unnormalised anchor difference) */
    double perp_x, perp_y;         /* last set-up: prismatic _perp, wheel _ay */
    double max_force, max_torque;  /* friction */
    double max_length, cur_length; /* rope: _max_length; _length of the last set-up */
    double spring_impulse;         /* wheel _spring_impulse */
    double sax_x, sax_y, s_ax, s_bx; /* wheel _ax, _s_ax, _s_bx: set by a set-up with a spring, kept otherwise */
    double ga_x, ga_y, gb_x, gb_y; /* pulley ground anchors */
    double ratio, constant;        /* pulley _ratio, _constant */
    double target_x, target_y;     /* mouse _target (max_force: _max_force; bias: _beta; gamma: _gamma) */
} gb_joint;

/* controller kinds (pypybox2d/controllers.py) */
#define GB_CONTROLLER_BUOYANCY 1
#define GB_CONTROLLER_GRAVITY 2

/* gb_controller.flags */
#define GB_CTRL_OWN_GRAVITY 1u  /* buoyancy: gravity_x/y given (a gravity of None or (0, 0) takes the world's) */
#define GB_CTRL_INV_SQR 2u      /* gravity: force falls off as 1/r^2 (else 1/r) */

/* One controller (controllers.py:24-280): a force rule applied to a list of
 * bodies at the start of the solve of every step (world.py:476-479), before
 * the islands are built.  Controllers of a batch are sorted by world; within
 * a world they are in World.controllers order, which is the order they run
 * in.  The controller's bodies are controller_bodies[body_start ..
 * body_start + body_count): world-local body indices in the controller's
 * own body order (Controller.add_body order), which is the order of the
 * gravity controller's pair loop. */
typedef struct gb_controller {
    int32_t world;                 /* world of the batch */
    int32_t type;                  /* GB_CONTROLLER_* */
    int32_t body_start, body_count;
    uint32_t flags;                /* GB_CTRL_* */
    int32_t _pad0;
    double normal_x, normal_y;     /* buoyancy: the fluid's outer surface normal (as given, not normalised) */
    double offset;                 /* buoyancy: height of the surface along the normal */
    double density;                /* buoyancy: fluid density */
    double velocity_x, velocity_y; /* buoyancy: fluid velocity (drag) */
    double linear_drag, angular_drag;
    double gravity_x, gravity_y;   /* buoyancy: with GB_CTRL_OWN_GRAVITY */
    double G;                      /* gravity controller: strength */
} gb_controller;

/* One world of a batch. */
typedef struct gb_world_desc {
    int32_t body_start, body_count;       /* into the batch body array */
    int32_t fixture_start, fixture_count; /* into the batch fixture array */
    int32_t contact_start, contact_count; /* initial contacts (into the batch contact array) */
    int32_t contact_capacity;             /* device contact slots reserved for this world (0: 6 per
                                             fixture, 10 for worlds of 16384 bodies or more) */
    uint32_t flags;                       /* GB_W_* */
    int32_t move_start, move_count;       /* pending broad-phase move buffer (into scene.moves);
                                             with GB_W_NEW_FIXTURE and move_count == 0 every
                                             fixture of the world is pending, in index order */
    double gx, gy;                        /* gravity */
    double inv_dt0;                       /* World._inv_dt0 */
} gb_world_desc;

/* A batch of independent worlds described by host arrays. */
typedef struct gb_scene {
    int32_t n_worlds;
    int32_t n_bodies, n_fixtures, n_contacts;
    const gb_world_desc *worlds;
    const gb_body *bodies;
    const gb_fixture *fixtures;
    const gb_contact *contacts;
    int32_t n_moves, _pad0;
    const int32_t *moves;                 /* world-local fixture indices (BroadPhase._move_buffer) */
    int32_t n_joints, _pad1;
    const gb_joint *joints;               /* sorted by world (NULL when n_joints is 0) */
    int32_t n_controllers, n_controller_bodies;
    const gb_controller *controllers;     /* sorted by world (NULL when n_controllers is 0) */
    const int32_t *controller_bodies;     /* world-local body indices of the controllers' body lists */
} gb_scene;

typedef struct gb_batch gb_batch; /* opaque device-resident batch of worlds */

/* Step options.  launch_mode: 0 = the batch's launch configuration
 * (gb_batch_set_launch_config, gb_batch_autotune), 1 = one CTA per world,
 * 2 = one warp per world, 3 = phased (batch-wide and per-world launches).
 * block_threads: CTA width (0 = the launch configuration's for mode 0,
 * 128 otherwise). */
typedef struct gb_step_opts {
    double dt;
    int32_t vel_iters, pos_iters;
    int32_t n_steps;
    int32_t launch_mode;
    int32_t block_threads;
    int32_t record_order; /* bit 0: keep the solver constraint order of the last step;
                             bit 1: accumulate per-phase SM clocks (gb_batch_phase_clocks)
                             bit 2: time every launch of the phased step (gb_batch_kernel_times) */
} gb_step_opts;

/* Library version and build information. */
const char *gb_version(void);
/* Message of the calling thread's last error (never NULL). */
const char *gb_last_error(void);
/* sizeof of gb_body, gb_fixture, gb_contact, gb_world_desc, gb_scene, gb_step_opts
 * (6 ints), so bindings can check their record layouts. */
int gb_struct_sizes(int32_t *sizes);
/* sizeof(gb_joint). */
int gb_joint_size(void);
/* sizeof(gb_controller). */
int gb_controller_size(void);
/* sizeof(gb_body_state), for binding checks. */
int gb_body_state_size(void);

/* One contact event of a step, replayed to the contact listeners after it.
 * `key` orders a world's events: (step of the call) << 48 | phase << 40 |
 * index, where phase 0 is the contact update (index = contact position),
 * phase 1 the island solve (index = contact position) and phase 2 the
 * continuous-collision loop (index = order of occurrence). */
typedef struct gb_event {
    int32_t type;                 /* GB_EV_* */
    int32_t fixture_a, fixture_b; /* world-local fixtures of the contact */
    int32_t point_count;          /* impulse points (post-solve) */
    int64_t key;
    double normal_impulse[2], tangent_impulse[2];
} gb_event;

/* Upload a scene to device memory.  Replaces the host-side construction of
 * the reference's World (world.py:64-91, 183-233). */
int gb_batch_create(const gb_scene *scene, int32_t precision, gb_batch **out);
/* Free every device buffer of the batch. */
int gb_batch_destroy(gb_batch *batch);
/* Advance every world by opts->n_steps calls of World.step(dt, vel_iters,
 * pos_iters) (world.py:307-354) on the given CUDA stream (NULL = default). */
int gb_batch_step(gb_batch *batch, const gb_step_opts *opts, void *cuda_stream);
/* Overwrite the device body state of the whole batch from host memory. */
int gb_batch_set_bodies(gb_batch *batch, const gb_body *bodies, int32_t n_bodies, void *cuda_stream);
/* Copy the device body state of the whole batch to host memory. */
int gb_batch_get_bodies(gb_batch *batch, gb_body *bodies, int32_t n_bodies, void *cuda_stream);
/* One host-buffer round trip of World.step (world.py:307-354) with the
 * body state read and written through host memory: the same results as
 * gb_batch_set_bodies(bodies_in), gb_batch_step(opts) and
 * gb_batch_get_bodies(bodies_out) in a row, bit for bit.  Under the phased
 * launch the worlds go in chunks (the batch's world groups, or four runs of
 * about equal body counts when the launch configuration has one group), each
 * chunk's upload, steps and download on a stream of its own, so the copies
 * of one chunk overlap the kernels of the others.  bodies_in and bodies_out
 * may be the same buffer; pinned host memory lets the copies run
 * asynchronously.  The call returns once bodies_out is written.  Other
 * mappings, contact events and launch timing take the three calls in a
 * row. */
int gb_batch_step_host(gb_batch *batch, const gb_body *bodies_in, gb_body *bodies_out, int32_t n_bodies,
                       const gb_step_opts *opts, void *cuda_stream);
/* gb_batch_step_host with gb_body_state records: the same chunks, streams
 * and results, with the step-invariant body fields left on the device (the
 * call neither reads nor writes them). */
int gb_batch_step_host_state(gb_batch *batch, const gb_body_state *states_in, gb_body_state *states_out,
                             int32_t n_bodies, const gb_step_opts *opts, void *cuda_stream);
/* Copy the fat AABBs (4 doubles per fixture) to host memory. */
int gb_batch_get_proxies(gb_batch *batch, double *aabbs, int32_t n_fixtures, void *cuda_stream);
/* Number of live contacts of every world (n_worlds ints). */
int gb_batch_get_contact_counts(gb_batch *batch, int32_t *counts, void *cuda_stream);
/* Copy the live contacts of one world, in creation order, to host memory. */
int gb_batch_get_contacts(gb_batch *batch, int32_t world, gb_contact *out, int32_t capacity,
                          int32_t *n_out, void *cuda_stream);
/* Solver constraint order of the last step of one world (contact indices in
 * the order the velocity and position passes visited them); only kept when
 * the step ran with record_order set. */
int gb_batch_get_solver_order(gb_batch *batch, int32_t world, int32_t *order, int32_t capacity,
                              int32_t *n_out, void *cuda_stream);
/* The same for the joints (world-local joint indices in the order the
 * passes visited them; every pass visits the joints before the contacts in
 * the velocity iterations and after them in the position iterations, as
 * island.py:107-148 does). */
int gb_batch_get_joint_order(gb_batch *batch, int32_t world, int32_t *order, int32_t capacity,
                             int32_t *n_out, void *cuda_stream);
/* Copy the joints of the whole batch (scene order) with their carried state
 * to host memory / overwrite them from host memory (definition and state:
 * the setters of the joint classes).  The world and bodies of each joint must be
 * the ones the batch was made with. */
int gb_batch_get_joints(gb_batch *batch, gb_joint *joints, int32_t n_joints, void *cuda_stream);
int gb_batch_set_joints(gb_batch *batch, const gb_joint *joints, int32_t n_joints, void *cuda_stream);
/* Overwrite the parameters of the batch's controllers (scene order): the
 * setters of BuoyancyController / GravityController between steps.  The
 * world, kind and body list range of each controller must be the ones the
 * batch was made with (a changed body list needs a new batch). */
int gb_batch_set_controllers(gb_batch *batch, const gb_controller *controllers, int32_t n_controllers, void *cuda_stream);
/* A world's custom contact filter (world.py:123-136: World.contact_filter,
 * called by contact_manager.py:145 for a new pair and :202 for a contact
 * flagged for filtering) as its answers: accept[a * n_fixtures + b] != 0
 * when fixture records a and b (world-local) may collide, for every ordered
 * pair.  It replaces the default category/mask/group rule for that world;
 * accept = NULL restores the default.  n_fixtures must be the world's
 * fixture record count, at most GB_PAIR_FILTER_MAX_FIXTURES.  Refused
 * (GB_E_UNSUPPORTED) while captured rollouts of the batch exist.  The call
 * waits for the device's earlier work, then replaces the tables. */
#define GB_PAIR_FILTER_MAX_FIXTURES 16384
int gb_batch_set_pair_filter(gb_batch *batch, int32_t world, const uint8_t *accept, int32_t n_fixtures, void *cuda_stream);
/* Step record of one world's bodies (world-local order) from the last step
 * run with record_order bit 0 set: out[0..n) the decisions of each body,
 * out[n..2n) its island in the solve (the smallest world-local index of the
 * island's non-static bodies, -1: not in a simulated island); *n_out = n,
 * capacity >= 2n.  Decisions per body: bits 0-7 the position
 * iterations its island ran before the early exit (island.py:141-153; 0:
 * not in a simulated island), bits 8-15 the TOI position-pass iterations
 * over the TOI events it took part in (contact.py:866-933, island.py:181-243),
 * bits 16-23 the number of those events (world.py:693-817), each capped at
 * 255; bit 24 the parity of its constraints' contact points that took the
 * restitution bias (relative normal velocity below -1 m/s, contact.py:470-475)
 * and bit 25 of its 2-point constraints that dropped to one point
 * (contact.py:487-496) in the island solve, bits 26/27 the same in TOI
 * sub-steps (non-static bodies).  These are decisions of the step that its
 * final state does not show; nothing in the reference (measurement for the
 * parity tests). */
int gb_batch_get_step_record(gb_batch *batch, int32_t world, int32_t *out, int32_t capacity, int32_t *n_out,
                             void *cuda_stream);
/* Poll limit of the solver's waits for its in-kernel bulk copies (default
 * 262144).  A wait that reaches it sets GB_ST_WAIT_TIMEOUT in its world's
 * status word, waits with the default limit for the copies still in flight
 * and ends that world's solve for the step; the context stays usable.  A
 * limit of 0 makes every such wait give up at once, so callers can exercise
 * that path without a fault.  No counterpart in the reference. */
int gb_batch_set_wait_polls(gb_batch *batch, int32_t polls);
/* Zero every world's status word (after the caller has handled a failure). */
int gb_batch_clear_status(gb_batch *batch, void *cuda_stream);
/* Per-world status words (GB_ST_* bits), n_worlds uint32. */
int gb_batch_status(gb_batch *batch, uint32_t *status, void *cuda_stream);
/* Accumulated SM clock cycles per step phase, 24 int64 per world
 * (0 pairing of new fixtures, 1 contact update, 2 islands, 3 colouring,
 * 4 velocity set-up, 5 velocity iterations, 6 position iterations, 7 sleep,
 * 8 fixture sync + pair finding, 9 continuous collision, 10 force clear;
 * continuous-collision loop: 11 passes, 12 finding the earliest event,
 * 13 events, 14 invalidation and pair search, 15 the number of events,
 * 16 pass statuses, 17 pass sweep alignment, 18 pass times of impact,
 * 19 event contact updates, 20 event position passes, 21 event velocity
 * passes and integration, 22 event fixture sync, 23 the number of fresh
 * times of impact; 11-14 hold what the finer slots do not). */
int gb_batch_phase_clocks(gb_batch *batch, int64_t *clocks, void *cuda_stream);
/* Counters: step launches so far, bytes of device memory held by the
 * batch, world-steps requested so far (3 int64). */
int gb_batch_counters(gb_batch *batch, int64_t *counters);
/* Device time of each launch of the phased step (launch_mode 3), summed over
 * the steps run with GB_OPT_KERNEL_TIMES set: 13 slots, in launch order
 * (new-fixture pairs, body prologue, contact update, contact update of
 * sleeping pairs, islands and colouring, velocity integration, solver
 * set-up, solver, fixture sync and pairs, TOI candidates, first-pass TOI,
 * TOI loop set-up, TOI event loop).  Measurement only: a timed step waits
 * for its events. */
int gb_batch_kernel_times(gb_batch *batch, double *total_ms, int32_t capacity, int32_t *n_slots, int64_t *n_steps);
/* Contact events of one world recorded by the last gb_batch_step call made
 * with GB_OPT_EVENTS (unsorted; order by `key`).  *n_out = number of events;
 * events beyond the world's slots (3 per contact slot + 64) are dropped and
 * flagged GB_ST_EVENT_OVERFLOW. */
int gb_batch_get_events(gb_batch *batch, int32_t world, gb_event *out, int32_t capacity, int32_t *n_out,
                        void *cuda_stream);

/* How the step is mapped onto the GPU.  Every mapping gives the same float64
 * results; only the time differs.  In float32 the phased configurations give
 * the same results as long as each world's solver keeps its shared-memory
 * body cache (worlds of up to 2048 bodies); launch modes 1 and 2 and uncached
 * worlds round differently, within the float32 step error.  A batch starts
 * with {3, 128, 2, 512, 1}.  No counterpart in the reference (one CPython
 * world has no launch geometry). */
typedef struct gb_launch_config {
    int32_t launch_mode;    /* 1 = one CTA per world, 2 = one warp per world, 3 = phased */
    int32_t block_threads;  /* CTA width: mode 1 the world's CTA, mode 2 warps per CTA x 32, mode 3 the
                               solver CTA of the smaller worlds (islands 4x, pair phases 2x, up to 256) */
    int32_t pipe_bufs;      /* mode 3 solver: constraint-chunk buffers in shared memory, 0..4
                               (0: records read from global memory) */
    int32_t big_bodies;     /* mode 3 solver: worlds of this many bodies or more get the wide launch */
    int32_t groups;         /* mode 3: world groups, 1..8 -- runs of consecutive worlds of about equal body
                               counts, each stepped on a stream of its own so one group's latency-bound
                               phases (the TOI event loop of its largest worlds) overlap the others' work;
                               1 for batches with worlds of 16384 bodies or more */
    int32_t _pad0;
    double ms_per_step;     /* autotune output (device ms per step); ignored on input */
} gb_launch_config;
#define GB_LAUNCH_CONFIG_BYTES 32
/* Set the configuration that steps with launch_mode 0 use (and pipe_bufs /
 * big_bodies for every phased step).  The batch state is not touched. */
int gb_batch_set_launch_config(gb_batch *batch, const gb_launch_config *cfg);
int gb_batch_get_launch_config(gb_batch *batch, gb_launch_config *cfg);
/* Autotuner.  Times candidate configurations on the batch's own next
 * opts->n_steps steps: the device arena is copied aside once, every trial
 * starts from that copy, and the copy is put back at the end, so the batch
 * state after the call is the state before it (the call needs device memory
 * for one more arena while it runs).  Stages, each keeping the best so far:
 * (1) mapping: phased with 32/64/128 threads, one CTA per world with 128/256
 * threads, one warp per world with 2/4 warps per CTA (phased only for
 * batches with cooperative-grid worlds); (2) big_bodies 256/512/1024/2048/
 * none; (3) pipe_bufs 0-4; (4) world groups 1/2/3/4 (phased, without
 * cooperative-grid worlds).  Each trial's steps are timed with CUDA events on
 * `cuda_stream`.  trials[] receives every trial in order (ms_per_step -1:
 * not runnable, e.g. too much shared memory; -2: its steps raised a status
 * bit, e.g. a copy wait that gave up, and it is not a candidate); the best
 * becomes the batch's launch configuration.  opts->record_order must be 0. */
int gb_batch_autotune(gb_batch *batch, const gb_step_opts *opts, gb_launch_config *trials, int32_t capacity,
                      int32_t *n_out, gb_launch_config *best, void *cuda_stream);

/* A multi-step rollout captured as one CUDA graph (the 13-14 launches of
 * each of opts->n_steps phased steps), replayed by gb_graph_launch with no
 * host work per step.  Replaces calling World.step n_steps times
 * (world.py:307-354).  The graph keeps the options, launch configuration and
 * device buffers of the capture: replays read and advance the batch's
 * current device state, so gb_batch_set_bodies and the getters may be used
 * between replays; a later gb_batch_set_launch_config does not change an
 * existing graph.  Not available: GB_OPT_KERNEL_TIMES (host timing), batches
 * with cooperative-grid worlds (16384+ bodies), launch modes 1 and 2. */
typedef struct gb_graph gb_graph;
int gb_graph_capture(gb_batch *batch, const gb_step_opts *opts, gb_graph **out);
/* Replay the captured steps on `cuda_stream` (asynchronous). */
int gb_graph_launch(gb_graph *graph, void *cuda_stream);
int gb_graph_destroy(gb_graph *graph);

/* One ray of gb_batch_ray_cast, from (p1x, p1y) to (p2x, p2y) in one world. */
typedef struct gb_ray {
    int32_t world, _pad0;
    double p1x, p1y, p2x, p2y;
} gb_ray;
/* The closest hit of a ray: what World.ray_cast (world.py:387-440) leaves in
 * a callback that returns the fraction it is given.  fixture = -1 (and
 * fraction 1) when no fixture is hit. */
typedef struct gb_ray_hit {
    int32_t fixture, _pad0;   /* world-local fixture index */
    double px, py;            /* (1 - fraction) * p1 + fraction * p2 */
    double nx, ny;            /* the shape's normal at the hit (edges: in the edge's frame, as shapes.py:655-702) */
    double fraction;
} gb_ray_hit;
/* One box of gb_batch_query_aabb: lower (lx, ly), upper (ux, uy). */
typedef struct gb_aabb_query {
    int32_t world, _pad0;
    double lx, ly, ux, uy;
} gb_aabb_query;
/* Closest hit of every ray against the fixtures of its world (circle,
 * polygon and edge ray casts of shapes.py:147-171, 265-314, 655-702, behind
 * the broad-phase segment test of dynamictree.py:209-250 with
 * max_fraction 1).  Ties go to the lower fixture index.  A ray of zero length
 * is rejected (GB_E_ARG), as dynamictree.py:222-224 raises.  Host arrays in
 * and out; the call waits for its results.  Replaces World.ray_cast with a
 * closest-hit callback, for many rays at once. */
int gb_batch_ray_cast(gb_batch *batch, const gb_ray *rays, int32_t n_rays, gb_ray_hit *hits, void *cuda_stream);
/* Every hit of every ray: what the generator form of World.ray_cast yields
 * when each fraction is left at 1 (world.py:387-440), in fixture order (the
 * reference's come in tree order).  Ray q's first max_per_ray hits go to
 * hits[q * max_per_ray ...], counts[q] is how many there are in all. */
int gb_batch_ray_cast_all(gb_batch *batch, const gb_ray *rays, int32_t n_rays, gb_ray_hit *hits, int32_t max_per_ray,
                          int32_t *counts, void *cuda_stream);
/* Fixtures whose fat AABB overlaps each query box (World.query_aabb,
 * world.py:371-385; DynamicTree.query, dynamictree.py:190-207), in fixture
 * order: query q's first max_per_query fixtures go to
 * fixtures[q * max_per_query ...], counts[q] is how many overlap in all. */
int gb_batch_query_aabb(gb_batch *batch, const gb_aabb_query *queries, int32_t n_queries, int32_t *fixtures,
                        int32_t max_per_query, int32_t *counts, void *cuda_stream);

/* Checkpoint and resume of a batch's whole device state: bodies and sweeps,
 * fixtures with their fat AABBs, contacts with manifolds, impulses and flags,
 * world headers (contact counts, status words, inv_dt0) and the pending
 * broad-phase move buffers.  The reference has no world serialisation (only
 * its math types pickle: common.py:176-179, 394-398, 649-652, 725-728, and
 * Body/Fixture copy, body.py:118-140, fixture.py:76-85); these calls give the
 * GPU batch one.  A snapshot is GB_SNAPSHOT_HEADER_BYTES of header (layout
 * identity: precision and record counts) followed by the device arena; it
 * restores only into a batch made from a scene of the same layout.  `dst` /
 * `src` may be host or device memory (copied with cudaMemcpyDefault); the
 * calls return once the copy is complete.  The launch configuration and
 * captured graphs are not part of the state and are kept. */
#define GB_SNAPSHOT_HEADER_BYTES 64
int gb_batch_snapshot_bytes(gb_batch *batch, uint64_t *bytes);
int gb_batch_snapshot(gb_batch *batch, void *dst, uint64_t bytes, void *cuda_stream);
int gb_batch_restore(gb_batch *batch, const void *src, uint64_t bytes, void *cuda_stream);

/* Size of the static device scratch of gb_batch_step_static_scratch (32 MiB). */
#define GB_STATIC_SCRATCH_BYTES (32u << 20)
/* gb_batch_step with the step's scratch arrays placed in one static device
 * array of GB_STATIC_SCRATCH_BYTES instead of the batch arena; the call
 * allocates no device memory.  No counterpart in the reference (its step
 * allocates Python objects per call).  launch_mode 0 takes the batch's
 * launch configuration, exactly as gb_batch_step does.  Contact events and
 * per-launch timing (GB_OPT_EVENTS, GB_OPT_KERNEL_TIMES) are refused with
 * GB_E_UNSUPPORTED.  The first call on a device looks up the array's address
 * (loading the module) and keeps it for that device, so make one call before
 * any stream capture, and do not call it again after a cudaDeviceReset of
 * that device (the kept address belongs to the old context).  A batch whose
 * scratch exceeds the array is rejected with GB_E_SCRATCH before any launch.
 * All calls on a device share the array: calls whose work may overlap (other
 * streams or host threads) race. */
int gb_batch_step_static_scratch(gb_batch *batch, const gb_step_opts *opts, void *cuda_stream);

#ifdef __cplusplus
}
#endif

#endif /* GB2D_H */

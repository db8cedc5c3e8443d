"""Host-side mirror of ``include/gb2d.h``: numpy record layouts of the C
structs and the ctypes binding of ``libgb2d.so``.

The record layouts are the plain-data form of the reference's objects:
``BODY`` is the state of ``pypybox2d.Body`` (body.py:46-84), ``FIXTURE`` a
fixture with its shape and proxy (fixture.py:42-71, shapes.py), ``CONTACT`` a
``Contact`` with its ``Manifold`` (contact.py:55-87, contact_util.py:120-155).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

SHAPE_CIRCLE, SHAPE_POLYGON, SHAPE_LOOP, SHAPE_EDGE = 0, 1, 2, 3
MAX_POLY_VERTS = 8
BODY_STATIC, BODY_DYNAMIC, BODY_KINEMATIC = 0, 1, 2

BODY_AWAKE = 1
BODY_ALLOW_SLEEP = 2
BODY_BULLET = 4
BODY_FIXED_ROTATION = 8
BODY_ACTIVE = 16

FIX_SENSOR = 1
FIX_EDGE_HAS_V0 = 2
FIX_EDGE_HAS_V3 = 4
FIX_LOOP_CHILD = 8      # one child edge of a loop fixture (no radius margin on its box)
FIX_LOOP_FIRST = 16     # the first child record of a loop fixture

C_TOUCHING = 1
C_ENABLED = 2
C_FILTER = 4
C_ISLAND = 8
C_TOI = 16
C_BULLET_HIT = 32

M_CIRCLES, M_FACE_A, M_FACE_B = 0, 1, 2

W_ALLOW_SLEEP = 1
W_WARM_STARTING = 2
W_CONTINUOUS = 4
W_AUTO_CLEAR_FORCES = 8
W_NEW_FIXTURE = 16
W_STEP_COMPLETE = 32

PREC_F64, PREC_F32 = 0, 1

ST_CONTACT_OVERFLOW = 1
ST_NONFINITE = 2
ST_ITER_LIMIT = 4
ST_PAIR_OVERFLOW = 8
ST_TOI_ISLAND_CAP = 16
ST_WAIT_TIMEOUT = 32

_BODY_FIELDS = [
    ("type", "<i4"), ("flags", "<u4"), ("fixture_start", "<i4"), ("fixture_count", "<i4"),
    ("px", "<f8"), ("py", "<f8"), ("qc", "<f8"), ("qs", "<f8"),
    ("lcx", "<f8"), ("lcy", "<f8"), ("c0x", "<f8"), ("c0y", "<f8"), ("cx", "<f8"), ("cy", "<f8"),
    ("a0", "<f8"), ("a", "<f8"), ("alpha0", "<f8"),
    ("vx", "<f8"), ("vy", "<f8"), ("w", "<f8"),
    ("fx", "<f8"), ("fy", "<f8"), ("torque", "<f8"),
    ("mass", "<f8"), ("inv_mass", "<f8"), ("I", "<f8"), ("inv_I", "<f8"),
    ("linear_damping", "<f8"), ("angular_damping", "<f8"), ("gravity_scale", "<f8"),
    ("sleep_time", "<f8"),
]
BODY = np.dtype(_BODY_FIELDS, align=True)

#: gb_body_state: the body fields a step reads and writes (gb_batch_step_host_state)
BODY_STATE = np.dtype([
    ("flags", "<u4"), ("_pad0", "<u4"),
    ("px", "<f8"), ("py", "<f8"), ("qc", "<f8"), ("qs", "<f8"),
    ("c0x", "<f8"), ("c0y", "<f8"), ("cx", "<f8"), ("cy", "<f8"),
    ("a0", "<f8"), ("a", "<f8"), ("alpha0", "<f8"),
    ("vx", "<f8"), ("vy", "<f8"), ("w", "<f8"),
    ("fx", "<f8"), ("fy", "<f8"), ("torque", "<f8"),
    ("sleep_time", "<f8"),
], align=True)

FIXTURE = np.dtype([
    ("body", "<i4"), ("shape_type", "<i4"), ("vertex_count", "<i4"), ("flags", "<u4"),
    ("radius", "<f8"), ("friction", "<f8"), ("restitution", "<f8"), ("density", "<f8"),
    ("category_bits", "<u4"), ("mask_bits", "<u4"), ("group_index", "<i4"), ("_pad0", "<i4"),
    ("vx", "<f8", (MAX_POLY_VERTS,)), ("vy", "<f8", (MAX_POLY_VERTS,)),
    ("nx", "<f8", (MAX_POLY_VERTS,)), ("ny", "<f8", (MAX_POLY_VERTS,)),
    ("aabb", "<f8", (4,)),
], align=True)

CONTACT = np.dtype([
    ("fixture_a", "<i4"), ("fixture_b", "<i4"), ("child_a", "<i4"), ("child_b", "<i4"),
    ("flags", "<u4"), ("toi_count", "<i4"), ("toi", "<f8"),
    ("friction", "<f8"), ("restitution", "<f8"),
    ("m_type", "<i4"), ("m_point_count", "<i4"),
    ("m_lnx", "<f8"), ("m_lny", "<f8"), ("m_lpx", "<f8"), ("m_lpy", "<f8"),
    ("p_lx", "<f8", (2,)), ("p_ly", "<f8", (2,)), ("p_ni", "<f8", (2,)), ("p_ti", "<f8", (2,)),
    ("p_id", "<u4", (2,)),
], align=True)

JOINT_REVOLUTE, JOINT_PRISMATIC, JOINT_DISTANCE, JOINT_WELD = 1, 2, 3, 4
JOINT_FRICTION, JOINT_ROPE, JOINT_WHEEL, JOINT_PULLEY, JOINT_MOUSE = 5, 6, 7, 8, 9
J_COLLIDE_CONNECTED, J_LIMIT, J_MOTOR = 1, 2, 4
LIMIT_INACTIVE, LIMIT_LOWER, LIMIT_UPPER, LIMIT_EQUAL = 0, 1, 2, 3

#: ``gb_joint``: a joint's definition and carried state (joints/joint.py and the four kinds)
JOINT = np.dtype([
    ("world", "<i4"), ("type", "<i4"), ("body_a", "<i4"), ("body_b", "<i4"), ("flags", "<u4"), ("limit_state", "<i4"),
    ("la_x", "<f8"), ("la_y", "<f8"), ("lb_x", "<f8"), ("lb_y", "<f8"), ("ref_angle", "<f8"),
    ("ax_x", "<f8"), ("ax_y", "<f8"), ("lower", "<f8"), ("upper", "<f8"), ("max_motor", "<f8"), ("motor_speed", "<f8"),
    ("length", "<f8"), ("frequency", "<f8"), ("damping_ratio", "<f8"),
    ("impulse", "<f8", (3,)), ("motor_impulse", "<f8"), ("gamma", "<f8"), ("bias", "<f8"),
    ("ux", "<f8"), ("uy", "<f8"), ("perp_x", "<f8"), ("perp_y", "<f8"),
    ("max_force", "<f8"), ("max_torque", "<f8"), ("max_length", "<f8"), ("cur_length", "<f8"),
    ("spring_impulse", "<f8"), ("sax_x", "<f8"), ("sax_y", "<f8"), ("s_ax", "<f8"), ("s_bx", "<f8"),
    ("ga_x", "<f8"), ("ga_y", "<f8"), ("gb_x", "<f8"), ("gb_y", "<f8"), ("ratio", "<f8"), ("constant", "<f8"),
    ("target_x", "<f8"), ("target_y", "<f8"),
], align=True)

CONTROLLER_BUOYANCY, CONTROLLER_GRAVITY = 1, 2
CTRL_OWN_GRAVITY, CTRL_INV_SQR = 1, 2

#: ``gb_controller``: one controller (controllers.py) with its body-list range
CONTROLLER = np.dtype([
    ("world", "<i4"), ("type", "<i4"), ("body_start", "<i4"), ("body_count", "<i4"), ("flags", "<u4"), ("_pad0", "<i4"),
    ("normal_x", "<f8"), ("normal_y", "<f8"), ("offset", "<f8"), ("density", "<f8"),
    ("velocity_x", "<f8"), ("velocity_y", "<f8"), ("linear_drag", "<f8"), ("angular_drag", "<f8"),
    ("gravity_x", "<f8"), ("gravity_y", "<f8"), ("G", "<f8"),
], align=True)

WORLD = np.dtype([
    ("body_start", "<i4"), ("body_count", "<i4"), ("fixture_start", "<i4"), ("fixture_count", "<i4"),
    ("contact_start", "<i4"), ("contact_count", "<i4"), ("contact_capacity", "<i4"), ("flags", "<u4"),
    ("move_start", "<i4"), ("move_count", "<i4"),
    ("gx", "<f8"), ("gy", "<f8"), ("inv_dt0", "<f8"),
], align=True)


class Scene(ctypes.Structure):
    """ctypes form of ``gb_scene``."""
    _fields_ = [
        ("n_worlds", ctypes.c_int32), ("n_bodies", ctypes.c_int32),
        ("n_fixtures", ctypes.c_int32), ("n_contacts", ctypes.c_int32),
        ("worlds", ctypes.c_void_p), ("bodies", ctypes.c_void_p),
        ("fixtures", ctypes.c_void_p), ("contacts", ctypes.c_void_p),
        ("n_moves", ctypes.c_int32), ("_pad0", ctypes.c_int32), ("moves", ctypes.c_void_p),
        ("n_joints", ctypes.c_int32), ("_pad1", ctypes.c_int32), ("joints", ctypes.c_void_p),
        ("n_controllers", ctypes.c_int32), ("n_controller_bodies", ctypes.c_int32),
        ("controllers", ctypes.c_void_p), ("controller_bodies", ctypes.c_void_p),
    ]


class StepOpts(ctypes.Structure):
    """ctypes form of ``gb_step_opts``."""
    _fields_ = [
        ("dt", ctypes.c_double), ("vel_iters", ctypes.c_int32), ("pos_iters", ctypes.c_int32),
        ("n_steps", ctypes.c_int32), ("launch_mode", ctypes.c_int32),
        ("block_threads", ctypes.c_int32), ("record_order", ctypes.c_int32),
    ]


class LaunchConfig(ctypes.Structure):
    """ctypes form of ``gb_launch_config``."""
    _fields_ = [
        ("launch_mode", ctypes.c_int32), ("block_threads", ctypes.c_int32),
        ("pipe_bufs", ctypes.c_int32), ("big_bodies", ctypes.c_int32),
        ("groups", ctypes.c_int32), ("_pad0", ctypes.c_int32),
        ("ms_per_step", ctypes.c_double),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if not k.startswith("_")}



#: gb_ray, gb_ray_hit, gb_aabb_query (world queries)
RAY = np.dtype([("world", "<i4"), ("_pad0", "<i4"), ("p1x", "<f8"), ("p1y", "<f8"), ("p2x", "<f8"), ("p2y", "<f8")],
               align=True)
RAY_HIT = np.dtype([("fixture", "<i4"), ("_pad0", "<i4"), ("px", "<f8"), ("py", "<f8"), ("nx", "<f8"), ("ny", "<f8"),
                    ("fraction", "<f8")], align=True)
AABB_QUERY = np.dtype([("world", "<i4"), ("_pad0", "<i4"), ("lx", "<f8"), ("ly", "<f8"), ("ux", "<f8"), ("uy", "<f8")],
                      align=True)

#: sizeof(gb_launch_config) (GB_LAUNCH_CONFIG_BYTES)
LAUNCH_CONFIG_BYTES = 32


def make_scene(worlds: np.ndarray, bodies: np.ndarray, fixtures: np.ndarray,
               contacts: np.ndarray | None = None, moves: np.ndarray | None = None,
               joints: np.ndarray | None = None, controllers: np.ndarray | None = None,
               controller_bodies: np.ndarray | None = None) -> tuple[Scene, tuple]:
    """Pack contiguous record arrays into a ``gb_scene``; the returned tuple
    keeps the arrays alive as long as the scene is used.  ``joints`` are
    sorted by their ``world`` field (stable: each world keeps its order);
    ``controllers`` must already be sorted by world, their ``body_start``
    indexing ``controller_bodies``."""
    worlds = np.ascontiguousarray(worlds, dtype=WORLD)
    bodies = np.ascontiguousarray(bodies, dtype=BODY)
    fixtures = np.ascontiguousarray(fixtures, dtype=FIXTURE)
    if contacts is None:
        contacts = np.zeros(0, dtype=CONTACT)
    contacts = np.ascontiguousarray(contacts, dtype=CONTACT)
    s = Scene()
    s.n_worlds = len(worlds)
    s.n_bodies = len(bodies)
    s.n_fixtures = len(fixtures)
    s.n_contacts = len(contacts)
    s.worlds = worlds.ctypes.data
    s.bodies = bodies.ctypes.data
    s.fixtures = fixtures.ctypes.data
    s.contacts = contacts.ctypes.data if len(contacts) else None
    moves = np.ascontiguousarray(moves if moves is not None else np.zeros(0, np.int32), dtype=np.int32)
    s.n_moves = len(moves)
    s.moves = moves.ctypes.data if len(moves) else None
    joints = np.ascontiguousarray(joints if joints is not None else np.zeros(0, JOINT), dtype=JOINT)
    if len(joints) and np.any(np.diff(joints["world"]) < 0):
        joints = joints[np.argsort(joints["world"], kind="stable")]
    s.n_joints = len(joints)
    s.joints = joints.ctypes.data if len(joints) else None
    controllers = np.ascontiguousarray(controllers if controllers is not None else np.zeros(0, CONTROLLER),
                                       dtype=CONTROLLER)
    cbodies = np.ascontiguousarray(controller_bodies if controller_bodies is not None else np.zeros(0, np.int32),
                                   dtype=np.int32)
    s.n_controllers = len(controllers)
    s.controllers = controllers.ctypes.data if len(controllers) else None
    s.n_controller_bodies = len(cbodies)
    s.controller_bodies = cbodies.ctypes.data if len(cbodies) else None
    return s, (worlds, bodies, fixtures, contacts, moves, joints, controllers, cbodies)


_PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG_DIR, "_build", "libgb2d.so")

EXPORTED = (
    "gb_version", "gb_last_error", "gb_struct_sizes",
    "gb_batch_create", "gb_batch_destroy", "gb_batch_step",
    "gb_batch_set_bodies", "gb_batch_get_bodies", "gb_batch_step_host", "gb_batch_step_host_state", "gb_body_state_size", "gb_batch_get_proxies",
    "gb_batch_get_contact_counts", "gb_batch_get_contacts", "gb_batch_get_solver_order",
    "gb_batch_status", "gb_batch_counters", "gb_batch_phase_clocks",
    "gb_batch_step_static_scratch", "gb_batch_kernel_times", "gb_batch_get_events",
    "gb_batch_set_launch_config", "gb_batch_get_launch_config", "gb_batch_autotune",
    "gb_graph_capture", "gb_graph_launch", "gb_graph_destroy",
    "gb_batch_ray_cast", "gb_batch_ray_cast_all", "gb_batch_query_aabb",
    "gb_batch_snapshot_bytes", "gb_batch_snapshot", "gb_batch_restore", "gb_batch_get_step_record",
    "gb_batch_set_wait_polls", "gb_batch_clear_status",
    "gb_joint_size", "gb_batch_get_joint_order", "gb_batch_get_joints", "gb_batch_set_joints",
    "gb_controller_size", "gb_batch_set_controllers", "gb_batch_set_pair_filter",
)

#: gb_step_opts.record_order bit that records contact events
OPT_EVENTS = 8
EV_BEGIN, EV_END, EV_POST_SOLVE = 1, 2, 3
ST_EVENT_OVERFLOW = 64
EVENT = np.dtype([
    ("type", "<i4"), ("fixture_a", "<i4"), ("fixture_b", "<i4"), ("point_count", "<i4"), ("key", "<i8"),
    ("normal_impulse", "<f8", (2,)), ("tangent_impulse", "<f8", (2,)),
], align=True)

#: gb_step_opts.record_order bit that times each launch of the phased step
OPT_KERNEL_TIMES = 4
KERNEL_SLOTS = ("pairs_new", "pre", "collide", "collide_sleeping", "islands", "vinit", "cinit", "solve",
                "sync_pairs", "toi_candidates", "toi_first_pass", "toi_setup", "toi_events")

#: bytes of the static device scratch behind gb_batch_step_static_scratch
STATIC_SCRATCH_BYTES = 32 << 20

#: C-ABI status codes (include/gb2d.h GB_E_*)
E_OK, E_ARG, E_CUDA, E_CONTACT_OVERFLOW, E_UNSUPPORTED, E_NONFINITE, E_ITER_LIMIT, E_SCRATCH = 0, -1, -2, -3, -4, -5, -6, -7

_lib = None


class GB2DError(RuntimeError):
    """A C-ABI call returned an error status (message from gb_last_error)."""


def load_library(path: str | None = None) -> ctypes.CDLL:
    """Load ``libgb2d.so`` (built in-tree by ``__graft_entry__.build``).

    There is no fallback: a missing library raises, so nothing silently runs
    on the CPU."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise GB2DError(f"libgb2d.so not built ({p}); run __graft_entry__.build()")
    lib = ctypes.CDLL(p)
    vp, i32, u32p, i32p = ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_int32)
    lib.gb_version.restype = ctypes.c_char_p
    lib.gb_last_error.restype = ctypes.c_char_p
    lib.gb_struct_sizes.argtypes = [i32p]
    lib.gb_batch_create.argtypes = [ctypes.POINTER(Scene), i32, ctypes.POINTER(vp)]
    lib.gb_batch_destroy.argtypes = [vp]
    lib.gb_batch_step.argtypes = [vp, ctypes.POINTER(StepOpts), vp]
    lib.gb_batch_set_bodies.argtypes = [vp, vp, i32, vp]
    lib.gb_batch_get_bodies.argtypes = [vp, vp, i32, vp]
    lib.gb_batch_step_host.argtypes = [vp, vp, vp, i32, ctypes.POINTER(StepOpts), vp]
    lib.gb_batch_step_host_state.argtypes = [vp, vp, vp, i32, ctypes.POINTER(StepOpts), vp]
    lib.gb_body_state_size.argtypes = []
    lib.gb_batch_get_proxies.argtypes = [vp, vp, i32, vp]
    lib.gb_batch_get_contact_counts.argtypes = [vp, i32p, vp]
    lib.gb_batch_get_contacts.argtypes = [vp, i32, vp, i32, i32p, vp]
    lib.gb_batch_get_solver_order.argtypes = [vp, i32, i32p, i32, i32p, vp]
    lib.gb_batch_status.argtypes = [vp, u32p, vp]
    lib.gb_batch_counters.argtypes = [vp, ctypes.POINTER(ctypes.c_int64)]
    lib.gb_batch_phase_clocks.argtypes = [vp, ctypes.POINTER(ctypes.c_int64), vp]
    lib.gb_batch_step_static_scratch.argtypes = [vp, ctypes.POINTER(StepOpts), vp]
    lib.gb_batch_kernel_times.argtypes = [vp, ctypes.POINTER(ctypes.c_double), i32, i32p, ctypes.POINTER(ctypes.c_int64)]
    lib.gb_batch_get_events.argtypes = [vp, i32, vp, i32, i32p, vp]
    cfgp = ctypes.POINTER(LaunchConfig)
    lib.gb_batch_set_launch_config.argtypes = [vp, cfgp]
    lib.gb_batch_get_launch_config.argtypes = [vp, cfgp]
    lib.gb_batch_autotune.argtypes = [vp, ctypes.POINTER(StepOpts), cfgp, i32, i32p, cfgp, vp]
    lib.gb_graph_capture.argtypes = [vp, ctypes.POINTER(StepOpts), ctypes.POINTER(vp)]
    lib.gb_graph_launch.argtypes = [vp, vp]
    lib.gb_graph_destroy.argtypes = [vp]
    lib.gb_batch_ray_cast.argtypes = [vp, vp, i32, vp, vp]
    lib.gb_batch_query_aabb.argtypes = [vp, vp, i32, i32p, i32, i32p, vp]
    lib.gb_batch_ray_cast_all.argtypes = [vp, vp, i32, vp, i32, i32p, vp]
    lib.gb_batch_snapshot_bytes.argtypes = [vp, ctypes.POINTER(ctypes.c_uint64)]
    lib.gb_batch_snapshot.argtypes = [vp, vp, ctypes.c_uint64, vp]
    lib.gb_batch_restore.argtypes = [vp, vp, ctypes.c_uint64, vp]
    lib.gb_batch_get_step_record.argtypes = [vp, i32, i32p, i32, i32p, vp]
    lib.gb_batch_set_wait_polls.argtypes = [vp, i32]
    lib.gb_batch_clear_status.argtypes = [vp, vp]
    lib.gb_joint_size.argtypes = []
    lib.gb_batch_get_joint_order.argtypes = [vp, i32, i32p, i32, i32p, vp]
    lib.gb_batch_get_joints.argtypes = [vp, vp, i32, vp]
    lib.gb_batch_set_joints.argtypes = [vp, vp, i32, vp]
    lib.gb_controller_size.argtypes = []
    lib.gb_batch_set_controllers.argtypes = [vp, vp, i32, vp]
    lib.gb_batch_set_pair_filter.argtypes = [vp, i32, vp, i32, vp]
    for name in EXPORTED:
        if name not in ("gb_version", "gb_last_error"):
            getattr(lib, name).restype = ctypes.c_int
    if path is None:
        _lib = lib
    return lib


def check(rc: int) -> None:
    """Raise GB2DError with the library's message when rc != 0."""
    if rc != 0:
        msg = load_library().gb_last_error().decode(errors="replace")
        raise GB2DError(f"gb2d error {rc}: {msg}")

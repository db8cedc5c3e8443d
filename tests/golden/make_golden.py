"""Generate the golden vectors of the World.step path by running the
reference pypybox2d itself (C-extension math mode) in this container.

Usage:  python tests/golden/make_golden.py --ref <pypybox2d source tree>   (or GB2D_REFERENCE=<tree>)

The reference is imported from its source tree (read only); its C extension
`_common` must first be compiled by oracle/build_ref.sh into oracle/_ref/.
Two harness hooks are installed, neither of which touches the physics:
  * BroadPhase.update_pairs yields the same pair set with the same pair
    orientation as the reference, in a fixed order (first position of the
    moved proxy in the move buffer, then the other proxy's index) instead of
    Python-set order (broadphase.py:83-109);
  * Island.solve records the contact-list position of each island contact in
    solver order, so the natural (depth-first) constraint order is pinned too.

Each scene is built through the reference's public API (World,
create_*_body, Fixture, Polygon/Circle/Edge), exported to the record layouts
of include/gb2d.h, stepped, and snapshotted at fixed steps.  The result is
one compressed .npz per scene under tests/golden/.
"""
from __future__ import annotations

import argparse
import glob
import importlib.util
import math
import os
import random
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
from pypybox2d_gb300 import abi  # noqa: E402


def load_reference(ref_root: str):
    sos = glob.glob(os.path.join(REPO, "oracle", "_ref", "_common*.so"))
    if not sos:
        raise SystemExit("build the reference extension first: oracle/build_ref.sh")
    spec = importlib.util.spec_from_file_location("pypybox2d._common", sos[0])
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    sys.modules["pypybox2d._common"] = mod
    sys.path.insert(0, ref_root)
    import pypybox2d as b2  # noqa: F401
    from pypybox2d import common
    assert common.Vec2 is mod.Vec2, "reference did not pick up the C extension"
    return b2


def fixture_index(world):
    """id(fixture) -> its first record; a loop fixture takes one record per
    child (its proxies, fixture.py:250-261), so proxy (f, child) is record
    idx[id(f)] + child."""
    idx = {}
    k = 0
    for body in world.bodies:
        for f in body.fixtures:
            idx[id(f)] = k
            k += f._shape.child_count
    return idx


class OrderLog(list):
    """Contact-list positions of the island contacts in solver order, and
    (.joints) the World.joints positions of the island joints."""

    def __init__(self):
        super().__init__()
        self.joints: list[int] = []


def install_hooks(world, b2, order_log):
    fidx = fixture_index(world)
    bp = world.contact_manager.broadphase

    def update_pairs(self, callback=None):
        first = {}
        for i, node in enumerate(self._move_buffer):
            if node not in first:
                first[node] = i
        pairs = []
        for node, pos in first.items():
            for res in self._tree.query(node.aabb):
                if res is node:
                    continue
                if res in first and first[res] < pos:
                    continue
                pairs.append((pos, fidx[id(res.user_data.fixture)] + res.user_data.child_index, node, res))
        self._move_buffer = []
        pairs.sort(key=lambda t: (t[0], t[1]))
        for _, _, a, b in pairs:
            yield (a.user_data, b.user_data)

    bp.update_pairs = types.MethodType(update_pairs, bp)

    from pypybox2d import island as island_mod
    orig_solve = island_mod.Island.solve

    def solve(self, step, gravity, allow_sleep):
        pos = {id(c): i for i, c in enumerate(world.contact_manager.contacts)}
        order_log.extend(pos[id(c)] for c in self.contacts)
        jpos = {id(j): i for i, j in enumerate(world.joints)}
        order_log.joints.extend(jpos[id(j)] for j in self.joints)
        return orig_solve(self, step, gravity, allow_sleep)

    island_mod.Island.solve = solve
    return orig_solve


def export_world(world, b2, contacts=True):
    """Reference world -> (worlds, bodies, fixtures, contacts) record arrays."""
    fidx = fixture_index(world)
    nb = len(world.bodies)
    nf = sum(f._shape.child_count for b in world.bodies for f in b.fixtures)
    B = np.zeros(nb, dtype=abi.BODY)
    F = np.zeros(nf, dtype=abi.FIXTURE)
    k = 0
    for i, body in enumerate(world.bodies):
        r = B[i]
        r["type"] = body._type
        fl = 0
        if body._awake:
            fl |= abi.BODY_AWAKE
        if body._allow_sleep:
            fl |= abi.BODY_ALLOW_SLEEP
        if body._bullet:
            fl |= abi.BODY_BULLET
        if body._fixed_rotation:
            fl |= abi.BODY_FIXED_ROTATION
        if body._active:
            fl |= abi.BODY_ACTIVE
        r["flags"] = fl
        r["fixture_start"] = k
        r["fixture_count"] = sum(f._shape.child_count for f in body.fixtures)
        xf = body._xf
        r["px"], r["py"] = xf.position.x, xf.position.y
        rot = xf.rotation
        r["qc"], r["qs"] = rot.col1.x, rot.col1.y
        sw = body._sweep
        r["lcx"], r["lcy"] = sw.local_center.x, sw.local_center.y
        r["c0x"], r["c0y"] = sw.c0.x, sw.c0.y
        r["cx"], r["cy"] = sw.c.x, sw.c.y
        r["a0"], r["a"], r["alpha0"] = sw.a0, sw.a, sw.alpha0
        r["vx"], r["vy"] = body._linear_velocity.x, body._linear_velocity.y
        r["w"] = body._angular_velocity
        r["fx"], r["fy"] = body._force.x, body._force.y
        r["torque"] = body._torque
        r["mass"], r["inv_mass"], r["I"], r["inv_I"] = body._mass, body._inv_mass, body._I, body._invI
        r["linear_damping"], r["angular_damping"] = body._linear_damping, body._angular_damping
        r["gravity_scale"] = body._gravity_scale
        r["sleep_time"] = body._sleep_time
        for f, child, sh in ((f, c, f._shape.child_edge(c) if f._shape._type == abi.SHAPE_LOOP else f._shape)
                             for f in body.fixtures for c in range(f._shape.child_count)):
            q = F[k]
            q["body"] = i
            q["shape_type"] = sh._type
            q["radius"] = sh.radius
            q["friction"], q["restitution"], q["density"] = f._friction, f._restitution, f._density
            q["category_bits"], q["mask_bits"], q["group_index"] = f._category_bits, f._mask_bits, f._group_index
            fl = abi.FIX_SENSOR if f._sensor else 0
            if f._shape._type == abi.SHAPE_LOOP:
                fl |= abi.FIX_LOOP_CHILD | (abi.FIX_LOOP_FIRST if child == 0 else 0)
            if sh._type == abi.SHAPE_CIRCLE:
                q["vertex_count"] = 1
                q["vx"][0], q["vy"][0] = sh.position.x, sh.position.y
            elif sh._type == abi.SHAPE_POLYGON:
                q["vertex_count"] = len(sh._vertices)
                for j, (v, n) in enumerate(zip(sh._vertices, sh._normals)):
                    q["vx"][j], q["vy"][j] = v.x, v.y
                    q["nx"][j], q["ny"][j] = n.x, n.y
            elif sh._type == abi.SHAPE_EDGE:
                q["vertex_count"] = 2
                q["vx"][0], q["vy"][0] = sh._vertex1.x, sh._vertex1.y
                q["vx"][1], q["vy"][1] = sh._vertex2.x, sh._vertex2.y
                if sh._vertex0 is not None:
                    fl |= abi.FIX_EDGE_HAS_V0
                    q["vx"][2], q["vy"][2] = sh._vertex0.x, sh._vertex0.y
                if sh._vertex3 is not None:
                    fl |= abi.FIX_EDGE_HAS_V3
                    q["vx"][3], q["vy"][3] = sh._vertex3.x, sh._vertex3.y
            else:
                raise NotImplementedError(f"shape type {sh._type} is not exported")
            q["flags"] = fl
            if f._proxies and f._proxies[child].proxy_ref is not None:
                aabb = f._proxies[child].proxy_ref.aabb
                q["aabb"][:] = (aabb.lower_bound.x, aabb.lower_bound.y, aabb.upper_bound.x, aabb.upper_bound.y)
            else:   # an inactive body's fixture has no proxy (body.py:846-872)
                q["aabb"][:] = np.nan
            k += 1
    clist = world.contact_manager.contacts if contacts else []
    C = np.zeros(len(clist), dtype=abi.CONTACT)
    for i, c in enumerate(clist):
        r = C[i]
        # a loop's child is its own record: the child index goes into the
        # record index, the child fields stay 0
        r["fixture_a"], r["fixture_b"] = fidx[id(c._fixture_a)] + c._index_a, fidx[id(c._fixture_b)] + c._index_b
        fl = 0
        for bit, name in ((abi.C_TOUCHING, "_touching_flag"), (abi.C_ENABLED, "_enabled_flag"),
                          (abi.C_FILTER, "_filter_flag"), (abi.C_ISLAND, "_island_flag"),
                          (abi.C_TOI, "_toi_flag"), (abi.C_BULLET_HIT, "_bullet_hit_flag")):
            if getattr(c, name):
                fl |= bit
        r["flags"] = fl
        r["toi_count"], r["toi"] = c._toi_count, c._toi
        r["friction"], r["restitution"] = c._friction, c._restitution
        m = c._manifold
        r["m_type"], r["m_point_count"] = m.type, m.point_count
        r["m_lnx"], r["m_lny"] = m.local_normal.x, m.local_normal.y
        r["m_lpx"], r["m_lpy"] = m.local_point.x, m.local_point.y
        for j in range(2):
            p = m.points[j]
            r["p_lx"][j], r["p_ly"][j] = p.local_point.x, p.local_point.y
            r["p_ni"][j], r["p_ti"][j] = p.normal_impulse, p.tangent_impulse
            ia, ib, ta, tb = p.id
            r["p_id"][j] = (ia & 255) | ((ib & 255) << 8) | ((ta & 255) << 16) | ((tb & 255) << 24)
    W = np.zeros(1, dtype=abi.WORLD)
    wf = 0
    if world._allow_sleep:
        wf |= abi.W_ALLOW_SLEEP
    if world._warm_starting:
        wf |= abi.W_WARM_STARTING
    if world._continuous_physics:
        wf |= abi.W_CONTINUOUS
    if world._auto_clear_forces:
        wf |= abi.W_AUTO_CLEAR_FORCES
    if world._new_fixture:
        wf |= abi.W_NEW_FIXTURE
    if world._step_complete:
        wf |= abi.W_STEP_COMPLETE
    W[0] = (0, nb, 0, nf, 0, len(C), max(64, 8 * nf), wf, 0, 0, world._gravity.x, world._gravity.y, world._inv_dt0)
    return W, B, F, C


def export_joints(world, b2):
    """Reference World.joints -> gb_joint records (definition and carried state)."""
    from pypybox2d import joints as jm
    bidx = {id(b): i for i, b in enumerate(world.bodies)}
    J = np.zeros(len(world.joints), dtype=abi.JOINT)
    kinds = ((jm.RevoluteJoint, abi.JOINT_REVOLUTE), (jm.PrismaticJoint, abi.JOINT_PRISMATIC),
             (jm.DistanceJoint, abi.JOINT_DISTANCE), (jm.WeldJoint, abi.JOINT_WELD),
             (jm.FrictionJoint, abi.JOINT_FRICTION), (jm.RopeJoint, abi.JOINT_ROPE), (jm.WheelJoint, abi.JOINT_WHEEL),
             (jm.PulleyJoint, abi.JOINT_PULLEY), (jm.MouseJoint, abi.JOINT_MOUSE))
    for i, j in enumerate(world.joints):
        r = J[i]
        r["type"] = next(t for cls, t in kinds if type(j) is cls)
        # a mouse joint has no body_a (mouse.py:67): its record repeats body_b
        r["body_a"] = bidx[id(j._body_a if j._body_a is not None else j._body_b)]
        r["body_b"] = bidx[id(j._body_b)]
        fl = abi.J_COLLIDE_CONNECTED if j._collide_connected else 0
        if getattr(j, "_limit_enabled", False):
            fl |= abi.J_LIMIT
        if getattr(j, "_motor_enabled", False):
            fl |= abi.J_MOTOR
        r["flags"] = fl
        if r["type"] != abi.JOINT_MOUSE:   # mouse.py keeps a local anchor on body_b only
            r["la_x"], r["la_y"] = j._local_anchor_a.x, j._local_anchor_a.y
        r["lb_x"], r["lb_y"] = j._local_anchor_b.x, j._local_anchor_b.y
        if r["type"] == abi.JOINT_FRICTION:
            r["max_force"], r["max_torque"] = j._max_force, j._max_torque
            r["impulse"][:] = (j._linear_impulse.x, j._linear_impulse.y, j._angular_impulse)
            continue
        if r["type"] == abi.JOINT_ROPE:
            r["max_length"], r["cur_length"] = j._max_length, j._length
            r["impulse"][0] = j._impulse
            r["limit_state"] = j._state
            r["ux"], r["uy"] = j._u.x, j._u.y
            continue
        if r["type"] == abi.JOINT_WHEEL:
            r["ax_x"], r["ax_y"] = j._local_x_axis.x, j._local_x_axis.y
            r["frequency"], r["damping_ratio"] = j._frequency, j._damping_ratio
            r["max_motor"], r["motor_speed"] = j._max_motor_torque, j._motor_speed
            r["impulse"][0] = j._impulse
            r["motor_impulse"], r["spring_impulse"] = j._motor_impulse, j._spring_impulse
            r["sax_x"], r["sax_y"], r["s_ax"], r["s_bx"] = j._ax.x, j._ax.y, j._s_ax, j._s_bx
            r["perp_x"], r["perp_y"] = j._ay.x, j._ay.y
            r["bias"], r["gamma"] = j._bias, j._gamma
            continue
        if r["type"] == abi.JOINT_MOUSE:
            r["lb_x"], r["lb_y"] = j._local_anchor_b.x, j._local_anchor_b.y
            r["target_x"], r["target_y"] = j._target.x, j._target.y
            r["max_force"], r["frequency"], r["damping_ratio"] = j._max_force, j._frequency, j._damping_ratio
            r["impulse"][:2] = (j._impulse.x, j._impulse.y)
            r["gamma"], r["bias"] = j._gamma, j._beta
            continue
        if r["type"] == abi.JOINT_PULLEY:
            r["ga_x"], r["ga_y"] = j._ground_anchor_a.x, j._ground_anchor_a.y
            r["gb_x"], r["gb_y"] = j._ground_anchor_b.x, j._ground_anchor_b.y
            r["ratio"], r["constant"] = j._ratio, j._constant
            r["impulse"][0] = j._impulse
            continue
        if r["type"] == abi.JOINT_DISTANCE:
            r["length"], r["frequency"], r["damping_ratio"] = j._length, j._frequency, j._damping_ratio
            r["impulse"][0] = j._impulse
            r["gamma"], r["bias"] = j._gamma, j._bias
            r["ux"], r["uy"] = j._u.x, j._u.y
            continue
        r["ref_angle"] = j._reference_angle
        r["impulse"][:] = (j._impulse.x, j._impulse.y, j._impulse.z)
        if r["type"] == abi.JOINT_REVOLUTE:
            r["lower"], r["upper"] = j._lower_angle, j._upper_angle
            r["max_motor"], r["motor_speed"] = j._max_motor_torque, j._motor_speed
            r["motor_impulse"], r["limit_state"] = j._motor_impulse, j._limit_state
        elif r["type"] == abi.JOINT_PRISMATIC:
            r["ax_x"], r["ax_y"] = j._local_x_axis.x, j._local_x_axis.y
            r["lower"], r["upper"] = j._lower_limit, j._upper_limit
            r["max_motor"], r["motor_speed"] = j._max_motor_force, j._motor_speed
            r["motor_impulse"], r["limit_state"] = j._motor_impulse, j._limit_state
            r["ux"], r["uy"] = j._axis.x, j._axis.y
            r["perp_x"], r["perp_y"] = j._perp.x, j._perp.y
    return J


# ---------------------------------------------------------------- scenes
def export_controllers(world, b2):
    """Reference World.controllers -> (gb_controller records, body lists)."""
    from pypybox2d import controllers as cm
    bidx = {id(b): i for i, b in enumerate(world.bodies)}
    C = np.zeros(len(world.controllers), dtype=abi.CONTROLLER)
    bodies = []
    for k, c in enumerate(world.controllers):
        r = C[k]
        if type(c) is cm.BuoyancyController:
            r["type"] = abi.CONTROLLER_BUOYANCY
            own = bool(c._gravity)      # None or a zero Vec2 take the world's (controllers.py:177)
            r["flags"] = abi.CTRL_OWN_GRAVITY if own else 0
            r["normal_x"], r["normal_y"] = c._normal.x, c._normal.y
            r["offset"], r["density"] = c._offset, c._density
            r["velocity_x"], r["velocity_y"] = c._velocity.x, c._velocity.y
            r["linear_drag"], r["angular_drag"] = c._linear_drag, c._angular_drag
            if own:
                r["gravity_x"], r["gravity_y"] = c._gravity.x, c._gravity.y
        elif type(c) is cm.GravityController:
            r["type"] = abi.CONTROLLER_GRAVITY
            r["flags"] = abi.CTRL_INV_SQR if c._inv_sqr else 0
            r["G"] = c._G
        else:
            raise NotImplementedError(type(c).__name__)
        mine = [bidx[id(b)] for b in c._bodies if id(b) in bidx]
        r["body_start"], r["body_count"] = len(bodies), len(mine)
        bodies.extend(mine)
    return C, np.array(bodies, dtype=np.int32)


def scene_pyramid(b2, rows=20):
    """Configuration 1: the pyramid of 20 rows of 0.5 m boxes (210 bodies)."""
    from pypybox2d.common import Vec2
    from copy import copy
    world = b2.World(gravity=(0, -10), do_sleep=True)
    world.create_static_body(position=(0, -0.5), shapes=b2.Polygon(box=(40, 0.5)))
    fixture = b2.Fixture(b2.Polygon(box=(0.5, 0.5)), density=5.0, friction=0.6, restitution=0.0)
    x = Vec2(-7.0, 0.75)
    dx, dy = Vec2(0.5625, 1.25), Vec2(1.125, 0.0)
    for i in range(rows):
        y = copy(x)
        for _ in range(i, rows):
            world.create_dynamic_body(position=y, fixtures=fixture)
            y = y + dy
        x = x + dx
    return world


def random_convex(rng, n, rad):
    """Convex CCW polygon: hull of n random points at radius `rad` (sorted
    angles on a circle are in convex position)."""
    angs = sorted(rng.uniform(0, 2 * math.pi) for _ in range(n))
    pts = [(rad * math.cos(a), rad * math.sin(a)) for a in angs]
    return pts


def scene_mixed(b2, n=40, seed=3, size=12.0):
    """Configuration-3 style: a static box container of 4 edge shapes with
    random circles and convex polygons, random velocities."""
    rng = random.Random(seed)
    world = b2.World(gravity=(0, -10), do_sleep=True)
    h = size / 2
    ground = world.create_static_body()
    for v1, v2 in (((-h, -h), (h, -h)), ((h, -h), (h, h)), ((h, h), (-h, h)), ((-h, h), (-h, -h))):
        ground.create_edge_fixture(v1, v2, friction=0.5)
    cols = int(math.ceil(math.sqrt(n)))
    spacing = (size - 2.5) / cols
    k = 0
    for gy in range(cols):
        for gx in range(cols):
            if k >= n:
                break
            px = -h + 1.25 + (gx + 0.5) * spacing
            py = -h + 1.25 + (gy + 0.5) * spacing
            body = world.create_dynamic_body(position=(px, py), angle=rng.uniform(-3, 3),
                                             linear_velocity=(rng.gauss(0, 2), rng.gauss(0, 2)),
                                             angular_velocity=rng.gauss(0, 1))
            dens, fr, rest = rng.uniform(0.5, 5), rng.uniform(0.2, 0.8), rng.uniform(0, 0.3)
            rad = min(rng.uniform(0.25, 1.0), 0.45 * spacing)
            prad = min(rng.uniform(0.3, 1.0), 0.45 * spacing)
            if k % 2 == 0:
                body.create_circle_fixture(radius=rad, density=dens, friction=fr, restitution=rest)
            else:
                nv = rng.randint(3, 8)
                while True:
                    pts = random_convex(rng, nv, prad)
                    try:
                        body.create_polygon_fixture(vertices=pts, density=dens, friction=fr, restitution=rest)
                        break
                    except (ValueError, AssertionError):
                        continue
            k += 1
    return world


def scene_bullets(b2, seed=5):
    """Configuration-5 style: a stack of 8 boxes on a ground box plus 2 fast
    bullet circles (continuous collision)."""
    rng = random.Random(seed)
    world = b2.World(gravity=(0, -10), do_sleep=True)
    world.create_static_body(position=(0, -0.5), shapes=b2.Polygon(box=(40, 0.5)))
    for i in range(8):
        body = world.create_dynamic_body(position=(0.0, 0.5 + 1.0 * i))
        body.create_polygon_fixture(box=(0.5, 0.5), density=1.0, friction=0.3)
    for j in range(2):
        body = world.create_dynamic_body(position=(-30.0, rng.uniform(0.5, 7.0)), bullet=True,
                                         linear_velocity=(rng.uniform(150, 250), 0.0))
        body.create_circle_fixture(radius=0.1, density=100.0)
    return world


def scene_sleep(b2):
    """Small scene whose bodies fall asleep: one isolated box, a two-box
    stack and a circle on a ground box."""
    world = b2.World(gravity=(0, -10), do_sleep=True)
    world.create_static_body(position=(0, -0.5), shapes=b2.Polygon(box=(20, 0.5)))
    world.create_dynamic_body(position=(-5, 0.6)).create_polygon_fixture(box=(0.5, 0.5), density=1.0)
    world.create_dynamic_body(position=(0, 0.5)).create_polygon_fixture(box=(0.5, 0.5), density=1.0)
    world.create_dynamic_body(position=(0, 1.5)).create_polygon_fixture(box=(0.5, 0.5), density=1.0)
    world.create_dynamic_body(position=(5, 0.5)).create_circle_fixture(radius=0.5, density=1.0)
    return world


def scene_kinematic(b2, seed=9):
    """Kinematic bodies: a platform sliding sideways and a spinning paddle
    (both moved by their velocities alone) under falling boxes and circles,
    above a static ground box."""
    rng = random.Random(seed)
    world = b2.World(gravity=(0, -10), do_sleep=True)
    world.create_static_body(position=(0, -0.5), shapes=b2.Polygon(box=(30, 0.5)))
    world.create_kinematic_body(position=(-4, 3), linear_velocity=(1.5, 0.0),
                                shapes=b2.Polygon(box=(3, 0.25)))
    world.create_kinematic_body(position=(5, 2.5), angular_velocity=1.2,
                                shapes=b2.Polygon(box=(2.5, 0.2)))
    for i in range(24):
        x, y = rng.uniform(-7, 8), 5 + 0.9 * i
        body = world.create_dynamic_body(position=(x, y), angle=rng.uniform(-1, 1))
        if i % 3 == 0:
            body.create_circle_fixture(radius=rng.uniform(0.2, 0.45), density=1.0, friction=0.4)
        else:
            body.create_polygon_fixture(box=(rng.uniform(0.2, 0.5), rng.uniform(0.2, 0.5)), density=1.0,
                                        friction=0.4, restitution=rng.uniform(0, 0.3))
    return world


def scene_uneven(b2, seed=11, n=250):
    """One world of the uneven-batch workload (pypybox2d_gb300.scenes draws:
    100 m container of 4 edges, circles and convex polygons on a 2.1 m grid,
    random velocities), built through the reference's API."""
    from pypybox2d_gb300 import scenes
    d = scenes._uneven_draws(seed, n)
    world = b2.World(gravity=(0, -10), do_sleep=True)
    h = scenes.CONTAINER_HALF
    edges = [((-h, -h), (h, -h)), ((h, -h), (h, h)), ((h, h), (-h, h)), ((-h, h), (-h, -h))]
    world.create_static_body(position=(0, 0), fixtures=[b2.Fixture(b2.Edge(v1, v2)) for v1, v2 in edges])
    for i in range(d["n"]):
        if d["circle"][i]:
            shape = b2.Circle(radius=float(d["crad"][i]))
        else:
            k = int(d["nv"][i])
            shape = b2.Polygon(vertices=list(zip(d["vx"][i, :k].tolist(), d["vy"][i, :k].tolist())))
        fx = b2.Fixture(shape, density=float(d["density"][i]), friction=float(d["friction"][i]),
                        restitution=float(d["restitution"][i]))
        world.create_dynamic_body(position=(float(d["px"][i]), float(d["py"][i])), angle=float(d["angle"][i]),
                                  linear_velocity=(float(d["v"][i, 0]), float(d["v"][i, 1])),
                                  angular_velocity=float(d["w"][i]), fixtures=fx)
    return world


def scene_sensor_filter(b2, seed=13):
    """Sensors and collision filtering (contact.py:222-233 sensor touching,
    world.py:958-970 default filter): a static sensor box the bodies fall
    through; a dynamic circle carrying a large sensor ring; four boxes of
    group -1 (never collide with each other) falling through one another
    onto the ground; two boxes of group 2 (always collide) stacked; a
    category-2 plank on posts and a box whose mask leaves category 2 out, so
    it falls through the plank."""
    rng = random.Random(seed)
    world = b2.World(gravity=(0, -10), do_sleep=True)
    world.create_static_body(position=(0, -0.5), shapes=b2.Polygon(box=(20, 0.5)))
    region = world.create_static_body(position=(-6.0, 3.0))
    region.create_polygon_fixture(box=(2.0, 1.5), sensor=True)
    for k in range(3):   # bodies falling through the sensor region
        b = world.create_dynamic_body(position=(-6.5 + 1.0 * k, 7.0 + 1.2 * k), angle=rng.uniform(-0.5, 0.5))
        if k % 2:
            b.create_circle_fixture(radius=0.4, density=1.0, friction=0.5)
        else:
            b.create_polygon_fixture(box=(0.4, 0.3), density=1.0, friction=0.5)
    ring = world.create_dynamic_body(position=(-1.0, 1.5))
    ring.create_circle_fixture(radius=0.5, density=2.0, friction=0.4)
    ring.create_circle_fixture(radius=1.6, sensor=True)
    for k in range(4):   # group -1: they pass through each other
        b = world.create_dynamic_body(position=(2.0 + 0.3 * k, 1.0 + 0.7 * k), angle=0.2 * k)
        b.create_polygon_fixture(box=(0.5, 0.5), density=1.0, friction=0.6, group_index=-1)
    for k in range(2):   # group 2: they collide
        b = world.create_dynamic_body(position=(5.0, 0.6 + 1.1 * k))
        b.create_polygon_fixture(box=(0.5, 0.5), density=1.0, friction=0.6, group_index=2)
    posts = world.create_static_body(position=(9.0, 0.0))
    posts.create_polygon_fixture(vertices=[(-2.2, 0.0), (-1.8, 0.0), (-1.8, 2.0), (-2.2, 2.0)])
    posts.create_polygon_fixture(vertices=[(1.8, 0.0), (2.2, 0.0), (2.2, 2.0), (1.8, 2.0)])
    plank = world.create_dynamic_body(position=(9.0, 2.3))
    plank.create_polygon_fixture(box=(2.5, 0.2), density=1.0, friction=0.6, category_bits=0x0002)
    ghost = world.create_dynamic_body(position=(9.0, 4.0))
    ghost.create_polygon_fixture(box=(0.4, 0.4), density=1.0, friction=0.6, mask_bits=0xFFFD)
    solid = world.create_dynamic_body(position=(9.8, 4.5))
    solid.create_polygon_fixture(box=(0.3, 0.3), density=1.0, friction=0.6)
    return world


def scene_joints(b2, seed=17):
    """The four joint kinds of the island solver (island.py:107-148): a
    revolute chain hanging from a static anchor (links collide with nothing
    they are jointed to, body.py:912-927); a motorised revolute arm with an
    angle limit and a revolute with equal limits; a prismatic lift with
    limits and a motor, and a prismatic slider on a tilted unit axis (the
    reference does not normalise the axis; a longer one makes its position
    correction diverge); a rigid and a soft distance joint; a
    cantilever of welded boxes; boxes and circles dropped onto all of it."""
    rng = random.Random(seed)
    world = b2.World(gravity=(0, -10), do_sleep=True)
    ground = world.create_static_body(position=(0, -0.5), shapes=b2.Polygon(box=(30, 0.5)))
    # revolute chain
    anchor = world.create_static_body(position=(-12.0, 12.0), shapes=b2.Polygon(box=(0.3, 0.3)))
    prev = anchor
    for k in range(10):
        link = world.create_dynamic_body(position=(-11.5 + 1.0 * k, 12.0))
        link.create_polygon_fixture(box=(0.5, 0.125), density=20.0, friction=0.2)
        world.create_revolute_joint(prev, link, anchor=(-12.0 + 1.0 * k, 12.0))
        prev = link
    # motorised arm with a limit, and an arm whose limits are equal
    hub = world.create_static_body(position=(-4.0, 4.0), shapes=b2.Circle(radius=0.3))
    arm = world.create_dynamic_body(position=(-2.5, 4.0))
    arm.create_polygon_fixture(box=(1.5, 0.2), density=2.0, friction=0.5)
    world.create_revolute_joint(hub, arm, anchor=(-4.0, 4.0), lower_angle=-0.6, upper_angle=0.9, limit_enabled=True,
                                motor_speed=1.5, max_motor_torque=400.0, motor_enabled=True)
    stiff = world.create_dynamic_body(position=(-4.0, 7.5), angle=0.3)
    stiff.create_polygon_fixture(box=(1.0, 0.15), density=1.0, friction=0.5)
    world.create_revolute_joint(hub, stiff, anchor=(-4.0, 7.0), lower_angle=0.3, upper_angle=0.3, limit_enabled=True)
    # prismatic lift (vertical, limits and motor) carrying a box, and a slider
    lift = world.create_dynamic_body(position=(2.0, 1.0))
    lift.create_polygon_fixture(box=(1.0, 0.2), density=3.0, friction=0.7)
    world.create_prismatic_joint(ground, lift, anchor=(2.0, 1.0), axis=(0.0, 1.0), lower_limit=0.0, upper_limit=3.0,
                                 limit_enabled=True, motor_speed=1.0, max_motor_force=500.0, motor_enabled=True)
    cargo = world.create_dynamic_body(position=(2.0, 1.8))
    cargo.create_polygon_fixture(box=(0.4, 0.4), density=1.0, friction=0.7)
    slider = world.create_dynamic_body(position=(6.0, 2.0), angle=0.1)
    slider.create_polygon_fixture(box=(0.5, 0.3), density=1.0, friction=0.3)
    world.create_prismatic_joint(ground, slider, anchor=(6.0, 2.0), axis=(0.8, 0.6), lower_limit=-1.0, upper_limit=1.5,
                                 limit_enabled=True)
    # distance joints: rigid pair and a soft spring to a static post
    c1 = world.create_dynamic_body(position=(9.0, 5.0))
    c1.create_circle_fixture(radius=0.4, density=1.0, friction=0.4)
    c2 = world.create_dynamic_body(position=(10.5, 5.5))
    c2.create_circle_fixture(radius=0.3, density=1.0, friction=0.4)
    world.create_distance_joint(c1, c2, anchor_a=(9.0, 5.0), anchor_b=(10.5, 5.5))
    post = world.create_static_body(position=(13.0, 8.0), shapes=b2.Polygon(box=(0.2, 0.2)))
    bob = world.create_dynamic_body(position=(13.5, 5.0))
    bob.create_polygon_fixture(box=(0.3, 0.3), density=2.0, friction=0.4)
    world.create_distance_joint(post, bob, anchor_a=(13.0, 8.0), anchor_b=(13.5, 5.3), frequency=2.0, damping_ratio=0.3)
    # welded cantilever
    wall = world.create_static_body(position=(17.0, 3.0), shapes=b2.Polygon(box=(0.3, 3.0)))
    prev = wall
    for k in range(4):
        seg = world.create_dynamic_body(position=(17.8 + 1.0 * k, 5.0))
        seg.create_polygon_fixture(box=(0.5, 0.15), density=1.0, friction=0.6)
        world.create_weld_joint(prev, seg, anchor=(17.3 + 1.0 * k, 5.0))
        prev = seg
    # things falling onto the joints
    for k in range(8):
        x = rng.uniform(-10.0, 20.0)
        b = world.create_dynamic_body(position=(x, 9.0 + 1.5 * k), angle=rng.uniform(-1.0, 1.0))
        if k % 2:
            b.create_circle_fixture(radius=rng.uniform(0.25, 0.5), density=1.0, friction=0.5)
        else:
            b.create_polygon_fixture(box=(rng.uniform(0.2, 0.5), rng.uniform(0.2, 0.5)), density=1.0, friction=0.5)
    return world


def scene_bridge(b2, planks=30, seed=19):
    """A suspension bridge: planks joined end to end by revolute joints and
    pinned to the ground at both ends, with boxes and circles dropped on it
    (the chains of joints stress the joint colouring)."""
    rng = random.Random(seed)
    world = b2.World(gravity=(0, -10), do_sleep=True)
    ground = world.create_static_body(position=(0, 0), shapes=b2.Polygon(box=(40, 0.5)))
    prev = ground
    x0, y = -15.0, 5.0
    for k in range(planks):
        p = world.create_dynamic_body(position=(x0 + 0.5 + 1.0 * k, y))
        p.create_polygon_fixture(box=(0.5, 0.125), density=20.0, friction=0.2)
        world.create_revolute_joint(prev, p, anchor=(x0 + 1.0 * k, y))
        prev = p
    world.create_revolute_joint(prev, ground, anchor=(x0 + 1.0 * planks, y))
    for k in range(12):
        b = world.create_dynamic_body(position=(x0 + 2.0 + 2.2 * k, 8.0 + 0.5 * (k % 3)), angle=rng.uniform(-0.5, 0.5))
        if k % 3 == 1:
            b.create_circle_fixture(radius=0.45, density=1.0, friction=0.5)
        else:
            b.create_polygon_fixture(box=(0.4, 0.4), density=1.0, friction=0.5)
    return world


def scene_joints2(b2, seed=37):
    """The friction, rope, wheel, pulley and mouse joints: a box sliding on
    the ground held back by a friction joint, a ball on a slack rope that
    pulls taut, a two-wheeled cart on sprung wheel joints with a motor on the
    rear wheel, a wheel without a spring (frequency 0, whose spring axis
    keeps its initial zero), two boxes on a pulley with ratio 1.5 and a box
    dragged by a mouse joint, plus a few boxes dropped among them."""
    rng = random.Random(seed)
    world = b2.World(gravity=(0, -10), do_sleep=True)
    ground = world.create_static_body(position=(0, -0.5), shapes=b2.Polygon(box=(40, 0.5)))
    # friction: a box sliding right, held back by a friction joint to the ground
    slider = world.create_dynamic_body(position=(-20, 0.5), linear_velocity=(6, 0), angular_velocity=1.0)
    slider.create_polygon_fixture(box=(0.5, 0.5), density=1.0, friction=0.1)
    world.create_friction_joint(ground, slider, local_anchor_a=(-20, 0.5), local_anchor_b=(0, 0), max_force=4.0,
                                max_torque=1.5)
    # rope: a pendulum on a rope longer than its initial distance
    hook = world.create_static_body(position=(-10, 10))
    hook.create_circle_fixture(0.2)
    ball = world.create_dynamic_body(position=(-8, 9))
    ball.create_circle_fixture(0.4, density=2.0)
    world.create_rope_joint(hook, ball, local_anchor_a=(0, 0), local_anchor_b=(0, 0), max_length=4.0)
    # wheel: a cart, rear wheel driven
    cart = world.create_dynamic_body(position=(0, 1.6))
    cart.create_polygon_fixture(box=(1.5, 0.3), density=1.0, friction=0.4)
    rear = world.create_dynamic_body(position=(-1.0, 0.9))
    rear.create_circle_fixture(0.4, density=1.0, friction=0.9)
    front = world.create_dynamic_body(position=(1.0, 0.9))
    front.create_circle_fixture(0.4, density=1.0, friction=0.9)
    world.create_wheel_joint(cart, rear, anchor=(-1.0, 0.9), axis=(0, 1), frequency=4.0, damping_ratio=0.7,
                             motor_enabled=True, motor_speed=-8.0, max_motor_torque=15.0)
    world.create_wheel_joint(cart, front, anchor=(1.0, 0.9), axis=(0, 1), frequency=4.0, damping_ratio=0.7)
    # a wheel joint without a spring on a separate body pair
    axle = world.create_dynamic_body(position=(8, 2.5))
    axle.create_polygon_fixture(box=(0.8, 0.2), density=1.0)
    hub = world.create_dynamic_body(position=(8, 1.8))
    hub.create_circle_fixture(0.35, density=1.0, friction=0.8)
    world.create_wheel_joint(axle, hub, anchor=(8, 1.8), axis=(0.2, 1.0), frequency=0.0, motor_enabled=True,
                             motor_speed=3.0, max_motor_torque=5.0)
    # pulley: two boxes hung from ground anchors, ratio 1.5
    pa = world.create_dynamic_body(position=(14, 6))
    pa.create_polygon_fixture(box=(0.4, 0.4), density=1.0)
    pb = world.create_dynamic_body(position=(18, 5))
    pb.create_polygon_fixture(box=(0.5, 0.5), density=1.0)
    world.create_pulley_joint(pa, pb, ground_anchor_a=(14, 12), ground_anchor_b=(18, 12), anchor_a=(14, 6.4),
                              anchor_b=(18, 5.5), ratio=1.5)
    # mouse: a box dragged towards a point above the ground
    dragged = world.create_dynamic_body(position=(24, 0.5), angle=0.3)
    dragged.create_polygon_fixture(box=(0.5, 0.3), density=1.0, friction=0.5)
    world.create_mouse_joint(dragged, target=(24.3, 0.6), max_force=40.0, frequency=3.0, damping_ratio=0.6)
    for i in range(6):
        b = world.create_dynamic_body(position=(-14 + 5.5 * i + rng.uniform(-0.5, 0.5), 7 + rng.uniform(0, 3)),
                                      angle=rng.uniform(-1, 1))
        b.create_polygon_fixture(box=(0.35, 0.35), density=1.0, friction=0.5)
    return world


def scene_loops(b2, seed=23):
    """Loop shapes: a static closed terrain loop (a valley with a hill whose
    top vertex is the body's origin, so its neighbouring child edges lose
    vertex0 / vertex3), a two-vertex loop as a shelf, a static sensor loop,
    a dynamic body carrying a triangle loop beside a circle, circles and
    convex polygons dropped into the valley and a bullet circle fired at
    the terrain (continuous collision against loop children)."""
    rng = random.Random(seed)
    world = b2.World(gravity=(0, -10), do_sleep=True)
    terrain = world.create_static_body(position=(0, -2))
    terrain.create_loop_fixture([(-15, 8), (-15, -2), (-9, -3), (-4, -3), (0, 0), (4, -3), (9, -2.5), (15, -2),
                                 (15, 8)], friction=0.6)
    shelf = world.create_static_body(position=(-10, 2))
    shelf.create_loop_fixture([(-2, 0), (2, 0.5)], friction=0.4)
    gate = world.create_static_body(position=(6, -1))
    gate.create_loop_fixture([(-1, -1), (1, -1), (1, 1), (-1, 1)], sensor=True)
    frame = world.create_dynamic_body(position=(7, 2), angle=0.3)
    frame.create_loop_fixture([(-0.8, -0.5), (0.8, -0.5), (0, 0.7)], friction=0.5)
    frame.create_circle_fixture(radius=0.25, density=2.0, friction=0.5)
    for i in range(22):
        x, y = rng.uniform(-13, 13), rng.uniform(-1, 4.5)
        body = world.create_dynamic_body(position=(x, y), angle=rng.uniform(-2, 2),
                                         linear_velocity=(rng.gauss(0, 1.5), rng.gauss(0, 1.5)))
        if i % 2 == 0:
            body.create_circle_fixture(radius=rng.uniform(0.2, 0.5), density=rng.uniform(0.5, 3), friction=0.4,
                                       restitution=rng.uniform(0, 0.3))
        else:
            body.create_polygon_fixture(vertices=random_convex(rng, rng.randint(3, 7), rng.uniform(0.3, 0.6)),
                                        density=rng.uniform(0.5, 3), friction=0.5)
    world.create_dynamic_body(position=(-12, 5), bullet=True, linear_velocity=(90.0, -40.0)).create_circle_fixture(
        radius=0.1, density=50.0)
    return world


def scene_buoyancy(b2, seed=29):
    """Buoyancy controllers: a pool (offset 6 along (0, 1), density 2, linear
    drag 2, angular drag 1) holding circles, boxes, triangles, a body whose
    only fixture is an edge, a body carrying a loop beside a circle and a
    chain of planks joined by revolute joints; a second controller with its
    own gravity and a current (fluid velocity) acts on some of them too, so
    two controllers run one after the other on the same bodies."""
    rng = random.Random(seed)
    world = b2.World(gravity=(0, -10), do_sleep=True)
    ground = world.create_static_body(shapes=b2.Edge((-20, 0), (20, 0)))
    pool = world.create_buoyancy_controller(offset=6, normal=(0, 1), density=2, linear_drag=2, angular_drag=1)
    current = world.create_buoyancy_controller(offset=4.5, normal=(0, 1), density=0.5, velocity=(1.5, 0.0),
                                               linear_drag=1, angular_drag=0.5, gravity=(0, -9.0))
    for i in range(6):
        b = world.create_dynamic_body(position=(-11 + 4.0 * i, 10 + rng.uniform(0, 2)),
                                      fixtures=b2.Fixture(shape=b2.Circle(radius=0.6 + 0.1 * (i % 3)), density=1.0))
        pool.add_body(b)
        if i % 2 == 0:
            current.add_body(b)
    prev = ground
    for k in range(10):
        p = world.create_dynamic_body(position=(-14.5 + 1.0 * k, 5))
        p.create_polygon_fixture(box=(0.5, 0.125), density=1.0, friction=0.2)
        world.create_revolute_joint(prev, p, anchor=(-15.0 + 1.0 * k, 5))
        pool.add_body(p)
        prev = p
    for i in range(4):
        b = world.create_dynamic_body(position=(-8 + 3.0 * i, 14), angle=rng.uniform(-1, 1),
                                      fixtures=b2.Fixture(shape=b2.Polygon(vertices=[(-0.5, 0), (0, -0.5), (0.5, 0)]),
                                                          density=1.0))
        pool.add_body(b)
    for i in range(3):
        b = world.create_dynamic_body(position=(4 + 2.5 * i, 9 + i), angle=0.3 * i)
        b.create_polygon_fixture(box=(0.5, 0.3), density=0.8 + 0.4 * i, friction=0.4)
        pool.add_body(b)
        current.add_body(b)
    edge = world.create_dynamic_body(fixtures=b2.Fixture(shape=b2.Edge((5, 0), (5, 3)), density=1.0))
    pool.add_body(edge)
    raft = world.create_dynamic_body(position=(12, 9), angle=0.2)
    raft.create_loop_fixture([(-1, -0.4), (1, -0.4), (1, 0.4), (-1, 0.4)], friction=0.4)
    raft.create_circle_fixture(radius=0.3, density=1.5)
    pool.add_body(raft)
    current.add_body(raft)
    return world


def scene_gravity(b2, seed=31):
    """Gravity controllers in a world without gravity: an inverse-square
    controller over circles, triangles, boxes (two of them created asleep,
    woken by the controller's forces) and a static anchor body (zero mass:
    its pairs give zero forces but still wake their partners), and an
    inverse-distance controller over a second group."""
    rng = random.Random(seed)
    world = b2.World(gravity=(0, 0), do_sleep=True)
    anchor = world.create_static_body(position=(0, 0), shapes=b2.Circle(radius=0.5))
    g1 = world.create_gravity_controller(G=0.8, inv_sqr=True)
    g2 = world.create_gravity_controller(G=0.3, inv_sqr=False)
    g1.add_body(anchor)
    for i in range(1, 5):
        b = world.create_dynamic_body(position=(0.25 * i, 2.0 + 3.5 * i), bullet=(i == 4),
                                      fixtures=b2.Fixture(shape=b2.Circle(radius=0.25 * i), density=1.0))
        g1.add_body(b)
    for i in range(4):
        b = world.create_dynamic_body(position=(-8 + 4.0 * i, -6 + rng.uniform(-1, 1)), angle=rng.uniform(-1, 1),
                                      awake=(i % 2 == 0),
                                      fixtures=b2.Fixture(shape=b2.Polygon(vertices=[(-0.5, 0), (0, -0.5), (0.5, 0)]),
                                                          density=1.0))
        g1.add_body(b)
    for i in range(5):
        b = world.create_dynamic_body(position=(10 + 1.5 * i, 5 + rng.uniform(-2, 2)),
                                      linear_velocity=(0, rng.uniform(-1, 1)))
        b.create_polygon_fixture(box=(0.4, 0.4), density=2.0, friction=0.5)
        g2.add_body(b)
    return world


SCENES = {
    "pyramid": (scene_pyramid, 300, (1, 2, 3, 5, 10, 30, 31, 100, 101, 200, 201, 300)),
    "pyramid5": (lambda b2: scene_pyramid(b2, rows=5), 150, (1, 2, 5, 20, 21, 60, 61, 150)),
    "mixed": (scene_mixed, 200, (1, 2, 5, 20, 21, 60, 61, 120, 121, 200)),
    "bullets": (scene_bullets, 60, (1, 2, 3, 5, 10, 11, 20, 21, 40, 41, 60)),
    "sleep": (scene_sleep, 90, (1, 10, 29, 30, 31, 45, 46, 60, 90)),
    "uneven": (scene_uneven, 240, (1, 2, 5, 30, 31, 60, 61, 120, 121, 180, 240)),
    "kinematic": (scene_kinematic, 180, (1, 2, 5, 20, 21, 60, 61, 120, 121, 180)),
    "sensor_filter": (scene_sensor_filter, 150, (1, 2, 5, 20, 21, 40, 60, 61, 90, 120, 121, 150)),
    "joints": (scene_joints, 300, (1, 2, 5, 20, 21, 60, 61, 120, 121, 200, 201, 300)),
    "bridge": (scene_bridge, 240, (1, 2, 5, 20, 21, 60, 61, 120, 121, 240)),
    "loops": (scene_loops, 180, (1, 2, 5, 20, 21, 60, 61, 120, 121, 180)),
    "buoyancy": (scene_buoyancy, 240, (1, 2, 5, 20, 21, 60, 61, 120, 121, 240)),
    "joints2": (scene_joints2, 240, (1, 2, 5, 20, 21, 60, 61, 120, 121, 240)),
    "gravity": (scene_gravity, 240, (1, 2, 5, 20, 21, 60, 61, 120, 121, 240)),
}


def run_scene(b2, name, builder, n_steps, snaps, vel_iters=8, pos_iters=3, dt=1.0 / 60):
    from pypybox2d import island as island_mod
    world = builder(b2)
    order_log = OrderLog()
    orig = install_hooks(world, b2, order_log)
    out = {}
    W, B, F, C = export_world(world, b2)
    out["init_world"], out["init_bodies"], out["init_fixtures"] = W, B, F
    if world.joints:
        out["init_joints"] = export_joints(world, b2)
    if world.controllers:
        out["init_controllers"], out["init_controller_bodies"] = export_controllers(world, b2)
    out["iters"] = np.array([vel_iters, pos_iters])
    try:
        for s in range(1, n_steps + 1):
            order_log.clear()
            order_log.joints.clear()
            world.step(dt, vel_iters, pos_iters)
            if s in snaps:
                W2, B2, F2, C2 = export_world(world, b2)
                out[f"s{s}_bodies"] = B2
                out[f"s{s}_aabb"] = F2["aabb"].copy()
                out[f"s{s}_contacts"] = C2
                out[f"s{s}_world"] = W2
                out[f"s{s}_order"] = np.array(order_log, dtype=np.int32)
                if world.joints:
                    out[f"s{s}_joints"] = export_joints(world, b2)
                    out[f"s{s}_jorder"] = np.array(order_log.joints, dtype=np.int32)
    finally:
        island_mod.Island.solve = orig
    out["snaps"] = np.array(sorted(snaps), dtype=np.int32)
    out["dt"] = np.array([dt])
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **out)
    print(f"{name}: {len(B)} bodies, {len(F)} fixtures, steps {n_steps} -> {os.path.getsize(path)} bytes")


def pair_order_hook(world):
    """update_pairs in the fixed order of install_hooks, with the fixture
    numbering read at each call (the script adds and removes fixtures)."""
    bp = world.contact_manager.broadphase

    def update_pairs(self, callback=None):
        fidx = fixture_index(world)
        first = {}
        for i, node in enumerate(self._move_buffer):
            if node not in first:
                first[node] = i
        pairs = []
        for node, pos in first.items():
            for res in self._tree.query(node.aabb):
                if res is node:
                    continue
                if res in first and first[res] < pos:
                    continue
                pairs.append((pos, fidx[id(res.user_data.fixture)] + res.user_data.child_index, node, res))
        self._move_buffer = []
        pairs.sort(key=lambda t: (t[0], t[1]))
        for _, _, a, b in pairs:
            yield (a.user_data, b.user_data)

    bp.update_pairs = types.MethodType(update_pairs, bp)


def events_array(log):
    """Listener log of api_script -> record array (kind 1 begin, 2 end, 3 post-solve)."""
    kinds = {"begin": 1, "end": 2, "post": 3}
    dt = np.dtype([("kind", "<i4"), ("step", "<i4"), ("ba", "<i4"), ("fa", "<i4"), ("bb", "<i4"), ("fb", "<i4"),
                   ("n", "<i4"), ("imp", "<f8", (4,))])
    out = np.zeros(len(log), dtype=dt)
    for k, (kind, step, ba, fa, bb, fb, imp) in enumerate(log):
        out[k]["kind"], out[k]["step"] = kinds[kind], step
        out[k]["ba"], out[k]["fa"], out[k]["bb"], out[k]["fb"] = ba, fa, bb, fb
        out[k]["n"] = len(imp) // 2
        out[k]["imp"][:len(imp)] = imp
    return out


def run_api_script(b2):
    """tests/golden/api_script.py on the reference -> api_script.npz."""
    sys.path.insert(0, HERE)
    import api_script
    out = {}

    def snap(label, world):
        W, B, F, C = export_world(world, b2)
        out[f"{label}_bodies"], out[f"{label}_aabb"], out[f"{label}_contacts"] = B, F["aabb"].copy(), C

    log = []
    api_script.script(b2, snap, on_world=pair_order_hook, log=log)
    out["events"] = events_array(log)
    path = os.path.join(HERE, "api_script.npz")
    np.savez_compressed(path, **out)
    print(f"api_script: {(len(out) - 1) // 3} snapshots, {len(out['events'])} events -> {os.path.getsize(path)} bytes")


def run_api_joints(b2):
    """tests/golden/api_joints.py on the reference -> api_joints.npz."""
    sys.path.insert(0, HERE)
    import api_joints
    out = {}

    def snap(label, world):
        W, B, F, C = export_world(world, b2)
        out[f"{label}_bodies"], out[f"{label}_aabb"], out[f"{label}_contacts"] = B, F["aabb"].copy(), C
        out[f"{label}_joints"] = export_joints(world, b2)
        out[f"{label}_getters"] = np.array([api_joints.getter_row(j) for j in world.joints], dtype=np.float64)

    log = []
    api_joints.script(b2, snap, on_world=pair_order_hook, log=log)
    out["destroyed"] = np.array(log)
    path = os.path.join(HERE, "api_joints.npz")
    np.savez_compressed(path, **out)
    print(f"api_joints: {len(api_joints.SNAPS)} snapshots, joints destroyed with bodies: {log} -> "
          f"{os.path.getsize(path)} bytes")


def run_api_joints2(b2):
    """tests/golden/api_joints2.py on the reference -> api_joints2.npz."""
    sys.path.insert(0, HERE)
    import api_joints2
    out = {}

    def snap(label, world):
        W, B, F, C = export_world(world, b2)
        out[f"{label}_bodies"], out[f"{label}_contacts"] = B, C
        out[f"{label}_joints"] = export_joints(world, b2)
        out[f"{label}_getters"] = np.array([api_joints2.getter_row(j) for j in world.joints], dtype=np.float64)

    api_joints2.script(b2, snap, on_world=pair_order_hook)
    path = os.path.join(HERE, "api_joints2.npz")
    np.savez_compressed(path, **out)
    print(f"api_joints2: {len(api_joints2.SNAPS)} snapshots -> {os.path.getsize(path)} bytes")


def run_api_active(b2):
    """tests/golden/api_active.py on the reference -> api_active.npz."""
    sys.path.insert(0, HERE)
    import api_active
    out = {}

    def snap(label, world):
        W, B, F, C = export_world(world, b2)
        out[f"{label}_bodies"], out[f"{label}_aabb"], out[f"{label}_contacts"] = B, F["aabb"].copy(), C

    api_active.script(b2, snap, on_world=pair_order_hook)
    path = os.path.join(HERE, "api_active.npz")
    np.savez_compressed(path, **out)
    print(f"api_active: {len(api_active.SNAPS)} snapshots -> {os.path.getsize(path)} bytes")


def run_api_loops(b2):
    """tests/golden/api_loops.py on the reference -> api_loops.npz."""
    sys.path.insert(0, HERE)
    import api_loops
    out = {}

    def snap(label, world):
        W, B, F, C = export_world(world, b2)
        out[f"{label}_bodies"], out[f"{label}_aabb"], out[f"{label}_contacts"] = B, F["aabb"].copy(), C
        rays, queries = api_loops.probes(b2, world)
        out[f"{label}_rays"] = np.array(rays, dtype=np.float64)
        out[f"{label}_queries"] = np.array(queries, dtype=np.float64)

    api_loops.script(b2, snap, on_world=pair_order_hook)
    path = os.path.join(HERE, "api_loops.npz")
    np.savez_compressed(path, **out)
    print(f"api_loops: {len(api_loops.SNAPS)} snapshots -> {os.path.getsize(path)} bytes")


def run_api_controllers(b2):
    """tests/golden/api_controllers.py on the reference -> api_controllers.npz."""
    sys.path.insert(0, HERE)
    import api_controllers
    out = {}

    def snap(label, world):
        W, B, F, C = export_world(world, b2)
        out[f"{label}_bodies"], out[f"{label}_contacts"] = B, C
        out[f"{label}_controllers"], out[f"{label}_controller_bodies"] = export_controllers(world, b2)

    api_controllers.script(b2, snap, on_world=pair_order_hook)
    path = os.path.join(HERE, "api_controllers.npz")
    np.savez_compressed(path, **out)
    print(f"api_controllers: {len(api_controllers.SNAPS)} snapshots -> {os.path.getsize(path)} bytes")


def run_api_filter(b2):
    """tests/golden/api_filter.py on the reference -> api_filter.npz."""
    sys.path.insert(0, HERE)
    import api_filter
    out = {}

    def snap(label, world):
        W, B, F, C = export_world(world, b2)
        out[f"{label}_bodies"], out[f"{label}_contacts"] = B, C

    api_filter.script(b2, snap, on_world=pair_order_hook)
    path = os.path.join(HERE, "api_filter.npz")
    np.savez_compressed(path, **out)
    print(f"api_filter: {len(api_filter.SNAPS)} snapshots -> {os.path.getsize(path)} bytes")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("GB2D_REFERENCE"), required="GB2D_REFERENCE" not in os.environ,
                    help="the pypybox2d source tree (default: $GB2D_REFERENCE)")
    ap.add_argument("--only", default=None)
    args = ap.parse_args()
    b2 = load_reference(args.ref)
    for name, (builder, n, snaps) in SCENES.items():
        if args.only and name != args.only:
            continue
        run_scene(b2, name, builder, n, snaps)
    if not args.only or args.only == "api_script":
        run_api_script(b2)
    if not args.only or args.only == "api_joints":
        run_api_joints(b2)
    if not args.only or args.only == "api_active":
        run_api_active(b2)
    if not args.only or args.only == "api_joints2":
        run_api_joints2(b2)
    if not args.only or args.only == "api_loops":
        run_api_loops(b2)
    if not args.only or args.only == "api_controllers":
        run_api_controllers(b2)
    if not args.only or args.only == "api_filter":
        run_api_filter(b2)


if __name__ == "__main__":
    main()

"""The reference's World / Body / Fixture API over the GPU step.

``World`` mirrors pypybox2d's ``World`` (pypybox2d/world.py:64-473),
``Body`` its ``Body`` (body.py) and ``Fixture`` its ``Fixture``
(fixture.py:43-): the same constructor arguments, properties and methods
for the parts the step uses, so a script written for pypybox2d runs with

    import pypybox2d_gb300 as b2

The host keeps the construction-time records (built with the reference's
float64 arithmetic by ``scenes.SceneBuilder``); the first ``step`` uploads
them (``gb_batch_create``) and from then on the device owns the state:

* ``World.step`` is one ``gb_batch_step`` call;
* reading a body property downloads all bodies once per step
  (``gb_batch_get_bodies``); changing a velocity, a force or the awake flag
  edits the host record and re-uploads the bodies before the next step
  (``gb_batch_set_bodies``);
* structural changes (a new body or fixture, a transform set by hand,
  gravity, a destroyed body) download the whole world -- bodies, fat AABBs,
  contacts with their manifolds and impulses -- edit it on the host with the
  reference's arithmetic and upload it again, with the moved proxies in the
  move buffer; pair finding for them runs on the device at the start of the
  next step, as the reference's ``find_new_contacts`` would before it.

Joints (revolute, prismatic, distance, weld: ``joints.py``) are records of
the world solved by the same step; creating or destroying one is a
structural change, and a joint setter edits the record and re-uploads the
joints before the next step (``gb_batch_set_joints``).

Controllers (buoyancy, gravity: ``controllers.py``) run inside the step;
before each step the World compares ``World.controllers`` with what the
device holds, uploading new parameters or rebuilding the batch for a new
controller or body list.

What the GPU step does not support raises instead of running elsewhere:
the friction, gear, mouse, pulley, rope and wheel joints, controllers with
a Python ``step`` of their own, sub-stepping, custom contact filters and
``pre_solve`` callbacks that run mid-step.
"""
from __future__ import annotations

import math

import numpy as np

from . import abi
from . import joints as _joints
from .controllers import BuoyancyController, Controller, GravityController, controller_records  # noqa: F401
from .joints import DistanceJoint, Joint, PrismaticJoint, RevoluteJoint, WeldJoint  # noqa: F401
from .scenes import AABB_EXTENSION, SceneBuilder, _Body
from .shapes import Circle, Edge, Loop, MassData, Polygon, Shape


from .errors import EmptyFixtureError, LockedError, PhysicsError, StepError, step_error  # noqa: E402,F401


class Vec2(tuple):
    """A 2-vector returned by the getters (x, y, arithmetic, length)."""

    def __new__(cls, x=0.0, y=0.0):
        return tuple.__new__(cls, (float(x), float(y)))

    x = property(lambda self: self[0])
    y = property(lambda self: self[1])

    def __add__(self, o):
        return Vec2(self[0] + o[0], self[1] + o[1])

    def __sub__(self, o):
        return Vec2(self[0] - o[0], self[1] - o[1])

    def __mul__(self, k):
        return Vec2(self[0] * k, self[1] * k)

    __rmul__ = __mul__

    def __neg__(self):
        return Vec2(-self[0], -self[1])

    def dot(self, o):
        return self[0] * o[0] + self[1] * o[1]

    def cross(self, o):
        return self[0] * o[1] - self[1] * o[0]

    @property
    def length(self):
        return math.sqrt(self[0] * self[0] + self[1] * self[1])

    @property
    def length_squared(self):
        return self[0] * self[0] + self[1] * self[1]

    def __repr__(self):
        return f"Vec2({self[0]:g}, {self[1]:g})"


class AABB:
    """The query box of World.query_aabb (common AABB, aabbmodule.c): lower
    and upper bound, each given as a pair."""

    __slots__ = ("lower_bound", "upper_bound")

    def __init__(self, lower_bound=None, upper_bound=None):
        self.lower_bound = Vec2(*lower_bound) if lower_bound is not None else Vec2()
        self.upper_bound = Vec2(*upper_bound) if upper_bound is not None else Vec2()

    @property
    def center(self):
        return Vec2(0.5 * (self.lower_bound[0] + self.upper_bound[0]), 0.5 * (self.lower_bound[1] + self.upper_bound[1]))

    @property
    def extents(self):
        return Vec2(0.5 * (self.upper_bound[0] - self.lower_bound[0]), 0.5 * (self.upper_bound[1] - self.lower_bound[1]))

    @property
    def perimeter(self):
        return 2.0 * ((self.upper_bound[0] - self.lower_bound[0]) + (self.upper_bound[1] - self.lower_bound[1]))

    def __repr__(self):
        return f"AABB(lower_bound={tuple(self.lower_bound)}, upper_bound={tuple(self.upper_bound)})"


class Fixture:
    """fixture.py:43-71: a shape with its material and filter data."""

    def __init__(self, shape=None, friction=0.2, restitution=0.0, density=0.0, category_bits=0x0001,
                 mask_bits=0xFFFF, group_index=0, sensor=False, user_data=None, body=None):
        self._body = None
        self._slot = -1
        self._shape = shape
        self._friction, self._restitution, self._density = float(friction), float(restitution), float(density)
        self._category_bits, self._mask_bits, self._group_index = category_bits, mask_bits, group_index
        self._sensor = bool(sensor)
        self.user_data = user_data

    # fixture.py:122-225: material and filter data.  On a fixture of a world
    # the change reaches the world's fixture records (re-uploaded before the
    # next step); the filter fields also refilter the fixture's contacts.
    @property
    def friction(self):
        return self._friction

    @friction.setter
    def friction(self, v):
        self._friction = float(v)
        self._push()

    @property
    def restitution(self):
        return self._restitution

    @restitution.setter
    def restitution(self, v):
        self._restitution = float(v)
        self._push()

    @property
    def density(self):
        return self._density

    @density.setter
    def density(self, v):
        if not math.isfinite(float(v)) or float(v) < 0:
            raise ValueError("Invalid density")
        self._density = float(v)
        self._push()

    @property
    def sensor(self):
        return self._sensor

    @sensor.setter
    def sensor(self, v):
        if bool(v) != self._sensor:
            if self._body is not None:
                self._body.awake = True
            self._sensor = bool(v)
            self._push()

    @property
    def category_bits(self):
        return self._category_bits

    @category_bits.setter
    def category_bits(self, v):
        self._category_bits = v
        self._push(refilter=True)

    @property
    def mask_bits(self):
        return self._mask_bits

    @mask_bits.setter
    def mask_bits(self, v):
        self._mask_bits = v
        self._push(refilter=True)

    @property
    def group_index(self):
        return self._group_index

    @group_index.setter
    def group_index(self, v):
        self._group_index = v
        self._push(refilter=True)

    def _push(self, refilter=False):
        body = self._body
        if body is not None and body._world is not None:
            body._world._set_fixture(self, refilter)

    def __copy__(self):
        return Fixture(self._shape, self.friction, self.restitution, self.density, self.category_bits,
                       self.mask_bits, self.group_index, self.sensor, self.user_data)

    @property
    def shape(self):
        return self._shape

    @property
    def body(self):
        return self._body

    def _kwargs(self):
        return dict(friction=self.friction, restitution=self.restitution, density=self.density,
                    category=self.category_bits, mask=self.mask_bits, group=self.group_index, sensor=self.sensor)


class Body:
    """body.py: a rigid body of a World.  Properties read the device state."""

    STATIC, DYNAMIC, KINEMATIC = abi.BODY_STATIC, abi.BODY_DYNAMIC, abi.BODY_KINEMATIC

    def __init__(self, world, index, fixtures, user_data=None):
        self._world = world
        self._index = index
        self.fixtures = fixtures
        self.user_data = user_data
        self._controllers = []

    def _attached_to_controller(self, controller):
        """body.py:348-350"""
        self._controllers.append(controller)

    def _detached_from_controller(self, controller):
        """body.py:352-353"""
        self._controllers.remove(controller)

    # -- record access
    def _rec(self):
        return self._world._body_record(self._index)

    def _edit(self):
        return self._world._body_record(self._index, write=True)

    # -- read-only state
    @property
    def world(self):
        return self._world

    @property
    def type(self):
        return int(self._rec()["type"])

    @type.setter
    def type(self, t):
        """body.py type setter: mass data reset for the new type, a static
        body stops, the body wakes, forces clear, and its fixtures are
        refiltered (contacts flagged for filtering, proxies touched)."""
        self._world._check_unlocked()
        if t == self.type:
            return
        if t not in (Body.STATIC, Body.DYNAMIC, Body.KINEMATIC):
            raise ValueError("Invalid body type")
        self._world._set_type(self, int(t))

    @property
    def static(self):
        return self.type == Body.STATIC

    @property
    def dynamic(self):
        return self.type == Body.DYNAMIC

    @property
    def kinematic(self):
        return self.type == Body.KINEMATIC

    @property
    def position(self):
        r = self._rec()
        return Vec2(r["px"], r["py"])

    @position.setter
    def position(self, pos):
        """body.py:420-423: a new origin, the rotation kept"""
        self._world._check_unlocked()
        self._world._set_transform(self._index, (float(pos[0]), float(pos[1])), None)

    @property
    def angle(self):
        """body.py:426-428: the transform's angle, atan2 of its rotation
        (transform.c Transform_get_angle), not the sweep angle"""
        r = self._rec()
        return math.atan2(float(r["qs"]), float(r["qc"]))

    @angle.setter
    def angle(self, angle):
        self.transform = (self.position, angle)

    @property
    def transform(self):
        r = self._rec()
        return (Vec2(r["px"], r["py"]), (float(r["qc"]), float(r["qs"])))

    @transform.setter
    def transform(self, position_angle):
        self._world._check_unlocked()
        pos, angle = position_angle
        self._world._set_transform(self._index, (float(pos[0]), float(pos[1])), float(angle))

    @property
    def world_center(self):
        r = self._rec()
        return Vec2(r["cx"], r["cy"])

    @property
    def local_center(self):
        r = self._rec()
        return Vec2(r["lcx"], r["lcy"])

    @property
    def mass(self):
        return float(self._rec()["mass"])

    @property
    def mass_data(self):
        """body.py mass_data: the mass, the rotational inertia about the body
        origin and the local centre of mass."""
        r = self._rec()
        cx, cy = float(r["lcx"]), float(r["lcy"])
        return MassData(float(r["mass"]), Vec2(cx, cy), float(r["I"]) + float(r["mass"]) * (cx * cx + cy * cy))

    @mass_data.setter
    def mass_data(self, md):
        """body.py mass_data setter: override the fixtures' mass data of a
        dynamic body; the centre of mass moves and its velocity follows."""
        self._world._check_unlocked()
        if self.type != Body.DYNAMIC:
            return
        r = self._edit()
        mass = float(md.mass)
        if mass <= 0.0:
            mass = 1.0
        inv_mass, I, invI = 1.0 / mass, 0.0, 0.0
        cx, cy = float(md.center[0]), float(md.center[1])
        if float(md.I) > 0.0 and not (int(r["flags"]) & abi.BODY_FIXED_ROTATION):
            I = float(md.I) - mass * (cx * cx + cy * cy)
            invI = 1.0 / I
        r["mass"], r["inv_mass"], r["I"], r["inv_I"] = mass, inv_mass, I, invI
        ox, oy = float(r["cx"]), float(r["cy"])
        r["lcx"], r["lcy"] = cx, cy
        c0x = r["px"] + r["qc"] * cx + (-r["qs"]) * cy          # xf * local_center
        c0y = r["py"] + r["qs"] * cx + r["qc"] * cy
        r["c0x"], r["c0y"], r["cx"], r["cy"] = c0x, c0y, c0x, c0y
        w = float(r["w"])                                       # v += cross(w, c - old_c)
        r["vx"], r["vy"] = r["vx"] + (-w * (c0y - oy)), r["vy"] + w * (c0x - ox)

    def reset_mass_data(self):
        """body.py:587-641: mass data from the fixtures' shapes and densities."""
        self._world._check_unlocked()
        self._world._reset_mass_data(self)

    @property
    def inertia(self):
        """body.py: rotational inertia about the local origin."""
        r = self._rec()
        return float(r["I"]) + float(r["mass"]) * (float(r["lcx"]) ** 2 + float(r["lcy"]) ** 2)

    @property
    def linear_velocity(self):
        r = self._rec()
        return Vec2(r["vx"], r["vy"])

    @linear_velocity.setter
    def linear_velocity(self, v):
        """body.py: static bodies ignore it; a non-zero velocity wakes the body."""
        if self.type == Body.STATIC:
            return
        vx, vy = float(v[0]), float(v[1])
        if vx * vx + vy * vy > 0.0:
            self.awake = True
        r = self._edit()
        r["vx"], r["vy"] = vx, vy

    @property
    def angular_velocity(self):
        return float(self._rec()["w"])

    @angular_velocity.setter
    def angular_velocity(self, w):
        if self.type == Body.STATIC:
            return
        w = float(w)
        if w * w > 0.0:
            self.awake = True
        self._edit()["w"] = w

    @property
    def awake(self):
        return bool(self._rec()["flags"] & abi.BODY_AWAKE)

    @awake.setter
    def awake(self, awake):
        """body.py:800-812"""
        r = self._edit()
        was = bool(r["flags"] & abi.BODY_AWAKE)
        if awake:
            if not was:
                r["sleep_time"] = 0.0
            r["flags"] |= abi.BODY_AWAKE
        else:
            r["sleep_time"] = 0.0
            r["vx"] = r["vy"] = r["w"] = 0.0
            r["fx"] = r["fy"] = r["torque"] = 0.0
            r["flags"] &= np.uint32(0xFFFFFFFF ^ abi.BODY_AWAKE)

    @property
    def sleeping(self):
        return not self.awake

    @sleeping.setter
    def sleeping(self, sleeping):
        self.awake = not sleeping

    @property
    def bullet(self):
        return bool(self._rec()["flags"] & abi.BODY_BULLET)

    @bullet.setter
    def bullet(self, flag):
        r = self._edit()
        r["flags"] = (r["flags"] | abi.BODY_BULLET) if flag else (r["flags"] & np.uint32(0xFFFFFFFF ^ abi.BODY_BULLET))

    @property
    def sleeping_allowed(self):
        return bool(self._rec()["flags"] & abi.BODY_ALLOW_SLEEP)

    @sleeping_allowed.setter
    def sleeping_allowed(self, flag):
        r = self._edit()
        if flag:
            r["flags"] |= abi.BODY_ALLOW_SLEEP
        else:
            r["flags"] &= np.uint32(0xFFFFFFFF ^ abi.BODY_ALLOW_SLEEP)
            self.awake = True

    @property
    def active(self):
        return bool(self._rec()["flags"] & abi.BODY_ACTIVE)

    @active.setter
    def active(self, active):
        """body.py:846-872: an inactive body keeps its place in the world but
        its fixtures leave the broad phase and its contacts are destroyed; an
        active one gets its proxies back (fattened at its transform, in the
        move buffer, so the next step pairs them)."""
        self._world._check_unlocked()
        if bool(active) == self.active:
            return
        self._world._set_active(self._index, bool(active))

    @property
    def joints(self):
        """Body.joints: the joints attached to this body, in creation order."""
        if self._world is None:
            return []
        return [j for j in self._world._joints if j._body_a is self or j._body_b is self]

    @property
    def fixed_rotation(self):
        return bool(self._rec()["flags"] & abi.BODY_FIXED_ROTATION)

    @fixed_rotation.setter
    def fixed_rotation(self, flag):
        """body.py fixed_rotation setter: the flag, then reset_mass_data."""
        r = self._edit()
        if flag:
            r["flags"] |= abi.BODY_FIXED_ROTATION
        else:
            r["flags"] &= np.uint32(0xFFFFFFFF ^ abi.BODY_FIXED_ROTATION)
        self._world._reset_mass_data(self)

    @property
    def linear_damping(self):
        return float(self._rec()["linear_damping"])

    @linear_damping.setter
    def linear_damping(self, v):
        self._edit()["linear_damping"] = float(v)

    @property
    def angular_damping(self):
        return float(self._rec()["angular_damping"])

    @angular_damping.setter
    def angular_damping(self, v):
        self._edit()["angular_damping"] = float(v)

    @property
    def gravity_scale(self):
        return float(self._rec()["gravity_scale"])

    @gravity_scale.setter
    def gravity_scale(self, v):
        self._edit()["gravity_scale"] = float(v)

    @property
    def force(self):
        r = self._rec()
        return Vec2(r["fx"], r["fy"])

    @property
    def torque(self):
        return float(self._rec()["torque"])

    # -- forces and impulses (body.py:477-545): dynamic bodies only, wake
    def _wake_for_force(self):
        if self.type != Body.DYNAMIC:
            return False
        if not self.awake:
            self.awake = True
        return True

    # -- frames (body.py: Transform and Mat22 products of the body's _xf)
    def get_world_point(self, local_point):
        """xf * local_point (Transform_mul)"""
        r = self._rec()
        x, y = float(local_point[0]), float(local_point[1])
        return Vec2(r["px"] + r["qc"] * x + (-r["qs"]) * y, r["py"] + r["qs"] * x + r["qc"] * y)

    def get_world_vector(self, local_vector):
        """R * local_vector (Mat22_mul)"""
        r = self._rec()
        x, y = float(local_vector[0]), float(local_vector[1])
        return Vec2(r["qc"] * x + (-r["qs"]) * y, r["qs"] * x + r["qc"] * y)

    def get_local_point(self, world_point):
        """xf^T * world_point (Transform_mul_t_vec)"""
        r = self._rec()
        x, y = float(world_point[0]) - r["px"], float(world_point[1]) - r["py"]
        return Vec2(r["qc"] * x + r["qs"] * y, (-r["qs"]) * x + r["qc"] * y)

    def get_local_vector(self, world_vector):
        """R^T * world_vector (Mat22_mul_t_vec)"""
        r = self._rec()
        x, y = float(world_vector[0]), float(world_vector[1])
        return Vec2(r["qc"] * x + r["qs"] * y, (-r["qs"]) * x + r["qc"] * y)

    def get_linear_velocity_from_world_point(self, world_point):
        """v + cross(w, p - c)"""
        r = self._rec()
        dx, dy = float(world_point[0]) - r["cx"], float(world_point[1]) - r["cy"]
        w = r["w"]
        return Vec2(r["vx"] + (-w * dy), r["vy"] + w * dx)

    def get_linear_velocity_from_local_point(self, local_point):
        return self.get_linear_velocity_from_world_point(self.get_world_point(local_point))

    @property
    def allow_sleep(self):
        return self.sleeping_allowed

    @allow_sleep.setter
    def allow_sleep(self, flag):
        self.sleeping_allowed = flag

    @property
    def contact_list(self):
        """The world's contacts that involve one of this body's fixtures."""
        mine = {id(f) for f in self.fixtures}
        return [c for c in self._world.contacts if id(c.fixture_a) in mine or id(c.fixture_b) in mine]

    def apply_force(self, force, point):
        if not self._wake_for_force():
            return
        r = self._edit()
        fx, fy = float(force[0]), float(force[1])
        r["fx"], r["fy"] = r["fx"] + fx, r["fy"] + fy
        dx, dy = float(point[0]) - float(r["cx"]), float(point[1]) - float(r["cy"])
        r["torque"] = r["torque"] + (dx * fy - dy * fx)

    def apply_force_to_center(self, force):
        if not self._wake_for_force():
            return
        r = self._edit()
        r["fx"], r["fy"] = r["fx"] + float(force[0]), r["fy"] + float(force[1])

    def apply_torque(self, torque):
        if not self._wake_for_force():
            return
        r = self._edit()
        r["torque"] = r["torque"] + float(torque)

    def apply_linear_impulse(self, impulse, point):
        if not self._wake_for_force():
            return
        r = self._edit()
        ix, iy = float(impulse[0]), float(impulse[1])
        im = float(r["inv_mass"])
        r["vx"], r["vy"] = r["vx"] + im * ix, r["vy"] + im * iy
        dx, dy = float(point[0]) - float(r["cx"]), float(point[1]) - float(r["cy"])
        r["w"] = r["w"] + float(r["inv_I"]) * (dx * iy - dy * ix)

    def apply_angular_impulse(self, impulse):
        if not self._wake_for_force():
            return
        r = self._edit()
        r["w"] = r["w"] + float(r["inv_I"]) * float(impulse)

    # -- fixtures (body.py:164-234)
    def create_fixture(self, shape, friction=0.2, restitution=0.0, density=0.0, category_bits=0x0001,
                       mask_bits=0xFFFF, group_index=0, sensor=False, user_data=None):
        fx = Fixture(shape, friction, restitution, density, category_bits, mask_bits, group_index, sensor, user_data)
        return self.attach_fixture(fx)

    def create_fixtures(self, shape_list, fixture=None, friction=0.2, restitution=0.0, density=0.0,
                        category_bits=0x0001, mask_bits=0xFFFF, group_index=0, sensor=False):
        """body.py create_fixtures: one fixture per shape, with the material
        and filter of `fixture` when given."""
        if isinstance(shape_list, Shape):
            shape_list = [shape_list]
        if fixture is not None:
            friction, restitution, density = fixture.friction, fixture.restitution, fixture.density
            category_bits, mask_bits, group_index = fixture.category_bits, fixture.mask_bits, fixture.group_index
            sensor = fixture.sensor
        for shape in shape_list:
            self.create_fixture(shape, friction, restitution, density, category_bits, mask_bits, group_index, sensor)

    def destroy_fixture(self, fixture):
        """body.py destroy_fixture: the fixture leaves the body, its contacts
        are destroyed (touching ones reported to end_contact,
        contact_manager.py:167-168), its proxy leaves the broad phase and
        the body's mass data is reset."""
        self._world._check_unlocked()
        if fixture._body is not self or fixture not in self.fixtures:
            raise ValueError("This fixture does not belong to this body")
        self._world._destroy_fixture(self, fixture)

    def attach_fixture(self, fixture):
        self._world._check_unlocked()
        if fixture._body is not None:
            raise ValueError("Fixture is already attached to a body")
        self._world._add_fixture(self, fixture)
        return fixture

    def create_circle_fixture(self, radius=0.2, position=(0, 0), **kwargs):
        return self.create_fixture(Circle(radius, position), **kwargs)

    def create_polygon_fixture(self, vertices=None, box=None, **kwargs):
        return self.create_fixture(Polygon(vertices, box), **kwargs)

    def create_edge_fixture(self, v1=None, v2=None, v0=None, v3=None, **kwargs):
        return self.create_fixture(Edge(v1, v2, v0, v3), **kwargs)

    def create_loop_fixture(self, vertices, *args, **kwargs):
        """body.py:231-234; the loop's children become edge records"""
        return self.create_fixture(Loop(vertices, *args), **kwargs)

    def __repr__(self):
        return f"Body(index={self._index}, position={self.position}, angle={self.angle:g})"


class Contact:
    """A read-only view of one contact after a step (contact.py:55-87)."""

    def __init__(self, world, rec):
        self._world = world
        self._rec = rec
        self.fixture_a, self.child_index_a = world._fixture_child_at(int(rec["fixture_a"]))
        self.fixture_b, self.child_index_b = world._fixture_child_at(int(rec["fixture_b"]))

    body_a = property(lambda self: self.fixture_a.body)
    body_b = property(lambda self: self.fixture_b.body)
    shape_a = property(lambda self: self.fixture_a.shape)
    shape_b = property(lambda self: self.fixture_b.shape)

    def other_body(self, body):
        """contact.py:91-98"""
        return self.fixture_b.body if body is self.fixture_a.body else self.fixture_a.body

    @property
    def manifold(self):
        """contact_util.py Manifold of this contact: type, local normal and
        point, and its points (local point, impulses, feature id as the
        (index_a, index_b, type_a, type_b) tuple of ClipVertex.id)."""
        c = self._rec
        n = int(c["m_point_count"])
        pts = []
        for k in range(n):
            i = int(c["p_id"][k])
            pts.append(ManifoldPoint(Vec2(c["p_lx"][k], c["p_ly"][k]), float(c["p_ni"][k]), float(c["p_ti"][k]),
                                     (i & 255, (i >> 8) & 255, (i >> 16) & 255, (i >> 24) & 255)))
        return Manifold(int(c["m_type"]), Vec2(c["m_lnx"], c["m_lny"]), Vec2(c["m_lpx"], c["m_lpy"]), pts)

    @property
    def world_manifold(self):
        """contact_util.py:195-245: the manifold's normal (A to B) and world
        points under the bodies' current transforms; (normal, [points])."""
        return world_manifold(self._rec, self._world._B, self._world._F)

    touching = property(lambda self: bool(self._rec["flags"] & abi.C_TOUCHING))
    enabled = property(lambda self: bool(self._rec["flags"] & abi.C_ENABLED))
    point_count = property(lambda self: int(self._rec["m_point_count"]))
    friction = property(lambda self: float(self._rec["friction"]))
    restitution = property(lambda self: float(self._rec["restitution"]))

    @property
    def normal_impulses(self):
        return [float(self._rec["p_ni"][k]) for k in range(self.point_count)]

    @property
    def tangent_impulses(self):
        return [float(self._rec["p_ti"][k]) for k in range(self.point_count)]

    @property
    def local_normal(self):
        return Vec2(self._rec["m_lnx"], self._rec["m_lny"])

    @property
    def local_point(self):
        return Vec2(self._rec["m_lpx"], self._rec["m_lpy"])


class ManifoldPoint:
    """contact_util.py ManifoldPoint (read-only copy)."""
    __slots__ = ("local_point", "normal_impulse", "tangent_impulse", "id")

    def __init__(self, local_point, normal_impulse, tangent_impulse, id):
        self.local_point, self.normal_impulse, self.tangent_impulse, self.id = local_point, normal_impulse, tangent_impulse, id


class Manifold:
    """contact_util.py Manifold (read-only copy): CIRCLES, FACE_A or FACE_B."""
    CIRCLES, FACE_A, FACE_B = abi.M_CIRCLES, abi.M_FACE_A, abi.M_FACE_B
    __slots__ = ("type", "local_normal", "local_point", "points")

    def __init__(self, type, local_normal, local_point, points):
        self.type, self.local_normal, self.local_point, self.points = type, local_normal, local_point, points

    @property
    def point_count(self):
        return len(self.points)

    @property
    def used_points(self):
        return list(self.points)


class EventContact:
    """The contact a listener receives when events are replayed after a
    step: its fixtures and whether it touched when the event occurred."""

    __slots__ = ("fixture_a", "fixture_b", "touching")

    def __init__(self, fixture_a, fixture_b, touching):
        self.fixture_a, self.fixture_b, self.touching = fixture_a, fixture_b, touching

    def __repr__(self):
        return f"EventContact({self.fixture_a!r}, {self.fixture_b!r}, touching={self.touching})"


class ContactManager:
    """contact_manager.py:46-100: the contact listeners of a World.

    The GPU step records begin, end and post-solve events on the device; the
    world replays them to these callbacks after the step, in a fixed order
    (contact updates in contact-list order, then post-solve reports in
    contact-list order, then continuous-collision events as they occurred).
    pre_solve, which may change a contact before the solver sees it, cannot
    run inside the GPU step: a world with one set raises on step."""

    def __init__(self):
        self.begin_contact = None
        self.end_contact = None
        self.pre_solve = None
        self.post_solve = None

    @property
    def contact_listener(self):
        return [self.begin_contact, self.end_contact, self.pre_solve, self.post_solve]

    @property
    def wants_events(self):
        return self.begin_contact is not None or self.end_contact is not None or self.post_solve is not None


def _fixture_list(shapes, fixtures, shape_fixture):
    """Body(shapes=..., fixtures=..., shape_fixture=...) of body.py:20-115."""
    out = []
    if shapes is not None:
        if isinstance(shapes, Shape):
            shapes = [shapes]
        base = shape_fixture if shape_fixture is not None else Fixture()
        for sh in shapes:
            f = base.__copy__()
            f._shape = sh
            out.append(f)
    if fixtures is not None:
        if not isinstance(fixtures, (list, tuple)):
            fixtures = [fixtures]
        out.extend(f.__copy__() for f in fixtures)
    return out


def _check_body_args(btype, kw):
    """body.py:49-63 with the C extension's Vec2.valid / is_valid_float
    (vec2module.c valid_float, common.py:942): only NaN is invalid.  The
    damping checks there read `not valid and > 0`, which no NaN satisfies, so
    they never raise; kept as they are."""
    def nan(x):
        return x != x
    px, py = kw.get("position", (0.0, 0.0))
    vx, vy = kw.get("linear_velocity", (0.0, 0.0))
    if nan(float(px)) or nan(float(py)):
        raise ValueError("Invalid position")
    if nan(float(vx)) or nan(float(vy)):
        raise ValueError("Invalid linear velocity")
    if nan(float(kw.get("angle", 0.0))):
        raise ValueError("Invalid angle")
    if nan(float(kw.get("angular_velocity", 0.0))):
        raise ValueError("Invalid angular velocity")
    for name in ("angular_damping", "linear_damping"):
        d = float(kw.get(name, 0.0))
        if nan(d) and d > 0.0:
            raise ValueError(f"Invalid {name.replace('_', ' ')}")
    if btype not in (Body.STATIC, Body.DYNAMIC, Body.KINEMATIC):
        raise ValueError("Invalid body type")



# World._contact_filter before any filter is set: the reference's default rule
# (world.py:88-89), applied on the device without a table.
_DEFAULT_FILTER = object()

class World:
    """world.py:64-473 for the step path, advanced by the GPU library.

    The host records (``abi.WORLD``/``BODY``/``FIXTURE``/``CONTACT`` arrays and
    the pending move buffer) are the state between device round trips;
    ``scenes.SceneBuilder`` supplies the reference's construction
    arithmetic for new bodies and fixtures."""

    def __init__(self, gravity=(0, -10), do_sleep=True, warm_starting=True, continuous_physics=True,
                 sub_stepping=False, auto_clear_forces=True, joint_destruction_listener=None,
                 fixture_destruction_listener=None, contact_filter=None, precision="f64", contact_capacity=0):
        """world.py:64-91.  Beyond the reference: ``precision`` ("f64" or
        "f32") and ``contact_capacity``, the device contact slots of the
        world (0: 6 per fixture); a step that needs more raises
        ContactOverflowError."""
        if sub_stepping:
            raise NotImplementedError("sub_stepping is not supported by the GPU world step")
        self._sb = SceneBuilder(gravity=gravity, do_sleep=do_sleep, warm_starting=warm_starting,
                                continuous_physics=continuous_physics, auto_clear_forces=auto_clear_forces)
        self._precision = precision
        self._contact_capacity = int(contact_capacity)
        self._bodies: list[Body] = []
        self._W = self._sb.world_record(0, 0, 0)
        self._B = np.zeros(0, dtype=abi.BODY)
        self._F = np.zeros(0, dtype=abi.FIXTURE)
        self._C = np.zeros(0, dtype=abi.CONTACT)
        self._M = np.zeros(0, dtype=np.int32)
        self._gpu = None
        self._owner = None          # the WorldBatch stepping this world, if any
        self._host_fresh = True     # host records equal the device state
        self._upload_bodies = False
        self._locked = False
        self._inv_dt0 = 0.0
        self.contact_manager = ContactManager()
        self._J = np.zeros(0, dtype=abi.JOINT)   # World.joints records (world field 0)
        self._joints: list[Joint] = []
        self._upload_joints = False
        self.controllers: list[Controller] = []   # World.controllers (world.py:73), run in this order
        self._ctl_key = None                      # controller kinds and body lists the device batch holds
        self._contact_filter = _DEFAULT_FILTER    # the contact filter (world.py:88-91, 123-136)
        self._pf_key = None                       # what the device batch's filter table was made from
        if contact_filter is not None:
            self.contact_filter = contact_filter
        self._ctl_params = None                   # and their parameters
        self.joint_destruction_listener = joint_destruction_listener
        self.fixture_destruction_listener = fixture_destruction_listener

    # -- properties
    @property
    def gravity(self):
        return Vec2(*self._sb.gravity)

    @gravity.setter
    def gravity(self, g):
        self._check_unlocked()
        self._structural()
        self._sb.gravity = (float(g[0]), float(g[1]))

    def _flag(self, bit):
        return bool(self._sb.flags & bit)

    def _set_flag(self, bit, value):
        """World flags live in the world descriptor: a change re-uploads the
        world before the next step (world.py:139-181 only store the flag)."""
        self._check_unlocked()
        if bool(value) == self._flag(bit):
            return
        self._structural()
        self._sb.flags = (self._sb.flags | bit) if value else (self._sb.flags & ~bit)

    @property
    def warm_starting(self):
        return self._flag(abi.W_WARM_STARTING)

    @warm_starting.setter
    def warm_starting(self, v):
        self._set_flag(abi.W_WARM_STARTING, v)

    @property
    def continuous_physics(self):
        return self._flag(abi.W_CONTINUOUS)

    @continuous_physics.setter
    def continuous_physics(self, v):
        self._set_flag(abi.W_CONTINUOUS, v)

    @property
    def allow_sleep(self):
        return self._flag(abi.W_ALLOW_SLEEP)

    @allow_sleep.setter
    def allow_sleep(self, v):
        self._set_flag(abi.W_ALLOW_SLEEP, v)

    @property
    def auto_clear_forces(self):
        return self._flag(abi.W_AUTO_CLEAR_FORCES)

    @auto_clear_forces.setter
    def auto_clear_forces(self, v):
        self._set_flag(abi.W_AUTO_CLEAR_FORCES, v)

    @staticmethod
    def default_contact_filter(filter_a, filter_b):
        """world.py:958-970, the rule the kernels apply to every new pair:
        a shared non-zero group decides by its sign, otherwise each
        fixture's mask must take the other's category."""
        ga, gb = filter_a.group_index, filter_b.group_index
        if ga == gb and ga != 0:
            return ga > 0
        return (filter_a.mask_bits & filter_b.category_bits) != 0 and (filter_a.category_bits & filter_b.mask_bits) != 0

    @property
    def contact_filter(self):
        """world.py:123-136: called as contact_filter(fixture_a, fixture_b)
        for a new pair (contact_manager.py:145) and for a contact flagged for
        filtering (contact_manager.py:202).  A custom filter reaches the GPU
        step as its answers for every pair of the world's fixtures, asked
        before the next step and again whenever the filter, the fixtures or
        their filter data change.  So the filter must answer alike for both
        orders of a pair and must not depend on other state that changes
        between steps (set it again after such a change).  None, as in the
        reference, turns filtering off: every pair may collide."""
        if self._contact_filter is _DEFAULT_FILTER:
            return self.default_contact_filter
        return self._contact_filter

    @contact_filter.setter
    def contact_filter(self, fcn):
        if fcn is not None and not callable(fcn):
            raise TypeError("contact_filter must be callable")
        default = fcn is not None and getattr(fcn, "__func__", fcn) is World.default_contact_filter
        self._contact_filter = _DEFAULT_FILTER if default else fcn
        self._pf_key = None if self._gpu is None else ("stale",)

    def _pair_filter_table(self):
        """The filter's answers for every ordered pair of fixture records
        (loop children share their fixture's answers; no filter accepts
        every pair), or None for the default rule."""
        fn = self._contact_filter
        if fn is _DEFAULT_FILTER:
            return None
        n = len(self._F)
        if fn is None:
            return np.ones((n, n), dtype=np.uint8)
        owners = [self._fixture_at(r) for r in range(n)]
        uniq, idx = [], []
        pos = {}
        for fx in owners:
            k = id(fx)
            if k not in pos:
                pos[k] = len(uniq)
                uniq.append(fx)
            idx.append(pos[k])
        m = len(uniq)
        T = np.zeros((m, m), dtype=np.uint8)
        for a in range(m):
            for b in range(m):
                T[a, b] = 1 if fn(uniq[a], uniq[b]) else 0
        ix = np.asarray(idx, dtype=np.int64)
        return np.ascontiguousarray(T[np.ix_(ix, ix)])

    def _pair_filter_key(self):
        """What the filter table depends on: the filter, the fixtures in
        record order and their filter data."""
        if self._contact_filter is _DEFAULT_FILTER:
            return None
        self._materialise()
        if self._contact_filter is None:
            return ("off", len(self._F))
        owners = tuple(id(self._fixture_at(r)) for r in range(len(self._F)))
        data = self._F[["category_bits", "mask_bits", "group_index"]]
        return (id(self._contact_filter), owners, tuple(map(tuple, data.tolist())))

    def _sync_pair_filter(self, gpu, world_index=0):
        """Before a step: the custom filter's table reaches the device batch
        when it changed (gb_batch_set_pair_filter)."""
        key = self._pair_filter_key()
        if key == self._pf_key:
            return
        gpu.set_pair_filter(world_index, self._pair_filter_table())
        self._pf_key = key

    @property
    def sub_stepping(self):
        return False

    @sub_stepping.setter
    def sub_stepping(self, v):
        if v:
            raise NotImplementedError("sub_stepping is not supported by the GPU world step")

    @property
    def locked(self):
        return self._locked

    @property
    def bodies(self):
        return list(self._bodies)

    @property
    def body_count(self):
        return len(self._bodies)

    @property
    def contacts(self):
        self._materialise()
        return [Contact(self, self._C[i]) for i in range(len(self._C))]

    @property
    def contact_count(self):
        self._materialise()
        return len(self._C)

    def _check_unlocked(self):
        if self._locked:
            raise LockedError("the world is locked during a step")

    # -- bodies
    def create_body(self, body=None, **kwargs):
        """world.py:208-224"""
        self._check_unlocked()
        if body is not None:
            raise NotImplementedError("copying an existing Body is not supported; pass keyword arguments")
        fixtures = _fixture_list(kwargs.pop("shapes", None), kwargs.pop("fixtures", None), kwargs.pop("shape_fixture", None))
        user_data = kwargs.pop("user_data", None)
        kwargs.pop("world", None)
        btype = kwargs.pop("type", Body.STATIC)
        if kwargs.pop("check_args", True):
            _check_body_args(btype, kwargs)
        self._structural()
        n_moves0 = len(self._sb.moves)
        bi = self._sb.create_body(btype, fixtures=[(f.shape, f._kwargs()) for f in fixtures], **kwargs)
        rb, rf = self._sb.body_records(bi)
        f0 = len(self._F)
        rb["fixture_start"] = f0
        self._B = np.concatenate([self._B, rb[None]])
        self._F = np.concatenate([self._F, rf])
        new_moves = [f0 + k for (b, k) in self._sb.moves[n_moves0:] if b == bi]
        self._M = np.concatenate([self._M, np.array(new_moves, np.int32)]).astype(np.int32)
        body = Body(self, bi, fixtures, user_data)
        for k, f in enumerate(fixtures):
            f._body, f._slot = body, k
        self._bodies.append(body)
        return body

    def create_dynamic_body(self, body=None, **kwargs):
        return self.create_body(body, type=Body.DYNAMIC, **kwargs)

    def create_static_body(self, body=None, **kwargs):
        return self.create_body(body, type=Body.STATIC, **kwargs)

    def create_kinematic_body(self, body=None, **kwargs):
        return self.create_body(body, type=Body.KINEMATIC, **kwargs)

    def destroy_body(self, body):
        """world.py:235-270: the body, its joints (body.py:313-320, each reported
        to joint_destruction_listener), its contacts (touching ones reported to
        end_contact, contact_manager.py:167-168) and its fixtures (each
        reported to fixture_destruction_listener, body.py:330-333) leave the
        world."""
        self._check_unlocked()
        for j in list(body.joints):
            if self.joint_destruction_listener is not None:
                self.joint_destruction_listener(j)
            self.destroy_joint(j)
        self._structural()
        bi = body._index
        B, F, C, M = self._B, self._F, self._C, self._M
        f0, nfix = int(B[bi]["fixture_start"]), int(B[bi]["fixture_count"])
        gone = lambda x: (x >= f0) & (x < f0 + nfix)   # noqa: E731
        if self.contact_manager.end_contact is not None:
            for c in C[gone(C["fixture_a"]) | gone(C["fixture_b"])]:
                if int(c["flags"]) & abi.C_TOUCHING:
                    self.contact_manager.end_contact(EventContact(self._fixture_at(int(c["fixture_a"])),
                                                                  self._fixture_at(int(c["fixture_b"])), False))
        if self.fixture_destruction_listener is not None:
            for f in list(body.fixtures):
                self.fixture_destruction_listener(f)
        C = C[~(gone(C["fixture_a"]) | gone(C["fixture_b"]))].copy()
        for key in ("fixture_a", "fixture_b"):
            C[key] = np.where(C[key] >= f0 + nfix, C[key] - nfix, C[key])
        M = M[~gone(M)]
        M = np.where(M >= f0 + nfix, M - nfix, M).astype(np.int32)
        F = np.delete(F, np.arange(f0, f0 + nfix))
        F["body"] = np.where(F["body"] > bi, F["body"] - 1, F["body"])
        B = np.delete(B, bi)
        B["fixture_start"] = np.where(B["fixture_start"] > f0, B["fixture_start"] - nfix, B["fixture_start"])
        self._B, self._F, self._C, self._M = B, F, C, M
        for key in ("body_a", "body_b"):
            self._J[key] = np.where(self._J[key] > bi, self._J[key] - 1, self._J[key])
        self._sb.bodies.pop(bi)
        self._sb.moves = [(b if b < bi else b - 1, k) for (b, k) in self._sb.moves if b != bi]
        self._bodies.pop(bi)
        for b in self._bodies[bi:]:
            b._index -= 1
        # body.py:342-344: the loop removes from the list it walks, so a body
        # in several controllers stays in every second one (as a body of no
        # world it has no record on the device)
        for controller in body._controllers:
            controller.remove_body(body)
        body._world = None

    def clear_forces(self):
        """world.py:356-369"""
        self._check_unlocked()
        self._materialise()
        self._B["fx"] = self._B["fy"] = self._B["torque"] = 0.0
        self._mark_bodies_edited()

    # -- the step
    def step(self, dt, vel_iters, pos_iters):
        """world.py:307-354: one gb_batch_step of this world, then the
        contact listeners' events."""
        self._check_unlocked()
        if self._owner is not None:
            raise RuntimeError("this world is stepped by a WorldBatch; call the batch's step")
        cm = self.contact_manager
        if cm.pre_solve is not None:
            raise NotImplementedError("pre_solve listeners cannot run inside the GPU step")
        self._check_mouse_joints(dt)
        self._sync_controllers()
        self._sync_device()
        self._sync_pair_filter(self._gpu)
        events = cm.wants_events
        self._locked = True
        try:
            self._gpu.step(float(dt), int(vel_iters), int(pos_iters), 1, launch_mode=1, events=events)
        finally:
            self._locked = False
        if dt > 0.0:
            self._inv_dt0 = 1.0 / dt
        self._host_fresh = False
        st = self._gpu.status()
        if st[0]:
            self._gpu.clear_status()
            raise step_error(st)
        if events:
            self._replay(self._gpu.events(0))

    # -- outside the GPU step: joints, controllers, loose bodies
    def add_body(self, body):
        """world.py:183-206 adds a Body built outside a world; bodies here are
        made by create_*_body only."""
        raise NotImplementedError("add_body: create bodies with World.create_*_body")

    # -- joints (world.py:252-306, 823-902)
    @property
    def joints(self):
        return list(self._joints)

    @property
    def joint_count(self):
        return len(self._joints)

    def add_joint(self, joint, duplicate=False):
        """world.py:252-283.  Creating a joint does not wake its bodies; when
        it turns collision off, the contacts between its bodies are flagged
        for filtering."""
        self._check_unlocked()
        if duplicate:
            raise NotImplementedError("add_joint(duplicate=True): create a second joint with the same arguments")
        if not isinstance(joint, Joint) or type(joint) not in _joints.KINDS.values():
            raise NotImplementedError(f"{type(joint).__name__} is not solved by the GPU world step")
        if joint._world is not None:
            raise ValueError("the joint already belongs to a world")
        for b in joint.bodies:
            if b is None and type(joint) is _joints.MouseJoint:
                continue   # the mouse joint's body_a is None (mouse.py:67)
            if b is None or b._world is not self:
                raise ValueError("Both bodies must be in the same world.")
        self._structural()
        r = joint._pending.copy()
        r["world"] = 0
        # a mouse joint's record repeats its one body (gb_joint, GB_JOINT_MOUSE)
        r["body_a"] = (joint._body_a if joint._body_a is not None else joint._body_b)._index
        r["body_b"] = joint._body_b._index
        self._J = np.concatenate([self._J, np.array([r], dtype=abi.JOINT)])
        joint._world, joint._index = self, len(self._joints)
        self._joints.append(joint)
        if not int(r["flags"]) & abi.J_COLLIDE_CONNECTED:
            self._flag_contacts_between(int(r["body_a"]), int(r["body_b"]))
        return joint

    def destroy_joint(self, joint):
        """world.py:285-305: the bodies are woken; contacts between them are
        flagged for filtering when the joint turned collision off."""
        self._check_unlocked()
        if joint._world is not self:
            raise ValueError("Joint not in world")
        self._structural()
        for b in joint.bodies:
            if b is not None:
                b.awake = True
        i = joint._index
        r = self._J[i].copy()
        self._J = np.delete(self._J, i)
        self._joints.pop(i)
        for k, j in enumerate(self._joints):
            j._index = k
        joint._pending = r
        joint._world, joint._index = None, -1
        if not int(r["flags"]) & abi.J_COLLIDE_CONNECTED:
            self._flag_contacts_between(int(r["body_a"]), int(r["body_b"]))

    def create_revolute_joint(self, *args, **kwargs):
        return self.add_joint(RevoluteJoint(*args, **kwargs))

    def create_prismatic_joint(self, *args, **kwargs):
        return self.add_joint(PrismaticJoint(*args, **kwargs))

    def create_distance_joint(self, *args, **kwargs):
        return self.add_joint(DistanceJoint(*args, **kwargs))

    def create_weld_joint(self, *args, **kwargs):
        return self.add_joint(WeldJoint(*args, **kwargs))

    def create_friction_joint(self, *args, **kwargs):
        return self.add_joint(_joints.FrictionJoint(*args, **kwargs))

    def create_rope_joint(self, *args, **kwargs):
        return self.add_joint(_joints.RopeJoint(*args, **kwargs))

    def create_wheel_joint(self, *args, **kwargs):
        return self.add_joint(_joints.WheelJoint(*args, **kwargs))

    def create_pulley_joint(self, *args, **kwargs):
        return self.add_joint(_joints.PulleyJoint(*args, **kwargs))

    def create_mouse_joint(self, *args, **kwargs):
        return self.add_joint(_joints.MouseJoint(*args, **kwargs))

    def _check_mouse_joints(self, dt):
        """mouse.py:161: the set-up asserts d + dt * k > EPSILON (a zero
        frequency fails it); the reference raises AssertionError from inside
        the step, here before it, for a mouse joint whose awake dynamic body
        the step solves."""
        if dt <= 0.0 or not any(type(j) is _joints.MouseJoint for j in self._joints):
            return
        for j in self._joints:
            if type(j) is not _joints.MouseJoint:
                continue
            b = j._body_b
            r = self._body_record(b._index)
            if r["type"] != Body.DYNAMIC or not (int(r["flags"]) & abi.BODY_AWAKE) or not (int(r["flags"]) & abi.BODY_ACTIVE):
                continue
            mass = float(r["mass"])
            omega = 2.0 * math.pi * j.frequency
            d = 2.0 * mass * j.damping_ratio * omega
            k = mass * omega ** 2
            if not d + dt * k > 2.220446049250313e-16:
                raise AssertionError("mouse joint: d + dt * k <= EPSILON (mouse.py:161)")

    def _unsupported(self, *args, **kwargs):
        raise NotImplementedError("gear joints are not part of the GPU world step")

    create_gear_joint = _unsupported

    # -- controllers (world.py:923-957)
    def create_gravity_controller(self, *args, **kwargs):
        """world.py:923-929"""
        return self.add_controller(GravityController(self, *args, **kwargs))

    def create_buoyancy_controller(self, *args, **kwargs):
        """world.py:931-937"""
        return self.add_controller(BuoyancyController(self, *args, **kwargs))

    def add_controller(self, controller):
        """world.py:939-945"""
        self.controllers.append(controller)
        return controller

    def destroy_controller(self, controller):
        """world.py:947-957: its bodies are detached, it leaves the world"""
        if controller not in self.controllers:
            raise ValueError("Controller not in this world")
        controller.clear()
        self.controllers.remove(controller)

    def _controller_state(self):
        """(records, body lists, structure key) of World.controllers"""
        C, cb = controller_records(self, self.controllers)
        key = (tuple(int(x) for x in C["type"]), tuple(int(x) for x in C["body_count"]), tuple(int(x) for x in cb))
        return C, cb, key

    def _sync_controllers(self):
        """Before a step: a new controller or body list rebuilds the device
        batch, new parameters are uploaded (gb_batch_set_controllers)."""
        if not self.controllers and self._ctl_key is None:
            return
        C, cb, key = self._controller_state()
        if self._gpu is None:
            return
        if key != self._ctl_key:
            self._structural()
        elif C.tobytes() != self._ctl_params:
            self._gpu.set_controllers(C)
            self._ctl_params = C.tobytes()

    # -- queries
    def query_aabb(self, aabb, callback=None):
        """world.py:371-385: the fixtures whose broad-phase (fat) AABB
        overlaps `aabb` (an object with lower_bound / upper_bound, or
        (lower, upper), or (lx, ly, ux, uy)); one gb_batch_query_aabb.  The
        fixtures come in fixture order (the reference's in tree order).
        Without a callback, an iterator; with one, called per fixture until
        it returns a false value, at once, and an empty iterator comes back:
        the reference's method is a generator, so callers that pass a
        callback iterate the result to run it."""
        lx, ly, ux, uy = _box_of(aabb)
        gpu, wi = self._query_gpu()
        q = np.zeros(1, dtype=abi.AABB_QUERY)
        q["world"], q["lx"], q["ly"], q["ux"], q["uy"] = wi, lx, ly, ux, uy
        out, n = gpu.query_aabb(q, max_per_query=max(1, len(self._F)))
        fixtures = [self._fixture_at(int(k)) for k in out[0, :int(n[0])]]
        if callback is None:
            return iter(fixtures)
        for f in fixtures:
            if not callback(f):
                break
        return iter(())

    def ray_cast_closest(self, point1, point2):
        """The closest fixture on the segment point1 -> point2: what
        World.ray_cast (world.py:387-440) leaves in a callback that returns
        the fraction it is given.  Returns (fixture, point, normal, fraction)
        or None; one gb_batch_ray_cast."""
        p1, p2 = Vec2(*point1), Vec2(*point2)
        gpu, wi = self._query_gpu()
        r = np.zeros(1, dtype=abi.RAY)
        r["world"], r["p1x"], r["p1y"], r["p2x"], r["p2y"] = wi, p1[0], p1[1], p2[0], p2[1]
        try:
            h = gpu.ray_cast(r)[0]
        except abi.GB2DError as ex:
            if "no length" in str(ex):
                raise ValueError("||p2 - p1||^2 > 0.0") from ex   # dynamictree.py:222-224
            raise
        if int(h["fixture"]) < 0:
            return None
        return (self._fixture_at(int(h["fixture"])), Vec2(float(h["px"]), float(h["py"])),
                Vec2(float(h["nx"]), float(h["ny"])), float(h["fraction"]))

    def ray_cast(self, point1, point2, callback=None):
        """world.py:387-440.  The fixtures on the segment come from one
        gb_batch_ray_cast_all and are handed over in order of fraction (the
        reference hands them over in its tree's order), with the reference's
        answers: -1 skips the fixture, 0 ends the cast, a fraction clips the
        ray (later hits beyond it are skipped), 1 goes on.  A closest-hit
        callback therefore ends as with the reference, and an all-hits one
        sees the same hits.  Without a callback, a generator of
        [fixture, point, normal, fraction] lists whose last entry the caller
        may set to the same answers.  A callback runs at once and an empty
        iterator comes back (callers of the reference's generator iterate
        it to run the callback)."""
        hits = self._ray_hits(point1, point2)
        if callback is not None:
            self._ray_walk(hits, lambda entry: callback(*entry))
            return iter(())
        return self._ray_generator(hits)

    def _ray_hits(self, point1, point2):
        p1, p2 = Vec2(*point1), Vec2(*point2)
        gpu, wi = self._query_gpu()
        r = np.zeros(1, dtype=abi.RAY)
        r["world"], r["p1x"], r["p1y"], r["p2x"], r["p2y"] = wi, p1[0], p1[1], p2[0], p2[1]
        cap = max(1, len(self._F))
        try:
            out, n = gpu.ray_cast_all(r, max_per_ray=cap)
        except abi.GB2DError as ex:
            if "no length" in str(ex):
                raise ValueError("||p2 - p1||^2 > 0.0") from ex   # dynamictree.py:222-224
            raise
        h = out[0, :int(n[0])]
        h = h[np.lexsort((h["fixture"], h["fraction"]))]
        return [(self._fixture_at(int(x["fixture"])), Vec2(float(x["px"]), float(x["py"])),
                 Vec2(float(x["nx"]), float(x["ny"])), float(x["fraction"])) for x in h]

    @staticmethod
    def _ray_walk(hits, answer):
        max_fraction = 1.0
        for hit in hits:
            if hit[3] > max_fraction:
                continue
            value = answer(list(hit))
            if value == 0.0:
                break
            if value > 0.0:
                max_fraction = value

    @staticmethod
    def _ray_generator(hits):
        max_fraction = 1.0
        for hit in hits:
            if hit[3] > max_fraction:
                continue
            entry = list(hit)
            yield entry
            value = entry[-1]
            if value == 0.0:
                break
            if value > 0.0:
                max_fraction = value

    def _replay(self, ev):
        """Hand the step's recorded events to the listeners, in key order.
        The world is locked meanwhile, as during the reference's step
        (world.py:321-354), where the listeners run: world.locked is True and
        structural changes raise LockedError."""
        was = self._locked
        self._locked = True
        try:
            self._replay_events(ev)
        finally:
            self._locked = was

    def _replay_events(self, ev):
        cm = self.contact_manager
        for e in ev:
            fa, fb = self._fixture_at(int(e["fixture_a"])), self._fixture_at(int(e["fixture_b"]))
            t = int(e["type"])
            if t == abi.EV_BEGIN and cm.begin_contact is not None:
                cm.begin_contact(EventContact(fa, fb, True))
            elif t == abi.EV_END and cm.end_contact is not None:
                cm.end_contact(EventContact(fa, fb, False))
            elif t == abi.EV_POST_SOLVE and cm.post_solve is not None:
                n = int(e["point_count"])
                cm.post_solve(EventContact(fa, fb, True),
                              [(float(e["normal_impulse"][k]), float(e["tangent_impulse"][k])) for k in range(n)])

    # ---------------------------------------------------------------- internals
    def _materialise(self):
        """Download the device state into the host records (once per step)."""
        if self._owner is not None and not self._host_fresh:
            self._owner._pull(self)
            return
        if self._gpu is None or self._host_fresh:
            return
        self._B = self._gpu.bodies()
        self._F["aabb"] = self._gpu.proxies()
        self._C = self._gpu.contacts(0)
        self._M = np.zeros(0, np.int32)
        if len(self._J):
            self._J = self._gpu.joints()
        self._host_fresh = True

    def _structural(self):
        """The next step re-uploads the whole world from the host records."""
        if self._owner is not None:
            raise NotImplementedError("structural changes (bodies, fixtures, transforms, gravity) of a world "
                                      "inside a WorldBatch: build a new batch after the change")
        self._materialise()
        if self._gpu is not None:
            self._gpu.close()
            self._gpu = None
        self._upload_bodies = False

    def _body_record(self, i, write=False):
        self._materialise()
        if write:
            self._mark_bodies_edited()
        return self._B[i]

    def _mark_bodies_edited(self):
        if self._gpu is not None or self._owner is not None:
            self._upload_bodies = True

    def _joint_record(self, i, write=False):
        self._materialise()
        if write and (self._gpu is not None or self._owner is not None):
            self._upload_joints = True
        return self._J[i]

    def _flag_contacts_between(self, ba, bb):
        """contact._flag_for_filtering of every contact between bodies ba and bb"""
        if not len(self._C):
            return
        fb = self._F["body"]
        a, b = fb[self._C["fixture_a"]], fb[self._C["fixture_b"]]
        hit = ((a == ba) & (b == bb)) | ((a == bb) & (b == ba))
        self._C["flags"] = np.where(hit, self._C["flags"] | abi.C_FILTER, self._C["flags"])

    def _query_gpu(self):
        """The device batch holding this world's current state, and the
        world's index in it."""
        if self._owner is not None:
            return self._owner._device_for(self)
        self._sync_device()
        return self._gpu, 0

    def _moves(self):
        """The move buffer with each proxy at its first position: pairs are
        found once per moved proxy, ordered by that position, so a proxy
        touched again before the step (a second filter change) adds
        nothing (broadphase.py:83-109 collects the pairs in a set)."""
        M = self._M
        if len(M) == 0:
            return M
        return M[np.sort(np.unique(M, return_index=True)[1])].astype(np.int32)

    def _fixture_at(self, f):
        return self._fixture_child_at(f)[0]

    def _fixture_child_at(self, f):
        """The fixture of record f and the child index of the record (a loop
        fixture has one record per child, fixture.py:250-261)."""
        bi = int(self._F[f]["body"])
        local = f - int(self._B[bi]["fixture_start"])
        for fx in self._bodies[bi].fixtures:
            n = fx.shape.child_count
            if local < n:
                return fx, local
            local -= n
        raise IndexError(f"fixture record {f} is past its body's fixtures")

    def _records_of(self, body, fixture):
        """(first record, record count) of a fixture of a body in the world"""
        o = int(self._B[body._index]["fixture_start"])
        for fx in body.fixtures:
            if fx is fixture:
                return o, fx.shape.child_count
            o += fx.shape.child_count
        raise ValueError("This fixture does not belong to this body")

    def _sync_device(self):
        if self._gpu is None:
            M = self._moves()
            W = self._sb.world_record(len(self._B), len(self._F), len(M))
            W["contact_count"] = len(self._C)
            W["contact_capacity"] = self._contact_capacity
            W["inv_dt0"] = self._inv_dt0
            C, cb, key = self._controller_state() if self.controllers else (None, None, None)
            self._gpu = self._make_batch(W, self._B, self._F, self._C, M, self._J, C, cb)
            self._ctl_key, self._ctl_params = key, (C.tobytes() if C is not None else None)
            self._pf_key = None
            self._host_fresh = True
            self._upload_bodies = False
            self._upload_joints = False
            return
        if self._upload_bodies:
            self._gpu.set_bodies(self._B)
            self._upload_bodies = False
        if self._upload_joints:
            self._gpu.set_joints(self._J)
            self._upload_joints = False

    def _make_batch(self, W, B, F, C, M, J=None, CT=None, CB=None):
        """The device batch holding this world (gb_batch_create)."""
        from .gpu import GpuBatch
        return GpuBatch(W, B, F, contacts=C if len(C) else None, precision=self._precision, moves=M,
                        joints=J if J is not None and len(J) else None, controllers=CT, controller_bodies=CB)

    def _add_fixture(self, body, fixture):
        """body.py:185-214: the fixture joins the body, its proxy the move
        buffer; a positive density resets the body's mass data."""
        self._structural()
        bi = body._index
        b = self._sb.bodies[bi]
        _load_body_state(b, self._B[bi])
        self._sb.add_fixture(bi, fixture.shape, **fixture._kwargs())
        rb, rf = self._sb.body_records(bi)
        r = self._B[bi]
        for key in ("lcx", "lcy", "c0x", "c0y", "cx", "cy", "vx", "vy", "mass", "inv_mass", "I", "inv_I"):
            r[key] = rb[key]
        n = fixture.shape.child_count
        pos = int(r["fixture_start"]) + int(r["fixture_count"])
        self._F = np.insert(self._F, pos, rf[-n:])
        self._B["fixture_count"][bi] += n
        self._B["fixture_start"] = np.where(np.arange(len(self._B)) > bi, self._B["fixture_start"] + n,
                                            self._B["fixture_start"])
        for key in ("fixture_a", "fixture_b"):
            self._C[key] = np.where(self._C[key] >= pos, self._C[key] + n, self._C[key])
        M = np.where(self._M >= pos, self._M + n, self._M)
        new = np.arange(pos, pos + n, dtype=np.int32) if b.active else np.zeros(0, np.int32)
        self._M = np.concatenate([M, new]).astype(np.int32)
        fixture._body, fixture._slot = body, len(body.fixtures)
        body.fixtures.append(fixture)

    def _reset_mass_data(self, body):
        bi = body._index
        r = self._body_record(bi, write=True)
        b = self._sb.bodies[bi]
        _load_body_state(b, r)
        b.reset_mass_data()
        rb, _ = self._sb.body_records(bi)
        for key in ("lcx", "lcy", "c0x", "c0y", "cx", "cy", "vx", "vy", "mass", "inv_mass", "I", "inv_I"):
            r[key] = rb[key]

    def _set_fixture(self, fixture, refilter):
        """A fixture's material or filter changed: its record (and the
        construction-time copy used by reset_mass_data) follow; with
        `refilter`, fixture._refilter (fixture.py:269-285)."""
        self._structural()
        body = fixture._body
        bi, k = body._index, fixture._slot
        fi, n = self._records_of(body, fixture)
        for r in self._F[fi:fi + n]:
            r["friction"], r["restitution"], r["density"] = fixture.friction, fixture.restitution, fixture.density
            r["category_bits"], r["mask_bits"], r["group_index"] = fixture.category_bits, fixture.mask_bits, fixture.group_index
            r["flags"] = (int(r["flags"]) | abi.FIX_SENSOR) if fixture.sensor else (int(r["flags"]) & ~abi.FIX_SENSOR)
        sf = self._sb.bodies[bi].fixtures[k]
        sf.friction, sf.restitution, sf.density = fixture.friction, fixture.restitution, fixture.density
        sf.category, sf.mask, sf.group, sf.sensor = fixture.category_bits, fixture.mask_bits, fixture.group_index, fixture.sensor
        if refilter:
            C = self._C
            mine = lambda x: (x >= fi) & (x < fi + n)   # noqa: E731
            C["flags"] = np.where(mine(C["fixture_a"]) | mine(C["fixture_b"]), C["flags"] | abi.C_FILTER, C["flags"])
            if int(self._B[bi]["flags"]) & abi.BODY_ACTIVE:
                self._M = np.concatenate([self._M, np.arange(fi, fi + n, dtype=np.int32)]).astype(np.int32)
                o = fi - int(self._B[bi]["fixture_start"])
                self._sb.moves.extend((bi, o + c) for c in range(n))

    def _set_type(self, body, t):
        self._structural()
        bi = body._index
        B, C = self._B, self._C
        r = B[bi]
        r["type"] = t
        b = self._sb.bodies[bi]
        _load_body_state(b, r)
        b.type = t
        b.reset_mass_data()
        rb, _ = self._sb.body_records(bi)
        for key in ("lcx", "lcy", "c0x", "c0y", "cx", "cy", "vx", "vy", "mass", "inv_mass", "I", "inv_I"):
            r[key] = rb[key]
        if t == Body.STATIC:
            r["vx"] = r["vy"] = r["w"] = 0.0
        if not int(r["flags"]) & abi.BODY_AWAKE:
            r["sleep_time"] = 0.0
        r["flags"] |= abi.BODY_AWAKE
        r["fx"] = r["fy"] = r["torque"] = 0.0
        # fixture._refilter (fixture.py:269-285): flag the fixtures' contacts,
        # touch their proxies (they join the move buffer)
        f0, nfix = int(r["fixture_start"]), int(r["fixture_count"])
        mine = lambda x: (x >= f0) & (x < f0 + nfix)   # noqa: E731
        C["flags"] = np.where(mine(C["fixture_a"]) | mine(C["fixture_b"]), C["flags"] | abi.C_FILTER, C["flags"])
        self._M = np.concatenate([self._M, np.arange(f0, f0 + nfix, dtype=np.int32)]).astype(np.int32)
        self._sb.moves.extend((bi, k) for k in range(nfix))

    def _destroy_fixture(self, body, fixture):
        self._structural()
        bi = body._index
        k = body.fixtures.index(fixture)
        B, F, C, M = self._B, self._F, self._C, self._M
        fi, n = self._records_of(body, fixture)
        o = fi - int(B[bi]["fixture_start"])
        gone = lambda x: (x >= fi) & (x < fi + n)   # noqa: E731
        hit = gone(C["fixture_a"]) | gone(C["fixture_b"])
        if self.contact_manager.end_contact is not None:
            for c in C[hit]:
                if int(c["flags"]) & abi.C_TOUCHING:
                    self.contact_manager.end_contact(EventContact(self._fixture_at(int(c["fixture_a"])),
                                                                  self._fixture_at(int(c["fixture_b"])), False))
        C = C[~hit].copy()
        for key in ("fixture_a", "fixture_b"):
            C[key] = np.where(C[key] >= fi + n, C[key] - n, C[key])
        M = M[~gone(M)]
        M = np.where(M >= fi + n, M - n, M).astype(np.int32)
        F = np.delete(F, np.arange(fi, fi + n))
        B["fixture_count"][bi] -= n
        B["fixture_start"] = np.where(np.arange(len(B)) > bi, B["fixture_start"] - n, B["fixture_start"])
        # the construction-time body: current state, fixture gone, mass data reset
        b = self._sb.bodies[bi]
        _load_body_state(b, B[bi])
        b.fixtures.pop(k)
        del b.aabbs[o:o + n]
        self._sb.moves = [(bb, kk - n if (bb == bi and kk >= o + n) else kk) for (bb, kk) in self._sb.moves
                          if not (bb == bi and o <= kk < o + n)]
        b.reset_mass_data()
        rb, _ = self._sb.body_records(bi)
        for key in ("lcx", "lcy", "c0x", "c0y", "cx", "cy", "vx", "vy", "mass", "inv_mass", "I", "inv_I"):
            B[bi][key] = rb[key]
        self._B, self._F, self._C, self._M = B, F, C, M
        body.fixtures.pop(k)
        fixture._body, fixture._slot = None, -1
        for j, f in enumerate(body.fixtures):
            f._slot = j

    def _set_active(self, bi, active):
        """Body.active setter (body.py:846-872).  The reference destroys the
        contacts in a loop over the body's contact list that removes from the
        same list, so it skips every second one and leaves them in the world;
        a later step then walks into the inactive body.  Here every contact
        of the body goes (touching ones reported to end_contact).  Making a
        body active again after it was made inactive with fixtures raises
        AssertionError, as in the reference: its Fixture._destroy_proxies
        leaves the fixture's proxy list non-empty and _create_proxies asserts
        it is empty (fixture.py:250-267).  Here nothing changes before the
        exception (the reference has already set the flag, and its next step
        fails on the dead proxy)."""
        b = self._sb.bodies[bi]
        if active and getattr(b, "stale_proxies", False):
            raise AssertionError("the body's fixtures still hold the proxies destroyed when it was made inactive")
        self._structural()
        B, F, C = self._B, self._F, self._C
        r = B[bi]
        f0, nfix = int(r["fixture_start"]), int(r["fixture_count"])
        mine = lambda x: (x >= f0) & (x < f0 + nfix)   # noqa: E731
        b.active = active
        if active:
            r["flags"] |= abi.BODY_ACTIVE
            pos, q = (float(r["px"]), float(r["py"])), (float(r["qc"]), float(r["qs"]))
            for k, (lx, ly, ux, uy) in enumerate(_record_aabbs(b.fixtures, pos, q)):
                F[f0 + k]["aabb"] = (lx - AABB_EXTENSION, ly - AABB_EXTENSION, ux + AABB_EXTENSION, uy + AABB_EXTENSION)
            self._M = np.concatenate([self._M, np.arange(f0, f0 + nfix, dtype=np.int32)]).astype(np.int32)
            self._sb.moves.extend((bi, k) for k in range(nfix))
            return
        r["flags"] &= np.uint32(0xFFFFFFFF ^ abi.BODY_ACTIVE)
        b.stale_proxies = nfix > 0
        hit = mine(C["fixture_a"]) | mine(C["fixture_b"])
        if self.contact_manager.end_contact is not None:
            for c in C[hit]:
                if int(c["flags"]) & abi.C_TOUCHING:
                    self.contact_manager.end_contact(EventContact(self._fixture_at(int(c["fixture_a"])),
                                                                  self._fixture_at(int(c["fixture_b"])), False))
        self._C = C[~hit].copy()
        self._M = self._M[~mine(self._M)].astype(np.int32)
        self._sb.moves = [(bb, k) for (bb, k) in self._sb.moves if bb != bi]

    def _set_transform(self, bi, pos, angle):
        """body.py:404-413 _transform_updated: new transform (angle None: the
        rotation kept) and sweep, whose angle is the transform's atan2
        (transform.c Transform_get_angle); the fixtures are synchronised with
        zero displacement (fixture.py:287-298, dynamictree.py:152-188) and
        re-fattened ones enter the move buffer."""
        self._structural()
        r = self._B[bi]
        q = (math.cos(angle), math.sin(angle)) if angle is not None else (float(r["qc"]), float(r["qs"]))
        angle = math.atan2(q[1], q[0])
        r["px"], r["py"], r["qc"], r["qs"] = pos[0], pos[1], q[0], q[1]
        lcx, lcy = float(r["lcx"]), float(r["lcy"])
        cx = pos[0] + q[0] * lcx + (-q[1]) * lcy
        cy = pos[1] + q[1] * lcx + q[0] * lcy
        r["c0x"], r["c0y"], r["cx"], r["cy"] = cx, cy, cx, cy
        r["a0"] = r["a"] = angle
        start = int(r["fixture_start"])
        moved = []
        for k, tight in enumerate(_record_aabbs(self._sb.bodies[bi].fixtures, pos, q)):
            fat = tuple(float(x) for x in self._F[start + k]["aabb"])
            if not _contains(fat, tight):
                self._F[start + k]["aabb"] = (tight[0] - AABB_EXTENSION, tight[1] - AABB_EXTENSION,
                                              tight[2] + AABB_EXTENSION, tight[3] + AABB_EXTENSION)
                moved.append(start + k)
        if moved:
            self._M = np.concatenate([self._M, np.array(moved, np.int32)]).astype(np.int32)


def _record_aabbs(fixtures, p, q):
    """The tight AABB of every fixture record under transform (p, q): one per
    child of a loop (shapes.py:822-837), one per other shape."""
    out = []
    for f in fixtures:
        sh = f.shape
        if isinstance(sh, Loop):
            out.extend(sh.compute_aabb(p, q, c) for c in range(sh.child_count))
        else:
            out.append(sh.compute_aabb(p, q))
    return out


_EPSILON_SQR = 2.220446049250313e-16 ** 2       # settings.py EPSILON_SQR


def _normalized(x, y):
    """Vec2_normalized (vec2module.c): unchanged below FLT_EPSILON."""
    length = math.sqrt(x * x + y * y)
    if length < 1.1920928955078125e-07:
        return x, y
    inv = 1.0 / length
    return x * inv, y * inv


def world_manifold(c, B, F):
    """WorldManifold (contact_util.py:195-245) of contact record `c` with the
    body records `B` and fixture records `F` of its world (world-local
    indices): (normal from A to B, [world points])."""
    fa, fb = int(c["fixture_a"]), int(c["fixture_b"])
    ra, rb = float(F[fa]["radius"]), float(F[fb]["radius"])
    ba, bb = B[int(F[fa]["body"])], B[int(F[fb]["body"])]
    n = int(c["m_point_count"])
    if n == 0:
        return Vec2(0.0, 0.0), []

    def xmul(b, x, y):      # Transform_mul
        return (b["px"] + b["qc"] * x + (-b["qs"]) * y, b["py"] + b["qs"] * x + b["qc"] * y)

    def rmul(b, x, y):      # Mat22_mul
        return (b["qc"] * x + (-b["qs"]) * y, b["qs"] * x + b["qc"] * y)

    t = int(c["m_type"])
    if t == abi.M_CIRCLES:
        nx, ny = 1.0, 0.0
        pa = xmul(ba, c["m_lpx"], c["m_lpy"])
        pb = xmul(bb, c["p_lx"][0], c["p_ly"][0])
        dx, dy = pa[0] - pb[0], pa[1] - pb[1]
        if dx * dx + dy * dy > _EPSILON_SQR:
            nx, ny = _normalized(pb[0] - pa[0], pb[1] - pa[1])
        ca = (pa[0] + ra * nx, pa[1] + ra * ny)
        cb = (pb[0] - rb * nx, pb[1] - rb * ny)
        return Vec2(nx, ny), [Vec2(0.5 * (ca[0] + cb[0]), 0.5 * (ca[1] + cb[1]))]
    face_a = t == abi.M_FACE_A
    bp, bc, rp, rc = (ba, bb, ra, rb) if face_a else (bb, ba, rb, ra)
    nx, ny = rmul(bp, c["m_lnx"], c["m_lny"])
    plane = xmul(bp, c["m_lpx"], c["m_lpy"])
    pts = []
    for k in range(n):
        clip = xmul(bc, c["p_lx"][k], c["p_ly"][k])
        s = rp - ((clip[0] - plane[0]) * nx + (clip[1] - plane[1]) * ny)
        c1 = (clip[0] + s * nx, clip[1] + s * ny)        # on the reference face's side
        c2 = (clip[0] - rc * nx, clip[1] - rc * ny)
        ca, cb = (c1, c2) if face_a else (c2, c1)
        pts.append(Vec2(0.5 * (ca[0] + cb[0]), 0.5 * (ca[1] + cb[1])))
    if not face_a:
        nx, ny = -nx, -ny
    return Vec2(nx, ny), pts


def _box_of(aabb):
    """(lx, ly, ux, uy) of an AABB given as an object with lower_bound /
    upper_bound, as (lower, upper) or as four numbers."""
    if hasattr(aabb, "lower_bound"):
        lo, hi = aabb.lower_bound, aabb.upper_bound
        return float(lo[0]), float(lo[1]), float(hi[0]), float(hi[1])
    if len(aabb) == 2:
        return float(aabb[0][0]), float(aabb[0][1]), float(aabb[1][0]), float(aabb[1][1])
    return tuple(float(x) for x in aabb)


def _contains(fat, tight):
    """AABB.contains (common.py): fat holds tight."""
    return fat[0] <= tight[0] and fat[1] <= tight[1] and tight[2] <= fat[2] and tight[3] <= fat[3]


def _load_body_state(b: _Body, r):
    """Copy a body record into the construction-time body (for reset_mass_data)."""
    b.p, b.q = (float(r["px"]), float(r["py"])), (float(r["qc"]), float(r["qs"]))
    b.lc = (float(r["lcx"]), float(r["lcy"]))
    b.c0, b.c = (float(r["c0x"]), float(r["c0y"])), (float(r["cx"]), float(r["cy"]))
    b.a0, b.a, b.alpha0 = float(r["a0"]), float(r["a"]), float(r["alpha0"])
    b.v, b.w = (float(r["vx"]), float(r["vy"])), float(r["w"])
    b.force, b.torque = (float(r["fx"]), float(r["fy"])), float(r["torque"])
    b.mass, b.inv_mass, b.I, b.invI = float(r["mass"]), float(r["inv_mass"]), float(r["I"]), float(r["inv_I"])
    b.sleep_time = float(r["sleep_time"])
    fl = int(r["flags"])
    b.awake, b.allow_sleep, b.bullet = bool(fl & abi.BODY_AWAKE), bool(fl & abi.BODY_ALLOW_SLEEP), bool(fl & abi.BODY_BULLET)
    b.fixed_rotation = bool(fl & abi.BODY_FIXED_ROTATION)


def _concat_worlds(recs):
    """Per-world (W, B, F, C, M) host records -> one batch's records (the
    world descriptors' ranges shifted; everything inside a world stays
    world-local)."""
    Ws, nb, nf, nc, nm = [], 0, 0, 0, 0
    for W, B, F, C, M in recs:
        W = W.copy()
        W["body_start"], W["fixture_start"], W["contact_start"], W["move_start"] = nb, nf, nc, nm
        Ws.append(W)
        nb, nf, nc, nm = nb + len(B), nf + len(F), nc + len(C), nm + len(M)
    cat = np.concatenate
    return (cat(Ws), cat([r[1] for r in recs]), cat([r[2] for r in recs]), cat([r[3] for r in recs]),
            cat([np.asarray(r[4], dtype=np.int32) for r in recs]).astype(np.int32))


class WorldBatch:
    """Independent worlds advanced together: one device batch and one launch
    sequence a step for all of them (the batched form of World.step,
    world.py:307-354).

    The worlds are built through the World API first.  While the batch holds
    them, their body getters, setters, forces, contacts, listeners and
    queries work as before; World.step and structural changes (new bodies or
    fixtures, transforms, gravity) raise, and every step is a
    WorldBatch.step.  ``close()`` hands the worlds back."""

    def __init__(self, worlds, precision=None):
        worlds = list(worlds)
        if not worlds:
            raise ValueError("a WorldBatch needs at least one world")
        for w in worlds:
            w._check_unlocked()
            if w._owner is not None:
                raise ValueError("a world can belong to one WorldBatch at a time")
        recs, Js = [], []
        for i, w in enumerate(worlds):
            w._materialise()
            M = w._moves()
            W = w._sb.world_record(len(w._B), len(w._F), len(M))
            W["contact_count"] = len(w._C)
            W["contact_capacity"] = w._contact_capacity
            W["inv_dt0"] = w._inv_dt0
            recs.append((W, w._B, w._F, w._C, M))
            J = w._J.copy()
            J["world"] = i
            Js.append(J)
        W, B, F, C, M = _concat_worlds(recs)
        J = np.concatenate(Js)
        self._ctl_keys = [w._controller_state()[2] if w.controllers else None for w in worlds]
        CT, CB = self._controller_records(worlds)
        self._ctl_params = CT.tobytes()
        from .gpu import GpuBatch
        self._gpu = GpuBatch(W, B, F, contacts=C if len(C) else None, precision=precision or worlds[0]._precision,
                             moves=M, joints=J if len(J) else None, controllers=CT if len(CT) else None,
                             controller_bodies=CB)
        self._worlds = worlds
        self._index = {id(w): i for i, w in enumerate(worlds)}
        for i, w in enumerate(worlds):
            w._pf_key = None
            w._sync_pair_filter(self._gpu, i)
        self._ranges = [(int(r["body_start"]), int(r["body_count"]), int(r["fixture_start"]), int(r["fixture_count"]))
                        for r in W]
        self._all = None        # (bodies, fat AABBs) of the whole batch, downloaded once after a step
        self._graphs = {}
        for w in worlds:
            if w._gpu is not None:
                w._gpu.close()
                w._gpu = None
            w._owner = self
            w._host_fresh = True
            w._upload_bodies = False
            w._upload_joints = False

    @property
    def worlds(self):
        return list(self._worlds)

    @property
    def device(self):
        """The underlying GpuBatch (C ABI handle)."""
        return self._gpu

    def autotune(self, dt, vel_iters=8, pos_iters=3, steps_per_trial=3):
        """Pick the launch configuration from trial steps (gb_batch_autotune);
        the worlds' state is unchanged."""
        self._push_edits()
        self._graphs.clear()
        return self._gpu.autotune(float(dt), int(vel_iters), int(pos_iters), steps_per_trial)

    def step(self, dt, vel_iters, pos_iters, n_steps=1, graph=False, stream=None):
        """n_steps calls of World.step on every world of the batch, in one
        gb_batch_step call, or (graph=True) as a captured CUDA graph replayed
        (captured once per (dt, iterations, n_steps)).  Listeners are called
        afterwards, world by world, in each world's event order."""
        for w in self._worlds:
            w._check_unlocked()
            if w.contact_manager.pre_solve is not None:
                raise NotImplementedError("pre_solve listeners cannot run inside the GPU step")
            w._check_mouse_joints(dt)
        self._push_edits()
        events = any(w.contact_manager.wants_events for w in self._worlds)
        for w in self._worlds:
            w._locked = True
        try:
            if graph:
                key = (float(dt), int(vel_iters), int(pos_iters), int(n_steps), events)
                g = self._graphs.get(key)
                if g is None:
                    g = self._gpu.capture(float(dt), int(vel_iters), int(pos_iters), int(n_steps), launch_mode=0,
                                          events=events)
                    self._graphs[key] = g
                g.launch(stream)
            else:
                self._gpu.step(float(dt), int(vel_iters), int(pos_iters), int(n_steps), launch_mode=0, events=events,
                               stream=stream)
        finally:
            for w in self._worlds:
                w._locked = False
        self._all = None
        for w in self._worlds:
            w._host_fresh = False
            if dt > 0.0 and n_steps > 0:
                w._inv_dt0 = 1.0 / dt
        st = self._gpu.status()
        if st.any():
            self._gpu.clear_status()
            raise step_error(st)
        if events:
            for i, w in enumerate(self._worlds):
                if w.contact_manager.wants_events:
                    w._replay(self._gpu.events(i))

    def close(self):
        """Copy the state back into the worlds and release them: each World
        steps on its own again (from its host records)."""
        if self._gpu is None:
            return
        for w in self._worlds:
            w._materialise()
        for w in self._worlds:
            w._owner = None
            w._upload_bodies = False
        for g in self._graphs.values():
            g.close()
        self._graphs.clear()
        self._gpu.close()
        self._gpu = None

    # ------------------------------------------------------------ internals
    def _pull(self, w):
        """Download world w's state (bodies, fat AABBs, contacts) into its
        host records; the whole batch's bodies and boxes come down once a step."""
        if self._all is None:
            self._all = (self._gpu.bodies(), self._gpu.proxies())
        B, A = self._all
        i = self._index[id(w)]
        b0, nb, f0, nf = self._ranges[i]
        w._B = B[b0:b0 + nb].copy()
        w._F["aabb"] = A[f0:f0 + nf]
        w._C = self._gpu.contacts(i)
        w._M = np.zeros(0, np.int32)
        if len(w._J):
            J = self._gpu.joints(i).copy()
            J["world"] = 0
            w._J = J
        w._host_fresh = True

    @staticmethod
    def _controller_records(worlds):
        """The controllers of every world, world by world (world field = its
        index in the batch), and their concatenated body lists."""
        Cs, Bs = [np.zeros(0, abi.CONTROLLER)], [np.zeros(0, np.int32)]
        nb = 0
        for i, w in enumerate(worlds):
            if not w.controllers:
                continue
            C, cb, _ = w._controller_state()
            C["world"] = i
            C["body_start"] += nb
            nb += len(cb)
            Cs.append(C)
            Bs.append(cb)
        return np.concatenate(Cs), np.concatenate(Bs).astype(np.int32)

    def _push_controllers(self):
        """Controller parameters edited since the last step go up
        (gb_batch_set_controllers); a new controller or body list is a
        structural change."""
        if not any(w.controllers for w in self._worlds) and not any(self._ctl_keys):
            return
        for w, key in zip(self._worlds, self._ctl_keys):
            if (w._controller_state()[2] if w.controllers else None) != key:
                raise NotImplementedError("a controller or controller body list changed in a world inside a "
                                          "WorldBatch: build a new batch after the change")
        CT, _ = self._controller_records(self._worlds)
        if CT.tobytes() != self._ctl_params:
            self._gpu.set_controllers(CT)
            self._ctl_params = CT.tobytes()

    def _push_edits(self):
        """Upload the bodies (joints, controllers) of the whole batch when a
        world's bodies (joints, controllers) were edited on the host:
        velocities, forces, awake flags (motor, limit and spring settings;
        controller parameters)."""
        self._push_controllers()
        for i, w in enumerate(self._worlds):
            if w._contact_filter is not _DEFAULT_FILTER or w._pf_key is not None:
                w._sync_pair_filter(self._gpu, i)
        bodies = any(w._upload_bodies for w in self._worlds)
        joints = any(w._upload_joints for w in self._worlds)
        if not (bodies or joints):
            return
        for w in self._worlds:
            w._materialise()
        if bodies:
            self._gpu.set_bodies(np.concatenate([w._B for w in self._worlds]))
            self._all = None
        if joints:
            Js = []
            for i, w in enumerate(self._worlds):
                J = w._J.copy()
                J["world"] = i
                Js.append(J)
            self._gpu.set_joints(np.concatenate(Js))
        for w in self._worlds:
            w._upload_bodies = False
            w._upload_joints = False

    def _device_for(self, w):
        self._push_edits()
        return self._gpu, self._index[id(w)]

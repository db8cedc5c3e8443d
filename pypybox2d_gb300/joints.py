"""The joint classes of the reference (pypybox2d/joints/): revolute,
prismatic, distance, weld, friction, rope, wheel, pulley and mouse, with their
constructors, properties, setters and reaction getters.

A joint is a view of one ``abi.JOINT`` record of its world (definition and
carried state: impulses, motor impulse, limit state); the GPU step solves
the records (gb_joint, include/gb2d.h).  Construction computes the local
anchors, reference angle and axis from the bodies' current frames with the
reference's arithmetic (joints/*.py __init__), so a joint built here holds
the same doubles as the reference's.
"""
from __future__ import annotations

import math

import numpy as np

from . import abi

LINEAR_SLOP = 0.005          # settings.py:61
INACTIVE_LIMIT, AT_LOWER_LIMIT, AT_UPPER_LIMIT, EQUAL_LIMITS = range(4)   # joints/joint.py:35
ALLOWED_STRETCH = 10.0 * LINEAR_SLOP


class _V(tuple):
    """A 2-vector result (x, y) with .x/.y, as the reference's Vec2."""

    def __new__(cls, x, y):
        return tuple.__new__(cls, (float(x), float(y)))

    x = property(lambda self: self[0])
    y = property(lambda self: self[1])


def _sub(a, b):
    return (a[0] - b[0], a[1] - b[1])


def _rot(angle, v):
    """Mat22(angle=a) * v (mat22module.c: col1 = (cos, sin), col2 = (-sin, cos))"""
    c, s = math.cos(angle), math.sin(angle)
    return (c * v[0] + (-s) * v[1], s * v[0] + c * v[1])


class Joint:
    """joints/joint.py:37-112.  Bodies must belong to the same World; the
    joint joins the world with World.add_joint (World.create_*_joint does
    both)."""

    _type = 0

    def __init__(self, body_a, body_b, collide_connected):
        if body_a is not None and body_b is not None:
            if body_a._world is not body_b._world or body_a._world is None:
                raise ValueError("Both bodies must be in the same world.")
        self._body_a, self._body_b = body_a, body_b
        self._world = None
        self._index = -1
        self._pending = np.zeros(1, dtype=abi.JOINT)[0]   # the record until the joint joins its world
        self._pending["type"] = self._type
        self._pending["flags"] = abi.J_COLLIDE_CONNECTED if collide_connected else 0

    # -- the record
    def _rec(self):
        if self._world is None:
            return self._pending
        return self._world._joint_record(self._index)

    def _edit(self):
        """The record, for a change the next step must see."""
        if self._world is None:
            return self._pending
        return self._world._joint_record(self._index, write=True)

    def _wake(self):
        for b in self.bodies:
            if b is not None:
                b.awake = True

    def _flag(self, bit):
        return bool(int(self._rec()["flags"]) & bit)

    def _set_flag(self, bit, on):
        r = self._edit()
        r["flags"] = (int(r["flags"]) | bit) if on else (int(r["flags"]) & ~bit)

    # -- joints/joint.py
    @property
    def body_a(self):
        return self._body_a

    @property
    def body_b(self):
        return self._body_b

    @property
    def bodies(self):
        return [self._body_a, self._body_b]

    def other_body(self, body):
        return self._body_b if body == self._body_a else self._body_a

    @property
    def active(self):
        return self._body_a.active and self._body_b.active

    @property
    def collide_connected(self):
        return self._flag(abi.J_COLLIDE_CONNECTED)

    @property
    def world(self):
        return self._world

    def get_reaction_force(self, inv_dt):
        r = self._rec()
        return _V(inv_dt * float(r["impulse"][0]), inv_dt * float(r["impulse"][1]))

    def get_reaction_torque(self, inv_dt):
        return inv_dt * float(self._rec()["impulse"][2])

    # -- anchors (local anchors relative to each body's origin)
    @property
    def local_anchor_a(self):
        r = self._rec()
        return _V(r["la_x"], r["la_y"])

    @property
    def local_anchor_b(self):
        r = self._rec()
        return _V(r["lb_x"], r["lb_y"])

    @property
    def anchor_a(self):
        return self._body_a.get_world_point(self.local_anchor_a)

    @property
    def anchor_b(self):
        return self._body_b.get_world_point(self.local_anchor_b)

    def _set_anchors(self, anchor_a, anchor_b, local_a, local_b):
        r = self._pending
        la = local_a if local_a is not None else self._body_a.get_local_point(anchor_a)
        lb = local_b if local_b is not None else self._body_b.get_local_point(anchor_b)
        r["la_x"], r["la_y"] = float(la[0]), float(la[1])
        r["lb_x"], r["lb_y"] = float(lb[0]), float(lb[1])

    def __repr__(self):
        return f"{type(self).__name__}(body_a={self._body_a!r}, body_b={self._body_b!r})"


class RevoluteJoint(Joint):
    """joints/revolute.py:32-453"""

    _type = abi.JOINT_REVOLUTE

    def __init__(self, body_a, body_b, anchor=(0, 0), reference_angle=None, lower_angle=0.0, upper_angle=0.0,
                 max_motor_torque=0.0, motor_speed=0.0, limit_enabled=False, motor_enabled=False,
                 local_anchor_a=None, local_anchor_b=None, collide_connected=False):
        if body_a is None or body_b is None:
            raise ValueError("body_a and body_b must be set")
        Joint.__init__(self, body_a, body_b, collide_connected)
        self._set_anchors(anchor, anchor, local_anchor_a, local_anchor_b)
        r = self._pending
        r["ref_angle"] = float(reference_angle) if reference_angle is not None else body_b.angle - body_a.angle
        r["lower"], r["upper"] = float(lower_angle), float(upper_angle)
        r["max_motor"], r["motor_speed"] = float(max_motor_torque), float(motor_speed)
        r["flags"] |= (abi.J_LIMIT if limit_enabled else 0) | (abi.J_MOTOR if motor_enabled else 0)

    @property
    def reference_angle(self):
        return float(self._rec()["ref_angle"])

    @property
    def joint_angle(self):
        """revolute.py:119-122: the sweep angles (not Body.angle)"""
        return self._body_b._rec()["a"] - self._body_a._rec()["a"] - self.reference_angle

    @property
    def joint_speed(self):
        return self._body_b.angular_velocity - self._body_a.angular_velocity

    @property
    def motor_speed(self):
        return float(self._rec()["motor_speed"])

    @motor_speed.setter
    def motor_speed(self, speed):
        self._wake()
        self._edit()["motor_speed"] = speed

    @property
    def limit_enabled(self):
        return self._flag(abi.J_LIMIT)

    @limit_enabled.setter
    def limit_enabled(self, on):
        if bool(on) != self.limit_enabled:
            self._wake()
            self._set_flag(abi.J_LIMIT, bool(on))
            self._edit()["impulse"][2] = 0.0

    @property
    def motor_enabled(self):
        return self._flag(abi.J_MOTOR)

    @motor_enabled.setter
    def motor_enabled(self, on):
        if bool(on) != self.motor_enabled:
            self._set_flag(abi.J_MOTOR, bool(on))
            self._wake()

    @property
    def lower_angle(self):
        return float(self._rec()["lower"])

    @lower_angle.setter
    def lower_angle(self, value):
        if self.lower_angle != value:
            self._wake()
            r = self._edit()
            r["impulse"][2] = 0.0
            r["lower"] = value

    @property
    def upper_angle(self):
        return float(self._rec()["upper"])

    @upper_angle.setter
    def upper_angle(self, value):
        if self.upper_angle != value:
            self._wake()
            r = self._edit()
            r["impulse"][2] = 0.0
            r["upper"] = value

    @property
    def max_motor_torque(self):
        return float(self._rec()["max_motor"])

    @max_motor_torque.setter
    def max_motor_torque(self, torque):
        self._wake()
        self._edit()["max_motor"] = torque

    def get_motor_torque(self, inv_dt):
        return inv_dt * float(self._rec()["motor_impulse"])

    def get_reaction_force(self, inv_dt):
        """revolute.py:206-208 slices the Vec3 impulse (`_impulse[:2]`), which
        Vec3.__getitem__ refuses (common.py:303-311): the reference raises
        IndexError here, and so does this getter."""
        raise IndexError("Index must be in (0,1,2)")


class PrismaticJoint(Joint):
    """joints/prismatic.py:32-513.  The axis is kept as given (in body_a's
    frame, not normalised), as the reference does."""

    _type = abi.JOINT_PRISMATIC

    def __init__(self, body_a, body_b, anchor=(0, 0), axis=(0, 1), lower_limit=0.0, upper_limit=0.0,
                 max_motor_force=0.0, max_motor_torque=0.0, motor_speed=0.0, reference_angle=None,
                 limit_enabled=False, motor_enabled=False, collide_connected=False, local_anchor_a=None,
                 local_anchor_b=None, local_x_axis=None):
        if body_a is None or body_b is None:
            raise ValueError("body_a and body_b must be set")
        Joint.__init__(self, body_a, body_b, collide_connected)
        self._set_anchors(anchor, anchor, local_anchor_a, local_anchor_b)
        r = self._pending
        r["ref_angle"] = float(reference_angle) if reference_angle is not None else body_b.angle - body_a.angle
        ax = local_x_axis if local_x_axis is not None else body_a.get_local_vector(axis)
        r["ax_x"], r["ax_y"] = float(ax[0]), float(ax[1])
        r["lower"], r["upper"] = float(lower_limit), float(upper_limit)
        r["max_motor"], r["motor_speed"] = float(max_motor_force), float(motor_speed)
        r["flags"] |= (abi.J_LIMIT if limit_enabled else 0) | (abi.J_MOTOR if motor_enabled else 0)

    def get_reaction_force(self, inv_dt):
        """inv_dt * (impulse.x * perp + (motor impulse + impulse.z) * axis), with
        the axis and perpendicular of the last step's set-up"""
        r = self._rec()
        ix, iz, mi = float(r["impulse"][0]), float(r["impulse"][2]), float(r["motor_impulse"])
        s = mi + iz
        px, py = ix * float(r["perp_x"]) + s * float(r["ux"]), ix * float(r["perp_y"]) + s * float(r["uy"])
        return _V(inv_dt * px, inv_dt * py)

    def get_reaction_torque(self, inv_dt):
        return inv_dt * float(self._rec()["impulse"][1])

    @property
    def local_x_axis(self):
        r = self._rec()
        return _V(r["ax_x"], r["ax_y"])

    @property
    def axis(self):
        return self._body_a.get_world_vector(self.local_x_axis)

    @property
    def reference_angle(self):
        return float(self._rec()["ref_angle"])

    @property
    def joint_translation(self):
        d = _sub(self.anchor_b, self.anchor_a)
        ax = self.axis
        return d[0] * ax[0] + d[1] * ax[1]

    @property
    def joint_speed(self):
        """prismatic.py:136-157"""
        ba, bb = self._body_a, self._body_b
        ca, cb = ba.world_center, bb.world_center
        ra = _rot(ba.angle, _sub(self.local_anchor_a, ba.local_center))
        rb = _rot(bb.angle, _sub(self.local_anchor_b, bb.local_center))
        p1 = (ca[0] + ra[0], ca[1] + ra[1])
        p2 = (cb[0] + rb[0], cb[1] + rb[1])
        d = _sub(p2, p1)
        axis = ba.get_world_vector(self.local_x_axis)
        va, vb = ba.linear_velocity, bb.linear_velocity
        wa, wb = ba.angular_velocity, bb.angular_velocity
        swa_axis = (-wa * axis[1], wa * axis[0])
        swb_rb = (-wb * rb[1], wb * rb[0])
        swa_ra = (-wa * ra[1], wa * ra[0])
        rel = ((vb[0] + swb_rb[0]) - va[0] - swa_ra[0], (vb[1] + swb_rb[1]) - va[1] - swa_ra[1])
        return (d[0] * swa_axis[0] + d[1] * swa_axis[1]) + (axis[0] * rel[0] + axis[1] * rel[1])

    @property
    def limit_enabled(self):
        return self._flag(abi.J_LIMIT)

    @limit_enabled.setter
    def limit_enabled(self, on):
        if bool(on) != self.limit_enabled:
            self._wake()
            self._set_flag(abi.J_LIMIT, bool(on))
            r = self._edit()
            r["impulse"][2] = r["impulse"][2] - r["impulse"][2]

    @property
    def lower_limit(self):
        return float(self._rec()["lower"])

    @lower_limit.setter
    def lower_limit(self, value):
        if self.lower_limit != value:
            self._wake()
            r = self._edit()
            r["impulse"][2] = r["impulse"][2] - r["impulse"][2]
            r["lower"] = value

    @property
    def upper_limit(self):
        return float(self._rec()["upper"])

    @upper_limit.setter
    def upper_limit(self, value):
        if self.upper_limit != value:
            self._wake()
            r = self._edit()
            r["impulse"][2] = r["impulse"][2] - r["impulse"][2]
            r["upper"] = value

    @property
    def motor_enabled(self):
        return self._flag(abi.J_MOTOR)

    @motor_enabled.setter
    def motor_enabled(self, on):
        if bool(on) != self.motor_enabled:
            self._set_flag(abi.J_MOTOR, bool(on))
            self._wake()

    @property
    def motor_speed(self):
        return float(self._rec()["motor_speed"])

    @motor_speed.setter
    def motor_speed(self, speed):
        self._wake()
        self._edit()["motor_speed"] = speed

    @property
    def max_motor_force(self):
        return float(self._rec()["max_motor"])

    @max_motor_force.setter
    def max_motor_force(self, force):
        self._wake()
        self._edit()["max_motor"] = force


class DistanceJoint(Joint):
    """joints/distance.py:33-311.  A length of LINEAR_SLOP or less raises."""

    _type = abi.JOINT_DISTANCE

    def __init__(self, body_a, body_b, anchor_a=(0, 0), anchor_b=(0, 0), frequency=0.0, damping_ratio=0.0, length=None,
                 collide_connected=False, local_anchor_a=None, local_anchor_b=None):
        if body_a is None or body_b is None:
            raise ValueError("body_a and body_b must be set")
        Joint.__init__(self, body_a, body_b, collide_connected)
        self._set_anchors(anchor_a, anchor_b, local_anchor_a, local_anchor_b)
        r = self._pending
        if length is not None:
            r["length"] = float(length)
        else:   # from the world anchors of the local anchors (distance.py:82-86)
            d = _sub(self.anchor_b, self.anchor_a)
            r["length"] = math.sqrt(d[0] * d[0] + d[1] * d[1])
        if r["length"] <= LINEAR_SLOP:
            raise ValueError("length must be > 0 and not a very small number")
        r["frequency"], r["damping_ratio"] = frequency, damping_ratio

    @property
    def length(self):
        return float(self._rec()["length"])

    @length.setter
    def length(self, value):
        self._edit()["length"] = value

    @property
    def frequency(self):
        return float(self._rec()["frequency"])

    @frequency.setter
    def frequency(self, value):
        self._edit()["frequency"] = value

    @property
    def damping_ratio(self):
        return float(self._rec()["damping_ratio"])

    @damping_ratio.setter
    def damping_ratio(self, value):
        self._edit()["damping_ratio"] = value

    def get_reaction_force(self, inv_dt):
        r = self._rec()
        s = inv_dt * float(r["impulse"][0])
        return _V(s * float(r["ux"]), s * float(r["uy"]))

    def get_reaction_torque(self, inv_dt):
        return 0.0


class WeldJoint(Joint):
    """joints/weld.py:33-257"""

    _type = abi.JOINT_WELD

    def __init__(self, body_a, body_b, anchor=None, reference_angle=None, local_anchor_a=None, local_anchor_b=None,
                 collide_connected=False):
        if body_a is None or body_b is None:
            raise ValueError("body_a and body_b must be set")
        Joint.__init__(self, body_a, body_b, collide_connected)
        if anchor is not None:
            self._set_anchors(anchor, anchor, None, None)
        else:
            self._set_anchors(None, None, local_anchor_a, local_anchor_b)
        r = self._pending
        r["ref_angle"] = float(reference_angle) if reference_angle is not None else body_b.angle - body_a.angle

    @property
    def reference_angle(self):
        return float(self._rec()["ref_angle"])


def _valid_float(v):
    """common.py is_valid_float: a finite number"""
    return isinstance(v, (int, float)) and math.isfinite(v)


class FrictionJoint(Joint):
    """joints/friction.py:30-233: translational and angular friction between
    two bodies.  The reference's velocity passes write the positions back
    where the velocities belong (friction.py:228-229), so the joint acts on
    the bodies only through the warm start of each set-up; the passes update
    the accumulated impulses."""

    _type = abi.JOINT_FRICTION

    def __init__(self, body_a, body_b, local_anchor_a=(0, 0), local_anchor_b=(0, 0), max_force=0.0, max_torque=0.0,
                 collide_connected=False):
        if body_a is None or body_b is None:
            raise ValueError("body_a and body_b must be set")
        Joint.__init__(self, body_a, body_b, collide_connected)
        self._set_anchors(None, None, local_anchor_a, local_anchor_b)
        r = self._pending
        r["max_force"], r["max_torque"] = max_force, max_torque

    def get_reaction_force(self, inv_dt):
        r = self._rec()
        return _V(inv_dt * float(r["impulse"][0]), inv_dt * float(r["impulse"][1]))

    def get_reaction_torque(self, inv_dt):
        return inv_dt * float(self._rec()["impulse"][2])

    @property
    def max_force(self):
        return float(self._rec()["max_force"])

    @max_force.setter
    def max_force(self, value):
        if not _valid_float(value) or value < 0.0:
            raise ValueError("Max force must be >= 0.0")
        self._edit()["max_force"] = value

    @property
    def max_torque(self):
        return float(self._rec()["max_torque"])

    @max_torque.setter
    def max_torque(self, value):
        if not _valid_float(value) or value < 0.0:
            raise ValueError("Max torque must be >= 0.0")
        self._edit()["max_torque"] = value


class RopeJoint(Joint):
    """joints/rope.py:32-248: a maximum distance between two anchors.  The
    reference's limit_state property reads an attribute it never sets
    (rope.py:93-95; the state is kept as _state) and raises AttributeError,
    as here."""

    _type = abi.JOINT_ROPE

    def __init__(self, body_a, body_b, local_anchor_a=(0, 0), local_anchor_b=(0, 0), max_length=0.0,
                 collide_connected=False):
        if body_a is None or body_b is None:
            raise ValueError("body_a and body_b must be set")
        Joint.__init__(self, body_a, body_b, collide_connected)
        self._set_anchors(None, None, local_anchor_a, local_anchor_b)
        self._pending["max_length"] = max_length

    def get_reaction_force(self, inv_dt):
        """(inv_dt * impulse) * _u, _u the unnormalised anchor difference of
        the last set-up (rope.py:140, 84-86)"""
        r = self._rec()
        s = inv_dt * float(r["impulse"][0])
        return _V(s * float(r["ux"]), s * float(r["uy"]))

    def get_reaction_torque(self, inv_dt):
        return 0.0

    @property
    def limit_state(self):
        raise AttributeError("'RopeJoint' object has no attribute '_limit_state'")

    @property
    def max_length(self):
        return float(self._rec()["max_length"])


class WheelJoint(Joint):
    """joints/wheel.py:32-417: translation along an axis fixed in body_a
    with a spring, rotation with a motor.  As in the reference, the
    spring_frequency and spring_damping_ratio properties read attributes the
    constructor never sets (wheel.py:184-199): reading one before setting it
    raises AttributeError, and setting one does not reach the solver, which
    runs the constructor's frequency and damping ratio."""

    _type = abi.JOINT_WHEEL

    def __init__(self, body_a, body_b, anchor=None, axis=None, frequency=2.0, damping_ratio=0.7, motor_enabled=False,
                 motor_speed=0.0, max_motor_torque=0.0, local_anchor_a=None, local_anchor_b=None, local_x_axis=None,
                 collide_connected=False):
        if body_a is None or body_b is None:
            raise ValueError("body_a and body_b must be set")
        Joint.__init__(self, body_a, body_b, collide_connected)
        self._set_anchors(anchor, anchor, local_anchor_a, local_anchor_b)
        r = self._pending
        ax = local_x_axis if local_x_axis is not None else body_a.get_local_vector(axis)
        r["ax_x"], r["ax_y"] = float(ax[0]), float(ax[1])
        r["frequency"], r["damping_ratio"] = float(frequency), float(damping_ratio)
        r["max_motor"], r["motor_speed"] = float(max_motor_torque), float(motor_speed)
        if motor_enabled:
            r["flags"] = int(r["flags"]) | abi.J_MOTOR

    def get_reaction_force(self, inv_dt):
        """inv_dt * (impulse * _ay + spring_impulse * _ax) of the last set-up"""
        r = self._rec()
        imp, si = float(r["impulse"][0]), float(r["spring_impulse"])
        return _V(inv_dt * (imp * float(r["perp_x"]) + si * float(r["sax_x"])),
                  inv_dt * (imp * float(r["perp_y"]) + si * float(r["sax_y"])))

    def get_reaction_torque(self, inv_dt):
        return inv_dt * float(self._rec()["motor_impulse"])

    @property
    def local_x_axis(self):
        r = self._rec()
        return _V(r["ax_x"], r["ax_y"])

    @property
    def joint_translation(self):
        d = _sub(self.anchor_b, self.anchor_a)
        axis = self._body_a.get_world_vector(self.local_x_axis)
        return d[0] * axis[0] + d[1] * axis[1]

    @property
    def joint_speed(self):
        """wheel.py:127-130: the bodies' angular velocity difference"""
        return self._body_b.angular_velocity - self._body_a.angular_velocity

    @property
    def motor_enabled(self):
        return self._flag(abi.J_MOTOR)

    @motor_enabled.setter
    def motor_enabled(self, on):
        if bool(on) != self.motor_enabled:
            self._wake()
            self._set_flag(abi.J_MOTOR, bool(on))

    @property
    def motor_speed(self):
        return float(self._rec()["motor_speed"])

    @motor_speed.setter
    def motor_speed(self, speed):
        self._wake()
        self._edit()["motor_speed"] = speed

    @property
    def max_motor_torque(self):
        return float(self._rec()["max_motor"])

    @max_motor_torque.setter
    def max_motor_torque(self, torque):
        self._wake()
        self._edit()["max_motor"] = torque

    def motor_torque(self, inv_dt):
        return inv_dt * float(self._rec()["motor_impulse"])

    @property
    def spring_frequency(self):
        try:
            return self.__dict__["_spring_frequency"]
        except KeyError:
            raise AttributeError("'WheelJoint' object has no attribute '_spring_frequency'") from None

    @spring_frequency.setter
    def spring_frequency(self, value):
        self.__dict__["_spring_frequency"] = value

    @property
    def spring_damping_ratio(self):
        try:
            return self.__dict__["_spring_damping_ratio"]
        except KeyError:
            raise AttributeError("'WheelJoint' object has no attribute '_spring_damping_ratio'") from None

    @spring_damping_ratio.setter
    def spring_damping_ratio(self, value):
        self.__dict__["_spring_damping_ratio"] = value


class PulleyJoint(Joint):
    """joints/pulley.py:32-320: two bodies hung from two ground anchors with
    length_a + ratio * length_b held at its initial value.  The reference's
    reaction force reads a direction it never sets (pulley.py:103-105, _u2
    stays the zero vector), so it is zero, as here."""

    _type = abi.JOINT_PULLEY

    def __init__(self, body_a, body_b, ground_anchor_a=(0, 0), ground_anchor_b=(0, 0), anchor_a=(0, 0),
                 anchor_b=(0, 0), ratio=1.0, length_a=None, length_b=None, collide_connected=False,
                 local_anchor_a=None, local_anchor_b=None):
        if body_a is None or body_b is None:
            raise ValueError("body_a and body_b must be set")
        Joint.__init__(self, body_a, body_b, collide_connected)
        if ratio == 0.0 or ratio < 2.220446049250313e-16:
            raise ValueError("Ratio must be positive, non-zero and not too small")
        self._set_anchors(anchor_a, anchor_b, local_anchor_a, local_anchor_b)
        r = self._pending
        r["ga_x"], r["ga_y"] = float(ground_anchor_a[0]), float(ground_anchor_a[1])
        r["gb_x"], r["gb_y"] = float(ground_anchor_b[0]), float(ground_anchor_b[1])
        if length_a is None:   # from the world anchor arguments (pulley.py:80-83)
            dx, dy = anchor_a[0] - r["ga_x"], anchor_a[1] - r["ga_y"]
            length_a = math.sqrt(dx * dx + dy * dy)
        if length_b is None:
            dx, dy = anchor_b[0] - r["gb_x"], anchor_b[1] - r["gb_y"]
            length_b = math.sqrt(dx * dx + dy * dy)
        self._length_a, self._length_b = length_a, length_b
        r["constant"] = length_a + ratio * length_b
        r["ratio"] = ratio

    def get_reaction_force(self, inv_dt):
        s = inv_dt * float(self._rec()["impulse"][0])
        return _V(s * 0.0, s * 0.0)

    def get_reaction_torque(self, inv_dt):
        return 0.0

    @property
    def ground_anchor_a(self):
        r = self._rec()
        return _V(r["ga_x"], r["ga_y"])

    @property
    def ground_anchor_b(self):
        r = self._rec()
        return _V(r["gb_x"], r["gb_y"])

    @property
    def length_a(self):
        d = _sub(self.anchor_a, self.ground_anchor_a)
        return math.sqrt(d[0] * d[0] + d[1] * d[1])

    @property
    def length_b(self):
        d = _sub(self.anchor_b, self.ground_anchor_b)
        return math.sqrt(d[0] * d[0] + d[1] * d[1])

    @property
    def ratio(self):
        return float(self._rec()["ratio"])


class MouseJoint(Joint):
    """joints/mouse.py:30-229: a point of one body pulled towards a world
    target by a soft constraint with a force limit.  The body is body_b;
    body_a is None, as in the reference (its record repeats body_b)."""

    _type = abi.JOINT_MOUSE

    def __init__(self, body, target=(0, 0), max_force=0.0, frequency=5.0, damping_ratio=0.7):
        if body is None:
            raise ValueError("body must be set")
        if not (_valid_float(target[0]) and _valid_float(target[1])):
            raise ValueError("Invalid target")
        if not _valid_float(max_force) or max_force < 0.0:
            raise ValueError("Invalid maximum force")
        if not _valid_float(frequency) or frequency < 0.0:
            raise ValueError("Invalid frequency")
        if not _valid_float(damping_ratio) or damping_ratio < 0.0:
            raise ValueError("Invalid damping ratio")
        Joint.__init__(self, None, body, False)
        r = self._pending
        r["target_x"], r["target_y"] = float(target[0]), float(target[1])
        lb = body.get_local_point(target)
        r["lb_x"], r["lb_y"] = float(lb[0]), float(lb[1])
        r["max_force"], r["frequency"], r["damping_ratio"] = max_force, frequency, damping_ratio

    def get_reaction_force(self, inv_dt):
        r = self._rec()
        return _V(inv_dt * float(r["impulse"][0]), inv_dt * float(r["impulse"][1]))

    def get_reaction_torque(self, inv_dt):
        return 0.0

    @property
    def target(self):
        r = self._rec()
        return _V(r["target_x"], r["target_y"])

    @target.setter
    def target(self, target):
        if not self._body_b.awake:
            self._body_b.awake = True
        r = self._edit()
        r["target_x"], r["target_y"] = float(target[0]), float(target[1])

    @property
    def max_force(self):
        return float(self._rec()["max_force"])

    @max_force.setter
    def max_force(self, value):
        self._edit()["max_force"] = value

    @property
    def frequency(self):
        return float(self._rec()["frequency"])

    @frequency.setter
    def frequency(self, value):
        self._edit()["frequency"] = value

    @property
    def damping_ratio(self):
        return float(self._rec()["damping_ratio"])

    @damping_ratio.setter
    def damping_ratio(self, value):
        self._edit()["damping_ratio"] = value


KINDS = {abi.JOINT_REVOLUTE: RevoluteJoint, abi.JOINT_PRISMATIC: PrismaticJoint, abi.JOINT_DISTANCE: DistanceJoint,
         abi.JOINT_WELD: WeldJoint, abi.JOINT_FRICTION: FrictionJoint, abi.JOINT_ROPE: RopeJoint,
         abi.JOINT_WHEEL: WheelJoint, abi.JOINT_PULLEY: PulleyJoint, abi.JOINT_MOUSE: MouseJoint}

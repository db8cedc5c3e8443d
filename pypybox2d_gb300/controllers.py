"""Controllers of the drop-in API (pypybox2d/controllers.py): force rules
that the world applies to their bodies at the start of every solve
(world.py:476-479).

The rules run inside the GPU step (``csrc/gb_controllers.cuh``): before each
step the World turns ``World.controllers`` into ``gb_controller`` records
(kind, parameters, the world-local indices of the controller's bodies in its
own order).  A parameter change reaches the device as a parameter upload
(``gb_batch_set_controllers``); a changed body list or controller list
rebuilds the device batch.  The base class ``Controller`` keeps the
reference's body bookkeeping; a subclass with a ``step`` of its own would
have to run Python in the middle of the device step and is refused when the
world steps.
"""
from __future__ import annotations

import numpy as np

from . import abi


def _vec(v):
    return (float(v[0]), float(v[1]))


class Controller:
    """controllers.py:24-78: a list of bodies a rule acts on."""

    def __init__(self, world, bodies=()):
        self._bodies = []
        self._world = world
        for body in bodies:
            self.add_body(body)

    @property
    def bodies(self):
        """The bodies affected by this controller"""
        return list(self._bodies)

    @property
    def world(self):
        """The world this controller acts in"""
        return self._world

    def step(self, timestep):
        """controllers.py:48-50: subclasses define the rule"""
        raise NotImplementedError

    def add_body(self, body):
        """controllers.py:52-63"""
        if body in self._bodies:
            raise ValueError("Body already in controller")
        elif not body:
            raise ValueError("Body unset")
        elif body._world != self._world:
            raise ValueError("Body not in same world")
        self._bodies.append(body)
        body._attached_to_controller(self)

    def remove_body(self, body):
        """controllers.py:65-74"""
        if not body:
            raise ValueError("Body unset")
        elif body not in self._bodies:
            raise ValueError("Body not in controller")
        self._bodies.remove(body)
        body._detached_from_controller(self)

    def clear(self):
        for body in list(self._bodies):
            self.remove_body(body)

    def _record(self, r):
        raise NotImplementedError(f"{type(self).__name__}: only BuoyancyController and GravityController run inside "
                                  "the GPU step")


class BuoyancyController(Controller):
    """controllers.py:80-222: buoyancy and drag of a fluid filling the half
    plane below ``offset`` along ``normal``."""

    def __init__(self, world, bodies=(), normal=(0, 1), offset=0, density=0, velocity=(0, 0), linear_drag=0,
                 angular_drag=0, use_density=False, gravity=None):
        Controller.__init__(self, world, bodies)
        self.normal = normal
        self.offset = offset
        self.density = density
        self.velocity = velocity
        self.linear_drag = linear_drag
        self.angular_drag = angular_drag
        self.use_density = use_density
        self.gravity = gravity

    normal = property(lambda self: self._normal, lambda self, v: setattr(self, "_normal", _vec(v)),
                      doc="The outer surface normal (not normalised)")
    offset = property(lambda self: self._offset, lambda self, v: setattr(self, "_offset", float(v)),
                      doc="The height of the fluid surface along the normal")
    density = property(lambda self: self._density, lambda self, v: setattr(self, "_density", float(v)),
                       doc="The fluid density")
    velocity = property(lambda self: self._velocity, lambda self, v: setattr(self, "_velocity", _vec(v)),
                        doc="Fluid velocity, for drag calculations")
    linear_drag = property(lambda self: self._linear_drag, lambda self, v: setattr(self, "_linear_drag", float(v)),
                           doc="Linear drag co-efficient")
    angular_drag = property(lambda self: self._angular_drag, lambda self, v: setattr(self, "_angular_drag", float(v)),
                            doc="Angular drag co-efficient")
    use_density = property(lambda self: self._use_density, lambda self, v: setattr(self, "_use_density", bool(v)),
                           doc="If true, the shapes' densities are used (pypybox2d's shapes carry none)")

    @property
    def gravity(self):
        """Gravity vector; None uses the world's gravity"""
        return self._gravity

    @gravity.setter
    def gravity(self, g):
        self._gravity = _vec(g) if g is not None else None

    def _record(self, r):
        if self._use_density:
            # controllers.py:189 reads Shape.density, which no pypybox2d shape
            # defines: the reference raises AttributeError in World.step
            raise AttributeError("use_density: the shapes have no 'density' attribute (controllers.py:189)")
        r["type"] = abi.CONTROLLER_BUOYANCY
        # `if not self._gravity` (controllers.py:177): None or a zero vector
        # takes the world's gravity
        own = self._gravity is not None and (self._gravity[0] != 0.0 or self._gravity[1] != 0.0)
        r["flags"] = abi.CTRL_OWN_GRAVITY if own else 0
        r["normal_x"], r["normal_y"] = self._normal
        r["offset"], r["density"] = self._offset, self._density
        r["velocity_x"], r["velocity_y"] = self._velocity
        r["linear_drag"], r["angular_drag"] = self._linear_drag, self._angular_drag
        if own:
            r["gravity_x"], r["gravity_y"] = self._gravity

    def step(self, timestep):
        """controllers.py:173-222, run by the device step (World.step)"""
        raise NotImplementedError("the buoyancy rule runs inside World.step")


class GravityController(Controller):
    """controllers.py:226-280: gravitation between every pair of its bodies."""

    def __init__(self, world, bodies=(), G=1.0, inv_sqr=True):
        Controller.__init__(self, world, bodies)
        self.G = G
        self.inv_sqr = inv_sqr

    G = property(lambda self: self._G, lambda self, v: setattr(self, "_G", float(v)),
                 doc="The strength of the gravitation force")
    inv_sqr = property(lambda self: self._inv_sqr, lambda self, v: setattr(self, "_inv_sqr", bool(v)),
                       doc="If True, gravity is proportional to 1/r^2, otherwise 1/r")

    def step(self, timestep):
        """controllers.py:263-280, run by the device step (World.step)"""
        raise NotImplementedError("the gravity rule runs inside World.step")

    def _record(self, r):
        r["type"] = abi.CONTROLLER_GRAVITY
        r["flags"] = abi.CTRL_INV_SQR if self._inv_sqr else 0
        r["G"] = self._G


def controller_records(world, controllers):
    """(gb_controller records, body lists) of a world's controllers, in
    World.controllers order.  A body no longer in the world (the reference's
    Body._detached_from_world skips every second controller of a destroyed
    body, body.py:342-344) is left out: it has no record on the device."""
    C = np.zeros(len(controllers), dtype=abi.CONTROLLER)
    bodies = []
    for k, c in enumerate(controllers):
        if type(c).step not in (BuoyancyController.step, GravityController.step):
            raise NotImplementedError(f"{type(c).__name__}.step is Python code; only the buoyancy and gravity rules "
                                      "run inside the GPU step")
        r = C[k]
        c._record(r)
        mine = [b._index for b in c._bodies if b._world is world]
        r["body_start"], r["body_count"] = len(bodies), len(mine)
        bodies.extend(mine)
    return C, np.array(bodies, dtype=np.int32)

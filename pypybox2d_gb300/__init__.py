"""pypybox2d_gb300 -- GB300 (sm_103a) implementation of pypybox2d's
World.step hot path behind the reference's World/Body/Fixture API."""

from .shapes import Circle, Edge, Loop, MassData, Polygon, Shape  # noqa: E402,F401
from .errors import (CapacityError, ContactOverflowError, EmptyFixtureError, LockedError, NonFiniteError,  # noqa: E402,F401
                     PhysicsError, StepError, WaitTimeoutError)
from .world import AABB, Body, Contact, ContactManager, EventContact, Fixture, Vec2, World, WorldBatch  # noqa: E402,F401
from . import joints  # noqa: E402,F401
from . import controllers  # noqa: E402,F401
from .controllers import BuoyancyController, Controller, GravityController  # noqa: E402,F401
from .joints import (DistanceJoint, FrictionJoint, Joint, MouseJoint, PrismaticJoint, PulleyJoint,  # noqa: E402,F401
                     RevoluteJoint, RopeJoint, WeldJoint, WheelJoint)

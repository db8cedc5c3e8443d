"""Host side of failure reporting (no GPU): the reference's exception
classes (pypybox2d/common.py:84-86), the mapping of per-world status words
(include/gb2d.h GB_ST_*) to StepError subclasses, and the argument checks of
body creation (body.py:49-63)."""
import math

import numpy as np
import pytest

import pypybox2d_gb300 as b2
from pypybox2d_gb300 import abi
from pypybox2d_gb300.errors import step_error


def test_exception_classes_follow_the_reference():
    assert issubclass(b2.LockedError, b2.PhysicsError)
    assert issubclass(b2.EmptyFixtureError, b2.PhysicsError)
    assert issubclass(b2.StepError, b2.PhysicsError)
    for cls in (b2.NonFiniteError, b2.ContactOverflowError, b2.WaitTimeoutError, b2.CapacityError):
        assert issubclass(cls, b2.StepError)
    assert not issubclass(b2.PhysicsError, RuntimeError)


@pytest.mark.parametrize("bits,cls", [
    (abi.ST_NONFINITE, b2.NonFiniteError),
    (abi.ST_CONTACT_OVERFLOW, b2.ContactOverflowError),
    (abi.ST_WAIT_TIMEOUT, b2.WaitTimeoutError),
    (abi.ST_ITER_LIMIT, b2.CapacityError),
    (abi.ST_PAIR_OVERFLOW, b2.CapacityError),
    (abi.ST_TOI_ISLAND_CAP, b2.CapacityError),
    (abi.ST_EVENT_OVERFLOW, b2.CapacityError),
    (abi.ST_CONTACT_OVERFLOW | abi.ST_NONFINITE, b2.NonFiniteError),   # the most severe bit names the class
])
def test_status_words_map_to_step_errors(bits, cls):
    status = np.array([0, bits, 0, bits], dtype=np.uint32)
    e = step_error(status)
    assert type(e) is cls
    assert e.worlds == [1, 3] and e.status == [bits, bits]
    assert f"{bits:#x}" in str(e)


def test_clean_status_is_no_error():
    assert step_error(np.zeros(5, dtype=np.uint32)) is None


@pytest.mark.parametrize("kw,msg", [
    (dict(position=(math.nan, 0.0)), "Invalid position"),
    (dict(linear_velocity=(0.0, math.nan)), "Invalid linear velocity"),
    (dict(angle=math.nan), "Invalid angle"),
    (dict(angular_velocity=math.nan), "Invalid angular velocity"),
    (dict(type=7), "Invalid body type"),
])
def test_create_body_rejects_what_the_reference_rejects(kw, msg):
    w = b2.World()
    kw = dict(kw)
    t = kw.pop("type", b2.Body.DYNAMIC)
    with pytest.raises(ValueError, match=msg):
        w.create_body(type=t, **kw)
    assert len(w.bodies) == 0


def test_create_body_checks_as_the_reference_does():
    w = b2.World()
    # only NaN is invalid (vec2module.c valid_float); infinities pass
    w.create_dynamic_body(position=(math.inf, 0.0))
    # body.py:59-62 read `not valid and > 0`, which no NaN satisfies: NaN damping passes
    w.create_dynamic_body(linear_damping=math.nan, angular_damping=math.nan)
    # check_args=False skips the checks
    w.create_dynamic_body(position=(math.nan, 0.0), check_args=False)
    assert len(w.bodies) == 3

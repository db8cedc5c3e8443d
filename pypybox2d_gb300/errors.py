"""Exceptions of the drop-in API.

``PhysicsError``, ``LockedError`` and ``EmptyFixtureError`` are the
reference's (pypybox2d/common.py:84-86).  ``StepError`` and its subclasses
are raised after a GPU step whose per-world status word (include/gb2d.h
``GB_ST_*``) reports a failure: the reference runs one CPython world and
either carries on (a NaN spreads, body.py:49-63 checks only the arguments of
new bodies) or grows its Python lists without bound; the device batch has
fixed capacities and bounded waits, and says so instead of failing silently.
"""
from __future__ import annotations

from . import abi


class PhysicsError(Exception):
    """common.py:84"""


class LockedError(PhysicsError):
    """A world was changed during a step (common.py:85)."""


class EmptyFixtureError(PhysicsError):
    """common.py:86"""


class StepError(PhysicsError):
    """A GPU step reported a failure.  ``worlds``: indices of the failing
    worlds; ``status``: their status words (GB_ST_* bits)."""

    def __init__(self, message, worlds=(), status=()):
        super().__init__(message)
        self.worlds = list(worlds)
        self.status = list(status)


class NonFiniteError(StepError):
    """A body's position, angle or velocity stopped being finite (GB_ST_NONFINITE)."""


class ContactOverflowError(StepError):
    """A world made more contacts than its device slots hold; the extra pairs
    were dropped (GB_ST_CONTACT_OVERFLOW)."""


class WaitTimeoutError(StepError):
    """An in-kernel wait for a bulk copy gave up; the world's solve ended early
    for that step (GB_ST_WAIT_TIMEOUT)."""


class CapacityError(StepError):
    """A bounded structure of the step ran out: solver chunk table or colours
    (GB_ST_ITER_LIMIT), a move buffer (GB_ST_PAIR_OVERFLOW), a TOI sub-island
    (GB_ST_TOI_ISLAND_CAP) or the event slots (GB_ST_EVENT_OVERFLOW)."""


_ORDER = (  # the class of the first bit found, most severe first
    (abi.ST_NONFINITE, NonFiniteError, "non-finite body state"),
    (abi.ST_CONTACT_OVERFLOW, ContactOverflowError, "contact slots exhausted"),
    (abi.ST_WAIT_TIMEOUT, WaitTimeoutError, "a bulk-copy wait gave up"),
    (abi.ST_ITER_LIMIT, CapacityError, "iteration or table limit reached"),
    (abi.ST_PAIR_OVERFLOW, CapacityError, "move buffer full"),
    (abi.ST_TOI_ISLAND_CAP, CapacityError, "TOI sub-island capacity reached"),
    (abi.ST_EVENT_OVERFLOW, CapacityError, "contact event slots exhausted"),
)


def step_error(status, world_ids=None):
    """The exception for an array of per-world status words (None when every
    word is zero)."""
    bad = [i for i, s in enumerate(status) if int(s)]
    if not bad:
        return None
    ids = [world_ids[i] for i in bad] if world_ids is not None else bad
    words = [int(status[i]) for i in bad]
    seen = 0
    for s in words:
        seen |= s
    for bit, cls, what in _ORDER:
        if seen & bit:
            return cls(f"GPU world step failed ({what}) in worlds {ids[:8]}: status bits {seen:#x}", ids, words)
    return StepError(f"GPU world step failed in worlds {ids[:8]}: status bits {seen:#x}", ids, words)

"""Failure detection on the GPU, with every failure made on the host.

* contact overflow: a world given fewer device contact slots
  (World(contact_capacity=...), gb_world_desc.contact_capacity) than its
  pairs need raises ContactOverflowError after the step;
* non-finite state: a NaN velocity set through the API (the reference's
  setter takes it, body.py) spreads into the position, which the step
  flags (GB_ST_NONFINITE) and World.step raises NonFiniteError;
* bounded waits: with the poll limit of the solver's bulk-copy waits set to
  0 (gb_batch_set_wait_polls) every such wait gives up at once; the kernel
  flags GB_ST_WAIT_TIMEOUT, waits for its copies still in flight and
  returns.  The context stays usable: after the status is cleared and the
  snapshot restored, the batch steps exactly as a twin that never failed;
* the autotuner discards trials whose steps raised a status bit.
No test faults, traps or hangs a GPU: the waits that give up are bounded
loops that return, and NaN arithmetic is ordinary arithmetic.
"""
import math

import numpy as np
import pytest

import pypybox2d_gb300 as b2
from pypybox2d_gb300 import abi, scenes

pytestmark = pytest.mark.gpu

DT = 1.0 / 60.0


def _pyramid(world, rows):
    ground = world.create_static_body(position=(0, -0.5))
    ground.create_polygon_fixture(box=(40, 0.5))
    x = [-7.0, 0.75]
    for i in range(rows):
        y = list(x)
        for _ in range(i, rows):
            b = world.create_dynamic_body(position=tuple(y))
            b.create_polygon_fixture(box=(0.5, 0.5), density=5.0, friction=0.6)
            y[0] += 1.125
        x[0] += 0.5625
        x[1] += 1.25


def test_contact_overflow_raises():
    w = b2.World(contact_capacity=64)
    _pyramid(w, 12)                                  # 78 boxes: more than 64 fat-box pairs
    with pytest.raises(b2.ContactOverflowError) as e:
        w.step(DT, 8, 3)
    assert e.value.worlds == [0] and e.value.status[0] & abi.ST_CONTACT_OVERFLOW
    assert isinstance(e.value, b2.PhysicsError)


def test_default_capacity_does_not_overflow():
    w = b2.World()
    _pyramid(w, 12)
    for _ in range(5):
        w.step(DT, 8, 3)


def test_nan_velocity_raises_non_finite():
    w = b2.World()
    _pyramid(w, 3)
    for _ in range(3):
        w.step(DT, 8, 3)
    w.bodies[2].linear_velocity = (math.nan, 0.0)
    with pytest.raises(b2.NonFiniteError):
        w.step(DT, 8, 3)


def test_wait_timeout_flags_and_the_context_stays_usable():
    from pypybox2d_gb300.gpu import GpuBatch
    W, B, F, M = scenes.pyramid_batch(8, rows=12, jitter=0.01, seed=3)
    ref = GpuBatch(W, B, F, precision="f32", moves=M)
    g = GpuBatch(W, B, F, precision="f32", moves=M)
    for x in (ref, g):
        x.set_launch_config(3, 64, 2, 512)           # constraint chunks stream through 2 shared-memory buffers
        x.step(DT, 8, 3, 40, launch_mode=0)          # landed: every world has constraints to stream
    snap = g.snapshot()
    g.set_wait_polls(0)                              # every chunk wait gives up at once
    g.step(DT, 8, 3, 2, launch_mode=0)
    st = g.status()
    assert (st & abi.ST_WAIT_TIMEOUT).all(), st
    assert not (st & ~np.uint32(abi.ST_WAIT_TIMEOUT)).any(), st
    e = b2.errors.step_error(st)
    assert isinstance(e, b2.WaitTimeoutError) and e.worlds == list(range(8))
    # back to the default limit: restored state, cleared status, same steps as the twin
    g.set_wait_polls(1 << 18)
    g.clear_status()
    g.restore(snap)
    for _ in range(2):
        ref.step(DT, 8, 3, 5, launch_mode=0)
        g.step(DT, 8, 3, 5, launch_mode=0)
        assert g.bodies().tobytes() == ref.bodies().tobytes()
    assert not g.status().any()


def test_autotuner_discards_trials_that_raise_status_bits():
    from pypybox2d_gb300.gpu import GpuBatch
    W, B, F, M = scenes.pyramid_batch(16, rows=10, jitter=0.01, seed=4)
    g = GpuBatch(W, B, F, precision="f32", moves=M)
    g.step(DT, 8, 3, 40, launch_mode=3, block_threads=64)   # landed: the solver has constraints
    g.set_wait_polls(0)
    best, trials = g.autotune(DT, 8, 3, steps_per_trial=2)
    chunked = [t for t in trials if t["launch_mode"] == 3 and t["pipe_bufs"] > 0]
    assert chunked and all(t["ms_per_step"] == -2.0 for t in chunked), chunked
    assert best["ms_per_step"] >= 0.0 and not (best["launch_mode"] == 3 and best["pipe_bufs"] > 0)
    assert not g.status().any()                      # the tuner puts the saved state back

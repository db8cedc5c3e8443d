"""gb_batch_step_static_scratch against gb_batch_step.

The static-scratch entry point runs the same step kernels with their
per-step scratch in one static device array instead of the batch arena, so
two twin batches -- one stepped through each entry point -- must hold the
same doubles after every call.  Tolerance: none (bit-exact) in both
precisions, since the kernels, launch sequence and reduction orders are the
same and only the scratch addresses differ.

Covered: the monolithic and phased launches; launch_mode 0 after
gb_batch_set_launch_config (the batch's configuration, as gb_batch_step
takes it); a batch whose solver runs as a wide launch on the caller's stream
beside a narrow one on the side stream; a world of 16384+ bodies run as a
cooperative grid, whose grid reductions use the arena next to the static
arrays (its contact capacity is set so its scratch fits the 32 MiB array; at
the default 10 slots per fixture such a world needs more and is refused, as
the oversize test shows for a large batch); and the option bits the entry
point refuses.

The file is named to be collected last; it also passes on its own.
"""
import ctypes
import os

import numpy as np
import pytest

from pypybox2d_gb300 import abi, scenes

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CALLS = 2          # calls in a row through each entry point
STEPS_PER_CALL = 25


def _golden(scene):
    d = np.load(os.path.join(GOLDEN, scene + ".npz"))
    return d["init_world"], d["init_bodies"], d["init_fixtures"], float(d["dt"][0]), tuple(int(x) for x in d["iters"])


def _same(a, b, what):
    for name in a.dtype.names:
        if name.startswith("_pad"):
            continue
        x, y = a[name], b[name]
        bad = ~((x == y) | ((x != x) & (y != y))) if x.dtype.kind == "f" else (x != y)
        assert not bad.any(), f"{what}.{name} differs at {np.argwhere(bad)[0]}"


def _twins(W, B, F, precision, moves=None):
    from pypybox2d_gb300.gpu import GpuBatch
    return GpuBatch(W, B, F, precision=precision, moves=moves), GpuBatch(W, B, F, precision=precision, moves=moves)


@pytest.mark.parametrize("mode", [1, 3], ids=["monolithic", "phased"])
@pytest.mark.parametrize("scene", ["bullets", "mixed", "sleep"])
def test_static_scratch_matches_arena_f64(scene, mode):
    W, B, F, dt, (vi, pi) = _golden(scene)
    ref, st = _twins(W, B, F, "f64")
    for call in range(CALLS):
        ref.step(dt, vi, pi, STEPS_PER_CALL, launch_mode=mode)
        st.step_static_scratch(dt, vi, pi, STEPS_PER_CALL, launch_mode=mode)
        _same(st.bodies(), ref.bodies(), f"{scene} call {call} bodies")
        _same(st.contacts(0), ref.contacts(0), f"{scene} call {call} contacts")
        assert np.array_equal(st.proxies(), ref.proxies())
    assert int(st.status()[0]) == 0


def test_static_scratch_matches_arena_f32_batch():
    W, B, F, M = scenes.pyramid_batch(24, rows=10, jitter=0.01)
    ref, st = _twins(W, B, F, "f32", moves=M)
    for call in range(CALLS):
        ref.step(1 / 60, 8, 3, STEPS_PER_CALL, launch_mode=3, block_threads=64)
        st.step_static_scratch(1 / 60, 8, 3, STEPS_PER_CALL, launch_mode=3, block_threads=64)
        _same(st.bodies(), ref.bodies(), f"f32 batch call {call} bodies")
        assert np.array_equal(st.contact_counts(), ref.contact_counts())


def test_batches_take_turns_on_the_shared_scratch():
    """Sequential calls of different batches on one stream share the array."""
    runs = []
    for scene in ("bullets", "mixed"):
        W, B, F, dt, iters = _golden(scene)
        runs.append((scene, dt, iters, *_twins(W, B, F, "f64")))
    for call in range(CALLS):
        for scene, dt, (vi, pi), ref, st in runs:
            ref.step(dt, vi, pi, 10, launch_mode=3)
            st.step_static_scratch(dt, vi, pi, 10, launch_mode=3)
        for scene, dt, iters, ref, st in runs:
            _same(st.bodies(), ref.bodies(), f"{scene} turn {call}")


def test_oversized_batch_is_rejected_before_any_launch():
    from pypybox2d_gb300.gpu import GpuBatch
    W, B, F, M = scenes.pyramid_batch(512, rows=20, jitter=0.0)
    g = GpuBatch(W, B, F, precision="f64", moves=M)
    before = g.bodies()
    o = abi.StepOpts(1 / 60, 8, 3, 1, 3, 0, 0)
    rc = g.lib.gb_batch_step_static_scratch(g.h, ctypes.byref(o), None)
    assert rc == abi.E_SCRATCH
    msg = g.lib.gb_last_error().decode()
    assert "static scratch holds" in msg and str(abi.STATIC_SCRATCH_BYTES) in msg
    _same(g.bodies(), before, "rejected call")
    assert int(g.arena_bytes()) > 0


@pytest.mark.parametrize("cfg", [(2, 64, 0, 512), (3, 64, 0, 512), (3, 32, 2, 256)],
                         ids=["warp-per-world", "phased-64", "phased-32-chunked"])
def test_static_scratch_follows_the_launch_config(cfg):
    """launch_mode 0 means the batch's launch configuration in both entry points."""
    W, B, F, M = scenes.uneven_batch(6, seed=3, counts=[40, 300, 25, 120, 60, 15])
    ref, st = _twins(W, B, F, "f64", moves=M)
    for g in (ref, st):
        g.set_launch_config(*cfg)
    for call in range(CALLS):
        ref.step(1 / 60, 8, 3, 10, launch_mode=0)
        st.step_static_scratch(1 / 60, 8, 3, 10, launch_mode=0)
        _same(st.bodies(), ref.bodies(), f"config {cfg} call {call} bodies")
        for w in range(len(W)):
            _same(st.contacts(w), ref.contacts(w), f"config {cfg} call {call} world {w} contacts")
    assert not st.status().any()


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_static_scratch_with_the_side_stream_solver(precision):
    """Worlds of 512+ bodies solve in the wide launch on the caller's stream,
    the rest beside them on the batch's side stream."""
    W, B, F, M = scenes.uneven_batch(5, seed=11, counts=[700, 560, 120, 60, 20])
    ref, st = _twins(W, B, F, precision, moves=M)
    for g in (ref, st):
        g.set_launch_config(3, 64, 0, 512)
    for call in range(CALLS):
        ref.step(1 / 60, 8, 3, 10, launch_mode=0)
        st.step_static_scratch(1 / 60, 8, 3, 10, launch_mode=0)
        _same(st.bodies(), ref.bodies(), f"{precision} side stream call {call} bodies")
        for w in range(len(W)):
            _same(st.contacts(w), ref.contacts(w), f"{precision} side stream call {call} world {w} contacts")
    assert not st.status().any()


def test_static_scratch_with_a_cooperative_grid_world():
    """A world of 16400 bodies runs every per-world phase as one cooperative
    grid; 40000 contact slots keep its step scratch inside the static array."""
    W, B, F, M = scenes.large_world(0, n=16400)
    W = W.copy()
    W["contact_capacity"] = 40000
    ref, st = _twins(W, B, F, "f64", moves=M)
    for call in range(CALLS):
        ref.step(1 / 60, 8, 3, STEPS_PER_CALL, launch_mode=3)
        st.step_static_scratch(1 / 60, 8, 3, STEPS_PER_CALL, launch_mode=3)
        _same(st.bodies(), ref.bodies(), f"grid world call {call} bodies")
        _same(st.contacts(0), ref.contacts(0), f"grid world call {call} contacts")
    assert int(st.status()[0]) == 0


@pytest.mark.parametrize("bit", [abi.OPT_EVENTS, abi.OPT_KERNEL_TIMES], ids=["events", "kernel-times"])
def test_static_scratch_refuses_recording_options(bit):
    from pypybox2d_gb300.gpu import GpuBatch
    W, B, F, dt, (vi, pi) = _golden("mixed")
    g = GpuBatch(W, B, F, precision="f64")
    before = g.bodies()
    o = abi.StepOpts(dt, vi, pi, 1, 3, 0, bit)
    rc = g.lib.gb_batch_step_static_scratch(g.h, ctypes.byref(o), None)
    assert rc == abi.E_UNSUPPORTED
    assert "gb_batch_step" in g.lib.gb_last_error().decode()
    _same(g.bodies(), before, "refused call")

"""Checkpoint and resume of a device batch (gb_batch_snapshot / gb_batch_restore).

A snapshot holds the batch's whole device state, so steps run after a
restore must reproduce, bit for bit, the steps run after the snapshot was
taken (the step is deterministic).  Host and device snapshot buffers both
work; a snapshot restores only into a batch of the same layout.
"""
import ctypes
import os

import numpy as np
import pytest

from pypybox2d_gb300 import abi, scenes

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _golden(scene):
    d = np.load(os.path.join(GOLDEN, scene + ".npz"))
    return d["init_world"], d["init_bodies"], d["init_fixtures"], float(d["dt"][0]), tuple(int(x) for x in d["iters"])


def _state(g):
    return g.bodies(), g.proxies(), [g.contacts(w) for w in range(g.n_worlds)], g.status(), g.contact_counts()


def _equal(a, b):
    ba, pa, ca, sa, na = a
    bb, pb, cb, sb, nb = b
    assert ba.tobytes() == bb.tobytes()
    assert np.array_equal(pa, pb)
    assert all(x.tobytes() == y.tobytes() for x, y in zip(ca, cb))
    assert np.array_equal(sa, sb) and np.array_equal(na, nb)


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_restore_replays_the_same_steps_host_snapshot(precision):
    from pypybox2d_gb300.gpu import GpuBatch
    W, B, F, dt, (vi, pi) = _golden("bullets")
    g = GpuBatch(W, B, F, precision=precision)
    g.step(dt, vi, pi, 7, launch_mode=3)
    snap = g.snapshot()
    assert snap.nbytes == g.snapshot_bytes() == g.arena_bytes() + 64
    g.step(dt, vi, pi, 30, launch_mode=3)
    first = _state(g)
    g.restore(snap)
    g.step(dt, vi, pi, 30, launch_mode=3)
    _equal(_state(g), first)


def test_restore_from_a_device_buffer_after_a_batch_of_worlds():
    import torch
    from pypybox2d_gb300.gpu import GpuBatch
    W, B, F, M = scenes.uneven_batch(12, seed=5, counts=[30, 600, 45, 120, 10, 80, 300, 20, 60, 15, 90, 40])
    g = GpuBatch(W, B, F, precision="f32", moves=M)
    g.step(1 / 60, 8, 3, 12, launch_mode=3, block_threads=64)
    buf = torch.empty(g.snapshot_bytes(), dtype=torch.uint8, device="cuda")
    g.snapshot(buf.data_ptr(), buf.numel())
    g.step(1 / 60, 8, 3, 20, launch_mode=3, block_threads=64)
    first = _state(g)
    g.restore(buf.data_ptr(), buf.numel())
    g.step(1 / 60, 8, 3, 20, launch_mode=3, block_threads=64)
    _equal(_state(g), first)


def test_snapshot_of_another_layout_is_refused():
    from pypybox2d_gb300.gpu import GpuBatch
    W, B, F, dt, (vi, pi) = _golden("mixed")
    a = GpuBatch(W, B, F, precision="f64")
    b = GpuBatch(W, B, F, precision="f32")
    snap = a.snapshot()
    with pytest.raises(abi.GB2DError, match="another layout|too small"):
        b.restore(snap)
    rc = a.lib.gb_batch_snapshot(a.h, snap.ctypes.data, 16, None)
    assert rc == abi.E_ARG
    rc = a.lib.gb_batch_restore(a.h, snap.ctypes.data, ctypes.c_uint64(snap.nbytes - 1), None)
    assert rc == abi.E_ARG

"""Body.active through the World API (body.py:826-872), pinned against the
reference (tests/golden/api_active.py, api_active.npz): an active body made
inactive (its contact destroyed, nothing collides with it, it stops moving),
a body created inactive and activated later (its proxy made at its
transform and paired by the next step).  Bodies, contacts and the fat boxes
of every fixture that has a proxy are the reference's bit for bit when the
World steps on the CPU restatement; on the float64 GPU step (every island
holds one contact, so the GPU's solver order is the reference's) the
discrete state is the reference's and positions are within GPU_TOL_M: the
GPU's portable sine/cosine differs from libm in the last bit of some
rotations (tests/test_sincos_gap.py).
"""
import os
import sys

import numpy as np
import pytest

import pypybox2d_gb300 as b2

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)
import api_active  # noqa: E402
from test_world_joints import oracle_world_class, same, used  # noqa: E402

GPU_TOL_M = 1e-9


def _run(world_class):
    snaps = {}

    class Recorder(world_class):
        pass

    def snap(label, world):
        world._materialise()
        snaps[label] = (world._B.copy(), world._F["aabb"].copy(), world._C.copy())

    orig = b2.World
    b2.World = Recorder
    try:
        api_active.script(b2, snap)
    finally:
        b2.World = orig
    return snaps


def _check(snaps):
    d = np.load(os.path.join(GOLDEN, "api_active.npz"))
    for label in api_active.SNAPS:
        B, A, C = snaps[label]
        same(B, d[f"{label}_bodies"], f"{label} bodies")
        want = d[f"{label}_aabb"]
        has = ~np.isnan(want[:, 0])            # fixtures with a proxy
        assert np.array_equal(A[has], want[has]), f"{label} fat AABBs"
        same(used(C), used(d[f"{label}_contacts"]), f"{label} contacts")


def test_active_session_matches_reference_bitwise():
    _check(_run(oracle_world_class()))


def test_reactivating_a_deactivated_body_raises_as_the_reference():
    w = b2.World()
    body = w.create_dynamic_body(position=(0, 1))
    body.create_circle_fixture(0.5, density=1.0)
    body.active = False
    assert not body.active
    with pytest.raises(AssertionError):
        body.active = True
    empty = w.create_dynamic_body(position=(3, 1))
    empty.active = False
    empty.active = True                            # no fixtures, no stale proxies
    assert empty.active


@pytest.mark.gpu
def test_active_session_on_the_gpu_follows_the_reference():
    d = np.load(os.path.join(GOLDEN, "api_active.npz"))
    snaps = _run(b2.World)
    for label in api_active.SNAPS:
        B, A, C = snaps[label]
        rb, rc = d[f"{label}_bodies"], d[f"{label}_contacts"]
        assert np.array_equal(B["flags"], rb["flags"]), label
        err = float(np.hypot(B["cx"] - rb["cx"], B["cy"] - rb["cy"]).max())
        assert err <= GPU_TOL_M, f"{label}: {err:.2e} m"
        for f in ("fixture_a", "fixture_b", "flags", "m_point_count", "m_type"):
            assert np.array_equal(C[f], rc[f]), f"{label} contacts.{f}"

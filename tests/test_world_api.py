"""The World / Body / Fixture API (pypybox2d_gb300.World) against the
reference: tests/golden/api_script.py runs the same API session on both
(the reference's snapshots are in tests/golden/api_script.npz).  The
construction-time state must be the reference's bit for bit on the CPU;
with the float64 GPU step every snapshot -- bodies, fat AABBs, contacts with
manifolds and impulses -- must be too."""
import os
import sys
import types

import numpy as np
import pytest

import pypybox2d_gb300 as b2
from pypybox2d_gb300 import abi

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)
import api_script  # noqa: E402


def same(a, b, what):
    for n in b.dtype.names:
        if n.startswith("_pad"):
            continue
        x, y = a[n], b[n]
        bad = ~((x == y) | ((x != x) & (y != y))) if x.dtype.kind == "f" else (x != y)
        assert not bad.any(), f"{what}.{n} differs at {np.argwhere(bad)[0]}"


def used(c):
    c = c.copy()
    for j in range(2):
        unused = c["m_point_count"] <= j
        for f in ("p_lx", "p_ly", "p_ni", "p_ti", "p_id"):
            c[f][unused, j] = 0
    return c


class Stop(Exception):
    pass


def test_construction_matches_reference():
    d = np.load(os.path.join(GOLDEN, "api_script.npz"))

    def snap(label, world):
        world._materialise()
        same(world._B, d[f"{label}_bodies"], label)
        assert np.array_equal(world._F["aabb"], d[f"{label}_aabb"])
        raise Stop

    with pytest.raises(Stop):
        api_script.script(b2, snap)


def test_unsupported_features_raise():
    with pytest.raises(NotImplementedError):
        b2.World(sub_stepping=True)
    w = b2.World((0, -10), True)
    w.contact_manager.pre_solve = lambda contact, old_manifold: None
    w.create_dynamic_body(position=(0, 1)).create_circle_fixture(0.5, density=1.0)
    with pytest.raises(NotImplementedError):      # pre_solve would run inside the step
        w.step(1 / 60, 8, 3)


def test_pre_step_edits_stay_on_the_host():
    w = b2.World((0, -10), True)
    body = w.create_dynamic_body(position=(1, 2))
    body.create_circle_fixture(0.5, density=2.0)
    body.linear_velocity = (1.5, 0.0)
    body.apply_force_to_center((0.0, 3.0))
    assert body.linear_velocity == (1.5, 0.0)
    assert body.force == (0.0, 3.0)
    assert body.awake
    body.awake = False
    assert body.linear_velocity == (0.0, 0.0) and body.force == (0.0, 0.0)
    assert w._gpu is None


def oracle_world_class(libm):
    """pypybox2d_gb300.World whose batch is the CPU restatement."""
    import oracle_lib

    class OracleBackedWorld(b2.World):
        def _make_batch(self, W, B, F, C, M, J=None, CT=None, CB=None):
            return oracle_lib.OracleBatch(W, B, F, C, M, libm=libm, joints=J, controllers=CT, controller_bodies=CB)

    return OracleBackedWorld


def run_session(world_class):
    """The API session with snapshots (bodies, fat AABBs, contacts)."""
    snaps = {}

    def snap(label, world):
        world._materialise()
        snaps[label] = (world._B.copy(), world._F["aabb"].copy(), world._C.copy())

    world = api_script.script(types.SimpleNamespace(World=world_class), snap)
    return world, snaps


def test_api_session_host_logic_matches_reference():
    """The World's host side (record edits for velocities, forces, impulses,
    transforms, new bodies and fixtures, destroyed bodies, gravity) driving
    the libm build of the restatement reproduces the reference's session."""
    d = np.load(os.path.join(GOLDEN, "api_script.npz"))
    world, snaps = run_session(oracle_world_class(libm=True))
    assert tuple(snaps) == api_script.SNAPS
    for label, (B, aabb, C) in snaps.items():
        same(B, d[f"{label}_bodies"], f"{label} bodies")
        assert np.array_equal(aabb, d[f"{label}_aabb"]), f"{label} fat AABBs"
        same(used(C), used(d[f"{label}_contacts"]), f"{label} contacts")
    assert world.body_count == 5


@pytest.mark.gpu
def test_api_session_on_gpu_matches_oracle_bit_for_bit():
    """The same session through the float64 GPU step equals the session
    driven by the restatement (portable sine/cosine build, the GPU's own)."""
    _, want = run_session(oracle_world_class(libm=False))
    world, got = run_session(b2.World)
    for label in api_script.SNAPS:
        (B, aabb, C), (B2, aabb2, C2) = got[label], want[label]
        same(B, B2, f"{label} bodies")
        assert np.array_equal(aabb, aabb2), f"{label} fat AABBs"
        same(used(C), used(C2), f"{label} contacts")
    assert all(isinstance(c.touching, bool) for c in world.contacts)


@pytest.mark.gpu
def test_listener_events_match_reference():
    """begin/end/post-solve events of the API session, replayed after each
    GPU step, against the reference's listener calls: the begin and end
    events in the same order at the same steps; per step the same
    post-solve reports, impulses within 1e-9 relative (the reference takes
    cos/sin from libm, the GPU from its portable sincos)."""
    d = np.load(os.path.join(GOLDEN, "api_script.npz"))
    want = d["events"]
    log = []
    api_script.script(b2, lambda label, world: None, log=log)
    kinds = {"begin": 1, "end": 2, "post": 3}
    got = [(kinds[k], s, ba, fa, bb, fb, imp) for (k, s, ba, fa, bb, fb, imp) in log]
    ge = [g[:6] for g in got if g[0] != 3]
    we = [tuple(int(x) for x in (r["kind"], r["step"], r["ba"], r["fa"], r["bb"], r["fb"])) for r in want if r["kind"] != 3]
    assert ge == we
    gp = sorted((g[1], g[2:6], g[6]) for g in got if g[0] == 3)
    wp = sorted((int(r["step"]), tuple(int(x) for x in (r["ba"], r["fa"], r["bb"], r["fb"])),
                 tuple(float(x) for x in r["imp"][:2 * int(r["n"])])) for r in want if r["kind"] == 3)
    assert [(a, b) for a, b, _ in gp] == [(a, b) for a, b, _ in wp]
    for (_, _, x), (_, _, y) in zip(gp, wp):
        np.testing.assert_allclose(x, y, rtol=1e-9, atol=1e-12)


def test_pre_solve_listener_raises_on_step():
    w = b2.World()
    w.contact_manager.pre_solve = lambda c, m: None
    with pytest.raises(NotImplementedError):
        w.step(1 / 60, 8, 3)

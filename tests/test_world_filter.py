"""Custom contact filters (World.contact_filter, world.py:123-136) through
the World API, pinned against the reference.

The filter is asked by the reference for a new pair (contact_manager.py:145)
and for a contact flagged for filtering (contact_manager.py:202); here its
answers for every pair of fixtures reach the step as a table
(gb_batch_set_pair_filter on the device, or_set_pair_filter in the CPU
restatement).  The scripted session tests/golden/api_filter.py (two filters
in turn, then no filter at all) gives the reference's bodies and contacts bit for bit on the CPU
restatement; on the float64 GPU step the discrete state (awake flags,
contact pairs in list order) is the reference's at every snapshot and
positions stay within GPU_TOL_M through s41.  After the second filter makes
the overlapping teams collide, the pile separates violently and the
portable sine and cosine's last-bit differences grow (measured: 6.5e-2 m
at s80, 0.55 m at s120) while every contact decision stays the reference's.
"""
import os
import sys

import numpy as np
import pytest

import pypybox2d_gb300 as b2

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)
import api_filter  # noqa: E402
from test_world_joints import oracle_world_class, same, used  # noqa: E402

GPU_TOL_M = 1e-2
BOUNDED = ("s0", "s1", "s40", "s41")


def _run(world_class, script=api_filter.script):
    snaps = {}

    def snap(label, world):
        world._materialise()
        snaps[label] = (world._B.copy(), world._C.copy())

    orig = b2.World
    b2.World = world_class
    try:
        script(b2, snap)
    finally:
        b2.World = orig
    return snaps


def test_filter_session_matches_reference_bitwise():
    d = np.load(os.path.join(GOLDEN, "api_filter.npz"))
    snaps = _run(oracle_world_class())
    for label in api_filter.SNAPS:
        B, C = snaps[label]
        same(B, d[f"{label}_bodies"], f"{label} bodies")
        same(used(C), used(d[f"{label}_contacts"]), f"{label} contacts")


def test_filter_decides_the_outcome():
    """The same session with the default rule throughout ends elsewhere: the
    filters are what the goldens pin."""
    d = np.load(os.path.join(GOLDEN, "api_filter.npz"))

    def no_custom(b2_, snap):
        class Plain(b2_.World):
            @property
            def contact_filter(self):
                return b2_.World.contact_filter.fget(self)

            @contact_filter.setter
            def contact_filter(self, fcn):
                pass
        orig = b2_.World
        b2_.World = Plain
        try:
            return api_filter.script(b2_, snap)
        finally:
            b2_.World = orig

    snaps = _run(oracle_world_class(), script=no_custom)
    B, _ = snaps["s40"]
    rb = d["s40_bodies"]
    assert float(np.abs(B["cy"] - rb["cy"]).max()) > 0.1


def test_contact_filter_property():
    w = b2.World()
    assert w.contact_filter is b2.World.default_contact_filter
    w.contact_filter = api_filter.same_team
    assert w.contact_filter is api_filter.same_team
    w.contact_filter = None                      # the reference's "no filtering"
    assert w.contact_filter is None
    w.contact_filter = w.default_contact_filter
    assert w.contact_filter is b2.World.default_contact_filter
    with pytest.raises(TypeError):
        w.contact_filter = 3
    w2 = b2.World(contact_filter=api_filter.heavy_ghosts)
    assert w2.contact_filter is api_filter.heavy_ghosts


@pytest.mark.gpu
def test_filter_session_on_the_gpu_follows_the_reference():
    d = np.load(os.path.join(GOLDEN, "api_filter.npz"))
    snaps = _run(b2.World)
    worst = 0.0
    for label in api_filter.SNAPS:
        B, C = snaps[label]
        rb = d[f"{label}_bodies"]
        err = float(np.hypot(B["cx"] - rb["cx"], B["cy"] - rb["cy"]).max())
        if label in BOUNDED:
            worst = max(worst, err)
        assert np.array_equal(B["flags"], rb["flags"]), label
        rc = d[f"{label}_contacts"]
        assert np.array_equal(C["fixture_a"], rc["fixture_a"]) and np.array_equal(C["fixture_b"], rc["fixture_b"]), label
        print(f"{label}: largest position difference {err:.2e} m")
    assert worst < GPU_TOL_M


@pytest.mark.gpu
def test_filter_in_a_world_batch():
    """A WorldBatch of the filter session's world and a plain world: the
    filtered world follows its lone twin bit for bit."""
    import make_golden
    worlds, twins = [], []
    class Stop(Exception):
        pass

    for target in (worlds, twins):
        def snap(label, world, target=target):   # the session's world at its first snapshot
            target.append(world)
            raise Stop

        try:
            api_filter.script(b2, snap)
        except Stop:
            pass
        target.append(make_golden.scene_gravity(b2))
    batch = b2.WorldBatch(worlds)
    batch.step(api_filter.DT, api_filter.VEL_ITERS, api_filter.POS_ITERS, n_steps=30)
    for w in twins:
        for _ in range(30):
            w.step(api_filter.DT, api_filter.VEL_ITERS, api_filter.POS_ITERS)
    for a, t in zip(worlds, twins):
        a._materialise()
        t._materialise()
        same(a._B, t._B, "batch world bodies")
        same(used(a._C), used(t._C), "batch world contacts")
    batch.close()

"""Pin the CPU restatement (oracle/) against the reference itself.

The golden vectors under tests/golden/ were produced by running pypybox2d's
World.step in CPython (tests/golden/make_golden.py).  The libm build of the
restatement must reproduce every recorded double, flag, feature id and the
depth-first solver order bit for bit, over hundreds of steps of chaotic
stacking -- any deviation in operation order would grow and show.
"""
import glob
import os

import numpy as np
import pytest

import oracle_lib
from pypybox2d_gb300 import abi

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SCENES = sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
                if not p.endswith(("api_script.npz", "api_joints.npz", "api_active.npz", "api_loops.npz", "api_controllers.npz", "api_joints2.npz", "api_filter.npz",
                                  "queries.npz")))   # own tests


def assert_records_equal(got, want, what):
    assert got.dtype == want.dtype, what
    assert len(got) == len(want), f"{what}: count {len(got)} != {len(want)}"
    for name in want.dtype.names:
        if name.startswith("_pad"):
            continue
        g, w = got[name], want[name]
        if g.dtype.kind == "f":
            bad = ~((g == w) | (np.isnan(g) & np.isnan(w)))
        else:
            bad = g != w
        if bad.any():
            idx = np.argwhere(bad)[0]
            raise AssertionError(f"{what}.{name} differs at {tuple(idx)}: got {g[tuple(idx)]!r} want {w[tuple(idx)]!r}")


@pytest.mark.parametrize("scene", SCENES)
def test_oracle_matches_reference_bitwise(scene):
    d = np.load(os.path.join(GOLDEN, scene + ".npz"))
    dt = float(d["dt"][0])
    vi, pi = (int(x) for x in d["iters"])
    extras = oracle_lib.golden_extras(d)
    joints = extras["joints"]
    w = oracle_lib.OracleWorld(d["init_world"], d["init_bodies"], d["init_fixtures"], libm=True, **extras)
    snaps = [int(s) for s in d["snaps"]]
    for s in range(1, max(snaps) + 1):
        w.step(dt, vi, pi)
        if s in snaps:
            assert_records_equal(w.bodies(), d[f"s{s}_bodies"], f"{scene} step {s} bodies")
            assert np.array_equal(w.fixtures()["aabb"], d[f"s{s}_aabb"]), f"{scene} step {s} fat AABBs"
            assert_records_equal(w.contacts(), d[f"s{s}_contacts"], f"{scene} step {s} contacts")
            assert np.array_equal(w.solver_order(), d[f"s{s}_order"]), f"{scene} step {s} solver order"
            assert (w.lib.or_world_flags(w.h) & 0x3F) == (int(d[f"s{s}_world"]["flags"][0]) & 0x3F)
            if joints is not None:
                assert_records_equal(w.joints(), d[f"s{s}_joints"], f"{scene} step {s} joints")
                assert np.array_equal(w.joint_order(), d[f"s{s}_jorder"]), f"{scene} step {s} joint order"
    assert w.status() == 0


def test_golden_vectors_present():
    assert {"pyramid", "mixed", "bullets", "sleep", "joints", "bridge"} <= set(SCENES)

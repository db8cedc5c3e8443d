"""The float64 GPU step against the reference's own golden snapshots.

The parity tests hold the float64 path bit-exact to the oracle solving in
the GPU's graph-coloured constraint order, and the oracle's libm build
bit-exact to these snapshots in the reference's order.  Here the GPU is
compared with the reference directly, each in its own order.  Two things
separate them: the Gauss-Seidel order (graph colours against the
reference's island order, island.py:107-148 and contact.py:470-620), and
the portable sine/cosine, which alone moves a run by at most 1e-11 m
(tests/test_sincos_gap.py).  Within one step the order is by far the
larger: solving the same constraints in another order converges to another
point of the same iteration, a difference of the solver's own residual.

1. One step from each snapshot whose successor the reference recorded
   (29 states up to step 201, most of them settled, with up to 590
   contacts): the pair set and contact order are the reference's; touching
   flags, manifold types, point counts, feature ids and awake flags too,
   except for DISCRETE_ONE_STEP contacts (one manifold type of the 20-row
   pyramid at step 100, a face pair on the knife edge of the reference's
   face choice, collision.py); positions within ONE_STEP_TOL_M, or
   JOINT_ONE_STEP_TOL_M in the joint scenes.  Measured: at most 1.0e-2 m
   among the contact scenes (that pyramid step: 590 contacts, 8 velocity
   iterations far from converged, so the order moves the result most),
   below 2.5e-3 m in every other one; 3.7e-2 m on the 30-plank bridge,
   whose chain of revolute joints the GPU solves in colour order (every
   other joint, then the rest) where the reference walks the chain, so
   eight iterations carry an impulse along it differently.
2. Free run from the initial state: the discrete state equal and positions
   within FREE_TOL_M at every snapshot up to the scene's FREE_HELD step
   (measured at most 3.1e-2 m, bullets at step 41).  After that the chaotic
   scenes separate (a solver-order difference grows until a manifold type
   or point count flips); their drift is printed, not bounded.
"""
import os

import numpy as np
import pytest

import oracle_lib
from pypybox2d_gb300 import abi

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SCENES = ("bridge", "buoyancy", "bullets", "gravity", "joints", "joints2", "kinematic", "loops", "mixed", "pyramid",
          "pyramid5", "sensor_filter", "sleep", "uneven")
ONE_STEP_TOL_M = 2e-2
JOINT_ONE_STEP_TOL_M = 5e-2
FREE_TOL_M = 5e-2
# scene -> last snapshot step at which the free run is held to the reference
FREE_HELD = {"bullets": 41, "kinematic": 61, "mixed": 21, "pyramid": 10, "pyramid5": 5, "sensor_filter": 150,
             "sleep": 90, "uneven": 61, "joints": 21, "bridge": 21, "loops": 21, "buoyancy": 61, "gravity": 240,
             "joints2": 61}
# scene -> contacts allowed to differ in discrete fields after one step, over all its one-step states
DISCRETE_ONE_STEP = {"pyramid": 1}


def _discrete_diffs(c, rc, b, rb):
    """Counts of discrete differences between the GPU's state and the reference's."""
    if len(c) != len(rc) or not (np.array_equal(c["fixture_a"], rc["fixture_a"]) and
                                 np.array_equal(c["fixture_b"], rc["fixture_b"])):
        return {"pairs": 1}
    n = c["m_point_count"]
    live = np.arange(2)[None, :] < n[:, None]
    out = {
        "touching": int((c["flags"] & abi.C_TOUCHING != rc["flags"] & abi.C_TOUCHING).sum()),
        "flags": int((c["flags"] != rc["flags"]).sum()),
        "point_count": int((c["m_point_count"] != rc["m_point_count"]).sum()),
        "manifold_type": int(((c["m_type"] != rc["m_type"]) & (n > 0)).sum()),
        "feature_ids": int((np.where(live, c["p_id"], 0) != np.where(live, rc["p_id"], 0)).any(axis=1).sum()),
        "awake": int((b["flags"] != rb["flags"]).sum()),
    }
    return {k: v for k, v in out.items() if v}


def _position_error(b, rb):
    return float(np.hypot(b["cx"] - rb["cx"], b["cy"] - rb["cy"]).max()), float(np.abs(b["a"] - rb["a"]).max())


def _snapshot_batch(d, s):
    from pypybox2d_gb300.gpu import GpuBatch
    C = d[f"s{s}_contacts"]
    W = d[f"s{s}_world"].copy()
    W["contact_start"], W["contact_count"], W["move_count"], W["contact_capacity"] = 0, len(C), 0, 0
    W["flags"] = W["flags"] & np.uint32(0xFFFFFFFF ^ abi.W_NEW_FIXTURE)
    F = d["init_fixtures"].copy()
    F["aabb"] = d[f"s{s}_aabb"]
    J = d[f"s{s}_joints"] if f"s{s}_joints" in d.files else None
    ctl = {k: v for k, v in oracle_lib.golden_extras(d).items() if k != "joints"}
    return GpuBatch(W, d[f"s{s}_bodies"], F, contacts=C if len(C) else None, precision="f64", joints=J, **ctl)


@pytest.mark.parametrize("scene", SCENES)
def test_one_step_from_reference_states(scene):
    d = np.load(os.path.join(GOLDEN, scene + ".npz"))
    dt, (vi, pi) = float(d["dt"][0]), (int(x) for x in d["iters"])
    snaps = [int(s) for s in d["snaps"]]
    worst, apart, lines = 0.0, 0, []
    for s in snaps:
        if s + 1 not in snaps:
            continue
        g = _snapshot_batch(d, s)
        g.step(dt, vi, pi, 1, launch_mode=3)
        assert int(g.status()[0]) == 0
        b, rb = g.bodies(), d[f"s{s + 1}_bodies"]
        dp, da = _position_error(b, rb)
        diffs = _discrete_diffs(g.contacts(0), d[f"s{s + 1}_contacts"], b, rb)
        lines.append(f"{s}->{s + 1}: position {dp:.1e} m, angle {da:.1e} rad, {len(d[f's{s}_contacts'])} contacts, "
                     f"discrete {diffs or 'equal'}")
        assert "pairs" not in diffs, f"{scene} {s}->{s + 1}: pair set or contact order differs"
        apart += max(diffs.values(), default=0)
        worst = max(worst, dp)
    print(f"\n{scene} one step from the reference's states:\n  " + "\n  ".join(lines))
    tol = JOINT_ONE_STEP_TOL_M if "init_joints" in d.files else ONE_STEP_TOL_M
    assert worst <= tol, f"{scene}: {worst:.2e} m"
    assert apart <= DISCRETE_ONE_STEP.get(scene, 0), f"{scene}: {apart} contacts or bodies decided apart"


@pytest.mark.parametrize("scene", SCENES)
def test_free_run_against_the_reference(scene):
    from pypybox2d_gb300.gpu import GpuBatch
    d = np.load(os.path.join(GOLDEN, scene + ".npz"))
    dt, (vi, pi) = float(d["dt"][0]), (int(x) for x in d["iters"])
    g = GpuBatch(d["init_world"], d["init_bodies"], d["init_fixtures"], precision="f64", **oracle_lib.golden_extras(d))
    done, lines = 0, []
    for s in (int(x) for x in d["snaps"]):
        g.step(dt, vi, pi, s - done, launch_mode=3)
        done = s
        b, rb = g.bodies(), d[f"s{s}_bodies"]
        dp, da = _position_error(b, rb)
        diffs = _discrete_diffs(g.contacts(0), d[f"s{s}_contacts"], b, rb)
        lines.append(f"step {s}: position {dp:.1e} m, angle {da:.1e} rad, discrete {diffs or 'equal'}")
        if s <= FREE_HELD[scene]:
            assert not diffs, f"{scene} step {s}: {diffs}"
            assert dp <= FREE_TOL_M, f"{scene} step {s}: {dp:.2e} m"
    assert int(g.status()[0]) == 0
    print(f"\n{scene} free run against the reference (held to step {FREE_HELD[scene]}):\n  " + "\n  ".join(lines))

"""Joints on the GPU beyond the single-world parity scenes.

* a batch mixing worlds with and without joints (the reference-made joint
  and bridge scenes, a contact-only scene between them, in two orders):
  every world steps bit for bit as the oracle steps it alone, so the
  per-world joint ranges, body joint lists and colour layouts of a batch are
  the ones each world has on its own;
* the float32 unit on the joint, loop and controller scenes: one step from
  identical float64 state against the float64 step, positions within
  F32_TOL_M (joints and controllers compute in float64 in both units; the
  float32 unit rounds the velocities and forces they act on; measured at
  most 1.4e-7 m at steps 20, 60 and 120) over the bodies whose step
  records agree.  The loops scene's step 60 has a TOI event whose first
  position pass ends exactly on the -1.5 slop early exit (a ball rolling
  into the terrain), so rounding decides one more pass there (4.7e-4 m, the
  threshold case of tests/test_gpu_f32_parity.py); at most one TOI event (its
  two bodies) a state may be decided apart, and its islands are left out of
  the bound;
* joint state through the C ABI: gb_batch_get_joints returns what was
  uploaded before any step, and gb_batch_set_joints refuses a record whose
  world, kind or bodies differ from the batch's.
"""
import os

import numpy as np
import pytest

import oracle_lib
from pypybox2d_gb300 import abi
from test_gpu_parity import assert_same, used_contact_view

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
F32_TOL_M = 1e-6


def _scene(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    J = d["init_joints"] if "init_joints" in d.files else np.zeros(0, abi.JOINT)
    return d["init_world"], d["init_bodies"], d["init_fixtures"], J


def _batch(names):
    Ws, Bs, Fs, Js = [], [], [], []
    nb = nf = 0
    for wi, n in enumerate(names):
        W, B, F, J = _scene(n)
        W = W.copy()
        W["body_start"], W["fixture_start"] = nb, nf
        J = J.copy()
        J["world"] = wi
        Ws.append(W); Bs.append(B); Fs.append(F); Js.append(J)
        nb += len(B)
        nf += len(F)
    cat = np.concatenate
    return cat(Ws), cat(Bs), cat(Fs), cat(Js)


@pytest.mark.parametrize("names", [("joints", "mixed", "bridge", "joints"), ("bridge", "bridge", "pyramid5", "joints"),
                                   ("joints2", "joints", "mixed", "joints2")])
def test_batch_of_worlds_with_and_without_joints(names):
    from pypybox2d_gb300.gpu import GpuBatch
    W, B, F, J = _batch(names)
    g = GpuBatch(W, B, F, precision="f64", joints=J)
    orcs = [oracle_lib.OracleWorld(W, B, F, libm=False, index=w, joints=J) for w in range(len(names))]
    for s in range(1, 121):
        g.step(1 / 60, 8, 3, 1, launch_mode=3, record_order=True)
        allb = g.bodies()
        for w, o in enumerate(orcs):
            o.step(1 / 60, 8, 3, order=g.solver_order(w), joint_order=g.joint_order(w))
            b0, n = int(W["body_start"][w]), int(W["body_count"][w])
            assert_same(allb[b0:b0 + n], o.bodies(), f"{names[w]} (world {w}) step {s} bodies")
            if s % 20 == 0:
                assert_same(used_contact_view(g.contacts(w)), used_contact_view(o.contacts()), f"world {w} step {s} contacts")
                assert_same(g.joints(w), o.joints(), f"world {w} step {s} joints")
    assert not g.status().any()


@pytest.mark.parametrize("scene", ["joints", "bridge", "joints2", "loops", "buoyancy", "gravity"])
def test_f32_joint_step_against_f64(scene):
    from pypybox2d_gb300.gpu import GpuBatch
    W, B, F, J = _scene(scene)
    ctl = {k: v for k, v in oracle_lib.golden_extras(np.load(os.path.join(GOLDEN, scene + ".npz"))).items()
           if k != "joints"}
    g64 = GpuBatch(W, B, F, precision="f64", joints=J, **ctl)
    worst = 0.0
    done = 0
    for s in (20, 60, 120):
        g64.step(1 / 60, 8, 3, s - done, launch_mode=3)
        done = s
        B0, J0, C0, P0 = g64.bodies(), g64.joints(), g64.contacts(0), g64.proxies()
        W0 = W.copy()
        W0["contact_count"], W0["move_count"] = len(C0), 0
        W0["flags"] &= np.uint32(0xFFFFFFFF ^ abi.W_NEW_FIXTURE)
        W0["inv_dt0"] = 1.0 / (1 / 60)
        F0 = F.copy()
        F0["aabb"] = P0
        a = GpuBatch(W0, B0, F0, contacts=C0 if len(C0) else None, precision="f64", joints=J0, **ctl)
        b = GpuBatch(W0, B0, F0, contacts=C0 if len(C0) else None, precision="f32", joints=J0, **ctl)
        a.step(1 / 60, 8, 3, 1, launch_mode=3, record_order=True)
        b.step(1 / 60, 8, 3, 1, launch_mode=3, record_order=True)
        ba, bb = a.bodies(), b.bodies()
        ra, rb = a.step_record(0), b.step_record(0)
        apart = ra[0] != rb[0]
        islands = set(ra[1][apart & (ra[1] >= 0)].tolist()) | set(rb[1][apart & (rb[1] >= 0)].tolist())
        keep = ~apart & ~np.isin(ra[1], list(islands)) & ~np.isin(rb[1], list(islands))
        d = np.hypot(ba["cx"] - bb["cx"], ba["cy"] - bb["cy"])
        err = float(d[keep].max()) if keep.any() else 0.0
        worst = max(worst, err)
        print(f"\n{scene} step {s}: float32 one-step position error {err:.2e} m over {int(keep.sum())} bodies, "
              f"{int(apart.sum())} body decided apart ({float(d.max()):.2e} m over all)")
        assert int(apart.sum()) <= 2      # one TOI event: its two bodies
        assert not b.status().any()
    assert worst <= F32_TOL_M, f"{scene}: {worst:.2e} m"


def test_joint_records_round_trip_and_fixed_fields():
    from pypybox2d_gb300.gpu import GpuBatch
    W, B, F, J = _scene("joints")
    g = GpuBatch(W, B, F, precision="f64", joints=J)
    assert g.joints().tobytes() == np.ascontiguousarray(J, dtype=abi.JOINT).tobytes()
    bad = g.joints()
    bad["body_b"][0] = bad["body_a"][0]
    with pytest.raises(abi.GB2DError):
        g.set_joints(bad)
    ok = g.joints()
    ok["motor_speed"][:] = 0.5
    g.set_joints(ok)
    assert (g.joints()["motor_speed"] == 0.5).all()

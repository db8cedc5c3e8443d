"""Parity of the sm_103a World.step kernels with the CPU restatement.

The float64 path (-fmad=false, portable sincos) must reproduce the oracle
bit for bit -- bodies, fat AABBs, contact list, manifolds, impulses, feature
ids, touching/enabled flags, sleep state, and the step record (position
iterations of each island, TOI position-pass iterations and events and the
solver set-up decisions of each body) -- step after step, with the
oracle solving each island in the GPU's graph-coloured constraint order
(the solver-order hook).  The scenes are the reference-exported initial
states of the golden vectors (pyramid, mixed edge/circle/polygon box,
bullets with time-of-impact events, sleeping bodies, kinematic bodies,
sensors with group and category/mask filtering, and the four joint kinds:
a scene of revolute, prismatic, distance and weld joints with limits and
motors, and a 30-plank revolute bridge).  Joints are compared record for
record (impulses, motor impulse, limit state, soft-constraint terms) with
the oracle solving them in the GPU's joint colour order.
"""
import os

import numpy as np
import pytest

import oracle_lib
from pypybox2d_gb300 import abi

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
STEPS = {"pyramid": 40, "pyramid5": 150, "mixed": 120, "bullets": 60, "sleep": 90, "uneven": 240, "kinematic": 180,
         "sensor_filter": 150, "joints": 300, "bridge": 240, "loops": 180, "buoyancy": 240, "gravity": 240,
         "joints2": 240}


def _gpu():
    from pypybox2d_gb300.gpu import GpuBatch
    return GpuBatch


def assert_same(got, want, what):
    for name in want.dtype.names:
        if name.startswith("_pad"):
            continue
        g, w = got[name], want[name]
        bad = ~((g == w) | ((g != g) & (w != w))) if g.dtype.kind == "f" else (g != w)
        if bad.any():
            idx = tuple(np.argwhere(bad)[0])
            raise AssertionError(f"{what}.{name} differs at {idx}: gpu {g[idx]!r} oracle {w[idx]!r}")


def used_contact_view(c):
    """Contact fields the step defines (manifold points beyond point_count
    keep stale values in both implementations and are not compared)."""
    c = c.copy()
    for j in range(2):
        unused = c["m_point_count"] <= j
        for f in ("p_lx", "p_ly", "p_ni", "p_ti", "p_id"):
            c[f][unused, j] = 0
    return c


def run_lockstep(scene, steps, launch_mode=1, block_threads=0):
    GpuBatch = _gpu()
    d = np.load(os.path.join(GOLDEN, scene + ".npz"))
    dt = float(d["dt"][0])
    vi, pi = (int(x) for x in d["iters"])
    W, B, F = d["init_world"], d["init_bodies"], d["init_fixtures"]
    extras = oracle_lib.golden_extras(d)
    J = extras["joints"]
    gpu = GpuBatch(W, B, F, precision="f64", **extras)
    orc = oracle_lib.OracleWorld(W, B, F, libm=False, **extras)
    for s in range(1, steps + 1):
        gpu.step(dt, vi, pi, 1, launch_mode=launch_mode, block_threads=block_threads, record_order=True)
        order = gpu.solver_order(0)
        orc.step(dt, vi, pi, order=order, joint_order=gpu.joint_order(0) if J is not None else None)
        if J is not None:
            assert_same(gpu.joints(), orc.joints(), f"{scene} step {s} joints")
        assert_same(gpu.bodies(), orc.bodies(), f"{scene} step {s} bodies")
        assert np.array_equal(gpu.proxies(), orc.fixtures()["aabb"]), f"{scene} step {s} fat AABBs"
        assert_same(used_contact_view(gpu.contacts(0)), used_contact_view(orc.contacts()), f"{scene} step {s} contacts")
        assert np.array_equal(gpu.step_record(0), orc.step_record()), f"{scene} step {s} step record"
    assert int(gpu.status()[0]) == 0
    return gpu, orc


@pytest.mark.parametrize("mode", [1, 3], ids=["monolithic", "phased"])
@pytest.mark.parametrize("scene", sorted(STEPS))
def test_f64_bit_exact_with_oracle(scene, mode):
    run_lockstep(scene, STEPS[scene], launch_mode=mode)


def test_warp_mapping_matches_cta_mapping():
    """One warp per world gives the same doubles as one CTA per world."""
    GpuBatch = _gpu()
    d = np.load(os.path.join(GOLDEN, "mixed.npz"))
    W, B, F = d["init_world"], d["init_bodies"], d["init_fixtures"]
    out = []
    for mode, threads in ((1, 128), (1, 256), (2, 64), (3, 128), (3, 64)):
        g = GpuBatch(W, B, F, precision="f64")
        g.step(1 / 60, 8, 3, 50, launch_mode=mode, block_threads=threads)
        out.append(g.bodies())
    for o in out[1:]:
        assert_same(o, out[0], "mapping")


@pytest.mark.parametrize("kind,n_bodies", [("uneven", 700), ("large", 900)])
def test_f64_large_world_bit_exact_with_oracle(kind, n_bodies):
    """Worlds large enough for the wide solver launch (512 bodies or more):
    100 lock steps of an uneven-workload world and of a piece of the
    large-world workload (boxes and circles falling into a walled ground)
    against the oracle."""
    from pypybox2d_gb300 import scenes
    GpuBatch = _gpu()
    W, B, F, M = scenes.uneven_world(5, n_bodies) if kind == "uneven" else scenes.large_world(5, n_bodies)
    gpu = GpuBatch(W, B, F, precision="f64", moves=M)
    orc = oracle_lib.OracleWorld(W, B, F, libm=False, moves=M)
    for s in range(1, 101):
        gpu.step(1 / 60, 8, 3, 1, launch_mode=3, block_threads=64, record_order=True)
        orc.step(1 / 60, 8, 3, order=gpu.solver_order(0))
        assert_same(gpu.bodies(), orc.bodies(), f"large world step {s} bodies")
        assert_same(used_contact_view(gpu.contacts(0)), used_contact_view(orc.contacts()), f"large world step {s} contacts")
        assert np.array_equal(gpu.step_record(0), orc.step_record()), f"large world step {s} step record"
    assert int(gpu.status()[0]) == 0


def test_f64_grid_world_bit_exact_with_oracle():
    """A world of 16384+ bodies runs every per-world phase as one cooperative
    grid; 6 lock steps of a 17000-body piece of the large-world workload."""
    from pypybox2d_gb300 import scenes
    GpuBatch = _gpu()
    W, B, F, M = scenes.large_world(9, 17000)
    gpu = GpuBatch(W, B, F, precision="f64", moves=M)
    orc = oracle_lib.OracleWorld(W, B, F, libm=False, moves=M)
    for s in range(1, 7):
        gpu.step(1 / 60, 8, 3, 1, launch_mode=3, block_threads=64, record_order=True)
        orc.step(1 / 60, 8, 3, order=gpu.solver_order(0))
        assert_same(gpu.bodies(), orc.bodies(), f"grid world step {s} bodies")
        assert_same(used_contact_view(gpu.contacts(0)), used_contact_view(orc.contacts()), f"grid world step {s} contacts")
        assert np.array_equal(gpu.step_record(0), orc.step_record()), f"grid world step {s} step record"
    assert int(gpu.status()[0]) == 0

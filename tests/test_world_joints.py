"""Joints through the World API, pinned against the reference.

* construction: the reference-made joint and bridge scenes built again with
  this package's API (the same builder functions, tests/golden/make_golden.py)
  give the reference's body and joint records bit for bit (anchors in each
  body's frame, reference angles, the prismatic axis, distance lengths);
* a scripted session (tests/golden/api_joints.py: create, step, setters,
  destroy_joint, a joint that filters an existing contact, destroy_body
  with its joints reported to joint_destruction_listener): every snapshot
  -- bodies, fat boxes, contacts, joint records and the joint getters -- is
  the reference's bit for bit when the World's step runs on the CPU
  restatement (the host logic: records, uploads, flags), and within
  tolerance of it on the float64 GPU step (the GPU solves the one island
  whose circles touch before they are joined in its colour order).
"""
import os
import sys

import numpy as np
import pytest

import pypybox2d_gb300 as b2
from pypybox2d_gb300 import abi

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)
import api_joints  # noqa: E402
import make_golden  # noqa: E402


def same(got, want, what):
    assert got.dtype == want.dtype and len(got) == len(want), what
    for n in want.dtype.names:
        if n.startswith("_pad"):
            continue
        g, w = got[n], want[n]
        bad = ~((g == w) | ((g != g) & (w != w))) if g.dtype.kind == "f" else (g != w)
        assert not bad.any(), f"{what}.{n} differs at {np.argwhere(bad)[0]}: {g[tuple(np.argwhere(bad)[0])]!r} vs " \
                              f"{w[tuple(np.argwhere(bad)[0])]!r}"


def used(c):
    c = c.copy()
    for j in range(2):
        unused = c["m_point_count"] <= j
        for f in ("p_lx", "p_ly", "p_ni", "p_ti", "p_id"):
            c[f][unused, j] = 0
    return c


def oracle_world_class():
    import oracle_lib

    class OracleBackedWorld(b2.World):
        def _make_batch(self, W, B, F, C, M, J=None, CT=None, CB=None):
            return oracle_lib.OracleBatch(W, B, F, C, M, libm=True, joints=J, controllers=CT, controller_bodies=CB)

    return OracleBackedWorld


@pytest.mark.parametrize("scene", ["joints", "bridge", "joints2"])
def test_joint_scene_construction_matches_reference(scene):
    d = np.load(os.path.join(GOLDEN, scene + ".npz"))
    w = getattr(make_golden, "scene_" + scene)(b2)
    w._materialise()
    same(w._B, d["init_bodies"], f"{scene} bodies")
    same(w._J, d["init_joints"], f"{scene} joints")
    assert np.array_equal(w._F["aabb"], d["init_fixtures"]["aabb"])


def _run_script(world_class):
    snaps, log = {}, []

    class Recorder(world_class):
        pass

    def snap(label, world):
        world._materialise()
        getters = np.array([api_joints.getter_row(j) for j in world.joints], dtype=np.float64)
        snaps[label] = (world._B.copy(), world._F["aabb"].copy(), world._C.copy(), world._J.copy(), getters)

    orig = b2.World
    b2.World = Recorder
    try:
        api_joints.script(b2, snap, log=log)
    finally:
        b2.World = orig
    return snaps, log


def test_joint_session_matches_reference_bitwise():
    d = np.load(os.path.join(GOLDEN, "api_joints.npz"))
    snaps, log = _run_script(oracle_world_class())
    assert log == list(d["destroyed"])
    for label in api_joints.SNAPS:
        B, A, C, J, G = snaps[label]
        same(B, d[f"{label}_bodies"], f"{label} bodies")
        assert np.array_equal(A, d[f"{label}_aabb"]), f"{label} fat AABBs"
        same(used(C), used(d[f"{label}_contacts"]), f"{label} contacts")
        same(J, d[f"{label}_joints"], f"{label} joints")
        want = d[f"{label}_getters"]
        assert G.shape == want.shape and np.array_equal(G, want, equal_nan=True), f"{label} joint getters"


def _run_script2(world_class):
    import api_joints2
    snaps = {}

    class Recorder(world_class):
        pass

    def snap(label, world):
        world._materialise()
        getters = np.array([api_joints2.getter_row(j) for j in world.joints], dtype=np.float64)
        snaps[label] = (world._B.copy(), world._C.copy(), world._J.copy(), getters)

    orig = b2.World
    b2.World = Recorder
    try:
        api_joints2.script(b2, snap)
    finally:
        b2.World = orig
    return snaps


def test_friction_rope_wheel_pulley_session_matches_reference_bitwise():
    """tests/golden/api_joints2.py: the friction, rope, wheel and pulley
    joints created, stepped, edited through their setters and destroyed;
    bodies, contacts, joint records and getters bit for bit on the CPU
    restatement."""
    import api_joints2
    d = np.load(os.path.join(GOLDEN, "api_joints2.npz"))
    snaps = _run_script2(oracle_world_class())
    for label in api_joints2.SNAPS:
        B, C, J, G = snaps[label]
        same(B, d[f"{label}_bodies"], f"{label} bodies")
        same(used(C), used(d[f"{label}_contacts"]), f"{label} contacts")
        same(J, d[f"{label}_joints"], f"{label} joints")
        want = d[f"{label}_getters"]
        assert G.shape == want.shape and np.array_equal(G, want, equal_nan=True), f"{label} joint getters"


def test_new_joint_kinds_api():
    w = b2.World()
    a = w.create_dynamic_body(position=(0, 0))
    a.create_circle_fixture(0.5, density=1.0)
    c = w.create_dynamic_body(position=(2, 0))
    c.create_circle_fixture(0.5, density=1.0)
    fr = w.create_friction_joint(a, c, max_force=1.0)
    with pytest.raises(ValueError):                 # friction.py:84-86
        fr.max_force = -1.0
    rope = w.create_rope_joint(a, c, max_length=3.0)
    with pytest.raises(AttributeError):             # rope.py:93-95 reads an attribute it never sets
        rope.limit_state
    wheel = w.create_wheel_joint(a, c, anchor=(2, 0), axis=(0, 1))
    with pytest.raises(AttributeError):             # wheel.py:184-188
        wheel.spring_frequency
    wheel.spring_frequency = 3.0
    assert wheel.spring_frequency == 3.0 and float(wheel._rec()["frequency"]) == 2.0
    with pytest.raises(ValueError):                 # pulley.py:62-63
        w.create_pulley_joint(a, c, ratio=0.0)
    p = w.create_pulley_joint(a, c, ground_anchor_a=(0, 5), ground_anchor_b=(2, 5), anchor_a=(0, 0),
                              anchor_b=(2, 0), ratio=2.0)
    assert p.ratio == 2.0 and tuple(p.get_reaction_force(60.0)) == (0.0, 0.0)
    assert float(p._rec()["constant"]) == 5.0 + 2.0 * 5.0
    assert w.joints == [fr, rope, wheel, p]
    with pytest.raises(NotImplementedError):
        w.create_gear_joint(wheel, wheel)


def test_joint_api_errors():
    w = b2.World()
    a = w.create_dynamic_body(position=(0, 0))
    a.create_circle_fixture(0.5, density=1.0)
    c = w.create_dynamic_body(position=(0, 0.001))
    c.create_circle_fixture(0.5, density=1.0)
    with pytest.raises(ValueError):
        w.create_revolute_joint(a, None)
    with pytest.raises(ValueError):                # distance.py:88-89
        w.create_distance_joint(a, c, anchor_a=(0, 0), anchor_b=(0, 0.001))
    other = b2.World().create_dynamic_body()
    with pytest.raises(ValueError):
        w.create_weld_joint(a, other, anchor=(0, 0))
    j = w.create_revolute_joint(a, c, anchor=(0, 0))
    assert w.joints == [j] and a.joints == [j] and c.joints == [j]
    with pytest.raises(IndexError):                # revolute.py:206-208
        j.get_reaction_force(60.0)
    w.destroy_joint(j)
    assert w.joints == [] and a.joints == []
    with pytest.raises(ValueError):
        w.destroy_joint(j)


@pytest.mark.gpu
def test_joint_session_on_the_gpu_follows_the_reference():
    d = np.load(os.path.join(GOLDEN, "api_joints.npz"))
    snaps, log = _run_script(b2.World)
    assert log == list(d["destroyed"])
    worst = 0.0
    for label in api_joints.SNAPS:
        B, A, C, J, G = snaps[label]
        rb = d[f"{label}_bodies"]
        err = float(np.hypot(B["cx"] - rb["cx"], B["cy"] - rb["cy"]).max())
        worst = max(worst, err)
        assert np.array_equal(J["limit_state"], d[f"{label}_joints"]["limit_state"]), label
        assert np.array_equal(B["flags"], rb["flags"]), label
        print(f"{label}: largest position difference {err:.2e} m")
    assert worst < 5e-2

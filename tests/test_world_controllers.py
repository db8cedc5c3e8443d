"""Controllers (controllers.py) through the World API, pinned against the
reference.

* construction: the reference-made buoyancy and gravity scenes built again
  with this package's API give the reference's bodies, fixtures and
  controller records (kind, parameters, body lists) bit for bit;
* the same scenes stepped through the World on the CPU restatement match
  the reference's snapshots bit for bit (the controllers' records reach the
  step as the device batch would get them);
* a scripted session (tests/golden/api_controllers.py: setters between
  steps, bodies leaving and joining, a destroyed body, destroy_controller,
  a controller made with its bodies and a zero gravity vector): bodies,
  contacts and each controller's body list are the reference's bit for bit
  on the CPU restatement, and on the float64 GPU step the discrete state is
  the reference's with positions within GPU_TOL_M;
* the API's refusals: use_density (the reference's shapes carry no density
  and its step raises AttributeError), a Controller subclass with a Python
  step, a controller of another world's body.
"""
import os
import sys

import numpy as np
import pytest

import pypybox2d_gb300 as b2
from pypybox2d_gb300 import abi
from pypybox2d_gb300.controllers import controller_records

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)
import api_controllers  # noqa: E402
import make_golden  # noqa: E402
from test_world_joints import oracle_world_class, same, used  # noqa: E402

GPU_TOL_M = 5e-2


@pytest.mark.parametrize("scene", ["buoyancy", "gravity"])
def test_controller_scene_construction_matches_reference(scene):
    d = np.load(os.path.join(GOLDEN, scene + ".npz"))
    w = getattr(make_golden, "scene_" + scene)(b2)
    w._materialise()
    same(w._B, d["init_bodies"], f"{scene} bodies")
    same(w._F, d["init_fixtures"], f"{scene} fixtures")
    C, cb = controller_records(w, w.controllers)
    same(C, d["init_controllers"], f"{scene} controllers")
    assert np.array_equal(cb, d["init_controller_bodies"])


@pytest.mark.parametrize("scene", ["buoyancy", "gravity"])
def test_controller_scene_steps_match_reference(scene):
    d = np.load(os.path.join(GOLDEN, scene + ".npz"))
    orig = b2.World
    b2.World = oracle_world_class()
    try:
        w = getattr(make_golden, "scene_" + scene)(b2)
    finally:
        b2.World = orig
    dt, (vi, pi) = float(d["dt"][0]), (int(x) for x in d["iters"])
    snaps = [int(s) for s in d["snaps"]]
    for s in range(1, max(snaps) + 1):
        w.step(dt, vi, pi)
        if s in snaps:
            w._materialise()
            same(w._B, d[f"s{s}_bodies"], f"{scene} step {s} bodies")


def _run(world_class):
    snaps = {}

    class Recorder(world_class):
        pass

    def snap(label, world):
        world._materialise()
        C, cb = controller_records(world, world.controllers)
        snaps[label] = (world._B.copy(), world._C.copy(), C, cb)

    orig = b2.World
    b2.World = Recorder
    try:
        api_controllers.script(b2, snap)
    finally:
        b2.World = orig
    return snaps


def test_controller_session_matches_reference_bitwise():
    d = np.load(os.path.join(GOLDEN, "api_controllers.npz"))
    snaps = _run(oracle_world_class())
    for label in api_controllers.SNAPS:
        B, C, CT, CB = snaps[label]
        same(B, d[f"{label}_bodies"], f"{label} bodies")
        same(used(C), used(d[f"{label}_contacts"]), f"{label} contacts")
        same(CT, d[f"{label}_controllers"], f"{label} controllers")
        assert np.array_equal(CB, d[f"{label}_controller_bodies"]), f"{label} controller bodies"


def test_controller_api_refusals():
    w = oracle_world_class()()
    body = w.create_dynamic_body(position=(0, 1))
    body.create_circle_fixture(0.5, density=1.0)
    pool = w.create_buoyancy_controller(offset=2, density=1, use_density=True)
    pool.add_body(body)
    with pytest.raises(ValueError):
        pool.add_body(body)                                  # controllers.py:55-56
    with pytest.raises(ValueError):
        pool.add_body(b2.World().create_dynamic_body())      # another world's body
    with pytest.raises(AttributeError):                      # controllers.py:189 in the reference's step
        w.step(1 / 60, 8, 3)
    pool.use_density = False
    w.step(1 / 60, 8, 3)

    class Custom(b2.Controller):
        def step(self, timestep):
            pass

    w.add_controller(Custom(w, [body]))
    with pytest.raises(NotImplementedError):
        w.step(1 / 60, 8, 3)
    w.destroy_controller(w.controllers[-1])
    with pytest.raises(ValueError):
        w.destroy_controller(Custom(w))
    assert body._controllers == [pool] and pool.bodies == [body]


def test_controller_records_follow_body_indices():
    w = b2.World((0, -10), True)
    bodies = [w.create_dynamic_body(position=(i, 3)) for i in range(4)]
    for b in bodies:
        b.create_circle_fixture(0.3, density=1.0)
    g = w.create_gravity_controller(G=0.5, inv_sqr=False, bodies=[bodies[3], bodies[1]])
    C, cb = controller_records(w, w.controllers)
    assert C["type"][0] == abi.CONTROLLER_GRAVITY and C["flags"][0] == 0 and list(cb) == [3, 1]
    w.destroy_body(bodies[0])
    C, cb = controller_records(w, w.controllers)
    assert list(cb) == [2, 0] and g.bodies == [bodies[3], bodies[1]]
    w.destroy_body(bodies[1])
    assert g.bodies == [bodies[3]]


@pytest.mark.gpu
def test_controller_session_on_the_gpu_follows_the_reference():
    d = np.load(os.path.join(GOLDEN, "api_controllers.npz"))
    snaps = _run(b2.World)
    worst = 0.0
    for label in api_controllers.SNAPS:
        B, C, CT, CB = snaps[label]
        rb = d[f"{label}_bodies"]
        err = float(np.hypot(B["cx"] - rb["cx"], B["cy"] - rb["cy"]).max())
        worst = max(worst, err)
        assert np.array_equal(B["flags"], rb["flags"]), label
        rc = d[f"{label}_contacts"]
        assert np.array_equal(C["fixture_a"], rc["fixture_a"]) and np.array_equal(C["fixture_b"], rc["fixture_b"]), label
        print(f"{label}: largest position difference {err:.2e} m")
    assert worst < GPU_TOL_M

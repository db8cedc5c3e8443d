"""Loop shapes (shapes.py:780-882) through the World API, pinned against the
reference.

A loop fixture of n vertices is n edge records flagged GB_FIX_LOOP_CHILD
(one per child proxy, fixture.py:250-261), child i the edge from vertex i to
vertex i + 1 with vertices i - 1 and i + 2 as vertex0 / vertex3
(shapes.py:851-863), its fat box made without the radius margin
(shapes.py:822-837).

* construction: the reference-made loops scene built again with this
  package's API gives the reference's body and fixture records bit for bit;
* a scripted session (tests/golden/api_loops.py: both call forms of
  create_loop_fixture, a transform that moves a dynamic loop, a filter
  change on a loop, a loop added to a body in the world, a loop destroyed):
  bodies, the fat box of every child proxy, contacts, closest ray hits and
  AABB query results are the reference's bit for bit when the World steps
  on the CPU restatement; on the float64 GPU step the pairs, awake flags,
  query results and the fixtures the rays hit are the reference's and
  positions stay within GPU_TOL_M (equal up to step 31; the islands of
  several contacts in the bowl are solved in colour order, not the
  reference's, measured 4.4e-3 m at step 60 and 2.8e-2 m at step 120);
* Contact.child_index_a / child_index_b name the loop child of a contact;
* the loop shape itself: child edges, child AABBs, zero mass.
"""
import math
import os
import sys

import numpy as np
import pytest

import pypybox2d_gb300 as b2
from pypybox2d_gb300 import abi

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)
import api_loops  # noqa: E402
import make_golden  # noqa: E402
from test_world_joints import oracle_world_class, same, used  # noqa: E402

GPU_TOL_M = 5e-2


def test_loop_scene_construction_matches_reference():
    d = np.load(os.path.join(GOLDEN, "loops.npz"))
    w = make_golden.scene_loops(b2)
    w._materialise()
    same(w._B, d["init_bodies"], "loops bodies")
    same(w._F, d["init_fixtures"], "loops fixtures")


def _run(world_class):
    snaps = {}

    class Recorder(world_class):
        pass

    def snap(label, world):
        world._materialise()
        rays, queries = api_loops.probes(b2, world)
        snaps[label] = (world._B.copy(), world._F["aabb"].copy(), world._C.copy(), np.array(rays, dtype=np.float64),
                        np.array(queries, dtype=np.float64))

    orig = b2.World
    b2.World = Recorder
    try:
        world = api_loops.script(b2, snap)
    finally:
        b2.World = orig
    return snaps, world


def test_loop_session_matches_reference_bitwise():
    d = np.load(os.path.join(GOLDEN, "api_loops.npz"))
    snaps, _ = _run(oracle_world_class())
    for label in api_loops.SNAPS:
        B, A, C, R, Q = snaps[label]
        same(B, d[f"{label}_bodies"], f"{label} bodies")
        assert np.array_equal(A, d[f"{label}_aabb"]), f"{label} fat AABBs"
        same(used(C), used(d[f"{label}_contacts"]), f"{label} contacts")
        assert np.array_equal(R, d[f"{label}_rays"], equal_nan=True), f"{label} ray hits"
        assert np.array_equal(Q, d[f"{label}_queries"]), f"{label} AABB queries"


def test_contact_child_indices_name_the_loop_child():
    _, world = _run(oracle_world_class())
    seen = 0
    for c in world.contacts:
        for fx, child in ((c.fixture_a, c.child_index_a), (c.fixture_b, c.child_index_b)):
            if isinstance(fx.shape, b2.Loop):
                assert 0 <= child < fx.shape.child_count
                seen += 1
            else:
                assert child == 0
    assert seen > 0


def test_loop_shape():
    with pytest.raises(ValueError):
        b2.Loop([(0, 0)])
    loop = b2.Loop((0, 0), (2, 0), (1, 1))           # vertices as separate arguments
    assert loop.child_count == 3 and loop.vertices == [(0.0, 0.0), (2.0, 0.0), (1.0, 1.0)]
    e = loop.child_edge(1)                            # from vertex 1 to 2, neighbours 0 and 0 (wrapped)
    assert e.vertex1 == (2.0, 0.0) and e.vertex2 == (1.0, 1.0)
    assert e.vertex0 is None and e.vertex3 is None    # vertex (0, 0) counts as absent (shapes.py:633-641)
    e = loop.child_edge(2)
    assert e.vertex0 == (2.0, 0.0) and e.vertex3 == (2.0, 0.0)
    assert loop.compute_mass(3.0).mass == 0.0
    q = (math.cos(0.5), math.sin(0.5))
    lx, ly, ux, uy = loop.compute_aabb((1.0, 2.0), q, 0)
    x2, y2 = 1.0 + q[0] * 2.0, 2.0 + q[1] * 2.0
    assert (lx, ly, ux, uy) == (min(1.0, x2), min(2.0, y2), max(1.0, x2), max(2.0, y2))


def test_loop_records_and_moves():
    w = b2.World((0, -10), True)
    body = w.create_static_body(position=(1, 1))
    body.create_polygon_fixture(box=(1, 1))
    loop = body.create_loop_fixture([(0, 5), (5, 5), (5, 9)])
    body.create_circle_fixture(0.5)
    w._materialise()
    F = w._F
    assert len(F) == 5 and int(w._B[0]["fixture_count"]) == 5
    assert list(F["flags"] & abi.FIX_LOOP_CHILD) == [0, 8, 8, 8, 0]
    assert [w._fixture_child_at(k) for k in range(5)][1:4] == [(loop, 0), (loop, 1), (loop, 2)]
    assert list(w._moves()) == [0, 1, 2, 3, 4]
    body.destroy_fixture(loop)
    w._materialise()
    assert len(w._F) == 2 and list(w._F["shape_type"]) == [abi.SHAPE_POLYGON, abi.SHAPE_CIRCLE]
    assert list(w._moves()) == [0, 1]


@pytest.mark.gpu
def test_loop_session_on_the_gpu_follows_the_reference():
    d = np.load(os.path.join(GOLDEN, "api_loops.npz"))
    snaps, _ = _run(b2.World)
    worst = 0.0
    for label in api_loops.SNAPS:
        B, A, C, R, Q = snaps[label]
        rb = d[f"{label}_bodies"]
        err = float(np.hypot(B["cx"] - rb["cx"], B["cy"] - rb["cy"]).max())
        worst = max(worst, err)
        assert np.array_equal(B["flags"], rb["flags"]), label
        rc = d[f"{label}_contacts"]
        assert np.array_equal(C["fixture_a"], rc["fixture_a"]) and np.array_equal(C["fixture_b"], rc["fixture_b"]), label
        assert np.array_equal(Q, d[f"{label}_queries"]), label
        assert np.array_equal(R[:, :2], d[f"{label}_rays"][:, :2]), label
        print(f"{label}: largest position difference {err:.2e} m")
    assert worst < GPU_TOL_M

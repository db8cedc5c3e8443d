"""WorldBatch: worlds built through the World API and advanced as one
device batch must follow exactly the trajectories they follow when each
World steps on its own (float64, bit-exact: the batch runs the phased
launches, a lone World the one-CTA launch, and both give the same doubles),
with host edits between steps, contact listeners, captured rollouts, queries
and the hand-back of the worlds by close()."""
import numpy as np
import pytest

import pypybox2d_gb300 as b2
from pypybox2d_gb300.world import _concat_worlds


def build(seed):
    rng = np.random.default_rng(seed)
    w = b2.World((0, -10), True)
    w.create_static_body(position=(0, -1)).create_polygon_fixture(box=(15, 1))
    for i in range(6 + 4 * seed):
        b = w.create_dynamic_body(position=(float(rng.uniform(-8, 8)), 1.0 + 1.1 * i), angle=float(rng.uniform(-1, 1)))
        if i % 2:
            b.create_circle_fixture(float(rng.uniform(0.3, 0.6)), density=1.0, friction=0.5)
        else:
            b.create_polygon_fixture(box=(float(rng.uniform(0.3, 0.6)), 0.4), density=2.0, friction=0.4)
    return w


def test_concat_worlds_shifts_only_the_world_ranges():
    ws = [build(s) for s in range(3)]
    recs = []
    for w in ws:
        W = w._sb.world_record(len(w._B), len(w._F), len(w._M))
        recs.append((W, w._B, w._F, w._C, w._M))
    W, B, F, C, M = _concat_worlds(recs)
    assert list(W["body_start"]) == [0, len(ws[0]._B), len(ws[0]._B) + len(ws[1]._B)]
    assert list(W["fixture_start"]) == [0, len(ws[0]._F), len(ws[0]._F) + len(ws[1]._F)]
    assert list(W["move_start"]) == [0, len(ws[0]._M), len(ws[0]._M) + len(ws[1]._M)]
    assert len(B) == sum(len(w._B) for w in ws) and len(M) == sum(len(w._M) for w in ws)
    assert np.array_equal(B["fixture_start"], np.concatenate([w._B["fixture_start"] for w in ws]))


def _log(world, out):
    cm = world.contact_manager
    idx = {}
    for bi, body in enumerate(world.bodies):
        for k, f in enumerate(body.fixtures):
            idx[id(f)] = (bi, k)
    cm.begin_contact = lambda c: out.append(("begin", idx[id(c.fixture_a)], idx[id(c.fixture_b)]))
    cm.end_contact = lambda c: out.append(("end", idx[id(c.fixture_a)], idx[id(c.fixture_b)]))


def _same_worlds(a, b, what):
    a._materialise()
    b._materialise()
    for name in a._B.dtype.names:
        assert np.array_equal(a._B[name], b._B[name]), f"{what}: bodies.{name}"
    assert np.array_equal(a._F["aabb"], b._F["aabb"]), f"{what}: fat AABBs"
    assert len(a._C) == len(b._C), f"{what}: contact count"
    for name in ("fixture_a", "fixture_b", "flags", "m_point_count", "p_ni", "p_ti"):
        assert np.array_equal(a._C[name], b._C[name]), f"{what}: contacts.{name}"


@pytest.mark.gpu
def test_world_batch_follows_the_lone_worlds():
    A = [build(s) for s in range(3)]
    S = [build(s) for s in range(3)]
    logA, logS = [], []
    _log(A[1], logA)
    _log(S[1], logS)
    for w in A + S:                       # some history before batching
        for _ in range(2):
            w.step(1 / 60, 8, 3)
    batch = b2.WorldBatch(A)
    with pytest.raises(RuntimeError):
        A[0].step(1 / 60, 8, 3)
    for k in range(3):
        batch.step(1 / 60, 8, 3, n_steps=10, graph=(k == 2))
        for w in S:
            for _ in range(10):
                w.step(1 / 60, 8, 3)
        for i in range(3):
            _same_worlds(A[i], S[i], f"round {k} world {i}")
        if k == 0:                        # a host edit reaches the next batch step
            A[0].bodies[3].linear_velocity = (1.0, 2.0)
            S[0].bodies[3].linear_velocity = (1.0, 2.0)
            A[2].bodies[2].apply_linear_impulse((0.5, 0.0), A[2].bodies[2].world_center)
            S[2].bodies[2].apply_linear_impulse((0.5, 0.0), S[2].bodies[2].world_center)
    assert logA == logS and len(logA) > 0
    # queries on a world inside the batch
    for p1, p2 in (((-9.0, 3.0), (9.0, 0.5)), ((0.0, 8.0), (0.5, -1.5))):
        ha, hs = A[2].ray_cast_closest(p1, p2), S[2].ray_cast_closest(p1, p2)
        assert (ha is None) == (hs is None)
        if ha is not None:
            assert ha[3] == hs[3] and tuple(ha[1]) == tuple(hs[1])
    assert len(list(A[1].query_aabb(((-3, -1), (3, 2))))) == len(list(S[1].query_aabb(((-3, -1), (3, 2)))))
    # hand the worlds back: they step on their own and stay in lock step
    batch.close()
    for w in A + S:
        for _ in range(5):
            w.step(1 / 60, 8, 3)
    for i in range(3):
        _same_worlds(A[i], S[i], f"after close world {i}")
    assert logA == logS


def test_listeners_run_with_the_world_locked():
    """As inside the reference's step (world.py:321-354): a listener sees
    world.locked and cannot change the world's structure."""
    from pypybox2d_gb300 import abi
    w = build(0)
    seen = []

    def begin(c):
        seen.append(w.locked)
        w.create_dynamic_body(position=(0, 5))

    w.contact_manager.begin_contact = begin
    ev = np.zeros(1, dtype=abi.EVENT)
    ev["type"], ev["fixture_a"], ev["fixture_b"] = abi.EV_BEGIN, 0, 1
    with pytest.raises(b2.LockedError):
        w._replay(ev)
    assert seen == [True] and not w.locked and w.body_count == 1 + 6


@pytest.mark.gpu
def test_world_batch_with_joints_loops_and_controllers():
    """Worlds with joints of every kind, loop shapes and controllers in one
    batch follow the lone worlds bit for bit (the batch's joint ranges,
    controller records and their body lists are offset per world), also
    after a controller parameter edit (gb_batch_set_controllers); a new
    controller body list inside the batch is refused."""
    import os
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import make_golden
    scenes = (make_golden.scene_joints2, make_golden.scene_buoyancy, make_golden.scene_loops, make_golden.scene_gravity)
    A = [s(b2) for s in scenes]
    S = [s(b2) for s in scenes]
    batch = b2.WorldBatch(A)
    for k in range(3):
        batch.step(1 / 60, 8, 3, n_steps=10)
        for w in S:
            for _ in range(10):
                w.step(1 / 60, 8, 3)
        for i in range(len(A)):
            _same_worlds(A[i], S[i], f"round {k} world {i}")
        if k == 0:
            for w in (A[1], S[1]):
                w.controllers[0].density = 3.0
                w.controllers[1].velocity = (-1.0, 0.0)
            for w in (A[3], S[3]):
                w.controllers[0].G = 2.0
    with pytest.raises(NotImplementedError):
        A[3].controllers[1].add_body(A[3].bodies[1])
        batch.step(1 / 60, 8, 3)
    batch.close()

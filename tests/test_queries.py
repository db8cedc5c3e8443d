"""World queries: the closest hit of a ray (World.ray_cast with a callback
returning the fraction, pypybox2d/world.py:387-440) and the fixtures whose
fat AABB overlaps a box (World.query_aabb, world.py:371-385).

tests/golden/queries.npz holds stepped states of the mixed and uneven scenes
with the reference's own answers to seeded rays and boxes
(tests/golden/make_golden_queries.py).  The CPU restatement must reproduce
them bit for bit (hit fixture, point, normal, fraction; fixture lists); the
float64 GPU kernels (gb_batch_ray_cast, gb_batch_query_aabb) must too.  The
float32 unit stores shape vertices in float32, so its hits are held to a
tolerance: the same fixture for at least 97% of the rays and hit points
within 1e-4 m where the fixture agrees.
"""
import os

import numpy as np
import pytest

import oracle_lib
from pypybox2d_gb300 import abi

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SCENES = ["mixed", "uneven"]
CAP = 64


def _load(scene):
    d = np.load(os.path.join(GOLDEN, "queries.npz"))
    W, B, F = d[f"{scene}_world"], d[f"{scene}_bodies"], d[f"{scene}_fixtures"]
    r = d[f"{scene}_rays"]
    rays = np.zeros(len(r), dtype=abi.RAY)
    rays["p1x"], rays["p1y"], rays["p2x"], rays["p2y"] = r[:, 0], r[:, 1], r[:, 2], r[:, 3]
    bx = d[f"{scene}_boxes"]
    boxes = np.zeros(len(bx), dtype=abi.AABB_QUERY)
    boxes["lx"], boxes["ly"], boxes["ux"], boxes["uy"] = bx[:, 0], bx[:, 1], bx[:, 2], bx[:, 3]
    counts = d[f"{scene}_box_counts"]
    lists = np.split(d[f"{scene}_box_fixtures"], np.cumsum(counts)[:-1])
    return W, B, F, rays, d[f"{scene}_hits"], boxes, counts, lists


def _load_all(scene):
    """Every hit of every ray, in fixture order: (counts, per-ray lists)."""
    d = np.load(os.path.join(GOLDEN, "queries.npz"))
    counts = d[f"{scene}_all_counts"]
    return counts, np.split(d[f"{scene}_all_hits"], np.cumsum(counts)[:-1])


def _check_all(out, n, counts, lists, what):
    assert np.array_equal(n, counts), f"{what}: hit counts differ"
    for q, hs in enumerate(lists):
        got = out[q, :len(hs)]
        for f in ("fixture", "px", "py", "nx", "ny", "fraction"):
            assert np.array_equal(got[f], hs[f]), f"{what}: ray {q} field {f} differs"


def _check_hits(got, want, what):
    assert np.array_equal(got["fixture"], want["fixture"]), f"{what}: hit fixtures differ at " \
        f"{np.argwhere(got['fixture'] != want['fixture'])[:5].ravel()}"
    hit = want["fixture"] >= 0
    for f in ("px", "py", "nx", "ny", "fraction"):
        bad = hit & (got[f] != want[f])
        assert not bad.any(), f"{what}.{f} differs at ray {np.argwhere(bad)[0][0]}: {got[f][bad][0]!r} vs {want[f][bad][0]!r}"


def _check_lists(out, n, counts, lists, what):
    assert np.array_equal(n, counts), f"{what}: overlap counts differ"
    for q, ks in enumerate(lists):
        m = min(len(ks), CAP)
        assert np.array_equal(out[q, :m], ks[:m]), f"{what}: box {q} fixtures differ"


@pytest.mark.parametrize("scene", SCENES)
def test_oracle_queries_match_reference(scene):
    W, B, F, rays, want, boxes, counts, lists = _load(scene)
    assert (want["fixture"] >= 0).sum() > 100
    _check_hits(oracle_lib.ray_cast_records(B, F, rays, libm=True), want, f"{scene} oracle rays")
    out, n = oracle_lib.query_aabb_records(F, boxes, CAP, libm=True)
    _check_lists(out, n, counts, lists, f"{scene} oracle boxes")
    ac, al = _load_all(scene)
    assert ac.sum() > 300 and ac.max() <= CAP
    out, n = oracle_lib.ray_cast_all_records(B, F, rays, CAP, libm=True)
    _check_all(out, n, ac, al, f"{scene} oracle all hits")


def _batch(scene, precision, copies=1):
    """The golden state as a batch of `copies` identical worlds."""
    from pypybox2d_gb300 import scenes
    from pypybox2d_gb300.gpu import GpuBatch
    W, B, F = _load(scene)[:3]
    W = W.copy()
    W["contact_count"] = 0          # queries read bodies and fat AABBs only
    if copies > 1:
        W, B, F, _ = scenes.concat([(W, B, F)] * copies)
    return GpuBatch(W, B, F, precision=precision)


@pytest.mark.gpu
@pytest.mark.parametrize("scene", SCENES)
def test_gpu_queries_match_reference_f64(scene):
    W, B, F, rays, want, boxes, counts, lists = _load(scene)
    g = _batch(scene, "f64", copies=3)
    for w in range(3):
        rays["world"] = w
        boxes["world"] = w
        _check_hits(g.ray_cast(rays), want, f"{scene} world {w} gpu rays")
        out, n = g.query_aabb(boxes, CAP)
        _check_lists(out, n, counts, lists, f"{scene} world {w} gpu boxes")
        ac, al = _load_all(scene)
        out, n = g.ray_cast_all(rays, CAP)
        _check_all(out, n, ac, al, f"{scene} world {w} gpu all hits")


@pytest.mark.gpu
@pytest.mark.parametrize("scene", SCENES)
def test_gpu_queries_f32_within_tolerance(scene):
    W, B, F, rays, want, boxes, counts, lists = _load(scene)
    g = _batch(scene, "f32")
    got = g.ray_cast(rays)
    same = got["fixture"] == want["fixture"]
    assert same.mean() >= 0.97, f"{scene}: f32 hit fixture agrees for {same.mean():.3f} of rays"
    hit = same & (want["fixture"] >= 0)
    err = np.hypot(got["px"] - want["px"], got["py"] - want["py"])[hit]
    assert err.max() <= 1e-4, f"{scene}: f32 hit point error {err.max():.3g} m"
    out, n = g.query_aabb(boxes, CAP)          # fat AABBs stay float64
    _check_lists(out, n, counts, lists, f"{scene} f32 boxes")


@pytest.mark.gpu
def test_gpu_queries_reject_bad_input():
    W, B, F, rays, want, boxes, counts, lists = _load("mixed")
    g = _batch("mixed", "f64")
    bad = rays[:2].copy()
    bad["p2x"], bad["p2y"] = bad["p1x"], bad["p1y"]
    with pytest.raises(abi.GB2DError, match="no length"):
        g.ray_cast(bad)
    bad = rays[:2].copy()
    bad["world"] = 5
    with pytest.raises(abi.GB2DError, match="world out of range"):
        g.ray_cast(bad)


@pytest.mark.gpu
def test_world_api_queries():
    """World.ray_cast / ray_cast_closest / query_aabb of the drop-in API
    against the restatement on the same records."""
    import pypybox2d_gb300 as b2
    world = b2.World((0, -10), True)
    world.create_static_body(position=(0, -1)).create_polygon_fixture(box=(20, 1))
    for i in range(12):
        b = world.create_dynamic_body(position=(-6 + i, 1 + 0.7 * (i % 3)), angle=0.3 * i)
        if i % 2:
            b.create_circle_fixture(0.4, density=1.0)
        else:
            b.create_polygon_fixture(box=(0.4, 0.3), density=1.0)
    for _ in range(20):
        world.step(1 / 60, 8, 3)
    world._materialise()
    B, F = world._B.copy(), world._F.copy()
    rng = np.random.default_rng(7)
    rays = np.zeros(64, dtype=abi.RAY)
    rays["p1x"], rays["p1y"] = rng.uniform(-8, 8, 64), rng.uniform(4, 6, 64)
    rays["p2x"], rays["p2y"] = rays["p1x"] + rng.uniform(-3, 3, 64), rng.uniform(-3, 0, 64)
    want = oracle_lib.ray_cast_records(B, F, rays, libm=False)
    n_hit = 0
    for r, w in zip(rays, want):
        got = world.ray_cast_closest((r["p1x"], r["p1y"]), (r["p2x"], r["p2y"]))
        if w["fixture"] < 0:
            assert got is None
            continue
        n_hit += 1
        fixture, point, normal, fraction = got
        assert fixture is world._fixture_at(int(w["fixture"]))
        assert (point[0], point[1], normal[0], normal[1], fraction) == (w["px"], w["py"], w["nx"], w["ny"], w["fraction"])
        seen = []
        world.ray_cast((r["p1x"], r["p1y"]), (r["p2x"], r["p2y"]), lambda f, p, n, fr: seen.append(f) or fr)
        assert seen == [fixture]
    assert n_hit > 10
    # every hit: a callback that answers 1, and the generator left at 1
    every, counts = oracle_lib.ray_cast_all_records(B, F, rays, 64, libm=False)
    for r, hs, c in zip(rays, every, counts):
        want = sorted((float(h["fraction"]), int(h["fixture"])) for h in hs[:c])
        seen = []
        world.ray_cast((r["p1x"], r["p1y"]), (r["p2x"], r["p2y"]),
                       lambda f, p, n, fr: seen.append((fr, f)) or 1.0)
        assert [(fr, f) for fr, f in seen] == [(fr, world._fixture_at(k)) for fr, k in want]
        gen = []
        for entry in world.ray_cast((r["p1x"], r["p1y"]), (r["p2x"], r["p2y"])):
            gen.append(entry[0])
            entry[-1] = 1.0
        assert gen == [f for _, f in seen]
    out, n = oracle_lib.query_aabb_records(F, np.array([(0, 0, -3.0, -0.5, 2.0, 3.0)], dtype=abi.AABB_QUERY), 64)
    got = list(world.query_aabb(((-3.0, -0.5), (2.0, 3.0))))
    assert got == [world._fixture_at(int(k)) for k in out[0, :n[0]]] and len(got) >= 3
    with pytest.raises(ValueError):
        world.ray_cast_closest((1.0, 1.0), (1.0, 1.0))

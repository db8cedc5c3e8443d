"""Scene construction reproduces the reference's construction arithmetic:
the records built by pypybox2d_gb300.scenes equal, bit for bit, the records
exported from the reference after building the same scene with its API
(tests/golden/*.npz, init_* arrays)."""
import os

import numpy as np
import pytest

from pypybox2d_gb300 import abi, scenes
from pypybox2d_gb300.shapes import Circle, Polygon

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def same(a, b, what):
    for n in b.dtype.names:
        if n.startswith("_pad"):
            continue
        x, y = a[n], b[n]
        bad = ~((x == y) | ((x != x) & (y != y))) if x.dtype.kind == "f" else (x != y)
        assert not bad.any(), f"{what}.{n} differs at {np.argwhere(bad)[0]}: {x[tuple(np.argwhere(bad)[0])]} vs {y[tuple(np.argwhere(bad)[0])]}"


@pytest.mark.parametrize("rows,name", [(20, "pyramid"), (5, "pyramid5")])
def test_pyramid_records_match_reference(rows, name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    W, B, F, M = scenes.pyramid_world(rows)
    same(B, d["init_bodies"], "bodies")
    same(F, d["init_fixtures"], "fixtures")
    assert W["flags"][0] == d["init_world"]["flags"][0]
    assert np.array_equal(M, np.arange(len(F)))


def test_sleep_scene_records_match_reference():
    d = np.load(os.path.join(GOLDEN, "sleep.npz"))
    s = scenes.SceneBuilder()
    s.create_body(abi.BODY_STATIC, position=(0, -0.5), fixtures=[(Polygon(box=(20, 0.5)), {})])
    for pos in ((-5, 0.6), (0, 0.5), (0, 1.5)):
        b = s.create_body(abi.BODY_DYNAMIC, position=pos)
        s.add_fixture(b, Polygon(box=(0.5, 0.5)), density=1.0)
    b = s.create_body(abi.BODY_DYNAMIC, position=(5, 0.5))
    s.add_fixture(b, Circle(radius=0.5), density=1.0)
    W, B, F, M = s.records()
    same(B, d["init_bodies"], "bodies")
    same(F, d["init_fixtures"], "fixtures")


def test_pyramid_batch_first_world_and_jitter():
    W, B, F, M = scenes.pyramid_batch(3, rows=5, jitter=0.01, seed=7)
    nb = len(B) // 3
    assert len(W) == 3 and (W["body_start"] == np.arange(3) * nb).all()
    # world 1 equals a world built one body at a time with the same offsets
    rng = np.random.default_rng(8)
    jit = rng.uniform(-0.01, 0.01, size=(nb - 1, 2))
    Wb, Bb, Fb, _ = scenes.pyramid_builder(5, jitter=lambda k: (jit[k, 0], jit[k, 1])).records()
    same(B[nb:2 * nb], Bb, "jittered bodies")
    same(F[len(Fb):2 * len(Fb)], Fb, "jittered fixtures")


def test_uneven_world_records_match_reference():
    d = np.load(os.path.join(GOLDEN, "uneven.npz"))
    W, B, F, M = scenes.uneven_world(11, 250)
    same(B, d["init_bodies"], "bodies")
    same(F, d["init_fixtures"], "fixtures")
    assert np.array_equal(M, np.arange(len(F)))


def test_uneven_batch_equals_worlds_built_one_body_at_a_time():
    W, B, F, M = scenes.uneven_batch(5, seed=40)
    W2, B2, F2, M2 = scenes.concat([scenes.uneven_world(40 + w) for w in range(5)])
    same(W, W2, "worlds")
    same(B, B2, "bodies")
    same(F, F2, "fixtures")
    assert np.array_equal(M, M2)
    n = W["body_count"] - 1
    assert ((n >= scenes.UNEVEN_MIN) & (n <= scenes.UNEVEN_MAX)).all()


def test_large_world_equals_world_built_one_body_at_a_time():
    W, B, F, M = scenes.large_world(3, 120)
    W2, B2, F2, M2 = scenes.large_builder(3, 120).records()
    same(W, W2, "world")
    same(B, B2, "bodies")
    same(F, F2, "fixtures")
    assert np.array_equal(M, M2)


def test_bullet_batch_layout():
    W, B, F, M = scenes.bullet_batch(3, seed=9)
    assert len(W) == 3 and (W["body_count"] == 25).all()
    bullets = B[(B["flags"] & abi.BODY_BULLET) != 0]
    assert len(bullets) == 12 and (bullets["vx"] >= 120).all()

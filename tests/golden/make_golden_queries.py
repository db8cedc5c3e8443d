"""Generate the golden vectors of the world queries by running the reference
pypybox2d itself (C-extension math mode) in this container.

Usage:  python tests/golden/make_golden_queries.py --ref <pypybox2d source tree>   (or GB2D_REFERENCE=<tree>)

For the mixed (edges, circles, polygons) and uneven scenes of
make_golden.py, the reference world is stepped (with the same pair-order
hook) and exported to the record layouts of include/gb2d.h; then seeded rays
and query boxes are put to the reference's own World.ray_cast
(world.py:387-440) and World.query_aabb (world.py:371-385):

  * every ray's hits are collected through the generator form with the
    fraction left at 1 (no clipping), so each fixture the tree reports and
    the shape hits is seen: all of them (in fixture order) are the expected
    answer of the all-hits query, the closest (lowest fraction) that of the
    closest-hit query.  Rays whose two closest hits share one fraction are left
    out (their winner would depend on the tree's visiting order).
  * every query box's fixtures are collected and sorted by fixture index.

Output: tests/golden/queries.npz (per scene: the exported state, the rays,
the expected hits, the query boxes, the expected fixture lists; plus the
Body frame helpers of tests/golden/api_frames.py).
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import make_golden as mg  # noqa: E402
from pypybox2d_gb300 import abi  # noqa: E402

SCENES = {"mixed": (mg.scene_mixed, 60), "uneven": (mg.scene_uneven, 90)}
N_RAYS, N_BOXES = 400, 120


def rays_for(rng, F):
    """Rays between points drawn over the scene's extent (fat AABBs), some
    starting inside shapes, some long, some short."""
    lo = F["aabb"][:, :2].min(axis=0)
    hi = F["aabb"][:, 2:].max(axis=0)
    p1 = rng.uniform(lo, hi, size=(N_RAYS, 2))
    d = rng.normal(size=(N_RAYS, 2))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    ln = rng.choice([0.5, 3.0, 15.0, 80.0], size=N_RAYS)
    return p1, p1 + d * ln[:, None]


def boxes_for(rng, F):
    lo = F["aabb"][:, :2].min(axis=0)
    hi = F["aabb"][:, 2:].max(axis=0)
    c = rng.uniform(lo, hi, size=(N_BOXES, 2))
    h = rng.uniform(0.05, 6.0, size=(N_BOXES, 2))
    return np.concatenate([c - h, c + h], axis=1)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("GB2D_REFERENCE"), required="GB2D_REFERENCE" not in os.environ,
                    help="the pypybox2d source tree (default: $GB2D_REFERENCE)")
    args = ap.parse_args()
    b2 = mg.load_reference(args.ref)
    from pypybox2d.common import AABB, Vec2
    out = {}
    for name, (builder, n_steps) in SCENES.items():
        world = builder(b2)
        mg.pair_order_hook(world)
        for _ in range(n_steps):
            world.step(1.0 / 60, 8, 3)
        W, B, F, C = mg.export_world(world, b2)
        fidx = mg.fixture_index(world)
        rng = np.random.default_rng(20261204 + len(name))
        p1, p2 = rays_for(rng, F)
        rays, hits, all_hits, all_counts = [], [], [], []
        for a, b in zip(p1, p2):
            found = []
            for ret in world.ray_cast((float(a[0]), float(a[1])), (float(b[0]), float(b[1]))):
                fixture, point, normal, fraction = ret
                found.append((fraction, fidx[id(fixture)], point.x, point.y, normal.x, normal.y))
                ret[-1] = 1.0
            found.sort()
            if len(found) > 1 and found[0][0] == found[1][0]:
                continue
            rays.append((a[0], a[1], b[0], b[1]))
            by_fixture = sorted(found, key=lambda h: h[1])
            all_counts.append(len(by_fixture))
            all_hits.extend((k, px, py, nx, ny, fr) for fr, k, px, py, nx, ny in by_fixture)
            if found:
                fr, k, px, py, nx, ny = found[0]
                hits.append((k, px, py, nx, ny, fr))
            else:
                hits.append((-1, 0.0, 0.0, 0.0, 0.0, 1.0))
        boxes = boxes_for(rng, F)
        lists, counts = [], []
        for bx in boxes:
            aabb = AABB(Vec2(float(bx[0]), float(bx[1])), Vec2(float(bx[2]), float(bx[3])))
            ks = sorted(fidx[id(f)] for f in world.query_aabb(aabb))
            counts.append(len(ks))
            lists.extend(ks)
        out[f"{name}_world"], out[f"{name}_bodies"], out[f"{name}_fixtures"] = W, B, F
        # Contact.world_manifold (contact_util.py:195-245) of every contact,
        # in contact-list order: normal, two points (NaN where unused)
        wm = np.full((len(C), 6), np.nan)
        for i, c in enumerate(world.contact_manager.contacts):
            m = c.world_manifold
            wm[i, 0], wm[i, 1] = m.normal.x, m.normal.y
            for k, p in enumerate(m.points):
                wm[i, 2 + 2 * k], wm[i, 3 + 2 * k] = p.x, p.y
        out[f"{name}_contacts"], out[f"{name}_world_manifolds"] = C, wm
        out[f"{name}_rays"] = np.array(rays, dtype=np.float64)
        out[f"{name}_hits"] = np.array(hits, dtype=[("fixture", "<i4"), ("px", "<f8"), ("py", "<f8"),
                                                    ("nx", "<f8"), ("ny", "<f8"), ("fraction", "<f8")])
        out[f"{name}_all_counts"] = np.array(all_counts, dtype=np.int32)
        out[f"{name}_all_hits"] = np.array(all_hits, dtype=out[f"{name}_hits"].dtype)
        out[f"{name}_boxes"] = boxes
        out[f"{name}_box_counts"] = np.array(counts, dtype=np.int32)
        out[f"{name}_box_fixtures"] = np.array(lists, dtype=np.int32)
        n_hit = int(np.sum(out[f"{name}_hits"]["fixture"] >= 0))
        print(f"{name}: {len(B)} bodies, {len(F)} fixtures, {len(rays)} rays ({n_hit} hit), "
              f"{len(boxes)} boxes ({int(np.sum(counts))} fixtures listed)")
    # Body frame helpers and World flags of a small API-built world (api_frames.py)
    import api_frames
    frame_rows, flags = api_frames.rows(b2)
    out["frames"] = np.array(frame_rows, dtype=np.float64)
    out["frame_world_flags"] = np.array(flags, dtype=np.int32)
    rows, world = api_frames.destroy_rows(b2, on_world=mg.pair_order_hook)
    out["destroy_fixture"] = np.array(rows, dtype=np.float64)
    for _ in range(api_frames.STEPS_AFTER_DESTROY):
        world.step(1.0 / 60, 8, 3)
    W2, B2, F2, C2 = mg.export_world(world, b2)
    out["destroy_fixture_bodies"] = B2
    out["destroy_fixture_contacts"] = C2
    rows, world = api_frames.mass_rows(b2, on_world=mg.pair_order_hook)
    out["mass_data"] = np.array(rows, dtype=np.float64)
    for _ in range(api_frames.STEPS_AFTER_DESTROY):
        world.step(1.0 / 60, 8, 3)
    out["mass_data_bodies"] = mg.export_world(world, b2)[1]
    rows, world = api_frames.type_rows(b2, on_world=mg.pair_order_hook)
    out["body_setters"] = np.array(rows, dtype=np.float64)
    for _ in range(api_frames.STEPS_AFTER_DESTROY):
        world.step(1.0 / 60, 8, 3)
    _, B2, _, C2 = mg.export_world(world, b2)
    out["body_setters_bodies"], out["body_setters_contacts"] = B2, C2
    rows, world = api_frames.fixture_rows(b2, on_world=mg.pair_order_hook)
    out["fixture_setters"] = np.array(rows, dtype=np.float64)
    for _ in range(api_frames.STEPS_AFTER_DESTROY):
        world.step(1.0 / 60, 8, 3)
    _, B2, _, C2 = mg.export_world(world, b2)
    out["fixture_setters_bodies"], out["fixture_setters_contacts"] = B2, C2
    # host-side edits between steps on a world with live contacts (api_edits.py)
    import api_edits

    def snap_edits(label, world):
        _, B3, F3, C3 = mg.export_world(world, b2)
        out[f"edits_{label}_bodies"], out[f"edits_{label}_aabb"], out[f"edits_{label}_contacts"] = B3, F3["aabb"].copy(), C3

    _, end_log = api_edits.script(b2, snap_edits, on_world=mg.pair_order_hook)
    out["edits_end_log"] = np.array(end_log, dtype=np.int32).reshape(-1, 2)
    path = os.path.join(HERE, "queries.npz")
    np.savez_compressed(path, **out)
    print(f"-> {path} ({os.path.getsize(path)} bytes)")


if __name__ == "__main__":
    main()

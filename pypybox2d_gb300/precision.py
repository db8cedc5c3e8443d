"""The float32-bulk batch against the float64 path.

The batched form computes its narrow phase, solver and velocities in float32
and keeps positions, angles, sweeps, fat AABBs, sleep timers and the time of
impact in float64.  This module measures what that costs, on the GPU:

* ``one_step``: from identical float64 state, one float32 step against one
  float64 step solved in the same constraint order.  The float64 GPU path is
  bit-exact with the CPU restatement of ``World.step``
  (pypybox2d/world.py:307-354), so it stands for the float64 reference here;
  a caller may instead pass the restatement's own results (``reference=``).
  Continuous errors per world (position, angle, velocity) and the discrete
  decisions both steps took.
* ``drift``: both forms stepped from the same initial state without re-syncing
  (the unmodified order of each), with the distribution of their position and
  angle differences at checkpoints.

Discrete state compared (the decisions the reference makes with float64
comparisons): the pair set and contact order (dynamictree.py:152-188 fat-box
rule, broadphase.py:83-109, contact_manager.py:102-158 creation,
contact_manager.py:174-223 destruction), touching flags, manifold type,
point count and feature ids (contact.py:210-268), the awake flags of bodies
(island.py:163-179), which proxies were re-fattened, and the step record
(gb_batch_get_step_record): the position iterations each island ran before
its early exit (island.py:141-153), the TOI position-pass iterations and
events of each body (contact.py:866-933, world.py:693-817) and the parity of
the restitution-bias and block-solver decisions of its constraints
(contact.py:470-496).
"""
from __future__ import annotations

import numpy as np

from . import abi


def with_proxies(F, P):
    """Fixture records with the fat AABBs of a device batch."""
    F2 = F.copy()
    F2["aabb"] = P
    return F2


def batch_records(g, F, inv_dt0: float, worlds=None):
    """Records (worlds, bodies, fixtures with the device fat AABBs, contacts)
    of the listed worlds of a device batch ``g`` built from fixture records
    ``F`` (default: all), as the batch stands after at least one step of
    ``1 / inv_dt0`` seconds (World._inv_dt0, world.py:349), laid out as a
    batch of their own: another batch built from them continues from the
    same state."""
    Wg = g.worlds
    idx = np.arange(len(Wg)) if worlds is None else np.asarray(worlds, dtype=np.int64)
    Ball, P = g.bodies(), g.proxies()
    W = Wg[idx].copy()
    Bs, Fs, Cs = [], [], []
    nb = nf = nc = 0
    for k, w in enumerate(idx):
        b0, bn = int(Wg["body_start"][w]), int(Wg["body_count"][w])
        f0, fn = int(Wg["fixture_start"][w]), int(Wg["fixture_count"][w])
        c = g.contacts(int(w))
        Bs.append(Ball[b0:b0 + bn])
        Fs.append(with_proxies(F[f0:f0 + fn], P[f0:f0 + fn]))
        Cs.append(c)
        W["body_start"][k], W["fixture_start"][k], W["contact_start"][k] = nb, nf, nc
        W["contact_count"][k] = len(c)
        nb, nf, nc = nb + bn, nf + fn, nc + len(c)
    W["flags"] = W["flags"] & np.uint32(0xFFFFFFFF ^ abi.W_NEW_FIXTURE)
    W["move_start"] = 0
    W["move_count"] = 0
    W["inv_dt0"] = inv_dt0
    C = np.concatenate(Cs) if Cs else np.zeros(0, abi.CONTACT)
    return W, np.concatenate(Bs), np.concatenate(Fs), C


def discrete(W, B, P, C):
    """Discrete state of every world: per world a dict of contact keys in
    list order, touching flags, manifold types, point counts, feature ids,
    and the awake flags of its bodies."""
    out = []
    for w in range(len(W)):
        c0, nc = int(W["contact_start"][w]), int(W["contact_count"][w])
        c = C[c0:c0 + nc]
        b0, nb = int(W["body_start"][w]), int(W["body_count"][w])
        cnt = c["m_point_count"].astype(np.int64)
        ids = np.where(np.arange(2)[None, :] < cnt[:, None], c["p_id"], 0)
        out.append({
            "keys": (c["fixture_a"].astype(np.int64) << 32) | c["fixture_b"].astype(np.int64),
            "touching": (c["flags"] & abi.C_TOUCHING) != 0,
            "type": np.where(cnt > 0, c["m_type"], -1),
            "count": cnt,
            "ids": ids,
            "awake": (B["flags"][b0:b0 + nb] & abi.BODY_AWAKE) != 0,
        })
    return out


_TOTALS = ("contacts", "touching_contacts", "bodies", "proxies", "worlds_with_any")


def mismatch(a, b, moved_a=None, moved_b=None):
    """Counts of discrete differences between two states of the same worlds
    (``discrete`` results), plus the totals they are counted over."""
    m = dict(pairs=0, order=0, touching=0, manifold_type=0, point_count=0, feature_ids=0, awake=0, refattened=0,
             contacts=0, touching_contacts=0, bodies=0, proxies=0, worlds_with_any=0)
    for x, y in zip(a, b):
        kx, ky = x["keys"], y["keys"]
        m["contacts"] += len(kx)
        m["bodies"] += len(x["awake"])
        before = sum(v for k, v in m.items() if k not in _TOTALS)
        common, ix, iy = np.intersect1d(kx, ky, return_indices=True)
        m["pairs"] += len(kx) + len(ky) - 2 * len(common)
        if len(kx) == len(ky) and not np.array_equal(kx, ky) and len(common) == len(kx):
            m["order"] += 1
        tx, ty = x["touching"][ix], y["touching"][iy]
        m["touching"] += int(np.count_nonzero(tx != ty))
        both = tx & ty
        m["touching_contacts"] += int(np.count_nonzero(both))
        m["manifold_type"] += int(np.count_nonzero(both & (x["type"][ix] != y["type"][iy])))
        same_n = both & (x["count"][ix] == y["count"][iy])
        m["point_count"] += int(np.count_nonzero(both & (x["count"][ix] != y["count"][iy])))
        m["feature_ids"] += int(np.count_nonzero(same_n & (x["ids"][ix] != y["ids"][iy]).any(axis=1)))
        m["awake"] += int(np.count_nonzero(x["awake"] != y["awake"]))
        after = sum(v for k, v in m.items() if k not in _TOTALS)
        m["worlds_with_any"] += 1 if after > before else 0
    if moved_a is not None and moved_b is not None:
        m["refattened"] = int(np.count_nonzero(moved_a != moved_b))
        m["proxies"] = int(len(moved_a))
    return m


REC_FIELDS = {   # step-record fields (gb_batch_get_step_record): (shift, mask)
    "position_iterations": (0, 0xff),
    "toi_position_iterations": (8, 0xff),
    "toi_events": (16, 0xff),
    "restitution_bias": (24, 1),
    "block_drop": (25, 1),
    "toi_restitution_bias": (26, 1),
    "toi_block_drop": (27, 1),
}


def record_mismatch(W, ra, rb):
    """Bodies whose step records differ.  ``ra``/``rb`` are per-world
    step records ([2, n]: decisions, islands); returns a boolean mask over the
    batch's bodies and the counts per field."""
    n = int(W["body_start"][-1] + W["body_count"][-1]) if len(W) else 0
    mask = np.zeros(n, dtype=bool)
    counts = {k: 0 for k in REC_FIELDS}
    for w, (x, y) in enumerate(zip(ra, rb)):
        b0 = int(W["body_start"][w])
        x, y = x[0], y[0]
        for name, (sh, m) in REC_FIELDS.items():
            d = ((x >> sh) & m) != ((y >> sh) & m)
            counts[name] += int(np.count_nonzero(d))
            mask[b0:b0 + len(x)] |= d
    return mask, counts


def contact_apart(W, F, C32, C64, n_bodies):
    """Bodies of contacts whose touching flag, manifold type, point count or
    feature ids differ between the two steps."""
    mask = np.zeros(n_bodies, dtype=bool)
    for w, (x, y) in enumerate(zip(C32, C64)):
        b0, f0 = int(W["body_start"][w]), int(W["fixture_start"][w])
        kx = (x["fixture_a"].astype(np.int64) << 32) | x["fixture_b"].astype(np.int64)
        ky = (y["fixture_a"].astype(np.int64) << 32) | y["fixture_b"].astype(np.int64)
        _, ix, iy = np.intersect1d(kx, ky, return_indices=True)
        a, b = x[ix], y[iy]
        n = a["m_point_count"]
        ids_a = np.where(np.arange(2)[None, :] < n[:, None], a["p_id"], 0)
        ids_b = np.where(np.arange(2)[None, :] < n[:, None], b["p_id"], 0)
        d = (((a["flags"] ^ b["flags"]) & abi.C_TOUCHING) != 0) | (a["m_point_count"] != b["m_point_count"]) | \
            ((a["m_point_count"] > 0) & (a["m_type"] != b["m_type"])) | (ids_a != ids_b).any(axis=1)
        for fa, fb in zip(a["fixture_a"][d], a["fixture_b"][d]):
            mask[b0 + int(F["body"][f0 + fa])] = True
            mask[b0 + int(F["body"][f0 + fb])] = True
    return mask


def world_errors(W, Ba, Bb):
    """Per world the largest position, angle and velocity difference over its
    dynamic bodies between two body arrays."""
    dyn = Ba["type"] == abi.BODY_DYNAMIC
    dp = np.hypot(Ba["cx"] - Bb["cx"], Ba["cy"] - Bb["cy"])
    da = np.abs(Ba["a"] - Bb["a"])
    dv = np.hypot(Ba["vx"] - Bb["vx"], Ba["vy"] - Bb["vy"])
    out = np.zeros((len(W), 3))
    for w in range(len(W)):
        s = slice(int(W["body_start"][w]), int(W["body_start"][w] + W["body_count"][w]))
        d = dyn[s]
        if d.any():
            out[w] = dp[s][d].max(), da[s][d].max(), dv[s][d].max()
    return out


def _stacked(W, B, P, Cs):
    W2 = W.copy()
    k = 0
    for w, c in enumerate(Cs):
        W2["contact_start"][w], W2["contact_count"][w] = k, len(c)
        k += len(c)
    return W2, B, P, (np.concatenate(Cs) if Cs else np.zeros(0, abi.CONTACT))


def one_step(W, B, F, C, dt, vel_iters, pos_iters, reference=None, launch=(3, 64)):
    """One float32 step and one float64 step from the same float64 state
    (records as ``batch_records`` gives them, fixtures carrying the fat
    AABBs), the float64 one in the float32 step's constraint order.

    ``reference``: optional callable (W, B, F, C, orders) -> (bodies, proxies,
    contacts per world, step records per world) giving the float64 step by
    other means (the CPU restatement); by default the float64 GPU path takes
    it.  Returns a dict: ``errors`` [n_worlds, 3] (largest position, angle,
    velocity difference over each world's dynamic bodies), ``errors_alike``
    (the same over the bodies of islands in which both steps took every
    decision alike: the continuous error of the float32 arithmetic),
    ``mismatch`` (discrete counts, step-record fields included),
    ``bodies_decided_apart`` (bodies of islands in which some decision
    differs: a step-record field or a contact's touching flag, manifold type,
    point count or feature ids), ``decisions_apart`` (how many such decisions:
    step-record fields per body plus bodies of differing contacts)."""
    from .gpu import GpuBatch
    g32 = GpuBatch(W, B, F, contacts=C, precision="f32")
    g32.step(dt, vel_iters, pos_iters, 1, launch_mode=launch[0], block_threads=launch[1], record_order=True)
    orders = [g32.solver_order(w) for w in range(len(W))]
    B32, P32 = g32.bodies(), g32.proxies()
    C32 = [g32.contacts(w) for w in range(len(W))]
    R32 = [g32.step_record(w) for w in range(len(W))]
    if reference is None:
        g64 = GpuBatch(W, B, F, contacts=C, precision="f64")
        g64.step(dt, vel_iters, pos_iters, 1, launch_mode=launch[0], block_threads=launch[1], record_order=True)
        B64, P64 = g64.bodies(), g64.proxies()
        C64 = [g64.contacts(w) for w in range(len(W))]
        R64 = [g64.step_record(w) for w in range(len(W))]
        g64.close()
    else:
        B64, P64, C64, R64 = reference(W, B, F, C, orders)
    g32.close()
    errs = world_errors(W, B32, B64)
    apart, rec_counts = record_mismatch(W, R32, R64)
    capart = contact_apart(W, F, C32, C64, len(B))
    decisions_apart = sum(rec_counts.values()) + int(np.count_nonzero(capart))
    apart |= capart
    # a decision taken apart moves its whole island (Gauss-Seidel couples it):
    # the islands of the solve, as both steps recorded them
    for R in (R32, R64):
        lab = np.full(len(B), -1, dtype=np.int64)
        for w, r in enumerate(R):
            b0 = int(W["body_start"][w])
            isl = r[1].astype(np.int64)
            lab[b0:b0 + len(isl)] = np.where(isl >= 0, b0 + isl, -1)
        hit = np.unique(lab[apart & (lab >= 0)])
        apart |= np.isin(lab, hit) & (lab >= 0)
    Ba, Bb = B32.copy(), B64.copy()
    Ba[apart] = Bb[apart]
    errs_alike = world_errors(W, Ba, Bb)
    moved32 = (P32 != F["aabb"]).any(axis=1)
    moved64 = (P64 != F["aabb"]).any(axis=1)
    d32 = discrete(*_stacked(W, B32, P32, C32))
    d64 = discrete(*_stacked(W, B64, P64, C64))
    mm = mismatch(d32, d64, moved32, moved64)
    mm.update(rec_counts)
    return {"errors": errs, "errors_alike": errs_alike, "mismatch": mm, "bodies_decided_apart": int(apart.sum()),
            "decisions_apart": decisions_apart,
            "f32": (B32, P32, C32, R32), "f64": (B64, P64, C64, R64)}


def drift(W, B, F, M, dt, vel_iters, pos_iters, steps, every, launch=(3, 64)):
    """Float32 and float64 GPU batches stepped from the same initial state for
    ``steps`` steps, each in its own order; every ``every`` steps the
    distribution over dynamic bodies of |dc| (m) and |da| (rad) between them.
    Returns a list of dicts (step, position quantiles, angle quantiles)."""
    from .gpu import GpuBatch
    g32 = GpuBatch(W, B, F, precision="f32", moves=M)
    g64 = GpuBatch(W, B, F, precision="f64", moves=M)
    dyn = B["type"] == abi.BODY_DYNAMIC
    q = (0.5, 0.9, 0.99, 1.0)
    out = []
    done = 0
    while done < steps:
        n = min(every, steps - done)
        g32.step(dt, vel_iters, pos_iters, n, launch_mode=launch[0], block_threads=launch[1])
        g64.step(dt, vel_iters, pos_iters, n, launch_mode=launch[0], block_threads=launch[1])
        done += n
        a, b = g32.bodies(), g64.bodies()
        dp = np.hypot(a["cx"] - b["cx"], a["cy"] - b["cy"])[dyn]
        da = np.abs(a["a"] - b["a"])[dyn]
        aw = (a["flags"] & abi.BODY_AWAKE) != (b["flags"] & abi.BODY_AWAKE)
        out.append({"step": done,
                    "position_m": dict(zip(("p50", "p90", "p99", "max"), np.quantile(dp, q).tolist())),
                    "angle_rad": dict(zip(("p50", "p90", "p99", "max"), np.quantile(da, q).tolist())),
                    "awake_differs": int(np.count_nonzero(aw[dyn]))})
    g32.close()
    g64.close()
    return out

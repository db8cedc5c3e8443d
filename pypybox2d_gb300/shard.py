"""Worlds of a batch spread over ranks (one process per GPU).

Worlds never interact, so a batch shards by world with no exchange during
the step: every rank builds a batch of its own worlds and steps it; only
measurements (times, counts) and results requested by the caller cross
ranks.  ``assign`` balances the ranks by body count (the step's cost grows
with bodies and contacts); ``split`` cuts the record arrays of a batch into
one rank's share; ``gather_bodies`` puts the shares back in batch order on
one rank.
"""
from __future__ import annotations

import numpy as np

from . import abi


def assign(body_counts, world_size: int) -> np.ndarray:
    """Rank of every world: largest worlds first, each to the rank with the
    fewest bodies so far (ties to the lower rank).  Deterministic."""
    counts = np.asarray(body_counts, dtype=np.int64)
    order = np.argsort(-counts, kind="stable")
    load = np.zeros(world_size, dtype=np.int64)
    rank_of = np.empty(len(counts), dtype=np.int32)
    for w in order:
        r = int(np.argmin(load))
        rank_of[w] = r
        load[r] += counts[w]
    return rank_of


def split(W, B, F, M, rank_of, rank: int):
    """Record arrays of the worlds assigned to `rank`, as a batch of their
    own (worlds in batch order), and the batch indices of those worlds."""
    mine = np.nonzero(np.asarray(rank_of) == rank)[0]
    Ws, Bs, Fs, Ms = [], [], [], []
    nb = nf = nm = 0
    for w in mine:
        b0, n_b = int(W["body_start"][w]), int(W["body_count"][w])
        f0, n_f = int(W["fixture_start"][w]), int(W["fixture_count"][w])
        m0, n_m = int(W["move_start"][w]), int(W["move_count"][w])
        wr = W[w:w + 1].copy()
        wr["body_start"], wr["fixture_start"], wr["move_start"] = nb, nf, nm
        Ws.append(wr)
        Bs.append(B[b0:b0 + n_b])
        Fs.append(F[f0:f0 + n_f])
        Ms.append(M[m0:m0 + n_m])
        nb, nf, nm = nb + n_b, nf + n_f, nm + n_m
    if not len(mine):
        return (np.zeros(0, abi.WORLD), np.zeros(0, abi.BODY), np.zeros(0, abi.FIXTURE),
                np.zeros(0, np.int32), mine)
    return np.concatenate(Ws), np.concatenate(Bs), np.concatenate(Fs), np.concatenate(Ms).astype(np.int32), mine


def gather_bodies(W, shard_bodies, shard_worlds, rank_of, group=None):
    """Body records of the whole batch on every rank (torch.distributed
    all_gather_object over `group`), in batch order."""
    import torch.distributed as dist
    parts = [None] * dist.get_world_size(group)
    dist.all_gather_object(parts, (np.asarray(shard_worlds), shard_bodies), group=group)
    out = np.zeros(int(np.sum(W["body_count"])), dtype=abi.BODY)
    for worlds, bodies in parts:
        k = 0
        for w in worlds:
            b0, n_b = int(W["body_start"][w]), int(W["body_count"][w])
            out[b0:b0 + n_b] = bodies[k:k + n_b]
            k += n_b
    return out

"""Worlds spread over two ranks (gloo, CPU): the sharded batch, stepped rank
by rank and gathered, equals the batch stepped whole; the balance and the
max-over-ranks timing reduction work as bench.py uses them.  The per-world
step here is the CPU restatement (oracle/), standing in for the GPU step,
which a call on one GPU cannot run on two ranks."""
import os
import socket
import sys

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

HERE = os.path.dirname(os.path.abspath(__file__))

DT, VI, PI, STEPS = 1.0 / 60.0, 8, 3, 6


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _oracle_step(W, B, F, M, steps):
    import ctypes
    import oracle_lib
    from pypybox2d_gb300 import abi
    lib = oracle_lib.load(False)
    out = np.zeros(len(B), dtype=abi.BODY)
    if len(W) == 0:
        return out
    s, keep = abi.make_scene(W, B, F, None, M)
    h = lib.or_batch_create(ctypes.byref(s))
    lib.or_batch_step(h, DT, VI, PI, steps, 1)
    for w in range(len(W)):
        b0, nb = int(W["body_start"][w]), int(W["body_count"][w])
        part = np.zeros(nb, dtype=abi.BODY)
        lib.or_batch_get_bodies(h, w, part.ctypes.data)
        out[b0:b0 + nb] = part
    lib.or_batch_destroy(h)
    return out


def _rank_main(rank, world_size, port, result_path):
    sys.path.insert(0, HERE)
    sys.path.insert(0, os.path.dirname(HERE))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world_size)
    import torch
    from pypybox2d_gb300 import scenes, shard
    W, B, F, M = scenes.uneven_batch(6, seed=70, counts=[12, 40, 25, 90, 17, 60])
    rank_of = shard.assign(W["body_count"], world_size)
    Ws, Bs, Fs, Ms, mine = shard.split(W, B, F, M, rank_of, rank)
    stepped = _oracle_step(Ws, Bs, Fs, Ms, STEPS)
    whole = shard.gather_bodies(W, stepped, mine, rank_of)
    t = torch.tensor([float(rank + 1)])
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    n = torch.tensor([float(len(Bs))])
    dist.all_reduce(n, op=dist.ReduceOp.SUM)
    if rank == 0:
        np.save(result_path, whole)
        with open(result_path + ".txt", "w") as f:
            f.write(f"{t.item()} {n.item()} {len(B)}")
    dist.destroy_process_group()


def test_sharded_batch_equals_whole_batch(tmp_path):
    from pypybox2d_gb300 import scenes, shard
    W, B, F, M = scenes.uneven_batch(6, seed=70, counts=[12, 40, 25, 90, 17, 60])
    rank_of = shard.assign(W["body_count"], 2)
    loads = [int(W["body_count"][rank_of == r].sum()) for r in range(2)]
    assert sorted(np.unique(rank_of)) == [0, 1] and abs(loads[0] - loads[1]) <= int(W["body_count"].max())
    path = str(tmp_path / "whole.npy")
    mp.spawn(_rank_main, args=(2, _free_port(), path), nprocs=2, join=True)
    got = np.load(path)
    t, n, nb = open(path + ".txt").read().split()
    assert float(t) == 2.0 and int(float(n)) == int(nb) == len(B)
    sys.path.insert(0, HERE)
    want = _oracle_step(W, B, F, M, STEPS)
    assert got.tobytes() == want.tobytes()

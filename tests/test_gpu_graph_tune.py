"""Captured rollouts (gb_graph_capture / gb_graph_launch) and the launch
autotuner (gb_batch_autotune, gb_batch_set_launch_config).

Both change how the step's launches reach the GPU, never what they
compute, so every check is against twin batches stepped the plain way.
Tolerance: none (bit-exact) in both precisions -- the kernels, their order
and their reduction orders are the same; a graph only removes the host from
between launches, and a launch configuration only changes CTA widths,
shared-memory chunk buffers and which solver launch a world goes to.
"""
import os

import numpy as np
import pytest

from pypybox2d_gb300 import abi, scenes

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
DT, VI, PI = 1 / 60, 8, 3
# worlds on both sides of the wide solver launch's 512-body threshold
COUNTS = [700, 40, 15, 300, 550, 20, 120, 1100]


def _golden(scene):
    d = np.load(os.path.join(GOLDEN, scene + ".npz"))
    return d["init_world"], d["init_bodies"], d["init_fixtures"], float(d["dt"][0]), tuple(int(x) for x in d["iters"])


def _same(a, b, what):
    for name in a.dtype.names:
        if name.startswith("_pad"):
            continue
        x, y = a[name], b[name]
        bad = ~((x == y) | ((x != x) & (y != y))) if x.dtype.kind == "f" else (x != y)
        assert not bad.any(), f"{what}.{name} differs at {np.argwhere(bad)[0]}"


def _same_state(a, b, what):
    _same(a.bodies(), b.bodies(), what + " bodies")
    assert np.array_equal(a.contact_counts(), b.contact_counts()), what + " contact counts"
    for w in range(a.n_worlds):
        _same(a.contacts(w), b.contacts(w), f"{what} world {w} contacts")
    assert np.array_equal(a.proxies(), b.proxies()), what + " fat AABBs"


def _twins(records, precision):
    from pypybox2d_gb300.gpu import GpuBatch
    W, B, F, M = records
    return (GpuBatch(W, B, F, precision=precision, moves=M), GpuBatch(W, B, F, precision=precision, moves=M))


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_graph_replays_match_direct_steps(precision):
    """A 10-step graph replayed 3 times equals 30 plain phased steps, with
    a body upload between replays."""
    g_batch, ref = _twins(scenes.uneven_batch(len(COUNTS), seed=3, counts=COUNTS), precision)
    graph = g_batch.capture(DT, VI, PI, n_steps=10, launch_mode=3)
    for rep in range(3):
        graph.launch()
        ref.step(DT, VI, PI, 10, launch_mode=3)
        _same_state(g_batch, ref, f"{precision} replay {rep}")
        if rep == 0:
            # a host edit between replays reaches the next replay
            b = ref.bodies()
            b["vx"][b["type"] == abi.BODY_DYNAMIC] += 0.5
            ref.set_bodies(b)
            g_batch.set_bodies(b)
    assert not g_batch.status().any()
    graph.close()


def test_graph_of_golden_bullets_matches_direct_steps():
    """Time-of-impact events inside a captured rollout (float64)."""
    W, B, F, dt, (vi, pi) = _golden("bullets")
    from pypybox2d_gb300.gpu import GpuBatch
    a, b = GpuBatch(W, B, F, precision="f64"), GpuBatch(W, B, F, precision="f64")
    graph = a.capture(dt, vi, pi, n_steps=20, launch_mode=3, block_threads=64)
    for _ in range(3):
        graph.launch()
        b.step(dt, vi, pi, 20, launch_mode=3, block_threads=64)
    _same_state(a, b, "bullets graph")


def test_graph_capture_rejects_what_it_cannot_capture():
    from pypybox2d_gb300.gpu import GpuBatch
    W, B, F, dt, (vi, pi) = _golden("mixed")
    g = GpuBatch(W, B, F, precision="f64")
    with pytest.raises(abi.GB2DError, match="phased"):
        g.capture(dt, vi, pi, n_steps=4, launch_mode=1)
    with pytest.raises(abi.GB2DError, match="n_steps"):
        g.capture(dt, vi, pi, n_steps=0)
    graph = g.capture(dt, vi, pi, n_steps=2)
    g.close()                      # destroying the batch disarms its graphs
    with pytest.raises(abi.GB2DError, match="destroyed"):
        graph.launch()
    graph.close()


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_launch_configs_compute_the_same_step(precision):
    """Phased-launch configurations (CTA widths, chunk buffers 0-4, the wide
    launch's threshold) give bit-identical states."""
    configs = [(3, 64, 0, 512), (3, 64, 1, 256), (3, 32, 3, 1 << 30), (3, 128, 4, 100), (3, 64, 2, 1024),
               (3, 64, 0, 512, 2), (3, 64, 2, 256, 3), (3, 128, 0, 512, 8)]
    recs = scenes.uneven_batch(len(COUNTS), seed=5, counts=COUNTS)
    from pypybox2d_gb300.gpu import GpuBatch
    W, B, F, M = recs
    ref = GpuBatch(W, B, F, precision=precision, moves=M)
    ref.step(DT, VI, PI, 30, launch_mode=3)
    for cfg in configs:
        g = GpuBatch(W, B, F, precision=precision, moves=M)
        g.set_launch_config(*cfg)
        assert g.launch_config()["pipe_bufs"] == cfg[2]
        g.step(DT, VI, PI, 30, launch_mode=0)
        _same_state(g, ref, f"{precision} config {cfg}")
        assert not g.status().any()
        g.close()


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_world_groups_in_graphs_and_static_scratch(precision):
    """World groups (runs of worlds stepped on streams of their own) inside
    a captured rollout and through the static-scratch entry point compute
    the plain single-stream steps."""
    from pypybox2d_gb300.gpu import GpuBatch
    W, B, F, M = scenes.uneven_batch(len(COUNTS), seed=11, counts=COUNTS)
    ref = GpuBatch(W, B, F, precision=precision, moves=M)
    ref.step(DT, VI, PI, 20, launch_mode=3, block_threads=64)
    g = GpuBatch(W, B, F, precision=precision, moves=M)
    g.set_launch_config(3, 64, 0, 512, 3)
    assert g.launch_config()["groups"] == 3
    graph = g.capture(DT, VI, PI, n_steps=10, launch_mode=0)
    graph.launch()
    g.step_static_scratch(DT, VI, PI, 10, launch_mode=0)
    _same_state(g, ref, f"{precision} groups in a graph, then static scratch")
    graph.close()
    with pytest.raises(abi.GB2DError):
        g.set_launch_config(1, 128, 0, 512, 2)    # groups run the phased launch only


def test_monolithic_mappings_compute_the_same_step_f64():
    """One CTA or one warp per world, as launch configurations, equal the
    phased launch in float64."""
    recs = scenes.uneven_batch(4, seed=7, counts=[600, 30, 200, 12])
    from pypybox2d_gb300.gpu import GpuBatch
    W, B, F, M = recs
    ref = GpuBatch(W, B, F, precision="f64", moves=M)
    ref.step(DT, VI, PI, 20, launch_mode=3)
    for cfg in [(1, 128, 2, 512), (2, 64, 2, 512)]:
        g = GpuBatch(W, B, F, precision="f64", moves=M)
        g.set_launch_config(*cfg)
        g.step(DT, VI, PI, 20, launch_mode=0)
        _same_state(g, ref, f"mapping {cfg}")


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_autotune_keeps_the_state_and_picks_a_runnable_config(precision):
    tuned, ref = _twins(scenes.uneven_batch(len(COUNTS), seed=9, counts=COUNTS), precision)
    tuned.step(DT, VI, PI, 15, launch_mode=3)
    ref.step(DT, VI, PI, 15, launch_mode=3)
    best, trials = tuned.autotune(DT, VI, PI, steps_per_trial=2)
    # the tuner's trial steps leave no trace in the batch
    _same_state(tuned, ref, f"{precision} after autotune")
    ran = [t for t in trials if t["ms_per_step"] >= 0]
    assert len(trials) >= 7 and ran          # stage 1 always; stages 2-3 when the phased launch wins
    assert best["ms_per_step"] == min(t["ms_per_step"] for t in ran)
    assert tuned.launch_config() == best
    # stepping with the tuned configuration (launch_mode 0) continues the
    # same trajectory: exactly in float64 (every mapping), and in float32
    # whenever the tuner kept the phased launch
    tuned.step(DT, VI, PI, 15, launch_mode=0)
    ref.step(DT, VI, PI, 15, launch_mode=3)
    if precision == "f64" or best["launch_mode"] == 3:
        _same_state(tuned, ref, f"{precision} tuned steps")
    assert not tuned.status().any()


def test_wide_launch_threshold_never_takes_grid_worlds_f64():
    """A world run as a cooperative grid (16384+ bodies) stays out of the
    per-world solver launches whatever big_bodies says."""
    from pypybox2d_gb300.gpu import GpuBatch
    W, B, F, M = scenes.large_world(9, 17000)
    ref = GpuBatch(W, B, F, precision="f64", moves=M)
    g = GpuBatch(W, B, F, precision="f64", moves=M)
    g.set_launch_config(3, 64, 2, 1 << 30)
    ref.step(DT, VI, PI, 3, launch_mode=3, block_threads=64)
    g.step(DT, VI, PI, 3, launch_mode=0)
    _same_state(g, ref, "grid world, no wide launch")


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_host_step_in_chunks_matches_upload_step_download(precision):
    """gb_batch_step_host (chunks of worlds uploading, stepping and
    downloading on streams of their own) computes what gb_batch_set_bodies,
    gb_batch_step and gb_batch_get_bodies compute one after the other: with a
    one-group configuration (four chunks) from pageable and from pinned host
    memory, in place (one buffer in and out), with three world groups as the
    chunks, and in a monolithic mapping (the three calls); body state records
    (gb_batch_step_host_state) give the same fields."""
    import torch
    from pypybox2d_gb300.gpu import GpuBatch
    W, B, F, M = scenes.uneven_batch(len(COUNTS), seed=13, counts=COUNTS)
    ref = GpuBatch(W, B, F, precision=precision, moves=M)
    g = GpuBatch(W, B, F, precision=precision, moves=M)
    for b in (ref, g):
        b.set_launch_config(3, 64, 0, 512, 1)
        b.step(DT, VI, PI, 20, launch_mode=0)          # live contacts, bodies asleep and awake

    def three_calls(host, n, mode=0):
        ref.set_bodies(host)
        ref.step(DT, VI, PI, n, launch_mode=mode)
        return ref.bodies()

    host = g.bodies()
    host["vx"][host["type"] == abi.BODY_DYNAMIC] += 0.25             # an edit on the host between steps
    out = g.step_host(host, DT, VI, PI, 5)
    _same(out, three_calls(host, 5), f"{precision} four chunks, pageable")
    _same_state(g, ref, f"{precision} four chunks, device state")

    pinned = torch.empty(len(out) * abi.BODY.itemsize, dtype=torch.uint8, pin_memory=True)
    buf = np.frombuffer(pinned.numpy(), dtype=abi.BODY)
    buf[:] = out
    buf["w"][buf["type"] == abi.BODY_DYNAMIC] *= 0.5
    expect = three_calls(buf.copy(), 3)
    g.step_host(buf, DT, VI, PI, 3, out=buf)
    _same(buf, expect, f"{precision} four chunks, pinned, in place")

    g.set_launch_config(3, 64, 0, 512, 3)
    expect = three_calls(buf.copy(), 4)
    g.step_host(buf, DT, VI, PI, 4, out=buf)
    _same(buf, expect, f"{precision} three world groups")
    _same_state(g, ref, f"{precision} three world groups, device state")

    # body state records (gb_batch_step_host_state): the step-invariant
    # fields stay on the device, the rest goes up and comes back
    def states(full):
        st = np.zeros(len(full), abi.BODY_STATE)
        for name in abi.BODY_STATE.names:
            if not name.startswith("_pad"):
                st[name] = full[name]
        return st

    buf["vy"][buf["type"] == abi.BODY_DYNAMIC] -= 0.125
    st = states(buf)
    expect = three_calls(buf.copy(), 3)
    g.step_host(st, DT, VI, PI, 3, out=st)
    _same(st, states(expect), f"{precision} state records, three world groups")
    buf[:] = expect

    expect = three_calls(buf.copy(), 2, mode=1)
    g.step_host(buf, DT, VI, PI, 2, launch_mode=1, out=buf)
    _same(buf, expect, f"{precision} CTA per world")
    st = states(buf)
    expect = three_calls(buf.copy(), 1, mode=1)
    g.step_host(st, DT, VI, PI, 1, launch_mode=1, out=st)
    _same(st, states(expect), f"{precision} state records, CTA per world")
    assert not g.status().any() and not ref.status().any()
    with pytest.raises(ValueError):
        g.step_host(buf[:-1], DT, VI, PI, 1)
    g.close()
    ref.close()

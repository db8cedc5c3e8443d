"""Benchmark of the World.step hot path on GB300.

Workloads (``--workload``):
  uneven   (default) 8192 worlds whose body counts are log-uniform on
           [10, 2000]: a static 100 x 100 m container of four edges, half
           circles and half convex polygons with random sizes, materials and
           velocities; 1000 steps.
  pyramid  4096 copies of the 20-row pyramid (210 boxes on a ground box),
           every box position jittered by a seeded U(-0.01, 0.01) m; 2000 steps.
  bullets  2048 twenty-box stacks, each hit by 4 bullet circles; 600 steps.
  large    one 100000-body world; 600 steps.
All: dt = 1/60, 8 velocity and 3 position iterations, float32 bulk
arithmetic with float64 positions, angles, sleep timers and time of impact.

Both arms (this one and ``--impl reference``) run the same untimed settle
(``--settle``; uneven and pyramid 300 steps, so the timed window is the
landed, piled steady state) and ``--warmup`` steps, then time ``--steps``
steps; ``config.timed_steps`` names the window and is the same in both.
Here, after the warm-up the launch autotuner (gb_batch_autotune) picks the
launch configuration from trials that leave the state unchanged; the state
at the start of the window is snapshotted on the device
(gb_batch_snapshot), the timed steps replay captured CUDA graphs of
``--graph-steps`` phased steps, and every later leg restores the snapshot
and measures the same steps.  A "step" is one World.step of every world.

Reported (one JSON line on rank 0):
  value    dynamic body-steps/s with the batch resident in HBM (device time,
           CUDA events on the launching stream, max over ranks)
  e2e      the same metric through the C ABI with host buffers: every step
           uploads the bodies' state records (the fields a step reads and
           writes) from pinned host memory, steps, and reads them back, in one
           gb_batch_step_host_state call (chunks of worlds whose copies
           overlap the other chunks' kernels); ``full_records_value``: the
           same with whole body records (gb_batch_step_host);
           ``three_calls_value``: whole records through gb_batch_set_bodies,
           gb_batch_step and gb_batch_get_bodies one after the other
  roofline HBM roofline of the whole step from the algorithmic bytes per
           world-step (152 B per body + shape bytes + 32 B per fixture + 128 B
           per contact, from live counts) over the event-timed step; the
           dominant launch against its own byte model (``kernels``)
  kernels  event-timed device ms per launch slot of the phased step
  autotune the tuner's trials and choice; graph: steps per captured graph and
           the same steps as one plain gb_batch_step call
  cpu_baseline  the CPU restatement (oracle/, C, float64) on the host cores
           stepping a bounded sample of the same worlds from the same state
  plain    the float64 path launched per world, one step per launch
  error    float32 against float64 from identical state on 64 worlds spread
           over the size range (one step, same constraint order): position,
           angle and velocity errors and the discrete-state mismatch counts;
           ``error.drift``: both forms from the same initial state without
           re-syncing, drift distributions at checkpoints

--impl reference runs the CPU restatement of the reference (oracle/) with
all host threads on a bounded sample of the same workload instead.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(HERE, "tests"))

METRIC = "body-steps/s on 1 GB300: batched FP32 vs plain FP64 GPU path at stated step error"
DT = 1.0 / 60.0
VI, PI = 8, 3
DEFAULTS = {"uneven": (8192, 1000), "pyramid": (4096, 2000), "bullets": (2048, 600), "large": (1, 600)}
# untimed steps both arms run before their warm-up and timed window (bodies
# landed and piled: the steady state that most of a 1000-step run is in; the
# bullet batch is timed from the start, while its bullets cross the stacks)
SETTLE_STEPS = {"uneven": 300, "pyramid": 300, "bullets": 0, "large": 20}


def _peaks():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms."""

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for name, v in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"), parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def build_workload(name: str, n_worlds: int, seed: int):
    from pypybox2d_gb300 import scenes
    if name == "pyramid":
        W, B, F, M = scenes.pyramid_batch(n_worlds, rows=20, jitter=0.01, seed=seed)
    elif name == "bullets":
        W, B, F, M = scenes.bullet_batch(n_worlds, seed=seed)
    elif name == "large":
        W, B, F, M = scenes.concat([scenes.large_world(seed + w) for w in range(n_worlds)])
    else:
        W, B, F, M = scenes.uneven_batch(n_worlds, seed=seed)
    return W, B, F, M, WORKLOAD_DESC[name].format(n=n_worlds)


def workload_counts(name: str, n_worlds: int, seed: int) -> np.ndarray:
    """Dynamic bodies of every world of a workload, without building it."""
    from pypybox2d_gb300 import scenes
    if name == "pyramid":
        return np.full(n_worlds, 210, dtype=np.int64)
    if name == "bullets":
        return np.full(n_worlds, 24, dtype=np.int64)
    if name == "large":
        return np.full(n_worlds, 100000, dtype=np.int64)
    return np.array([scenes.uneven_count(seed + w) for w in range(n_worlds)], dtype=np.int64)


def workload_config(name: str, n_worlds: int, seed: int, settle: int, warmup: int, steps: int) -> dict:
    """The `config` both arms print: the workload and the window of steps timed."""
    dyn = workload_counts(name, n_worlds, seed)
    first = settle + warmup + 1
    return {"workload": WORKLOAD_DESC[name].format(n=n_worlds), "worlds_per_gpu": n_worlds,
            "dynamic_bodies_per_gpu": int(dyn.sum()),
            "bodies_per_world": {"min": int(dyn.min()), "mean": float(dyn.mean()), "max": int(dyn.max())},
            "settle_steps": settle, "timed_steps": [first, first + steps - 1],
            "l2": "inputs larger than L2 (129 MB): the batch state is several GiB and each step reads all of it"}


WORKLOAD_DESC = {
    "uneven": ("uneven x{n} per GPU: bodies/world log-uniform on [10,2000] in a 100 m edge box, 50% circles r U(0.25,1) / "
               "50% convex 3-8-gons r U(0.3,1), v N(0,2), w N(0,1), gravity (0,-10), dt=1/60, 8 vel / 3 pos iters, "
               "f32 bulk / f64 positions"),
    "pyramid": ("pyramid x{n} per GPU, 210 boxes/world on a ground box, jitter U(-0.01,0.01) m, dt=1/60, 8 vel / 3 pos iters, "
                "f32 bulk / f64 positions"),
    "bullets": ("bullets x{n} per GPU: 20-box stack (friction 0.3) on a ground box + 4 bullet circles (r 0.1, density 100) "
                "from x=-30, y U(0.5,10), speed U(150,250) m/s, dt=1/60, 8 vel / 3 pos iters, f32 bulk / f64 positions and TOI"),
    "large": ("large world x{n}: 100000 bodies (60% boxes half-extent U(0.2,0.6), 40% circles r U(0.2,0.6), density 1, "
              "friction 0.5) on a jittered 1.5 m grid above a 600 m ground box with 200 m walls, dt=1/60, 8 vel / 3 pos "
              "iters, f32 bulk / f64 positions"),
}


def dynamic_counts(W, B):
    """Dynamic bodies of every world."""
    from pypybox2d_gb300 import abi
    dyn = (B["type"] == abi.BODY_DYNAMIC).astype(np.int64)
    cs = np.concatenate([[0], np.cumsum(dyn)])
    return cs[W["body_start"] + W["body_count"]] - cs[W["body_start"]]


def algorithmic_bytes_per_step(n_bodies, fixtures, n_contacts):
    """152 B per body (read c, a, v, w, mass constants, flags, sleep timer;
    write c, a, c0, a0, v, w, sleep timer, flags) + per fixture its shape
    (polygon and edge: 16 B per vertex for vertex + normal in float32,
    circle 12 B) and its fat AABB read and write (32 B) + 128 B per contact
    (pair indices, manifold read and write, flags)."""
    shape = np.where(fixtures["shape_type"] == 0, 12, fixtures["vertex_count"] * 16)
    return 152.0 * n_bodies + float(np.sum(shape + 32)) + 128.0 * n_contacts


def solve_bytes_per_step(n_bodies, n_constraints, real_bytes=4):
    """Byte model of the solver launch: per body velocity and angular
    velocity read and written (6 reals), position and angle read and
    written (48 B), type/flags and sleep timer (16 B); per constraint the
    solver record read (216 B in float32) and its impulses written back to
    the record and to the contact (32 B)."""
    return n_bodies * (6 * real_bytes + 48 + 16) + n_constraints * (216 + 32)


def pairs_bytes_per_step(fixtures, n_bodies, n_contacts):
    """Byte model of the fixture-sync and pair-finding launch: per body its
    type, flags, pose and sweep start read (64 B); per fixture its shape
    (as in algorithmic_bytes_per_step) and fat AABB read, the new fat AABB
    written (32 B), its move flag and move-buffer entry (8 B); per contact the
    pair key read for the existence check (8 B)."""
    shape = np.where(fixtures["shape_type"] == 0, 12, fixtures["vertex_count"] * 16)
    return 64.0 * n_bodies + float(np.sum(shape + 32 + 32 + 8)) + 8.0 * n_contacts


def group_ranges(counts, n: int):
    """The library's world groups (gb_launch_config.groups): n runs of
    consecutive worlds of about equal body counts, as [w0, w1) ranges."""
    nw = len(counts)
    n = min(n, nw)
    if n < 2:
        return [(0, nw)]
    total, w, acc, out = int(np.sum(counts)), 0, 0, []
    for k in range(n):
        w0, target, last = w, total * (k + 1) // n, nw - (n - 1 - k)
        while True:
            acc += int(counts[w])
            w += 1
            if not (w < last and acc < target):
                break
        if k == n - 1:
            w = nw
        out.append((w0, w))
    return out


def launches_per_step(W, big_bodies: int = 512, groups: int = 1):
    """Kernel launches of one phased step: 13 per world group, plus a second
    solver launch in each group that mixes worlds below and above the wide
    launch's threshold (big_bodies)."""
    n = 0
    for w0, w1 in group_ranges(W["body_count"], groups):
        nbig = int(np.count_nonzero(W["body_count"][w0:w1] >= big_bodies))
        n += 13 + (1 if 0 < nbig < w1 - w0 else 0)
    return n


def cpu_oracle_rate(W, B, F, C, dyn, steps, threads, target_s=8.0):
    """Body-steps/s of the CPU restatement stepping the first worlds of W
    (one world per thread task, all threads)."""
    import oracle_lib
    from pypybox2d_gb300 import abi
    lib = oracle_lib.load(False)
    nw = len(W)
    probe = min(nw, threads)
    s, keep = abi.make_scene(W[:probe], B, F, C, None)
    h = lib.or_batch_create(ctypes.byref(s))
    t = lib.or_batch_step(h, DT, VI, PI, 2, threads)
    lib.or_batch_destroy(h)
    per_world_step = max(t / 2.0 / probe, 1e-7)     # wall seconds per world-step on `threads` threads
    n = int(max(threads, min(nw, target_s / (per_world_step * steps))))
    s, keep = abi.make_scene(W[:n], B, F, C, None)
    h = lib.or_batch_create(ctypes.byref(s))
    t = lib.or_batch_step(h, DT, VI, PI, steps, threads)
    lib.or_batch_destroy(h)
    return float(dyn[:n].sum()) * steps / t, n, t


def run_reference(args):
    """The reference arm: the CPU restatement of World.step (oracle/, float64
    C, bit-exact with the reference's golden vectors) on all host threads,
    stepping the first worlds of the same workload through the same settle,
    warm-up and timed window as the GPU arm."""
    ws, rank, _ = _dist()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    n_worlds = args.worlds or DEFAULTS[args.workload][0]
    steps = args.steps or DEFAULTS[args.workload][1]
    settle = SETTLE_STEPS[args.workload] if args.settle < 0 else args.settle
    cfg = workload_config(args.workload, n_worlds, 0, settle, args.warmup, steps)
    per = {"uneven": 8, "pyramid": 4, "bullets": 8, "large": 1}[args.workload]
    if args.workload == "large":
        from pypybox2d_gb300 import scenes
        W, B, F, M = scenes.large_world(0, n=LARGE_SAMPLE_BODIES)
    else:
        W, B, F, M, _ = build_workload(args.workload, min(n_worlds, per * threads), 0)
    dyn = dynamic_counts(W, B)
    import oracle_lib
    from pypybox2d_gb300 import abi
    lib = oracle_lib.load(False)
    s, keep = abi.make_scene(W, B, F, None, M)
    h = lib.or_batch_create(ctypes.byref(s))
    lib.or_batch_step(h, DT, VI, PI, settle + args.warmup, threads)
    t = lib.or_batch_step(h, DT, VI, PI, steps, threads)
    lib.or_batch_destroy(h)
    value = float(dyn.sum()) * steps / t
    first, last = cfg["timed_steps"]
    if args.workload != "large":
        sample = (f"the first {len(W)} of the {n_worlds} worlds ({int(dyn.sum())} dynamic bodies, the GPU arm's seeds), "
                  f"steps {first}-{last} after {settle} settle and {args.warmup} warm-up steps, one world per thread "
                  f"task, {threads} threads")
    else:
        sample = (f"one {int(dyn.sum())}-body world of the large-world generator, steps {first}-{last}, one thread "
                  f"(a world does not split across threads)")
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "body-steps/s", "n_gpus": ws,
        "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": cfg,
        "cpu_baseline": {"value": value, "unit": "body-steps/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "body-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "CPU restatement of pypybox2d World.step (oracle/, float64 C, pinned bit-exact to the reference's "
                "golden vectors); the reference itself is CPython and does not travel to the GPU box",
    }
    print(json.dumps(out))


LARGE_SAMPLE_BODIES = 20000   # the reference arm's large-world sample (one world on one thread)


def stratified(dyn, n):
    """n worlds spread over the range of body counts (evenly spaced ranks)."""
    order = np.argsort(dyn, kind="stable")
    take = np.unique(np.linspace(0, len(dyn) - 1, min(n, len(dyn))).round().astype(np.int64))
    return np.sort(order[take])


def error_block(batch, F, dyn, settle_label, sample=64):
    """Float32 against float64 from identical state on a stratified sample of
    worlds (one step each, same constraint order), with the discrete-state
    mismatch counts; the float64 side is the float64 GPU path, which is
    bit-exact with the CPU restatement of World.step."""
    from pypybox2d_gb300 import precision
    ws = stratified(dyn, sample)
    W, B, Fw, C = precision.batch_records(batch, F, 1.0 / DT, ws)
    r = precision.one_step(W, B, Fw, C, DT, VI, PI)
    errs, alike, mm = r["errors"], r["errors_alike"], r["mismatch"]
    return {
        "f32_one_step_max_position_error_m": float(alike[:, 0].max()),
        "f32_one_step_max_angle_error_rad": float(alike[:, 1].max()),
        "f32_one_step_max_velocity_error_mps": float(alike[:, 2].max()),
        "per_world_position_error_m": {"median": float(np.median(alike[:, 0])), "p90": float(np.quantile(alike[:, 0], 0.9))},
        "bodies_compared": int(mm["bodies"]),
        "bodies_decided_apart": r["bodies_decided_apart"],
        "max_position_error_all_bodies_m": float(errs[:, 0].max()),
        "target_m": 1e-5,
        "worlds_over_target": int(np.count_nonzero(alike[:, 0] > 1e-5)),
        "discrete_mismatch": mm,
        "state": f"{len(ws)} worlds spread over the body-count range ({int(dyn[ws].min())}-{int(dyn[ws].max())} "
                 f"bodies), {settle_label}; one step each from identical state against the float64 GPU path "
                 f"(bit-exact with the CPU restatement) in the same constraint order",
        "note": "errors over the islands in which both steps took every decision alike (the step record: island "
                "position iterations, TOI position passes and events, restitution and block-solver set-up; and the "
                "contacts' touching flags, manifold types, point counts and feature ids); bodies decided apart are "
                "counted, with the all-bodies maximum beside them",
    }


def drift_block(workload, steps):
    """Float32 and float64 from the same initial state, each in its own order,
    without re-syncing: drift distributions over dynamic bodies."""
    from pypybox2d_gb300 import precision
    if workload == "pyramid":
        W, B, F, M, _ = build_workload("pyramid", 32, 0)
    elif workload == "bullets":
        W, B, F, M, _ = build_workload("bullets", 64, 0)
    else:
        W, B, F, M, _ = build_workload("uneven", 64, 0)
    every = max(1, steps // 5)
    rows = precision.drift(W, B, F, M, DT, VI, PI, steps, every)
    return {"worlds": len(W), "steps": steps, "checkpoints": rows,
            "note": "chaotic stacks: the two forms' trajectories separate over time; these are the distributions of "
                    "the separation, not a per-step error"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=0, help="0 = the workload's default (uneven 1000, pyramid 2000, bullets 600, large 600)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--settle", type=int, default=-1, help="untimed steps before the warm-up, in both arms "
                                                           "(-1 = the workload's: uneven 300, pyramid 300, bullets 0, large 20)")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="uneven", choices=["uneven", "pyramid", "bullets", "large"])
    ap.add_argument("--worlds", type=int, default=0, help="0 = the workload's default (uneven 8192, pyramid 4096, bullets 2048, large 1)")
    ap.add_argument("--precision", default="f32", choices=["f32", "f64"])
    ap.add_argument("--mode", type=int, default=3, help="1 = one CTA per world (monolithic), 2 = one warp per world, "
                                                        "3 = phase kernels over the whole batch")
    ap.add_argument("--threads", type=int, default=64)
    ap.add_argument("--e2e-steps", type=int, default=0, help="steps of the end-to-end leg (0 = the timed steps, up to 50)")
    ap.add_argument("--ktime-steps", type=int, default=20, help="steps of the per-launch timing pass")
    ap.add_argument("--no-extras", action="store_true", help="skip cpu baseline, plain path, error and drift legs")
    ap.add_argument("--drift-steps", type=int, default=-1, help="steps of the drift leg (-1: 1000, pyramid 2000; 0: skip)")
    ap.add_argument("--no-tune", action="store_true", help="skip the launch autotuner (use --mode / --threads)")
    ap.add_argument("--tune-steps", type=int, default=3, help="timed steps per autotuner trial")
    ap.add_argument("--launch-config", default="", help="mode,threads,pipe_bufs,big_bodies[,groups]: pin this "
                                                         "launch configuration instead of tuning")
    ap.add_argument("--graph-steps", type=int, default=50, help="steps per captured CUDA graph in the timed region "
                                                                "(0 = one gb_batch_step call)")
    args = ap.parse_args()

    if args.impl == "reference":
        run_reference(args)
        return
    n_worlds = args.worlds or DEFAULTS[args.workload][0]
    steps = args.steps or DEFAULTS[args.workload][1]
    settle = SETTLE_STEPS[args.workload] if args.settle < 0 else args.settle

    ws, rank, local = _dist()
    import torch
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)

    from pypybox2d_gb300 import abi
    from pypybox2d_gb300.gpu import GpuBatch

    # rank r steps its own worlds (seeded from r x n_worlds): no data-path exchange
    W, B, F, M, desc = build_workload(args.workload, n_worlds, rank * n_worlds)
    dyn = dynamic_counts(W, B)
    cfg_out = workload_config(args.workload, n_worlds, rank * n_worlds, settle, args.warmup, steps)
    batch = GpuBatch(W, B, F, precision=args.precision, moves=M)
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    # settle and warm-up, untimed (the first step also finds the initial contacts)
    if settle + args.warmup > 0:
        batch.step(DT, VI, PI, settle + args.warmup, launch_mode=args.mode, block_threads=args.threads, stream=sh)
    torch.cuda.synchronize()

    # launch autotuner: trials from the warmed-up state, which it restores
    mode, threads = args.mode, args.threads
    tune = None
    if args.launch_config:
        batch.set_launch_config(*[int(x) for x in args.launch_config.split(",")])
        mode, threads = 0, 0
    elif not args.no_tune:
        import time
        t0 = time.time()
        try:
            best, trials = batch.autotune(DT, VI, PI, steps_per_trial=args.tune_steps, stream=sh)
        except abi.GB2DError as ex:   # e.g. no device memory for the arena copy: keep --mode / --threads
            tune = {"unavailable": str(ex)}
        else:
            mode, threads = 0, 0          # steps take the tuned launch configuration
            tune = {"best": best, "trials": len(trials), "steps_per_trial": args.tune_steps,
                    "seconds": round(time.time() - t0, 2),
                    "table": [[t["launch_mode"], t["block_threads"], t["pipe_bufs"], t["big_bodies"], t["groups"],
                               round(t["ms_per_step"], 3)] for t in trials],
                    "columns": ["launch_mode", "block_threads", "pipe_bufs", "big_bodies", "groups", "ms_per_step"]}
    tuned = tune is not None and "best" in tune
    cfg = batch.launch_config() if (tuned or args.launch_config) else {"launch_mode": args.mode,
                                                                      "block_threads": args.threads,
                                                                      "pipe_bufs": 2, "big_bodies": 512, "groups": 1}
    eff_mode = cfg["launch_mode"]

    # the timed steps: captured rollouts of graph_steps phased steps replayed
    # back to back (the remainder, if any, as one plain call)
    graph, graph_info, n_graph = None, None, 0
    if args.graph_steps > 0 and eff_mode == 3:
        g_steps = min(args.graph_steps, steps)
        try:
            graph = batch.capture(DT, VI, PI, n_steps=g_steps, launch_mode=mode, block_threads=threads)
            n_graph = steps // g_steps
            graph_info = {"steps_per_graph": g_steps, "graph_launches": n_graph, "plain_steps": steps - n_graph * g_steps}
        except abi.GB2DError as ex:
            graph_info = {"unavailable": str(ex)}
    rest = steps - (n_graph * graph.n_steps if graph else 0)

    # the state at the start of the timed window: every later leg restores it
    # and measures the same steps
    snap = torch.empty(batch.snapshot_bytes(), dtype=torch.uint8, device=dev)
    batch.snapshot(snap.data_ptr(), snap.numel(), stream=sh)

    def restore():
        batch.restore(snap.data_ptr(), snap.numel(), stream=sh)

    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        barrier()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(n_graph):
            graph.launch(stream=sh)
        if rest:
            batch.step(DT, VI, PI, rest, launch_mode=mode, block_threads=threads, stream=sh)
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
    t = e0.elapsed_time(e1) / 1e3
    if ws > 1:
        import torch.distributed as dist
        tt = torch.tensor([t], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t = float(tt.item())
    status = batch.status()
    counts = batch.contact_counts()
    print(f"[bench] {steps} steps of {n_worlds} worlds: {t:.3f} s", file=sys.stderr, flush=True)
    total_dyn = float(dyn.sum()) * ws
    value = total_dyn * steps / t

    # roofline of the whole step: algorithmic bytes per world-step from live counts
    bytes_step = algorithmic_bytes_per_step(len(B), F, float(np.sum(counts)))
    achieved = bytes_step * steps / t / 1e9
    peak, peak_kind = _peaks()

    # per-launch device times over the first steps of the same window
    # (separate pass, one host wait per step)
    kt = {}
    if eff_mode == 3 and args.ktime_steps > 0:
        restore()
        batch.step(DT, VI, PI, min(args.ktime_steps, steps), launch_mode=mode, block_threads=threads, stream=sh,
                   kernel_times=True)
        torch.cuda.synchronize()
        tot, nsteps = batch.kernel_times()
        kt = {k: v / max(nsteps, 1) for k, v in tot.items()}
    kernels = None
    if kt:
        ksum = sum(kt.values())
        top = max(kt, key=kt.get)
        kernels = {"ms_per_launch": {k: round(v, 4) for k, v in kt.items()},
                   "share": {k: round(v / ksum, 4) for k, v in kt.items()},
                   "dominant": top, "timed_steps": min(args.ktime_steps, steps),
                   "window": "the first steps of the timed window, restored from its snapshot"}
        if top == "solve":
            ncons = float(np.sum(counts))   # touching contacts bound the constraints
            sb = solve_bytes_per_step(len(B), ncons, 4 if args.precision == "f32" else 8)
            kernels["dominant_roofline"] = {"bound": "hbm", "achieved": sb / (kt[top] / 1e3) / 1e9, "peak": peak,
                                            "unit": "GB/s", "frac": sb / (kt[top] / 1e3) / 1e9 / peak,
                                            "algorithmic_bytes_per_launch": sb}
        elif top == "sync_pairs":
            pb = pairs_bytes_per_step(F, len(B), float(np.sum(counts)))
            kernels["dominant_roofline"] = {"bound": "hbm", "achieved": pb / (kt[top] / 1e3) / 1e9, "peak": peak,
                                            "unit": "GB/s", "frac": pb / (kt[top] / 1e3) / 1e9 / peak,
                                            "algorithmic_bytes_per_launch": pb}

    # the same steps as one plain gb_batch_step call, for the graphs' effect
    if graph is not None:
        nd = min(steps, 100)
        restore()
        e6, e7 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e6.record(stream)
        batch.step(DT, VI, PI, nd, launch_mode=mode, block_threads=threads, stream=sh)
        e7.record(stream)
        torch.cuda.synchronize()
        graph_info["plain_call_ms_per_step"] = e6.elapsed_time(e7) / nd
        graph_info["plain_call_steps"] = nd

    # e2e through the C ABI with pinned host buffers, on the same window
    restore()
    e2e_steps = args.e2e_steps or min(steps, 50)
    n_b = len(B)
    pinned = torch.empty(n_b * abi.BODY.itemsize, dtype=torch.uint8, pin_memory=True)
    host = np.frombuffer(pinned.numpy(), dtype=abi.BODY)
    lib = batch.lib
    host[:] = batch.bodies(stream=sh)
    ptr = pinned.data_ptr()
    opts = abi.StepOpts(DT, VI, PI, 1, mode, threads, 0)

    def e2e_leg(one_step):
        e2 = torch.cuda.Event(enable_timing=True)
        e3 = torch.cuda.Event(enable_timing=True)
        barrier()
        torch.cuda.synchronize()
        e2.record(stream)
        for _ in range(e2e_steps):
            one_step()
        e3.record(stream)
        torch.cuda.synchronize()
        barrier()
        return total_dyn * e2e_steps / (e2.elapsed_time(e3) / 1e3)

    def chunked():      # gb_batch_step_host: chunks of worlds upload, step and download on streams of their own
        abi.check(lib.gb_batch_step_host(batch.h, ptr, ptr, n_b, ctypes.byref(opts), ctypes.c_void_p(sh)))

    def three_calls():  # the same round trip as three calls on one stream
        abi.check(lib.gb_batch_set_bodies(batch.h, ptr, n_b, ctypes.c_void_p(sh)))
        abi.check(lib.gb_batch_step(batch.h, ctypes.byref(opts), ctypes.c_void_p(sh)))
        abi.check(lib.gb_batch_get_bodies(batch.h, ptr, n_b, ctypes.c_void_p(sh)))

    pinned_s = torch.empty(n_b * abi.BODY_STATE.itemsize, dtype=torch.uint8, pin_memory=True)
    host_s = np.frombuffer(pinned_s.numpy(), dtype=abi.BODY_STATE)
    for name in abi.BODY_STATE.names:
        if not name.startswith("_pad"):
            host_s[name] = host[name]
    ptr_s = pinned_s.data_ptr()

    def chunked_state():  # gb_batch_step_host_state: the fields a step changes, same chunks
        abi.check(lib.gb_batch_step_host_state(batch.h, ptr_s, ptr_s, n_b, ctypes.byref(opts), ctypes.c_void_p(sh)))

    e2e_value = e2e_leg(chunked_state)
    restore()
    e2e_full = e2e_leg(chunked)
    restore()
    host[:] = batch.bodies(stream=sh)
    e2e_three = e2e_leg(three_calls)

    def ms_of(fn, reps=3):
        ea = torch.cuda.Event(enable_timing=True)
        eb = torch.cuda.Event(enable_timing=True)
        fn()                    # untimed: a first copy into a new buffer maps its pages
        torch.cuda.synchronize()
        ea.record(stream)
        for _ in range(reps):
            fn()
        eb.record(stream)
        torch.cuda.synchronize()
        return ea.elapsed_time(eb) / reps

    # where the round trip's time goes: the bare copies of the records, and
    # each half of the three-call form (copy plus unpack and candidate-flag
    # refresh; pack plus copy)
    restore()
    dbuf = torch.empty(n_b * abi.BODY.itemsize, dtype=torch.uint8, device=local)
    h2d_ms = ms_of(lambda: dbuf.copy_(pinned, non_blocking=True))    # torch's current stream is `stream`
    d2h_ms = ms_of(lambda: pinned.copy_(dbuf, non_blocking=True))
    host[:] = batch.bodies(stream=sh)
    set_ms = ms_of(lambda: abi.check(lib.gb_batch_set_bodies(batch.h, ptr, n_b, ctypes.c_void_p(sh))))
    get_ms = ms_of(lambda: abi.check(lib.gb_batch_get_bodies(batch.h, ptr, n_b, ctypes.c_void_p(sh))))
    del dbuf
    e2e_breakdown = {"h2d_copy_ms": h2d_ms, "d2h_copy_ms": d2h_ms, "set_bodies_ms": set_ms, "get_bodies_ms": get_ms,
                     "h2d_gbs": n_b * abi.BODY.itemsize / h2d_ms / 1e6, "d2h_gbs": n_b * abi.BODY.itemsize / d2h_ms / 1e6}

    out = {
        "metric": METRIC, "value": value, "unit": "body-steps/s", "n_gpus": ws, "steps": steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t / steps, "higher_is_better": True, "scaling": "weak",
        "world_steps_per_s": float(n_worlds) * ws * steps / t,
        "vs_baseline": None, "dtype": args.precision, "data": "synthetic",
        "config": cfg_out,
        "launch": {"launch_config": cfg,
                   "form": {1: "one persistent launch per timed region, one CTA per world",
                            2: "one persistent launch per timed region, one warp per world",
                            3: f"{launches_per_step(W, cfg['big_bodies'], cfg['groups'])} launches per step (batch-wide + "
                               f"per-world" + (f"; {cfg['groups']} world groups on streams of their own" if cfg['groups'] > 1
                                                else "") + ")"
                            + (f", captured as CUDA graphs of {graph.n_steps} steps" if graph else "")}[eff_mode],
                   "arena_gib": round(batch.arena_bytes() / 2**30, 2),
                   "mean_contacts_per_world": float(np.mean(counts))},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None, "peak_kind": peak_kind,
                     "kernel": f"whole step ({launches_per_step(W, cfg['big_bodies'], cfg['groups'])} launches)",
                     "algorithmic_bytes_per_step": bytes_step,
                     "traffic_note": "DRAM bytes are measured by ncu on a smaller case and kept in profiles/, "
                                     "not read into this line"},
        "kernels": kernels,
        "e2e": {"value": e2e_value, "unit": "body-steps/s", "h2d_bytes_per_step": n_b * abi.BODY_STATE.itemsize,
                "d2h_bytes_per_step": n_b * abi.BODY_STATE.itemsize, "steps": e2e_steps,
                "window": "the first steps of the timed window, restored from its snapshot",
                "entry": "gb_batch_step_host_state (gb_body_state records, the fields a step reads and writes, from "
                         "and to one pinned host buffer; chunks of worlds on streams of their own)",
                "full_records_value": e2e_full, "full_records_bytes_per_step": n_b * abi.BODY.itemsize,
                "three_calls_value": e2e_three, "breakdown": e2e_breakdown},
        "gpu_launches": launches_per_step(W, cfg["big_bodies"], cfg["groups"]) * steps if eff_mode == 3 else 1,
        "autotune": tune,
        "graph": graph_info,
        "clocks": clocks.summary(),
        "status_nonzero_worlds": int(np.count_nonzero(status)),
    }

    if rank == 0 and not args.no_extras:
        from pypybox2d_gb300 import precision
        restore()
        threads_cpu = os.cpu_count() or 1
        cpu_steps = min(steps, 20)
        n_cpu = min(n_worlds, 64 * threads_cpu)
        Wc, Bc, Fc, Cc = precision.batch_records(batch, F, 1.0 / DT, np.arange(n_cpu))
        rate, n, tcpu = cpu_oracle_rate(Wc, Bc, Fc, Cc, dyn, cpu_steps, threads_cpu, target_s=8.0)
        first = cfg_out["timed_steps"][0]
        out["cpu_baseline"] = {"value": rate, "unit": "body-steps/s", "cores": threads_cpu, "kind": "port",
                               "sample": f"first {n} of the {n_worlds} worlds, steps {first}-{first + cpu_steps - 1} "
                                         f"(from the timed window's start state; {tcpu:.1f} s, {threads_cpu} threads, "
                                         f"float64 C restatement)"}
        # plain float64 path: one world per batch, one launch per world-step,
        # from the same state
        n_plain, plain_steps = min(16, n_worlds), 5
        plain = []
        for w in range(n_plain):
            Wp, Bp, Fp, Cp = precision.batch_records(batch, F, 1.0 / DT, [w])
            plain.append(GpuBatch(Wp, Bp, Fp, contacts=Cp, precision="f64"))
        for p in plain:
            p.step(DT, VI, PI, 1, stream=sh)
        torch.cuda.synchronize()
        e4, e5 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e4.record(stream)
        for _ in range(plain_steps):
            for p in plain:
                p.step(DT, VI, PI, 1, stream=sh)
        e5.record(stream)
        torch.cuda.synchronize()
        tp_ = e4.elapsed_time(e5) / 1e3
        plain_rate = float(dyn[:n_plain].sum()) * plain_steps / tp_
        out["plain_f64_per_world"] = {"value": plain_rate, "unit": "body-steps/s",
                                      "sample": f"first {n_plain} worlds ({int(dyn[:n_plain].sum())} bodies) x "
                                                f"{plain_steps} steps from the timed window's start state, one launch "
                                                f"per world-step",
                                      "batched_over_plain": value / plain_rate}
        out["error"] = error_block(batch, F, dyn, f"at the timed window's start (step {first})")
        drift_steps = args.drift_steps if args.drift_steps >= 0 else (2000 if args.workload == "pyramid" else 1000)
        if drift_steps > 0 and args.workload != "large":
            out["error"]["drift"] = drift_block(args.workload, drift_steps)
    if rank == 0:
        print(json.dumps(out))
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

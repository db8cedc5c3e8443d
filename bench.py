"""Benchmark of the World.step hot path on GB300.

Workloads (``--workload``):
  uneven   (default) 8192 worlds whose body counts are log-uniform on
           [10, 2000]: a static 100 x 100 m container of four edges, half
           circles and half convex polygons with random sizes, materials and
           velocities; 1000 steps.
  pyramid  4096 copies of the 20-row pyramid (210 boxes on a ground box),
           every box position jittered by a seeded U(-0.01, 0.01) m; 2000 steps.
Both: dt = 1/60, 8 velocity and 3 position iterations, float32 bulk
arithmetic with float64 positions, angles, sleep timers and time of impact.
After the warm-up the launch autotuner (gb_batch_autotune) picks the launch
configuration from trials that start from the warmed-up state and leave it
unchanged; the timed steps then replay captured CUDA graphs of
``--graph-steps`` phased steps (12-13 launches each).  A "step" is one
World.step of every world of the batch.

Reported (one JSON line on rank 0):
  value    dynamic body-steps/s with the batch resident in HBM (device time,
           CUDA events on the launching stream, max over ranks)
  e2e      the same metric through the C ABI with host buffers: every step
           uploads the body records from pinned host memory
           (gb_batch_set_bodies), steps, and reads them back (gb_batch_get_bodies)
  roofline HBM roofline of the whole step from the algorithmic bytes per
           world-step (152 B per body + shape bytes + 32 B per fixture + 128 B
           per contact, from live counts) over the event-timed step, and of
           the dominant launch with its own byte model (``kernels``)
  kernels  event-timed device ms per launch slot of the phased step
  autotune the tuner's trials and choice; graph: steps per captured graph and
           the same steps as one plain gb_batch_step call
  cpu_baseline  the CPU restatement (oracle/, C, float64) on the host cores
           stepping a bounded sample of the same worlds
  plain    the float64 path launched per world, one step per launch
  error    float32 position error after one step against the float64
           restatement from identical state, solved in the same order

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
SETTLE_STEPS = {"uneven": 300, "pyramid": 300, "bullets": 0, "large": 20}   # reference arm: untimed steps before its sample


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
        desc = (f"pyramid x{n_worlds} per GPU, 210 boxes/world on a ground box, jitter U(-0.01,0.01) m, "
                f"dt=1/60, 8 vel / 3 pos iters, f32 bulk / f64 positions")
    elif name == "bullets":
        W, B, F, M = scenes.bullet_batch(n_worlds, seed=seed)
        desc = (f"bullets x{n_worlds} per GPU: 20-box stack (friction 0.3) on a ground box + 4 bullet circles "
                f"(r 0.1, density 100) from x=-30, y U(0.5,10), speed U(150,250) m/s, dt=1/60, 8 vel / 3 pos iters, "
                f"f32 bulk / f64 positions and TOI")
    elif name == "large":
        W, B, F, M = scenes.concat([scenes.large_world(seed + w) for w in range(n_worlds)])
        desc = (f"large world x{n_worlds}: 100000 bodies (60% boxes half-extent U(0.2,0.6), 40% circles r U(0.2,0.6), "
                f"density 1, friction 0.5) on a jittered 1.5 m grid above a 600 m ground box with 200 m walls, "
                f"dt=1/60, 8 vel / 3 pos iters, f32 bulk / f64 positions")
    else:
        W, B, F, M = scenes.uneven_batch(n_worlds, seed=seed)
        desc = (f"uneven x{n_worlds} per GPU: bodies/world log-uniform on [10,2000] in a 100 m edge box, "
                f"50% circles r U(0.25,1) / 50% convex 3-8-gons r U(0.3,1), v N(0,2), w N(0,1), gravity (0,-10), "
                f"dt=1/60, 8 vel / 3 pos iters, f32 bulk / f64 positions")
    return W, B, F, M, desc


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


def launches_per_step(W, big_bodies: int = 512):
    """Kernel launches of one phased step: 12, plus a second solver launch
    when the batch mixes worlds below and above the wide launch's threshold
    (big_bodies)."""
    nbig = int(np.count_nonzero(W["body_count"] >= big_bodies))
    return 12 + (1 if 0 < nbig < len(W) else 0)


def world_slice(W, B, F, M, w):
    """Records of world w of a batch, as a one-world batch."""
    b0, nb = int(W["body_start"][w]), int(W["body_count"][w])
    f0, nf = int(W["fixture_start"][w]), int(W["fixture_count"][w])
    m0, nm = int(W["move_start"][w]), int(W["move_count"][w])
    Wi = W[w:w + 1].copy()
    Wi["body_start"] = 0
    Wi["fixture_start"] = 0
    Wi["move_start"] = 0
    return Wi, B[b0:b0 + nb].copy(), F[f0:f0 + nf].copy(), M[m0:m0 + nm].copy()


def device_state(batch, W, F, n):
    """Records of the first n worlds of a device batch as it stands (bodies,
    fat AABBs, contacts), ready to continue on the CPU restatement."""
    from pypybox2d_gb300 import abi
    B = batch.bodies()
    F2 = F.copy()
    F2["aabb"] = batch.proxies()
    Cs, W2 = [], W[:n].copy()
    k = 0
    for w in range(n):
        c = batch.contacts(w)
        W2["contact_start"][w], W2["contact_count"][w] = k, len(c)
        k += len(c)
        Cs.append(c)
    W2["flags"] = W2["flags"] & np.uint32(0xFFFFFFFF ^ abi.W_NEW_FIXTURE)
    W2["move_count"] = 0
    W2["inv_dt0"] = 1.0 / DT
    return W2, B, F2, np.concatenate(Cs) if Cs else np.zeros(0, abi.CONTACT)


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
    ws, rank, _ = _dist()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    n_worlds = args.worlds or DEFAULTS[args.workload][0]
    n = min(n_worlds, 4 * threads if args.workload == "uneven" else 2 * threads)
    W, B, F, M, desc = build_workload(args.workload, n, 0)
    dyn = dynamic_counts(W, B)
    import oracle_lib
    from pypybox2d_gb300 import abi
    lib = oracle_lib.load(False)
    s, keep = abi.make_scene(W, B, F, None, M)
    h = lib.or_batch_create(ctypes.byref(s))
    # settle the sample like the timed GPU window (bodies landed and piled)
    settle = SETTLE_STEPS[args.workload]
    lib.or_batch_step(h, DT, VI, PI, settle, threads)
    for _ in range(args.warmup):
        lib.or_batch_step(h, DT, VI, PI, 1, threads)
    steps = min(args.steps or DEFAULTS[args.workload][1], 10)
    t = 0.0
    for _ in range(steps):
        t += lib.or_batch_step(h, DT, VI, PI, 1, threads)
    lib.or_batch_destroy(h)
    value = float(dyn.sum()) * steps / t
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "body-steps/s", "n_gpus": ws,
        "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"first {len(W)} worlds of: {desc}", "worlds": len(W), "dynamic_bodies": int(dyn.sum())},
        "cpu_baseline": {"value": value, "unit": "body-steps/s", "cores": threads, "kind": "port",
                         "sample": f"{len(W)} worlds x {steps} steps after {settle} settling and {args.warmup} "
                                   f"warm-up steps, "
                                   f"one world per thread task, {threads} threads"},
        "e2e": {"value": value, "unit": "body-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "CPU restatement of pypybox2d World.step (oracle/, float64 C, pinned bit-exact to the reference's "
                "golden vectors); the reference itself is CPython and is not on the GPU box",
    }
    print(json.dumps(out))


def f32_step_error(W, B, F, M, w, settle_steps=60):
    """Position/angle error of one float32 step against the float64
    restatement, both started from the float64 state of world w after
    `settle_steps` steps (bodies, fat AABBs and contacts) and solving in the
    same constraint order."""
    import oracle_lib
    from pypybox2d_gb300 import abi
    from pypybox2d_gb300.gpu import GpuBatch
    Wi, Bi, Fi, Mi = world_slice(W, B, F, M, w)
    g64 = GpuBatch(Wi, Bi, Fi, precision="f64", moves=Mi)
    g64.step(DT, VI, PI, settle_steps)
    st, C = g64.bodies(), g64.contacts(0)
    F2 = Fi.copy()
    F2["aabb"] = g64.proxies()
    W2 = Wi.copy()
    W2["flags"] = W2["flags"] & np.uint32(0xFFFFFFFF ^ abi.W_NEW_FIXTURE)
    W2["move_count"] = 0
    W2["contact_count"] = len(C)
    W2["inv_dt0"] = 1.0 / DT
    g32 = GpuBatch(W2, st, F2, contacts=C, precision="f32")
    g32.step(DT, VI, PI, 1, record_order=True)
    orc = oracle_lib.OracleWorld(W2, st, F2, contacts=C, libm=False)
    orc.step(DT, VI, PI, order=g32.solver_order(0))
    a, b = g32.bodies(), orc.bodies()
    return {"f32_one_step_max_position_error_m": float(np.hypot(a["cx"] - b["cx"], a["cy"] - b["cy"]).max()),
            "f32_one_step_max_angle_error_rad": float(np.abs(a["a"] - b["a"]).max()),
            "f32_one_step_max_velocity_error_mps": float(np.hypot(a["vx"] - b["vx"], a["vy"] - b["vy"]).max()),
            "target_m": 1e-5,
            "state": f"world {w} ({len(Bi)} bodies, {len(C)} contacts) after {settle_steps} float64 steps; "
                     f"one step each from identical state, same constraint order"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=0, help="0 = the workload's default (uneven 1000, pyramid 2000, bullets 600, large 600)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="uneven", choices=["uneven", "pyramid", "bullets", "large"])
    ap.add_argument("--worlds", type=int, default=0, help="0 = the workload's default (uneven 8192, pyramid 4096, bullets 2048, large 1)")
    ap.add_argument("--precision", default="f32", choices=["f32", "f64"])
    ap.add_argument("--mode", type=int, default=3, help="1 = one CTA per world (monolithic), 2 = one warp per world, "
                                                        "3 = phase kernels over the whole batch")
    ap.add_argument("--threads", type=int, default=64)
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--ktime-steps", type=int, default=20, help="steps of the per-launch timing pass")
    ap.add_argument("--no-extras", action="store_true", help="skip cpu baseline, plain path and error legs")
    ap.add_argument("--no-tune", action="store_true", help="skip the launch autotuner (use --mode / --threads)")
    ap.add_argument("--tune-steps", type=int, default=3, help="timed steps per autotuner trial")
    ap.add_argument("--launch-config", default="", help="mode,threads,pipe_bufs,big_bodies: pin this launch "
                                                         "configuration instead of tuning")
    ap.add_argument("--graph-steps", type=int, default=50, help="steps per captured CUDA graph in the timed region "
                                                                "(0 = one gb_batch_step call)")
    args = ap.parse_args()

    if args.impl == "reference":
        run_reference(args)
        return
    n_worlds = args.worlds or DEFAULTS[args.workload][0]
    steps = args.steps or DEFAULTS[args.workload][1]

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
    batch = GpuBatch(W, B, F, precision=args.precision, moves=M)
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    # warm-up (also finds the initial contacts)
    batch.step(DT, VI, PI, args.warmup, launch_mode=args.mode, block_threads=args.threads, stream=sh)
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
                    "table": [[t["launch_mode"], t["block_threads"], t["pipe_bufs"], t["big_bodies"],
                               round(t["ms_per_step"], 3)] for t in trials],
                    "columns": ["launch_mode", "block_threads", "pipe_bufs", "big_bodies", "ms_per_step"]}
    tuned = tune is not None and "best" in tune
    cfg = batch.launch_config() if (tuned or args.launch_config) else {"launch_mode": args.mode,
                                                                      "block_threads": args.threads,
                                                                      "pipe_bufs": 2, "big_bodies": 512}
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
    traffic = None
    tp = os.path.join(HERE, "profiles", f"traffic_{args.workload}.txt")
    if os.path.exists(tp) and args.precision == "f32":
        for ln in open(tp):
            if ln.startswith("dram_bytes_per_step:"):
                traffic = float(ln.split(":")[1])

    # per-launch device times (separate pass, one host wait per step)
    kt = {}
    if eff_mode == 3 and args.ktime_steps > 0:
        batch.step(DT, VI, PI, args.ktime_steps, launch_mode=mode, block_threads=threads, stream=sh, kernel_times=True)
        torch.cuda.synchronize()
        tot, nsteps = batch.kernel_times()
        kt = {k: v / max(nsteps, 1) for k, v in tot.items()}
    kernels = None
    if kt:
        ksum = sum(kt.values())
        top = max(kt, key=kt.get)
        kernels = {"ms_per_launch": {k: round(v, 4) for k, v in kt.items()},
                   "share": {k: round(v / ksum, 4) for k, v in kt.items()},
                   "dominant": top, "timed_steps": args.ktime_steps}
        if top == "solve":
            ncons = float(np.sum(counts))   # touching contacts bound the constraints
            sb = solve_bytes_per_step(len(B), ncons, 4 if args.precision == "f32" else 8)
            kernels["dominant_roofline"] = {"bound": "hbm", "achieved": sb / (kt[top] / 1e3) / 1e9, "peak": peak,
                                            "unit": "GB/s", "frac": sb / (kt[top] / 1e3) / 1e9 / peak,
                                            "algorithmic_bytes_per_launch": sb}

    # the same steps as one plain gb_batch_step call, for the graphs' effect
    if graph is not None:
        nd = min(steps, 100)
        e6, e7 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e6.record(stream)
        batch.step(DT, VI, PI, nd, launch_mode=mode, block_threads=threads, stream=sh)
        e7.record(stream)
        torch.cuda.synchronize()
        graph_info["plain_call_ms_per_step"] = e6.elapsed_time(e7) / nd
        graph_info["plain_call_steps"] = nd

    # e2e through the C ABI with pinned host buffers
    n_b = len(B)
    pinned = torch.empty(n_b * abi.BODY.itemsize, dtype=torch.uint8, pin_memory=True)
    host = np.frombuffer(pinned.numpy(), dtype=abi.BODY)
    lib = batch.lib
    host[:] = batch.bodies(stream=sh)
    ptr = pinned.data_ptr()
    e2 = torch.cuda.Event(enable_timing=True)
    e3 = torch.cuda.Event(enable_timing=True)
    opts = abi.StepOpts(DT, VI, PI, 1, mode, threads, 0)
    barrier()
    torch.cuda.synchronize()
    e2.record(stream)
    for _ in range(args.e2e_steps):
        abi.check(lib.gb_batch_set_bodies(batch.h, ptr, n_b, ctypes.c_void_p(sh)))
        abi.check(lib.gb_batch_step(batch.h, ctypes.byref(opts), ctypes.c_void_p(sh)))
        abi.check(lib.gb_batch_get_bodies(batch.h, ptr, n_b, ctypes.c_void_p(sh)))
    e3.record(stream)
    torch.cuda.synchronize()
    barrier()
    te = e2.elapsed_time(e3) / 1e3
    e2e_value = total_dyn * args.e2e_steps / te

    out = {
        "metric": METRIC, "value": value, "unit": "body-steps/s", "n_gpus": ws, "steps": steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t / steps, "higher_is_better": True, "scaling": "weak",
        "world_steps_per_s": float(n_worlds) * ws * steps / t,
        "vs_baseline": None, "dtype": args.precision, "data": "synthetic",
        "config": {"workload": desc, "worlds_per_gpu": n_worlds, "dynamic_bodies_per_gpu": int(dyn.sum()),
                   "bodies_per_world": {"min": int(dyn.min()), "mean": float(dyn.mean()), "max": int(dyn.max())},
                   "launch": {1: "one persistent launch per timed region, one CTA per world",
                              2: "one persistent launch per timed region, one warp per world",
                              3: f"{launches_per_step(W, cfg['big_bodies'])} launches per step (batch-wide + per-world)"
                              + (f", captured as CUDA graphs of {graph.n_steps} steps" if graph else "")}[eff_mode],
                   "launch_config": cfg,
                   "l2": f"inputs larger than L2: {batch.arena_bytes() / 2**30:.2f} GiB resident per GPU",
                   "mean_contacts_per_world": float(np.mean(counts))},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_kind": peak_kind,
                     "kernel": f"whole step ({launches_per_step(W, cfg['big_bodies'])} launches)",
                     "algorithmic_bytes_per_step": bytes_step},
        "kernels": kernels,
        "e2e": {"value": e2e_value, "unit": "body-steps/s", "h2d_bytes_per_step": n_b * abi.BODY.itemsize,
                "d2h_bytes_per_step": n_b * abi.BODY.itemsize, "steps": args.e2e_steps},
        "gpu_launches": launches_per_step(W, cfg["big_bodies"]) * steps if eff_mode == 3 else 1,
        "autotune": tune,
        "graph": graph_info,
        "clocks": clocks.summary(),
        "status_nonzero_worlds": int(np.count_nonzero(status)),
    }

    if rank == 0 and not args.no_extras:
        threads = os.cpu_count() or 1
        cpu_steps = 20
        n_cpu = min(n_worlds, 64 * threads)
        Wc, Bc, Fc, Cc = device_state(batch, W, F, n_cpu)
        rate, n, tcpu = cpu_oracle_rate(Wc, Bc, Fc, Cc, dyn, cpu_steps, threads, target_s=8.0)
        out["cpu_baseline"] = {"value": rate, "unit": "body-steps/s", "cores": threads, "kind": "port",
                               "sample": f"first {n} of the {n_worlds} worlds x {cpu_steps} steps, continuing from "
                                         f"the batch's state after the timed steps ({tcpu:.1f} s, {threads} threads, "
                                         f"float64 C restatement)"}
        # plain float64 path: one world per batch, one launch per world-step
        n_plain, plain_steps = min(16, n_worlds), 5
        plain = [GpuBatch(*world_slice(W, B, F, M, w)[:3], precision="f64", moves=world_slice(W, B, F, M, w)[3])
                 for w in range(n_plain)]
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
                                                f"{plain_steps} steps, one launch per world-step",
                                      "batched_over_plain": value / plain_rate}
        wi = int(np.argmax(dyn >= 200)) if (dyn >= 200).any() else 0
        out["error"] = f32_step_error(W, B, F, M, wi)
    if rank == 0:
        print(json.dumps(out))
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

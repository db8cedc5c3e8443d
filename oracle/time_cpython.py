"""TEST INFRASTRUCTURE: the reference itself (CPython pypybox2d with its C
extension `_common`, built by oracle/build_ref.sh) against the oracle port on
the same uneven worlds and steps, in the container that holds the reference
source (it cannot travel to the GPU machine, so the bench's reference arm times
the port; this script gives the factor between the two).

Usage:  GB2D_REFERENCE=<pypybox2d source tree> python oracle/time_cpython.py [n_worlds]

Each of n_worlds uneven worlds (the bench's generator, world w from seed w)
is built through the reference's API (tests/golden/make_golden.py
scene_uneven), settled for SETTLE steps and timed for TIMED steps, one world
per process; the port steps the same worlds on one thread.  Prints one JSON
line: CPython body-steps/s per core, the port's, and their ratio.
"""
import ctypes
import json
import multiprocessing as mp
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "tests"))
sys.path.insert(0, os.path.join(REPO, "tests", "golden"))
SETTLE, TIMED = 305, 20


def reference_world(w):
    import make_golden as mg
    from pypybox2d_gb300 import scenes
    b2 = mg.load_reference(os.environ["GB2D_REFERENCE"])
    n = scenes.uneven_count(w)
    world = mg.scene_uneven(b2, seed=w, n=n)
    for _ in range(SETTLE):
        world.step(1 / 60, 8, 3)
    t = time.perf_counter()
    for _ in range(TIMED):
        world.step(1 / 60, 8, 3)
    return w, n, time.perf_counter() - t


def main():
    if "GB2D_REFERENCE" not in os.environ:
        raise SystemExit("set GB2D_REFERENCE to the pypybox2d source tree")
    nw = int(sys.argv[1]) if len(sys.argv) > 1 else 8
    t0 = time.time()
    with mp.get_context("spawn").Pool(nw) as pool:
        res = pool.map(reference_world, range(nw))
    cpython = sum(r[1] * TIMED for r in res) / sum(r[2] for r in res)
    import oracle_lib
    from pypybox2d_gb300 import abi, scenes
    W, B, F, M = scenes.uneven_batch(nw, seed=0)
    lib = oracle_lib.load(False)
    s, keep = abi.make_scene(W, B, F, None, M)
    h = lib.or_batch_create(ctypes.byref(s))
    lib.or_batch_step(h, 1 / 60, 8, 3, SETTLE, 1)
    tp = lib.or_batch_step(h, 1 / 60, 8, 3, TIMED, 1)
    lib.or_batch_destroy(h)
    port = sum(scenes.uneven_count(w) for w in range(nw)) * TIMED / tp
    cpu = ""
    try:
        with open("/proc/cpuinfo") as f:
            cpu = next((l.split(":", 1)[1].strip() for l in f if l.startswith("model name")), "")
    except OSError:
        pass
    print(json.dumps({"worlds": nw, "bodies": int(sum(r[1] for r in res)), "steps": f"{SETTLE + 1}-{SETTLE + TIMED}",
                      "cpython_body_steps_per_s_per_core": cpython, "port_one_thread_body_steps_per_s": port,
                      "port_over_cpython": port / cpython, "cpu": cpu, "wall_s": round(time.time() - t0, 1)}))


if __name__ == "__main__":
    main()

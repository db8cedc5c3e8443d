"""Thin host wrapper of the C ABI: a device-resident batch of worlds.

``GpuBatch`` is the plumbing under ``World`` / ``WorldBatch``: it uploads
record arrays (``abi.BODY``, ``abi.FIXTURE``, ``abi.CONTACT``, ``abi.WORLD``)
through ``gb_batch_create`` and advances them with ``gb_batch_step``.  Every
call goes to libgb2d.so; a missing library or a CUDA error raises.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import abi


class GpuBatch:
    """A batch of independent worlds resident in device memory."""

    def __init__(self, worlds, bodies, fixtures, contacts=None, precision: str = "f64", moves=None, joints=None,
                 controllers=None, controller_bodies=None):
        self.lib = abi.load_library()
        self.prec = abi.PREC_F64 if precision in ("f64", "float64", abi.PREC_F64) else abi.PREC_F32
        scene, keep = abi.make_scene(worlds, bodies, fixtures, contacts, moves, joints, controllers, controller_bodies)
        self.worlds, self.n_bodies, self.n_fixtures = keep[0], len(keep[1]), len(keep[2])
        self.joint_worlds = keep[5]["world"].copy()
        self.n_joints = len(keep[5])
        h = ctypes.c_void_p()
        abi.check(self.lib.gb_batch_create(ctypes.byref(scene), self.prec, ctypes.byref(h)))
        self.h = h
        self.n_worlds = len(self.worlds)

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.gb_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, dt: float, vel_iters: int = 8, pos_iters: int = 3, n_steps: int = 1, launch_mode: int = 1,
             block_threads: int = 0, record_order: bool = False, stream: int | None = None,
             profile: bool = False, kernel_times: bool = False, events: bool = False) -> None:
        flags = ((1 if record_order else 0) | (2 if profile else 0) | (abi.OPT_KERNEL_TIMES if kernel_times else 0) |
                 (abi.OPT_EVENTS if events else 0))
        o = abi.StepOpts(dt, vel_iters, pos_iters, n_steps, launch_mode, block_threads, flags)
        abi.check(self.lib.gb_batch_step(self.h, ctypes.byref(o), ctypes.c_void_p(stream or 0)))

    def step_static_scratch(self, dt: float, vel_iters: int = 8, pos_iters: int = 3, n_steps: int = 1,
                            launch_mode: int = 1, block_threads: int = 0, stream: int | None = None) -> None:
        """``step`` with the step scratch in the library's static device array
        (gb_batch_step_static_scratch): no device allocation in the call; the
        batch's scratch must fit ``abi.STATIC_SCRATCH_BYTES``."""
        o = abi.StepOpts(dt, vel_iters, pos_iters, n_steps, launch_mode, block_threads, 0)
        abi.check(self.lib.gb_batch_step_static_scratch(self.h, ctypes.byref(o), ctypes.c_void_p(stream or 0)))

    def launch_config(self) -> dict:
        """The configuration steps with launch_mode=0 use (gb_batch_get_launch_config)."""
        c = abi.LaunchConfig()
        abi.check(self.lib.gb_batch_get_launch_config(self.h, ctypes.byref(c)))
        return c.as_dict()

    def set_launch_config(self, launch_mode: int = 3, block_threads: int = 128, pipe_bufs: int = 2,
                          big_bodies: int = 512, groups: int = 1) -> None:
        """Pin a launch configuration (for example one an earlier autotune chose)."""
        c = abi.LaunchConfig(launch_mode, block_threads, pipe_bufs, big_bodies, groups, 0, 0.0)
        abi.check(self.lib.gb_batch_set_launch_config(self.h, ctypes.byref(c)))

    def autotune(self, dt: float, vel_iters: int = 8, pos_iters: int = 3, steps_per_trial: int = 3,
                 stream: int | None = None) -> tuple[dict, list[dict]]:
        """Time candidate launch configurations on this batch's next
        ``steps_per_trial`` steps (gb_batch_autotune) and keep the fastest.
        The batch state is unchanged afterwards.  Returns (best, trials)."""
        o = abi.StepOpts(dt, vel_iters, pos_iters, steps_per_trial, 0, 0, 0)
        cap = 32
        trials = (abi.LaunchConfig * cap)()
        n = ctypes.c_int32()
        best = abi.LaunchConfig()
        abi.check(self.lib.gb_batch_autotune(self.h, ctypes.byref(o), trials, cap, ctypes.byref(n), ctypes.byref(best),
                                             ctypes.c_void_p(stream or 0)))
        return best.as_dict(), [trials[k].as_dict() for k in range(min(n.value, cap))]

    def capture(self, dt: float, vel_iters: int = 8, pos_iters: int = 3, n_steps: int = 1, launch_mode: int = 3,
                block_threads: int = 0, record_order: bool = False, events: bool = False) -> "StepGraph":
        """Capture ``n_steps`` phased steps as one CUDA graph (gb_graph_capture)."""
        flags = (1 if record_order else 0) | (abi.OPT_EVENTS if events else 0)
        o = abi.StepOpts(dt, vel_iters, pos_iters, n_steps, launch_mode, block_threads, flags)
        h = ctypes.c_void_p()
        abi.check(self.lib.gb_graph_capture(self.h, ctypes.byref(o), ctypes.byref(h)))
        return StepGraph(self, h, n_steps)

    def ray_cast(self, rays: np.ndarray, stream: int | None = None) -> np.ndarray:
        """Closest hit of each ray (``abi.RAY`` records) -> ``abi.RAY_HIT``
        records (gb_batch_ray_cast)."""
        r = np.ascontiguousarray(rays, dtype=abi.RAY)
        out = np.zeros(len(r), dtype=abi.RAY_HIT)
        abi.check(self.lib.gb_batch_ray_cast(self.h, r.ctypes.data, len(r), out.ctypes.data, ctypes.c_void_p(stream or 0)))
        return out

    def ray_cast_all(self, rays: np.ndarray, max_per_ray: int = 64,
                     stream: int | None = None) -> tuple[np.ndarray, np.ndarray]:
        """Every hit of each ray (``abi.RAY`` records), in fixture order:
        (``abi.RAY_HIT`` [n, max_per_ray], counts[n]) (gb_batch_ray_cast_all)."""
        r = np.ascontiguousarray(rays, dtype=abi.RAY)
        out = np.zeros((len(r), max_per_ray), dtype=abi.RAY_HIT)
        counts = np.zeros(len(r), dtype=np.int32)
        abi.check(self.lib.gb_batch_ray_cast_all(self.h, r.ctypes.data, len(r), out.ctypes.data, max_per_ray,
                                                 counts.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                                 ctypes.c_void_p(stream or 0)))
        return out, counts

    def query_aabb(self, boxes: np.ndarray, max_per_query: int = 64,
                   stream: int | None = None) -> tuple[np.ndarray, np.ndarray]:
        """Fixtures whose fat AABB overlaps each box (``abi.AABB_QUERY``
        records): (fixtures[n, max_per_query], counts[n]) (gb_batch_query_aabb)."""
        q = np.ascontiguousarray(boxes, dtype=abi.AABB_QUERY)
        out = np.full((len(q), max_per_query), -1, dtype=np.int32)
        counts = np.zeros(len(q), dtype=np.int32)
        i32p = ctypes.POINTER(ctypes.c_int32)
        abi.check(self.lib.gb_batch_query_aabb(self.h, q.ctypes.data, len(q), out.ctypes.data_as(i32p), max_per_query,
                                               counts.ctypes.data_as(i32p), ctypes.c_void_p(stream or 0)))
        return out, counts

    def bodies(self, stream: int | None = None) -> np.ndarray:
        out = np.zeros(self.n_bodies, dtype=abi.BODY)
        abi.check(self.lib.gb_batch_get_bodies(self.h, out.ctypes.data, self.n_bodies, ctypes.c_void_p(stream or 0)))
        return out

    def set_bodies(self, bodies: np.ndarray, stream: int | None = None) -> None:
        b = np.ascontiguousarray(bodies, dtype=abi.BODY)
        abi.check(self.lib.gb_batch_set_bodies(self.h, b.ctypes.data, len(b), ctypes.c_void_p(stream or 0)))

    def step_host(self, bodies: np.ndarray, dt: float, vel_iters: int = 8, pos_iters: int = 3, n_steps: int = 1,
                  launch_mode: int = 0, block_threads: int = 0, out: np.ndarray | None = None,
                  stream: int | None = None) -> np.ndarray:
        """set_bodies(bodies), step and bodies() in one call through host
        buffers (gb_batch_step_host): chunks of worlds upload, step and
        download on streams of their own.  ``bodies`` holds abi.BODY records,
        or abi.BODY_STATE records (gb_batch_step_host_state: the fields a
        step changes; the others stay on the device).  ``out`` (same record
        kind) may be ``bodies``."""
        kind = abi.BODY_STATE if bodies.dtype == abi.BODY_STATE else abi.BODY
        b = np.ascontiguousarray(bodies, dtype=kind)
        if len(b) != self.n_bodies:
            raise ValueError("body count mismatch")
        if out is None:
            out = np.zeros(self.n_bodies, dtype=kind)
        if out.dtype != kind or len(out) != self.n_bodies or not out.flags.c_contiguous:
            raise ValueError("out must be a contiguous array of the input's record kind and the batch's length")
        o = abi.StepOpts(dt, vel_iters, pos_iters, n_steps, launch_mode, block_threads, 0)
        fn = self.lib.gb_batch_step_host_state if kind is abi.BODY_STATE else self.lib.gb_batch_step_host
        abi.check(fn(self.h, b.ctypes.data, out.ctypes.data, self.n_bodies, ctypes.byref(o), ctypes.c_void_p(stream or 0)))
        return out

    def proxies(self) -> np.ndarray:
        out = np.zeros((self.n_fixtures, 4), dtype=np.float64)
        abi.check(self.lib.gb_batch_get_proxies(self.h, out.ctypes.data, self.n_fixtures, None))
        return out

    def contact_counts(self) -> np.ndarray:
        out = np.zeros(self.n_worlds, dtype=np.int32)
        abi.check(self.lib.gb_batch_get_contact_counts(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), None))
        return out

    def contacts(self, world: int = 0) -> np.ndarray:
        cap = int(self.contact_counts()[world])
        out = np.zeros(max(cap, 1), dtype=abi.CONTACT)
        n = ctypes.c_int32()
        abi.check(self.lib.gb_batch_get_contacts(self.h, world, out.ctypes.data, len(out), ctypes.byref(n), None))
        return out[:n.value].copy()

    def solver_order(self, world: int = 0) -> np.ndarray:
        cap = max(16, int(self.contact_counts()[world]) + 16)
        out = np.zeros(cap, dtype=np.int32)
        n = ctypes.c_int32()
        abi.check(self.lib.gb_batch_get_solver_order(self.h, world, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                                     cap, ctypes.byref(n), None))
        return out[:n.value].copy()

    def joint_order(self, world: int = 0) -> np.ndarray:
        """World-local joint indices in the order the last record_order step
        solved them (gb_batch_get_joint_order)."""
        cap = self.n_joints + 1
        out = np.zeros(cap, dtype=np.int32)
        n = ctypes.c_int32()
        abi.check(self.lib.gb_batch_get_joint_order(self.h, world, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                                    cap, ctypes.byref(n), None))
        return out[:n.value].copy()

    def joints(self, world: int | None = None) -> np.ndarray:
        """The joints with their carried state (``abi.JOINT``; all, or one world's)."""
        out = np.zeros(self.n_joints, dtype=abi.JOINT)
        abi.check(self.lib.gb_batch_get_joints(self.h, out.ctypes.data, self.n_joints, None))
        return out if world is None else out[out["world"] == world]

    def set_joints(self, joints: np.ndarray) -> None:
        """Overwrite every joint's definition and state (same worlds, kinds and bodies)."""
        j = np.ascontiguousarray(joints, dtype=abi.JOINT)
        abi.check(self.lib.gb_batch_set_joints(self.h, j.ctypes.data, len(j), None))

    def set_controllers(self, controllers: np.ndarray) -> None:
        """Overwrite every controller's parameters (same worlds, kinds and body lists)."""
        c = np.ascontiguousarray(controllers, dtype=abi.CONTROLLER)
        abi.check(self.lib.gb_batch_set_controllers(self.h, c.ctypes.data, len(c), None))

    def set_pair_filter(self, world: int, accept: np.ndarray | None) -> None:
        """A world's custom contact filter as its answers for every ordered
        pair of its fixture records (an n x n array, nonzero = may collide),
        or None for the default rule (gb_batch_set_pair_filter)."""
        if accept is None:
            abi.check(self.lib.gb_batch_set_pair_filter(self.h, world, None, 0, None))
            return
        m = np.ascontiguousarray(accept, dtype=np.uint8)
        if m.ndim != 2 or m.shape[0] != m.shape[1]:
            raise ValueError("accept must be a square array over the world's fixture records")
        abi.check(self.lib.gb_batch_set_pair_filter(self.h, world, m.ctypes.data, m.shape[0], None))

    def events(self, world: int = 0) -> np.ndarray:
        """Contact events of one world from the last step call made with
        events=True, in replay order (sorted by key)."""
        n = ctypes.c_int32()
        cap = 3 * 64 + 64
        while True:
            out = np.zeros(cap, dtype=abi.EVENT)
            rc = self.lib.gb_batch_get_events(self.h, world, out.ctypes.data, cap, ctypes.byref(n), None)
            if rc == 0:
                break
            if n.value <= cap:
                abi.check(rc)
            cap = n.value
        ev = out[:n.value]
        return ev[np.argsort(ev["key"], kind="stable")]

    def phase_clocks(self) -> np.ndarray:
        """Accumulated SM clocks per step phase and world (n_worlds x 24)."""
        out = np.zeros((self.n_worlds, 24), dtype=np.int64)
        abi.check(self.lib.gb_batch_phase_clocks(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), None))
        return out

    def kernel_times(self) -> tuple[dict, int]:
        """Summed device ms per phased-step launch slot and the number of
        timed steps (steps run with kernel_times=True)."""
        out = (ctypes.c_double * 16)()
        n = ctypes.c_int32()
        steps = ctypes.c_int64()
        abi.check(self.lib.gb_batch_kernel_times(self.h, out, 16, ctypes.byref(n), ctypes.byref(steps)))
        return {name: out[k] for k, name in enumerate(abi.KERNEL_SLOTS[:n.value])}, int(steps.value)

    def arena_bytes(self) -> int:
        c = (ctypes.c_int64 * 3)()
        abi.check(self.lib.gb_batch_counters(self.h, c))
        return int(c[1])

    def status(self) -> np.ndarray:
        out = np.zeros(self.n_worlds, dtype=np.uint32)
        abi.check(self.lib.gb_batch_status(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), None))
        return out

    def step_record(self, world: int = 0) -> np.ndarray:
        """Per body of the world (world-local order) the step record of the
        last step run with ``record_order`` (gb_batch_get_step_record):
        bits 0-7 position iterations of its island, 8-15 TOI position-pass
        iterations, 16-23 TOI events, 24-27 parities of its constraints'
        restitution-bias and block-solver decisions (island solve, TOI).
        Returns [2, n]: row 0 the decisions, row 1 each body's island in the
        solve (smallest non-static body index of the island, -1: none)."""
        nb = int(self.worlds["body_count"][world])
        out = np.zeros(max(2 * nb, 1), dtype=np.int32)
        n = ctypes.c_int32()
        abi.check(self.lib.gb_batch_get_step_record(self.h, world, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                                    2 * nb, ctypes.byref(n), None))
        return out[:2 * n.value].reshape(2, n.value).copy()

    def set_wait_polls(self, polls: int) -> None:
        """Poll limit of the solver's in-kernel copy waits (gb_batch_set_wait_polls)."""
        abi.check(self.lib.gb_batch_set_wait_polls(self.h, int(polls)))

    def clear_status(self) -> None:
        abi.check(self.lib.gb_batch_clear_status(self.h, None))

    def snapshot_bytes(self) -> int:
        n = ctypes.c_uint64()
        abi.check(self.lib.gb_batch_snapshot_bytes(self.h, ctypes.byref(n)))
        return int(n.value)

    def snapshot(self, dst_ptr: int | None = None, nbytes: int = 0, stream: int | None = None):
        """The batch's whole device state (gb_batch_snapshot).  Without
        ``dst_ptr`` it goes to a new host array, which is returned; with it, to
        the caller's buffer of ``nbytes`` (host or device address)."""
        if dst_ptr is None:
            out = np.empty(self.snapshot_bytes(), dtype=np.uint8)
            abi.check(self.lib.gb_batch_snapshot(self.h, out.ctypes.data, out.nbytes, ctypes.c_void_p(stream or 0)))
            return out
        abi.check(self.lib.gb_batch_snapshot(self.h, ctypes.c_void_p(dst_ptr), nbytes, ctypes.c_void_p(stream or 0)))
        return None

    def restore(self, src, nbytes: int = 0, stream: int | None = None) -> None:
        """Put back a snapshot (gb_batch_restore): a host array from
        ``snapshot()``, or a host/device address with its size."""
        if isinstance(src, np.ndarray):
            ptr, nbytes = src.ctypes.data, src.nbytes
        else:
            ptr = int(src)
        abi.check(self.lib.gb_batch_restore(self.h, ctypes.c_void_p(ptr), nbytes, ctypes.c_void_p(stream or 0)))


class StepGraph:
    """A captured multi-step rollout of a GpuBatch; ``launch()`` replays it
    on a stream and advances the batch by ``n_steps`` steps."""

    def __init__(self, batch: GpuBatch, handle: ctypes.c_void_p, n_steps: int):
        self.batch, self.h, self.n_steps = batch, handle, n_steps

    def launch(self, stream: int | None = None) -> None:
        abi.check(self.batch.lib.gb_graph_launch(self.h, ctypes.c_void_p(stream or 0)))

    def close(self) -> None:
        if getattr(self, "h", None) is not None and self.h.value:
            self.batch.lib.gb_graph_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

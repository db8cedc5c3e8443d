"""ctypes binding of the CPU restatement (oracle/) for the tests.

The oracle is test infrastructure: it is the checker of the GPU library and
is never called by the product.  ``load(libm=True)`` gives the build that
uses libm cos/sin/pow like CPython (pinned bit for bit against the golden
vectors of the reference); ``load(libm=False)`` the build with the portable
sincos and x*x that the float64 GPU kernels reproduce bit for bit.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

from pypybox2d_gb300 import abi

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(REPO, "oracle")
_libs: dict[bool, ctypes.CDLL] = {}


def build() -> None:
    subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)


def load(libm: bool = False) -> ctypes.CDLL:
    if libm in _libs:
        return _libs[libm]
    name = "liboracle_libm.so" if libm else "liboracle.so"
    path = os.path.join(ORACLE_DIR, "_build", name)
    build()
    lib = ctypes.CDLL(path)
    vp, i32, dbl = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    lib.or_create.restype = vp
    lib.or_create.argtypes = [vp, vp, vp, vp, vp]
    lib.or_destroy.argtypes = [vp]
    lib.or_step.argtypes = [vp, dbl, i32, i32]
    for n in ("or_body_count", "or_contact_count", "or_status"):
        getattr(lib, n).argtypes = [vp]
        getattr(lib, n).restype = i32
    lib.or_world_flags.argtypes = [vp]
    lib.or_world_flags.restype = ctypes.c_uint32
    lib.or_inv_dt0.argtypes = [vp]
    lib.or_inv_dt0.restype = dbl
    lib.or_get_bodies.argtypes = [vp, vp]
    lib.or_set_bodies.argtypes = [vp, vp]
    lib.or_get_fixtures.argtypes = [vp, vp]
    lib.or_get_contacts.argtypes = [vp, vp, i32]
    lib.or_get_contacts.restype = i32
    lib.or_set_solver_order.argtypes = [vp, vp, i32]
    lib.or_get_solver_order.argtypes = [vp, vp, i32]
    lib.or_get_solver_order.restype = i32
    lib.or_get_step_record.argtypes = [vp, vp]
    lib.or_get_step_record.restype = None
    lib.or_clear_status.argtypes = [vp]
    lib.or_clear_status.restype = None
    lib.or_toi_calls.argtypes = [vp]
    lib.or_toi_calls.restype = ctypes.c_longlong
    lib.or_toi_events.argtypes = [vp]
    lib.or_toi_events.restype = ctypes.c_longlong
    lib.or_run_scene.argtypes = [ctypes.POINTER(abi.Scene), dbl, i32, i32, i32, i32, vp]
    lib.or_run_scene.restype = dbl
    lib.or_batch_create.argtypes = [ctypes.POINTER(abi.Scene)]
    lib.or_batch_create.restype = vp
    lib.or_batch_destroy.argtypes = [vp]
    lib.or_batch_step.argtypes = [vp, dbl, i32, i32, i32, i32]
    lib.or_batch_step.restype = dbl
    lib.or_batch_get_bodies.argtypes = [vp, i32, vp]
    lib.or_batch_get_bodies.restype = i32
    lib.or_set_joints.argtypes = [vp, vp, i32]
    lib.or_set_joints.restype = i32
    lib.or_flag_joint_contacts.argtypes = [vp, i32]
    lib.or_flag_joint_contacts.restype = None
    lib.or_joint_count.argtypes = [vp]
    lib.or_joint_count.restype = i32
    lib.or_get_joints.argtypes = [vp, vp]
    lib.or_get_joints.restype = None
    lib.or_set_joint_order.argtypes = [vp, vp, i32]
    lib.or_set_joint_order.restype = None
    lib.or_get_joint_order.argtypes = [vp, vp, i32]
    lib.or_get_joint_order.restype = i32
    lib.or_set_controllers.argtypes = [vp, vp, i32, vp, i32]
    lib.or_set_controllers.restype = i32
    lib.or_set_pair_filter.argtypes = [vp, vp, i32]
    lib.or_set_pair_filter.restype = i32
    _libs[libm] = lib
    return lib


def golden_extras(d) -> dict:
    """The joints and controllers of a golden scene (npz), as keyword
    arguments of OracleWorld and GpuBatch."""
    out = {"joints": d["init_joints"] if "init_joints" in d.files else None}
    if "init_controllers" in d.files:
        out["controllers"], out["controller_bodies"] = d["init_controllers"], d["init_controller_bodies"]
    return out


class OracleWorld:
    """One world of the restatement, built from gb2d record arrays."""

    def __init__(self, world, bodies, fixtures, contacts=None, libm=False, index=0, moves=None, joints=None,
                 controllers=None, controller_bodies=None):
        self.lib = load(libm)
        self._keep = [np.ascontiguousarray(world, dtype=abi.WORLD),
                      np.ascontiguousarray(bodies, dtype=abi.BODY),
                      np.ascontiguousarray(fixtures, dtype=abi.FIXTURE),
                      np.ascontiguousarray(contacts if contacts is not None else np.zeros(0, abi.CONTACT),
                                           dtype=abi.CONTACT)]
        self._keep.append(np.ascontiguousarray(moves if moves is not None else np.zeros(0, np.int32), dtype=np.int32))
        w, b, f, c, mv = self._keep
        wd = w[index:index + 1]
        self._wd = np.ascontiguousarray(wd)
        self.h = self.lib.or_create(self._wd.ctypes.data, b.ctypes.data, f.ctypes.data,
                                    c.ctypes.data if len(c) else None, mv.ctypes.data if len(mv) else None)
        self.nb = int(wd["body_count"][0])
        self.nf = int(wd["fixture_count"][0])
        if joints is not None and len(joints):
            J = np.ascontiguousarray(joints, dtype=abi.JOINT)
            J = np.ascontiguousarray(J[J["world"] == index])
            if len(J):
                assert self.lib.or_set_joints(self.h, J.ctypes.data, len(J)) == 0, "bad joint records"
        if controllers is not None and len(controllers):
            self.set_controllers(controllers, controller_bodies, index)

    def set_controllers(self, controllers, controller_bodies, index=0):
        """The controllers of world `index` (records sorted by world, body
        lists in controller_bodies)."""
        C = np.ascontiguousarray(controllers, dtype=abi.CONTROLLER)
        C = np.ascontiguousarray(C[C["world"] == index])
        cb = np.ascontiguousarray(controller_bodies if controller_bodies is not None else np.zeros(0, np.int32),
                                  dtype=np.int32)
        self._ctl = (C, cb)
        assert self.lib.or_set_controllers(self.h, C.ctypes.data if len(C) else None, len(C),
                                           cb.ctypes.data if len(cb) else None, len(cb)) == 0, "bad controller records"

    def set_pair_filter(self, accept):
        """A custom contact filter's answers over the fixture records (n x n),
        or None for the default rule (or_set_pair_filter)."""
        if accept is None:
            self._pf = None
            assert self.lib.or_set_pair_filter(self.h, None, 0) == 0
            return
        self._pf = np.ascontiguousarray(accept, dtype=np.uint8)
        assert self.lib.or_set_pair_filter(self.h, self._pf.ctypes.data, self._pf.shape[0]) == 0, "bad filter table"

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.or_destroy(self.h)
            self.h = None

    def step(self, dt, vel_iters=8, pos_iters=3, order=None, joint_order=None):
        if order is not None:
            o = np.ascontiguousarray(order, dtype=np.int32)
            self.lib.or_set_solver_order(self.h, o.ctypes.data, len(o))
        if joint_order is not None:
            jo = np.ascontiguousarray(joint_order, dtype=np.int32)
            self.lib.or_set_joint_order(self.h, jo.ctypes.data, len(jo))
        self.lib.or_step(self.h, dt, vel_iters, pos_iters)

    def joints(self):
        n = self.lib.or_joint_count(self.h)
        out = np.zeros(n, dtype=abi.JOINT)
        if n:
            self.lib.or_get_joints(self.h, out.ctypes.data)
        return out

    def joint_order(self):
        cap = self.lib.or_joint_count(self.h) + 1
        out = np.zeros(cap, dtype=np.int32)
        n = self.lib.or_get_joint_order(self.h, out.ctypes.data, cap)
        return out[:n].copy()

    def bodies(self):
        out = np.zeros(self.nb, dtype=abi.BODY)
        self.lib.or_get_bodies(self.h, out.ctypes.data)
        return out

    def fixtures(self):
        out = np.zeros(self.nf, dtype=abi.FIXTURE)
        self.lib.or_get_fixtures(self.h, out.ctypes.data)
        return out

    def contacts(self):
        n = self.lib.or_contact_count(self.h)
        out = np.zeros(n, dtype=abi.CONTACT)
        self.lib.or_get_contacts(self.h, out.ctypes.data, n)
        return out

    def set_bodies(self, bodies):
        b = np.ascontiguousarray(bodies, dtype=abi.BODY)
        self.lib.or_set_bodies(self.h, b.ctypes.data)

    def solver_order(self):
        cap = max(16, 4 * self.lib.or_contact_count(self.h) + 16)
        out = np.zeros(cap, dtype=np.int32)
        n = self.lib.or_get_solver_order(self.h, out.ctypes.data, cap)
        return out[:n].copy()

    def status(self):
        return self.lib.or_status(self.h)

    def step_record(self):
        """Per body the step record of the last step (or_get_step_record)."""
        out = np.zeros(max(2 * self.nb, 1), dtype=np.int32)
        self.lib.or_get_step_record(self.h, out.ctypes.data)
        return out[:2 * self.nb].reshape(2, self.nb).copy()


class OracleBatch:
    """The restatement behind the batch interface pypybox2d_gb300.World uses
    (step / bodies / set_bodies / proxies / contacts / status), so the
    World's host logic can be checked on the CPU.  Test infrastructure."""

    def __init__(self, W, B, F, C, M, libm=False, joints=None, controllers=None, controller_bodies=None):
        self.o = OracleWorld(W, B, F, C if len(C) else None, libm=libm, moves=M, joints=joints, controllers=controllers,
                             controller_bodies=controller_bodies)
        self.libm = libm

    def query_aabb(self, q, max_per_query):
        return query_aabb_records(self.o.fixtures(), q, max_per_query, libm=self.libm)

    def set_pair_filter(self, world, accept):
        self.o.set_pair_filter(accept)

    def ray_cast(self, r):
        return ray_cast_records(self.o.bodies(), self.o.fixtures(), r, libm=self.libm)

    def ray_cast_all(self, r, max_per_ray):
        return ray_cast_all_records(self.o.bodies(), self.o.fixtures(), r, max_per_ray, libm=self.libm)

    def step(self, dt, vel_iters, pos_iters, n_steps=1, **_):
        for _ in range(n_steps):
            self.o.step(dt, vel_iters, pos_iters)

    def bodies(self):
        return self.o.bodies()

    def set_bodies(self, B):
        self.o.set_bodies(B)

    def proxies(self):
        return self.o.fixtures()["aabb"].copy()

    def contacts(self, world=0):
        return self.o.contacts()

    def contact_counts(self):
        return np.array([len(self.o.contacts())], dtype=np.int32)

    def status(self):
        return np.array([self.o.status()], dtype=np.uint32)

    def clear_status(self):
        self.o.lib.or_clear_status(self.o.h)

    def joints(self, world=None):
        return self.o.joints()

    def set_controllers(self, controllers):
        self.o.set_controllers(controllers, getattr(self.o, "_ctl", (None, None))[1])

    def set_joints(self, J):
        J = np.ascontiguousarray(J, dtype=abi.JOINT)
        assert self.o.lib.or_set_joints(self.o.h, J.ctypes.data, len(J)) == 0

    def close(self):
        pass


def ray_cast_records(B, F, rays, libm: bool = True) -> np.ndarray:
    """The restatement's closest hits (or_ray_cast_records) of one world."""
    lib = load(libm)
    lib.or_ray_cast_records.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                        ctypes.c_void_p]
    B = np.ascontiguousarray(B, dtype=abi.BODY)
    F = np.ascontiguousarray(F, dtype=abi.FIXTURE)
    r = np.ascontiguousarray(rays, dtype=abi.RAY)
    out = np.zeros(len(r), dtype=abi.RAY_HIT)
    lib.or_ray_cast_records(B.ctypes.data, F.ctypes.data, len(F), r.ctypes.data, len(r), out.ctypes.data)
    return out


def query_aabb_records(F, boxes, cap: int, libm: bool = True) -> tuple[np.ndarray, np.ndarray]:
    """The restatement's overlapping fixtures (or_query_aabb_records) of one world."""
    lib = load(libm)
    lib.or_query_aabb_records.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                          ctypes.c_int, ctypes.c_void_p]
    F = np.ascontiguousarray(F, dtype=abi.FIXTURE)
    q = np.ascontiguousarray(boxes, dtype=abi.AABB_QUERY)
    out = np.full((len(q), cap), -1, dtype=np.int32)
    counts = np.zeros(len(q), dtype=np.int32)
    lib.or_query_aabb_records(F.ctypes.data, len(F), q.ctypes.data, len(q), out.ctypes.data, cap, counts.ctypes.data)
    return out, counts


def ray_cast_all_records(B, F, rays, cap: int, libm: bool = True) -> tuple[np.ndarray, np.ndarray]:
    """The restatement's every hit (or_ray_cast_all_records) of one world."""
    lib = load(libm)
    lib.or_ray_cast_all_records.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                            ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    B = np.ascontiguousarray(B, dtype=abi.BODY)
    F = np.ascontiguousarray(F, dtype=abi.FIXTURE)
    r = np.ascontiguousarray(rays, dtype=abi.RAY)
    out = np.zeros((len(r), cap), dtype=abi.RAY_HIT)
    counts = np.zeros(len(r), dtype=np.int32)
    lib.or_ray_cast_all_records(B.ctypes.data, F.ctypes.data, len(F), r.ctypes.data, len(r), out.ctypes.data, cap,
                                counts.ctypes.data)
    return out, counts

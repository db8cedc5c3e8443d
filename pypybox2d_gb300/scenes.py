"""Scene construction as record arrays, with the reference's construction
arithmetic, and the synthetic workloads of the benchmark.

``SceneBuilder`` reproduces what pypybox2d does when bodies and fixtures are
created through its API -- Body.__init__ (body.py:20-97), attach_fixture /
reset_mass_data (body.py:166-195, 587-641), proxy creation with the fat
AABB (fixture.py:250-261, dynamictree.py:115-134) -- so a scene built here
is bit-identical to the same scene built with the reference.  The workload
generators below build the batches the benchmark runs:

  pyramid_world   20 rows of 0.5 m boxes on a 40 x 0.5 m ground box (210 bodies)
  pyramid_batch   N jittered copies of the pyramid
  mixed_batch     uneven worlds: a 100 m edge box with circles and convex polygons
  bullet_batch    box stacks hit by bullet circles (continuous collision)
"""
from __future__ import annotations

import math

import numpy as np

from . import abi
from .shapes import Circle, Edge, Polygon, _xmul

AABB_EXTENSION = 0.1


class _Fix:
    __slots__ = ("shape", "friction", "restitution", "density", "category", "mask", "group", "sensor")

    def __init__(self, shape, friction=0.2, restitution=0.0, density=0.0, category=0x0001, mask=0xFFFF,
                 group=0, sensor=False):
        self.shape, self.friction, self.restitution, self.density = shape, float(friction), float(restitution), float(density)
        self.category, self.mask, self.group, self.sensor = category, mask, group, sensor


class _Body:
    """Construction-time state of one body (the fields of body.py:46-84)."""

    def __init__(self, type=abi.BODY_STATIC, position=(0, 0), angle=0.0, linear_velocity=(0, 0),
                 angular_velocity=0.0, linear_damping=0.0, angular_damping=0.0, allow_sleep=True, awake=True,
                 fixed_rotation=False, bullet=False, active=True, gravity_scale=1.0):
        self.type = type
        angle = float(angle)
        self.p = (float(position[0]), float(position[1]))
        self.q = (math.cos(angle), math.sin(angle))
        self.lc = (0.0, 0.0)
        self.a0 = self.a = angle
        self.c0 = _xmul(self.p, self.q, self.lc)
        self.c = self.c0
        self.alpha0 = 0.0
        self.v = (float(linear_velocity[0]), float(linear_velocity[1]))
        self.w = float(angular_velocity)
        self.force = (0.0, 0.0)
        self.torque = 0.0
        self.I = self.invI = 0.0
        self.mass, self.inv_mass = (1.0, 1.0) if type == abi.BODY_DYNAMIC else (0.0, 0.0)
        self.ld, self.ad, self.gs = float(linear_damping), float(angular_damping), float(gravity_scale)
        self.allow_sleep, self.awake, self.fixed_rotation = bool(allow_sleep), bool(awake), bool(fixed_rotation)
        self.bullet, self.active = bool(bullet), bool(active)
        self.sleep_time = 0.0
        self.fixtures: list[_Fix] = []
        self.aabbs: list[tuple] = []

    def reset_mass_data(self):
        """body.py:587-641"""
        self.mass = self.inv_mass = self.I = self.invI = 0.0
        self.lc = (0.0, 0.0)
        if self.type in (abi.BODY_STATIC, abi.BODY_KINEMATIC):
            self.c = self.p
            self.c0 = self.c
            return
        cx = cy = 0.0
        for f in self.fixtures:
            if f.density == 0.0:
                continue
            md = f.shape.compute_mass(f.density)
            self.mass += md.mass
            cx, cy = cx + md.mass * md.center[0], cy + md.mass * md.center[1]
            self.I += md.I
        if self.mass > 0.0:
            self.inv_mass = 1.0 / self.mass
            cx, cy = cx * self.inv_mass, cy * self.inv_mass
        else:
            self.mass = 1.0
            self.inv_mass = 1.0
        if self.I > 0.0 and not self.fixed_rotation:
            self.I -= self.mass * (cx * cx + cy * cy)
            self.invI = 1.0 / self.I
        else:
            self.I = 0.0
            self.invI = 0.0
        old = self.c
        self.lc = (cx, cy)
        self.c0 = _xmul(self.p, self.q, self.lc)
        self.c = self.c0
        dx, dy = self.c[0] - old[0], self.c[1] - old[1]
        w = self.w
        self.v = (self.v[0] + (-w * dy), self.v[1] + w * dx)


class SceneBuilder:
    """Bodies and fixtures of one world, created as with pypybox2d's API.

    Bodies are attached to the world at creation (World.create_body); a
    fixture added afterwards creates its proxy at once and, when its
    density is positive, resets the body's mass data (body.py:166-195)."""

    def __init__(self, gravity=(0.0, -10.0), do_sleep=True, warm_starting=True, continuous_physics=True,
                 auto_clear_forces=True):
        self.gravity = (float(gravity[0]), float(gravity[1]))
        self.flags = ((abi.W_ALLOW_SLEEP if do_sleep else 0) | (abi.W_WARM_STARTING if warm_starting else 0) |
                      (abi.W_CONTINUOUS if continuous_physics else 0) | (abi.W_AUTO_CLEAR_FORCES if auto_clear_forces else 0) |
                      abi.W_STEP_COMPLETE)
        self.bodies: list[_Body] = []
        self.moves: list[tuple[int, int]] = []   # (body, fixture slot) in proxy creation order

    def create_body(self, type=abi.BODY_STATIC, fixtures=(), **kw) -> int:
        """World.create_body(**kw) with `fixtures` = [(shape, fixture kwargs)] attached
        before the body joins the world (Body.__init__ shapes=/fixtures=)."""
        b = _Body(type=type, **kw)
        for shape, fkw in fixtures:
            b.fixtures.append(_Fix(shape.__copy__(), **fkw))
            if b.fixtures[-1].density > 0.0:
                b.reset_mass_data()
        self.bodies.append(b)
        bi = len(self.bodies) - 1
        reset = False
        for k, f in enumerate(b.fixtures):
            if b.active:
                self._create_proxy(bi, k)
            if f.density > 0.0:
                reset = True
        if reset:
            b.reset_mass_data()
        return bi

    def add_fixture(self, bi: int, shape, **fkw) -> None:
        """Body.create_fixture on a body already in the world."""
        b = self.bodies[bi]
        b.fixtures.append(_Fix(shape.__copy__(), **fkw))
        if b.active:
            self._create_proxy(bi, len(b.fixtures) - 1)
        if b.fixtures[-1].density > 0.0:
            b.reset_mass_data()

    def _create_proxy(self, bi, k):
        b = self.bodies[bi]
        lx, ly, ux, uy = b.fixtures[k].shape.compute_aabb(b.p, b.q)
        while len(b.aabbs) <= k:
            b.aabbs.append(None)
        b.aabbs[k] = (lx - AABB_EXTENSION, ly - AABB_EXTENSION, ux + AABB_EXTENSION, uy + AABB_EXTENSION)
        self.moves.append((bi, k))

    def records(self):
        """(worlds[1], bodies, fixtures, moves) record arrays of this world."""
        nb = len(self.bodies)
        nf = sum(len(b.fixtures) for b in self.bodies)
        B = np.zeros(nb, dtype=abi.BODY)
        F = np.zeros(nf, dtype=abi.FIXTURE)
        start = []
        k = 0
        for i, b in enumerate(self.bodies):
            start.append(k)
            fl = ((abi.BODY_AWAKE if b.awake else 0) | (abi.BODY_ALLOW_SLEEP if b.allow_sleep else 0) |
                  (abi.BODY_BULLET if b.bullet else 0) | (abi.BODY_FIXED_ROTATION if b.fixed_rotation else 0) |
                  (abi.BODY_ACTIVE if b.active else 0))
            B[i] = (b.type, fl, k, len(b.fixtures), b.p[0], b.p[1], b.q[0], b.q[1], b.lc[0], b.lc[1],
                    b.c0[0], b.c0[1], b.c[0], b.c[1], b.a0, b.a, b.alpha0, b.v[0], b.v[1], b.w,
                    b.force[0], b.force[1], b.torque, b.mass, b.inv_mass, b.I, b.invI, b.ld, b.ad, b.gs, b.sleep_time)
            for j, f in enumerate(b.fixtures):
                r = F[k]
                sh = f.shape
                r["body"], r["shape_type"], r["radius"] = i, sh.type, sh.radius
                r["friction"], r["restitution"], r["density"] = f.friction, f.restitution, f.density
                r["category_bits"], r["mask_bits"], r["group_index"] = f.category, f.mask, f.group
                fl = abi.FIX_SENSOR if f.sensor else 0
                if isinstance(sh, Circle):
                    r["vertex_count"] = 1
                    r["vx"][0], r["vy"][0] = sh.position
                elif isinstance(sh, Polygon):
                    r["vertex_count"] = len(sh._vertices)
                    for m, ((vx, vy), (nx, ny)) in enumerate(zip(sh._vertices, sh._normals)):
                        r["vx"][m], r["vy"][m], r["nx"][m], r["ny"][m] = vx, vy, nx, ny
                elif isinstance(sh, Edge):
                    r["vertex_count"] = 2
                    r["vx"][0], r["vy"][0] = sh.vertex1
                    r["vx"][1], r["vy"][1] = sh.vertex2
                    if sh.vertex0 is not None:
                        fl |= abi.FIX_EDGE_HAS_V0
                        r["vx"][2], r["vy"][2] = sh.vertex0
                    if sh.vertex3 is not None:
                        fl |= abi.FIX_EDGE_HAS_V3
                        r["vx"][3], r["vy"][3] = sh.vertex3
                r["flags"] = fl
                r["aabb"][:] = b.aabbs[j] if j < len(b.aabbs) and b.aabbs[j] is not None else (0, 0, 0, 0)
                k += 1
        moves = np.array([start[bi] + k for bi, k in self.moves], dtype=np.int32)
        W = np.zeros(1, dtype=abi.WORLD)
        flags = self.flags | (abi.W_NEW_FIXTURE if len(moves) else 0)
        W[0] = (0, nb, 0, nf, 0, 0, 0, flags, 0, len(moves), self.gravity[0], self.gravity[1], 0.0)
        return W, B, F, moves


def concat(worlds: list) -> tuple:
    """Concatenate per-world (W, B, F[, moves]) tuples into one batch."""
    Ws, Bs, Fs, Ms = [], [], [], []
    nb = nf = nm = 0
    for item in worlds:
        W, B, F = item[0], item[1], item[2]
        M = item[3] if len(item) > 3 else np.zeros(0, np.int32)
        W = W.copy()
        W["body_start"] += nb
        W["fixture_start"] += nf
        W["move_start"] = nm
        Ws.append(W); Bs.append(B); Fs.append(F); Ms.append(M)
        nb += len(B); nf += len(F); nm += len(M)
    return np.concatenate(Ws), np.concatenate(Bs), np.concatenate(Fs), np.concatenate(Ms).astype(np.int32)


# ------------------------------------------------------------------ workloads
def pyramid_builder(rows: int = 20, jitter=None) -> SceneBuilder:
    """The pyramid: ground box 40 x 0.5 half extents centred at (0, -0.5);
    rows of 0.5 m boxes (density 5, friction 0.6, restitution 0) starting at
    (-7, 0.75) with row offset (0.5625, 1.25) and column offset (1.125, 0).
    `jitter(k)` returns the (dx, dy) added to box k's position."""
    s = SceneBuilder(gravity=(0.0, -10.0), do_sleep=True)
    s.create_body(abi.BODY_STATIC, position=(0, -0.5), fixtures=[(Polygon(box=(40, 0.5)), {})])
    box = Polygon(box=(0.5, 0.5))
    fk = dict(density=5.0, friction=0.6, restitution=0.0)
    x = (-7.0, 0.75)
    k = 0
    for i in range(rows):
        y = x
        for _ in range(i, rows):
            pos = y
            if jitter is not None:
                dx, dy = jitter(k)
                pos = (y[0] + dx, y[1] + dy)
            s.create_body(abi.BODY_DYNAMIC, position=pos, fixtures=[(box, fk)])
            y = (y[0] + 1.125, y[1] + 0.0)
            k += 1
        x = (x[0] + 0.5625, x[1] + 1.25)
    return s


def pyramid_world(rows: int = 20):
    W, B, F, M = pyramid_builder(rows).records()
    return W, B, F, M


def pyramid_batch(n_worlds: int, rows: int = 20, jitter: float = 0.01, seed: int = 0):
    """n_worlds copies of the pyramid; every box position gets a seeded
    U(-jitter, jitter) offset (world w uses seed + w).  The first world is
    built through SceneBuilder; the others reuse its shapes and mass data
    (position independent) and recompute position, sweep and fat AABB with
    the same float64 expressions, vectorised."""
    W0, B0, F0, M0 = pyramid_world(rows)
    nb, nf = len(B0), len(F0)
    Bs = np.tile(B0, n_worlds)
    Fs = np.tile(F0, n_worlds)
    Ws = np.tile(W0, n_worlds)
    Ms = np.tile(M0, n_worlds)
    Ws["body_start"] = np.arange(n_worlds) * nb
    Ws["fixture_start"] = np.arange(n_worlds) * nf
    Ws["move_start"] = np.arange(n_worlds) * len(M0)
    if jitter:
        jit = np.zeros((n_worlds, nb, 2))
        for w in range(n_worlds):
            r = np.random.default_rng(seed + w)
            jit[w, 1:] = r.uniform(-jitter, jitter, size=(nb - 1, 2))
        Bv = Bs.reshape(n_worlds, nb)
        Fv = Fs.reshape(n_worlds, nf)
        dyn = Bv["type"] == abi.BODY_DYNAMIC
        px = np.where(dyn, Bv["px"] + jit[:, :, 0], Bv["px"])
        py = np.where(dyn, Bv["py"] + jit[:, :, 1], Bv["py"])
        Bv["px"], Bv["py"] = px, py
        qc, qs = Bv["qc"], Bv["qs"]
        lcx, lcy = Bv["lcx"], Bv["lcy"]
        cx = px + qc * lcx + (-qs) * lcy
        cy = py + qs * lcx + qc * lcy
        Bv["cx"] = np.where(dyn, cx, Bv["cx"]); Bv["cy"] = np.where(dyn, cy, Bv["cy"])
        Bv["c0x"] = Bv["cx"]; Bv["c0y"] = Bv["cy"]
        # fat AABB of each box fixture (Polygon.compute_aabb + fattening)
        fb = Fv["body"]
        bpx = np.take_along_axis(px, fb, axis=1)
        bpy = np.take_along_axis(py, fb, axis=1)
        bqc = np.take_along_axis(qc, fb, axis=1)
        bqs = np.take_along_axis(qs, fb, axis=1)
        vx, vy = Fv["vx"], Fv["vy"]
        X = bpx[..., None] + bqc[..., None] * vx + (-bqs[..., None]) * vy
        Y = bpy[..., None] + bqs[..., None] * vx + bqc[..., None] * vy
        cnt = Fv["vertex_count"]
        lx, ly, ux, uy = X[..., 0].copy(), Y[..., 0].copy(), X[..., 0].copy(), Y[..., 0].copy()
        for m in range(abi.MAX_POLY_VERTS):
            use = m < cnt
            lx = np.where(use & ~(lx < X[..., m]), X[..., m], lx)
            ly = np.where(use & ~(ly < Y[..., m]), Y[..., m], ly)
            ux = np.where(use & ~(ux > X[..., m]), X[..., m], ux)
            uy = np.where(use & ~(uy > Y[..., m]), Y[..., m], uy)
        r = Fv["radius"]
        dynf = np.take_along_axis(dyn, fb, axis=1)
        aabb = np.stack([(lx - r) - AABB_EXTENSION, (ly - r) - AABB_EXTENSION,
                         (ux + r) + AABB_EXTENSION, (uy + r) + AABB_EXTENSION], axis=-1)
        Fv["aabb"] = np.where(dynf[..., None], aabb, Fv["aabb"])
        Bs = Bv.reshape(-1)
        Fs = Fv.reshape(-1)
    return Ws, Bs, Fs, Ms

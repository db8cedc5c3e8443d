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
from .shapes import FLT_EPSILON, POLYGON_RADIUS, Circle, Edge, Loop, Polygon, _xmul

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
        self.aabbs: list[tuple] = []      # per record (a loop fixture has one record per child)

    def record_offset(self, k: int) -> int:
        """The first record of fixture k (loop fixtures take one per child)."""
        return sum(f.shape.child_count for f in self.fixtures[:k])

    @property
    def record_count(self) -> int:
        return sum(f.shape.child_count for f in self.fixtures)

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
        self.moves: list[tuple[int, int]] = []   # (body, record within the body) in proxy creation order

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
        """fixture.py:250-261: one proxy per child, fattened (dynamictree.py:115-134)"""
        b = self.bodies[bi]
        sh = b.fixtures[k].shape
        o = b.record_offset(k)
        for c in range(sh.child_count):
            lx, ly, ux, uy = sh.compute_aabb(b.p, b.q, c) if isinstance(sh, Loop) else sh.compute_aabb(b.p, b.q)
            while len(b.aabbs) <= o + c:
                b.aabbs.append(None)
            b.aabbs[o + c] = (lx - AABB_EXTENSION, ly - AABB_EXTENSION, ux + AABB_EXTENSION, uy + AABB_EXTENSION)
            self.moves.append((bi, o + c))

    def body_records(self, bi: int, body_index: int | None = None):
        """Record of body bi and the records of its fixtures (``body`` field =
        body_index, default bi)."""
        b = self.bodies[bi]
        B = np.zeros(1, dtype=abi.BODY)
        F = np.zeros(b.record_count, dtype=abi.FIXTURE)
        fl = ((abi.BODY_AWAKE if b.awake else 0) | (abi.BODY_ALLOW_SLEEP if b.allow_sleep else 0) |
              (abi.BODY_BULLET if b.bullet else 0) | (abi.BODY_FIXED_ROTATION if b.fixed_rotation else 0) |
              (abi.BODY_ACTIVE if b.active else 0))
        B[0] = (b.type, fl, 0, len(F), b.p[0], b.p[1], b.q[0], b.q[1], b.lc[0], b.lc[1],
                b.c0[0], b.c0[1], b.c[0], b.c[1], b.a0, b.a, b.alpha0, b.v[0], b.v[1], b.w,
                b.force[0], b.force[1], b.torque, b.mass, b.inv_mass, b.I, b.invI, b.ld, b.ad, b.gs, b.sleep_time)
        j = 0
        for f in b.fixtures:
            # a loop: one edge record per child (shapes.py:851-863), no radius
            # margin on its fat box
            children = [(f.shape.child_edge(c), abi.FIX_LOOP_CHILD | (abi.FIX_LOOP_FIRST if c == 0 else 0))
                        for c in range(f.shape.child_count)] if isinstance(f.shape, Loop) else [(f.shape, 0)]
            for sh, extra in children:
                j = self._fixture_record(F, j, b, f, sh, extra, bi if body_index is None else body_index)
        return B[0], F

    def _fixture_record(self, F, j, b, f, sh, extra, body_index):
        """Fill record j of F from fixture f with shape sh; returns j + 1."""
        r = F[j]
        r["body"], r["shape_type"], r["radius"] = body_index, sh.type, sh.radius
        r["friction"], r["restitution"], r["density"] = f.friction, f.restitution, f.density
        r["category_bits"], r["mask_bits"], r["group_index"] = f.category, f.mask, f.group
        ffl = (abi.FIX_SENSOR if f.sensor else 0) | extra
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
                ffl |= abi.FIX_EDGE_HAS_V0
                r["vx"][2], r["vy"][2] = sh.vertex0
            if sh.vertex3 is not None:
                ffl |= abi.FIX_EDGE_HAS_V3
                r["vx"][3], r["vy"][3] = sh.vertex3
        r["flags"] = ffl
        r["aabb"][:] = b.aabbs[j] if j < len(b.aabbs) and b.aabbs[j] is not None else (0, 0, 0, 0)
        return j + 1

    def world_record(self, nb: int, nf: int, n_moves: int):
        W = np.zeros(1, dtype=abi.WORLD)
        flags = self.flags | (abi.W_NEW_FIXTURE if n_moves else 0)
        W[0] = (0, nb, 0, nf, 0, 0, 0, flags, 0, n_moves, self.gravity[0], self.gravity[1], 0.0)
        return W

    def records(self):
        """(worlds[1], bodies, fixtures, moves) record arrays of this world."""
        nb = len(self.bodies)
        nf = sum(b.record_count for b in self.bodies)
        B = np.zeros(nb, dtype=abi.BODY)
        F = np.zeros(nf, dtype=abi.FIXTURE)
        start = []
        k = 0
        for i in range(nb):
            start.append(k)
            B[i], Fi = self.body_records(i)
            B[i]["fixture_start"] = k
            F[k:k + len(Fi)] = Fi
            k += len(Fi)
        moves = np.array([start[bi] + k for bi, k in self.moves], dtype=np.int32)
        return self.world_record(nb, nf, len(moves)), B, F, moves


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


# ------------------------------------------------------------ uneven batch
# Worlds of log-uniform size in [10, 2000] bodies: a static 100 x 100 m
# container of four edges, half circles (radius U(0.25, 1)) and half convex
# polygons of 3-8 vertices on a circle of radius U(0.3, 1); density U(0.5, 5),
# friction U(0.2, 0.8), restitution U(0, 0.3); bodies start on distinct
# cells of a 2.1 m grid (so they do not overlap) with velocity N(0, 2) m/s,
# angular velocity N(0, 1) rad/s and angle U(-pi, pi); gravity (0, -10).
CONTAINER_HALF = 50.0
GRID_CELL = 2.1
GRID_N = 45                                   # 45 x 45 cells span +-47.25 m
UNEVEN_MIN, UNEVEN_MAX = 10, 2000


def uneven_count(seed: int) -> int:
    r = np.random.default_rng(seed)
    return int(math.floor(math.exp(r.uniform(math.log(UNEVEN_MIN), math.log(UNEVEN_MAX)))))


def _uneven_draws(seed: int, n: int | None = None) -> dict:
    """Every random draw of one uneven world, in a fixed order (shared by the
    SceneBuilder form and the vectorised batch, so both see the same numbers)."""
    if n is None:
        n = uneven_count(seed)
    r = np.random.default_rng((seed, 1))
    cells = r.choice(GRID_N * GRID_N, size=n, replace=False)
    jit = r.uniform(-0.04, 0.04, size=(n, 2))
    x0 = -0.5 * GRID_N * GRID_CELL + 0.5 * GRID_CELL
    px = x0 + (cells % GRID_N) * GRID_CELL + jit[:, 0]
    py = x0 + (cells // GRID_N) * GRID_CELL + jit[:, 1]
    circle = r.random(n) < 0.5
    crad = r.uniform(0.25, 1.0, n)
    prad = r.uniform(0.3, 1.0, n)
    nv = r.integers(3, abi.MAX_POLY_VERTS + 1, n)
    # polygon vertices: nv angles in CCW order on the circle (points on a
    # circle are in strictly convex position); the gaps are 0.2 rad plus a
    # Dirichlet(4) share of the rest (no short edges), redrawn while one
    # exceeds 3 rad (the polygon holds its origin)
    theta = np.zeros((n, abi.MAX_POLY_VERTS))
    cols = np.arange(abi.MAX_POLY_VERTS)[None, :]
    todo = np.arange(n)
    while len(todo):
        k = nv[todo][:, None]
        e = np.where(cols < k, r.gamma(4.0, 1.0, (len(todo), abi.MAX_POLY_VERTS)), 0.0)
        gaps = 0.2 + (2.0 * math.pi - 0.2 * k) * (e / e.sum(axis=1, keepdims=True))
        gaps = np.where(cols < k, gaps, 0.0)
        ok = gaps.max(axis=1) <= 3.0
        start = r.uniform(0.0, 2.0 * math.pi, len(todo))
        ang = start[:, None] + np.concatenate([np.zeros((len(todo), 1)), np.cumsum(gaps, axis=1)[:, :-1]], axis=1)
        theta[todo[ok]] = np.where(cols < k, ang, 0.0)[ok]
        todo = todo[~ok]
    vx = prad[:, None] * np.cos(theta)
    vy = prad[:, None] * np.sin(theta)
    return dict(n=n, px=px, py=py, circle=circle, crad=crad, nv=nv, vx=vx, vy=vy,
                density=r.uniform(0.5, 5.0, n), friction=r.uniform(0.2, 0.8, n),
                restitution=r.uniform(0.0, 0.3, n), v=r.normal(0.0, 2.0, (n, 2)),
                w=r.normal(0.0, 1.0, n), angle=r.uniform(-math.pi, math.pi, n))


def _container_edges():
    h = CONTAINER_HALF
    return [Edge((-h, -h), (h, -h)), Edge((h, -h), (h, h)), Edge((h, h), (-h, h)), Edge((-h, h), (-h, -h))]


def uneven_builder(seed: int, n: int | None = None) -> SceneBuilder:
    """One uneven world built body by body through SceneBuilder."""
    d = _uneven_draws(seed, n)
    s = SceneBuilder(gravity=(0.0, -10.0), do_sleep=True)
    s.create_body(abi.BODY_STATIC, position=(0, 0), fixtures=[(e, {}) for e in _container_edges()])
    for i in range(d["n"]):
        if d["circle"][i]:
            shape = Circle(radius=float(d["crad"][i]))
        else:
            k = int(d["nv"][i])
            shape = Polygon(vertices=list(zip(d["vx"][i, :k].tolist(), d["vy"][i, :k].tolist())))
        fk = dict(density=float(d["density"][i]), friction=float(d["friction"][i]),
                  restitution=float(d["restitution"][i]))
        s.create_body(abi.BODY_DYNAMIC, position=(float(d["px"][i]), float(d["py"][i])), angle=float(d["angle"][i]),
                      linear_velocity=(float(d["v"][i, 0]), float(d["v"][i, 1])), angular_velocity=float(d["w"][i]),
                      fixtures=[(shape, fk)])
    return s


def uneven_world(seed: int, n: int | None = None):
    return uneven_builder(seed, n).records()


def uneven_batch(n_worlds: int = 8192, seed: int = 0, counts=None):
    """The uneven batch, world w drawn from seed + w.  Records are assembled
    with numpy in the same float64 operation order as SceneBuilder (circle and
    polygon mass data, centre of mass, the velocity shift of reset_mass_data,
    edge normals and fat AABBs), so world w equals uneven_world(seed + w)."""
    draws = [_uneven_draws(seed + w, None if counts is None else int(counts[w])) for w in range(n_worlds)]
    cs = SceneBuilder(gravity=(0.0, -10.0), do_sleep=True)
    cs.create_body(abi.BODY_STATIC, position=(0, 0), fixtures=[(e, {}) for e in _container_edges()])
    return _assemble(cs, draws)


def _assemble(cs: SceneBuilder, draws: list):
    """Batch records: per world the static body of `cs` (built once) and one
    dynamic body with one circle or polygon fixture per draw."""
    n_worlds = len(draws)
    ns = np.array([d["n"] for d in draws])
    cat = {k: np.concatenate([d[k] for d in draws]) for k in draws[0] if k != "n"}
    nbody = int(ns.sum())
    Wc, Bc, Fc, _ = cs.records()
    nfc = len(Fc)
    nb_w = ns + 1
    nf_w = ns + nfc
    b_start = np.concatenate([[0], np.cumsum(nb_w)[:-1]])
    f_start = np.concatenate([[0], np.cumsum(nf_w)[:-1]])
    # the static body 0 of every world with its fixtures
    B = np.zeros(int(nb_w.sum()), dtype=abi.BODY)
    F = np.zeros(int(nf_w.sum()), dtype=abi.FIXTURE)
    B[b_start] = Bc[0]
    for k in range(nfc):
        F[f_start + k] = Fc[k]
    # dynamic bodies: index of body i of world w = b_start[w] + 1 + i
    widx = np.repeat(np.arange(n_worlds), ns)
    local = np.arange(nbody) - np.repeat(np.concatenate([[0], np.cumsum(ns)[:-1]]), ns)
    bi = b_start[widx] + 1 + local
    fi = f_start[widx] + nfc + local
    angle = cat["angle"]
    qc = np.fromiter((math.cos(a) for a in angle.tolist()), float, nbody)
    qs = np.fromiter((math.sin(a) for a in angle.tolist()), float, nbody)
    px, py = cat["px"], cat["py"]
    circ = cat["circle"]
    dens = cat["density"]
    # mass data (Circle.compute_mass, Polygon.compute_mass)
    r = cat["crad"]
    r2 = np.fromiter((x ** 2 for x in r.tolist()), float, nbody)   # CPython float pow, as Circle.compute_mass
    cm = dens * math.pi * r2
    cI = cm * (0.5 * r2 + (0.0 * 0.0 + 0.0 * 0.0))
    nv = cat["nv"]
    vx, vy = cat["vx"], cat["vy"]
    sx, sy = vx[:, 0].copy(), vy[:, 0].copy()
    for m in range(1, abi.MAX_POLY_VERTS):
        use = m < nv
        sx = np.where(use, sx + vx[:, m], sx)
        sy = np.where(use, sy + vy[:, m], sy)
    fn = nv.astype(float)
    sx, sy = sx / fn, sy / fn
    ccx = np.zeros(nbody); ccy = np.zeros(nbody); area = np.zeros(nbody); pI = np.zeros(nbody)
    inv3 = 1.0 / 3.0
    for m in range(abi.MAX_POLY_VERTS):
        use = m < nv
        j = np.where(m + 1 < nv, m + 1, 0)
        e1x, e1y = vx[:, m] - sx, vy[:, m] - sy
        e2x = np.take_along_axis(vx, j[:, None], axis=1)[:, 0] - sx
        e2y = np.take_along_axis(vy, j[:, None], axis=1)[:, 0] - sy
        D = e1x * e2y - e1y * e2x
        tri = 0.5 * D
        area = np.where(use, area + tri, area)
        kk = tri * inv3
        ccx = np.where(use, ccx + kk * (e1x + e2x), ccx)
        ccy = np.where(use, ccy + kk * (e1y + e2y), ccy)
        intx2 = e1x * e1x + e2x * e1x + e2x * e2x
        inty2 = e1y * e1y + e2y * e1y + e2y * e2y
        pI = np.where(use, pI + (0.25 * inv3 * D) * (intx2 + inty2), pI)
    with np.errstate(divide="ignore", invalid="ignore"):
        pm = dens * area
        ccx, ccy = ccx / area, ccy / area
        mcx, mcy = ccx + sx, ccy + sy
        pIm = dens * pI
        pIm = pIm + pm * ((mcx * mcx + mcy * mcy) - (ccx * ccx + ccy * ccy))
    md_mass = np.where(circ, cm, pm)
    md_cx = np.where(circ, 0.0, mcx)
    md_cy = np.where(circ, 0.0, mcy)
    md_I = np.where(circ, cI, pIm)
    # Body.reset_mass_data (twice: once when the fixture is attached, once when
    # the body joins the world; the second leaves the state unchanged but its
    # velocity shift is by a zero vector)
    mass = 0.0 + md_mass
    cx = 0.0 + mass * md_cx
    cy = 0.0 + mass * md_cy
    I = 0.0 + md_I
    inv_mass = 1.0 / mass
    cx, cy = cx * inv_mass, cy * inv_mass
    I = I - mass * (cx * cx + cy * cy)
    invI = 1.0 / I
    c0x = px + qc * 0.0 + (-qs) * 0.0
    c0y = py + qs * 0.0 + qc * 0.0
    ncx = px + qc * cx + (-qs) * cy
    ncy = py + qs * cx + qc * cy
    w = cat["w"]
    v0, v1 = cat["v"][:, 0], cat["v"][:, 1]
    v0, v1 = v0 + (-w * (ncy - c0y)), v1 + w * (ncx - c0x)
    v0, v1 = v0 + (-w * (ncy - ncy)), v1 + w * (ncx - ncx)
    Bd = B[bi]
    Bd["type"] = abi.BODY_DYNAMIC
    Bd["flags"] = abi.BODY_AWAKE | abi.BODY_ALLOW_SLEEP | abi.BODY_ACTIVE
    Bd["fixture_start"] = nfc + local
    Bd["fixture_count"] = 1
    Bd["px"], Bd["py"], Bd["qc"], Bd["qs"] = px, py, qc, qs
    Bd["lcx"], Bd["lcy"] = cx, cy
    Bd["c0x"], Bd["c0y"], Bd["cx"], Bd["cy"] = ncx, ncy, ncx, ncy
    Bd["a0"], Bd["a"] = angle, angle
    Bd["vx"], Bd["vy"], Bd["w"] = v0, v1, w
    Bd["mass"], Bd["inv_mass"], Bd["I"], Bd["inv_I"] = mass, inv_mass, I, invI
    Bd["gravity_scale"] = 1.0
    B[bi] = Bd
    # fixtures
    Fd = F[fi]
    Fd["body"] = 1 + local
    Fd["shape_type"] = np.where(circ, abi.SHAPE_CIRCLE, abi.SHAPE_POLYGON)
    Fd["vertex_count"] = np.where(circ, 1, nv)
    Fd["radius"] = np.where(circ, r, POLYGON_RADIUS)
    Fd["friction"], Fd["restitution"], Fd["density"] = cat["friction"], cat["restitution"], dens
    Fd["category_bits"], Fd["mask_bits"] = 0x0001, 0xFFFF
    used = np.arange(abi.MAX_POLY_VERTS)[None, :] < nv[:, None]
    pvx = np.where(used, vx, 0.0)
    pvy = np.where(used, vy, 0.0)
    # edge normals (Polygon.vertices setter)
    nxs = np.zeros_like(pvx); nys = np.zeros_like(pvy)
    for m in range(abi.MAX_POLY_VERTS):
        j = np.where(m + 1 < nv, m + 1, 0)
        ex = np.take_along_axis(pvx, j[:, None], axis=1)[:, 0] - pvx[:, m]
        ey = np.take_along_axis(pvy, j[:, None], axis=1)[:, 0] - pvy[:, m]
        nx, ny = 1.0 * ey, -1.0 * ex
        ln = np.sqrt(nx * nx + ny * ny)
        with np.errstate(divide="ignore", invalid="ignore"):
            inv = 1.0 / ln
        small = ln < FLT_EPSILON
        nxs[:, m] = np.where(used[:, m], np.where(small, nx, nx * inv), 0.0)
        nys[:, m] = np.where(used[:, m], np.where(small, ny, ny * inv), 0.0)
    Fd["vx"] = np.where(circ[:, None], 0.0, pvx)
    Fd["vy"] = np.where(circ[:, None], 0.0, pvy)
    Fd["nx"] = np.where(circ[:, None], 0.0, nxs)
    Fd["ny"] = np.where(circ[:, None], 0.0, nys)
    # fat AABBs (compute_aabb at the body transform, then +-0.1)
    X = px[:, None] + qc[:, None] * pvx + (-qs[:, None]) * pvy
    Y = py[:, None] + qs[:, None] * pvx + qc[:, None] * pvy
    lx, ly, ux, uy = X[:, 0].copy(), Y[:, 0].copy(), X[:, 0].copy(), Y[:, 0].copy()
    for m in range(abi.MAX_POLY_VERTS):
        use = m < nv
        lx = np.where(use & ~(lx < X[:, m]), X[:, m], lx)
        ly = np.where(use & ~(ly < Y[:, m]), Y[:, m], ly)
        ux = np.where(use & ~(ux > X[:, m]), X[:, m], ux)
        uy = np.where(use & ~(uy > Y[:, m]), Y[:, m], uy)
    pr = POLYGON_RADIUS
    paabb = np.stack([(lx - pr) - AABB_EXTENSION, (ly - pr) - AABB_EXTENSION,
                      (ux + pr) + AABB_EXTENSION, (uy + pr) + AABB_EXTENSION], axis=-1)
    ccx_, ccy_ = px + (qc * 0.0 + (-qs) * 0.0), py + (qs * 0.0 + qc * 0.0)
    caabb = np.stack([(ccx_ - r) - AABB_EXTENSION, (ccy_ - r) - AABB_EXTENSION,
                      (ccx_ + r) + AABB_EXTENSION, (ccy_ + r) + AABB_EXTENSION], axis=-1)
    Fd["aabb"] = np.where(circ[:, None], caabb, paabb)
    F[fi] = Fd
    Wv = np.zeros(n_worlds, dtype=abi.WORLD)
    Wv[:] = Wc[0]
    Wv["body_start"], Wv["body_count"] = b_start, nb_w
    Wv["fixture_start"], Wv["fixture_count"] = f_start, nf_w
    Wv["move_start"], Wv["move_count"] = f_start, nf_w
    M = np.concatenate([np.arange(k, dtype=np.int32) for k in nf_w]) if n_worlds else np.zeros(0, np.int32)
    return Wv, B, F, M


# ------------------------------------------------------------ bullet batch
# A 20-high stack of 0.5 m boxes (density 1, friction 0.3) on a 40 x 0.5 m
# ground box, and 4 bullet circles (radius 0.1, density 100) fired from
# x = -30 at heights U(0.5, 10) with speeds U(150, 250) m/s.
def bullet_builder(seed: int, stack: int = 20, bullets: int = 4) -> SceneBuilder:
    r = np.random.default_rng((seed, 5))
    ys = r.uniform(0.5, 10.0, bullets)
    vs = r.uniform(150.0, 250.0, bullets)
    s = SceneBuilder(gravity=(0.0, -10.0), do_sleep=True)
    s.create_body(abi.BODY_STATIC, position=(0, -0.5), fixtures=[(Polygon(box=(40, 0.5)), {})])
    box = Polygon(box=(0.5, 0.5))
    for i in range(stack):
        s.create_body(abi.BODY_DYNAMIC, position=(0.0, 0.5 + 1.0 * i), fixtures=[(box, dict(density=1.0, friction=0.3))])
    for k in range(bullets):
        s.create_body(abi.BODY_DYNAMIC, position=(-30.0, float(ys[k])), bullet=True,
                      linear_velocity=(float(vs[k]), 0.0), fixtures=[(Circle(radius=0.1), dict(density=100.0))])
    return s


def bullet_batch(n_worlds: int = 2048, seed: int = 0):
    """n_worlds bullet worlds, world w drawn from seed + w."""
    return concat([bullet_builder(seed + w).records() for w in range(n_worlds)])


# ------------------------------------------------------------ one large world
# n dynamic bodies (60% boxes with half extents U(0.2, 0.6), 40% circles of
# radius U(0.2, 0.6); density 1, friction 0.5) on a jittered 1.5 m grid,
# above a static 600 m ground box with two 200 m side walls; gravity (0, -10).
LARGE_COLS = 390


def _large_draws(seed: int, n: int) -> dict:
    r = np.random.default_rng((seed, 4))
    cols = max(1, min(LARGE_COLS, n))
    k = np.arange(n)
    jit = r.uniform(-0.1, 0.1, size=(n, 2))
    px = -0.5 * (cols - 1) * 1.5 + (k % cols) * 1.5 + jit[:, 0]
    py = 2.0 + (k // cols) * 1.5 + jit[:, 1]
    circle = r.random(n) < 0.4
    crad = r.uniform(0.2, 0.6, n)
    hx = r.uniform(0.2, 0.6, n)
    hy = r.uniform(0.2, 0.6, n)
    vx = np.zeros((n, abi.MAX_POLY_VERTS))
    vy = np.zeros((n, abi.MAX_POLY_VERTS))
    vx[:, 0], vx[:, 1], vx[:, 2], vx[:, 3] = -hx, hx, hx, -hx
    vy[:, 0], vy[:, 1], vy[:, 2], vy[:, 3] = -hy, -hy, hy, hy
    z = np.zeros(n)
    return dict(n=n, px=px, py=py, circle=circle, crad=crad, nv=np.full(n, 4), vx=vx, vy=vy,
                density=np.ones(n), friction=np.full(n, 0.5), restitution=z.copy(), v=np.zeros((n, 2)),
                w=z.copy(), angle=z.copy())


def _large_container() -> SceneBuilder:
    cs = SceneBuilder(gravity=(0.0, -10.0), do_sleep=True)
    ground = Polygon(vertices=[(-300.0, -1.0), (300.0, -1.0), (300.0, 0.0), (-300.0, 0.0)])
    left = Polygon(vertices=[(-301.0, 0.0), (-300.0, 0.0), (-300.0, 200.0), (-301.0, 200.0)])
    right = Polygon(vertices=[(300.0, 0.0), (301.0, 0.0), (301.0, 200.0), (300.0, 200.0)])
    cs.create_body(abi.BODY_STATIC, position=(0, 0), fixtures=[(ground, {}), (left, {}), (right, {})])
    return cs


def large_builder(seed: int = 0, n: int = 100000) -> SceneBuilder:
    """The large world built body by body through SceneBuilder (small n)."""
    d = _large_draws(seed, n)
    s = _large_container()
    for i in range(n):
        if d["circle"][i]:
            shape = Circle(radius=float(d["crad"][i]))
        else:
            shape = Polygon(vertices=list(zip(d["vx"][i, :4].tolist(), d["vy"][i, :4].tolist())))
        s.create_body(abi.BODY_DYNAMIC, position=(float(d["px"][i]), float(d["py"][i])), angle=0.0,
                      fixtures=[(shape, dict(density=1.0, friction=0.5, restitution=0.0))])
    return s


def large_world(seed: int = 0, n: int = 100000):
    """One large world, assembled with numpy (equals large_builder's records)."""
    return _assemble(_large_container(), [_large_draws(seed, n)])

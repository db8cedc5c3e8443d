"""A scripted loop-shape session of the World API, run on the reference by
make_golden.py (api_loops.npz) and on pypybox2d_gb300 by
tests/test_world_loops.py.

Loop fixtures (shapes.py:780-882) are made through create_loop_fixture in
both call forms (a vertex list, and vertices as separate arguments): a
static bowl whose bottom vertex is its body's origin (so the two child
edges beside it lose vertex0 / vertex3), a two-vertex shelf, and a triangle
loop on a dynamic frame whose circle gives it mass.  Between steps the
frame is moved through its transform (its three child proxies re-fattened
and moved), the bowl's filter is changed (its children's contacts
refiltered: the balls fall through the bowl), a loop is added to a body
already in the world, and the frame's loop is destroyed (the contacts of
all its children end).  Every snapshot records the bodies, the fat boxes of
every child proxy and the contacts, and `probes` records closest ray hits
and AABB query results through the public query API.
"""
DT = 1.0 / 60.0
VEL_ITERS, POS_ITERS = 8, 3
SNAPS = ("s0", "s30", "s31", "s60", "s61", "s90", "s91", "s120")
RAYS = (((-12.0, 3.0), (-4.0, 3.0)), ((-8.0, 6.0), (-8.0, -3.0)), ((10.0, 5.0), (10.0, 0.0)),
        ((4.0, 6.0), (4.0, -1.0)), ((0.0, 8.0), (0.0, 7.0)))
BOXES = (((-12.0, -1.0), (-4.0, 5.0)), ((2.0, 0.0), (7.0, 4.0)), ((8.0, 1.0), (12.0, 3.0)))
QUERY_WIDTH = 24     # entries per query row (body * 100 + fixture, sorted, -1 padded)


def _where(world, fixture):
    bodies = list(world.bodies)
    bi = next(i for i, b in enumerate(bodies) if b is fixture.body)
    fi = next(i for i, f in enumerate(bodies[bi].fixtures) if f is fixture)
    return bi, fi


def probes(b2, world):
    """Closest hit of each ray (body index, fixture index, point, normal,
    fraction; -1 and NaN for none) and the fixtures each box query reports,
    as rows of floats."""
    rows = []
    for p1, p2 in RAYS:
        best = None
        for ret in world.ray_cast(p1, p2):
            if best is None or ret[3] < best[3]:
                best = list(ret)
            ret[-1] = ret[3]
        if best is None:
            rows.append([-1.0, -1.0] + [float("nan")] * 5)
        else:
            bi, fi = _where(world, best[0])
            rows.append([float(bi), float(fi), float(best[1][0]), float(best[1][1]), float(best[2][0]),
                         float(best[2][1]), float(best[3])])
    queries = []
    for lo, hi in BOXES:
        found = sorted(100 * bi + fi for bi, fi in (_where(world, f) for f in world.query_aabb(b2.AABB(lo, hi))))
        queries.append([float(x) for x in found] + [-1.0] * (QUERY_WIDTH - len(found)))
    return rows, queries


def script(b2, snap, on_world=lambda world: None):
    world = b2.World((0, -10), True)
    on_world(world)
    ground = world.create_static_body(position=(0, -1))
    ground.create_polygon_fixture(box=(30, 1))
    bowl = world.create_static_body(position=(-8, 0.5))
    rim = bowl.create_loop_fixture([(-3, 4), (-3, 0.5), (0, 0), (3, 0.5), (3, 4)], friction=0.5)
    for i, x in enumerate((-9.5, -8.0, -6.5)):
        ball = world.create_dynamic_body(position=(x, 2.5 + 0.3 * i))
        ball.create_circle_fixture(0.4, density=1.0, friction=0.3)
    crate = world.create_dynamic_body(position=(-8, 3.8), angle=0.2)
    crate.create_polygon_fixture(box=(0.4, 0.3), density=1.0, friction=0.4)
    frame = world.create_dynamic_body(position=(4, 3), angle=0.1)
    tri = frame.create_loop_fixture((-1, -0.6), (1, -0.6), (0, 0.8), friction=0.5)
    frame.create_circle_fixture(0.3, density=2.0)
    box = world.create_dynamic_body(position=(4.2, 5.5))
    box.create_polygon_fixture(box=(0.3, 0.3), density=1.0, friction=0.5)
    shelf = world.create_static_body(position=(10, 2))
    shelf.create_loop_fixture([(-2, 0), (2, -0.5)], friction=0.3)
    pebble = world.create_dynamic_body(position=(10, 4))
    pebble.create_circle_fixture(0.3, density=1.0)

    def run(n):
        for _ in range(n):
            world.step(DT, VEL_ITERS, POS_ITERS)

    snap("s0", world)
    run(30)
    snap("s30", world)
    frame.transform = ((6.0, 2.5), 0.5)
    run(1)
    snap("s31", world)
    run(29)
    snap("s60", world)
    rim.category_bits = 0x0002
    rim.mask_bits = 0x0002
    run(1)
    snap("s61", world)
    run(29)
    snap("s90", world)
    ground.create_loop_fixture([(-25, 3), (-20, 1), (-15, 3)], friction=0.2)
    frame.destroy_fixture(tri)
    run(1)
    snap("s91", world)
    run(29)
    snap("s120", world)
    return world

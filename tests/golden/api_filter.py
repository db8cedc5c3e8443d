"""A scripted session of a custom contact filter (World.contact_filter,
world.py:123-136, asked by contact_manager.py:145 for a new pair and by
contact_manager.py:202 for a contact flagged for filtering), run on the
reference by make_golden.py (api_filter.npz) and on pypybox2d_gb300 by
tests/test_world_filter.py.

Two teams of boxes (densities 1 and 2) fall through each other onto the
ground under `same_team`; then `heavy_ghosts` replaces it and the heavy
circles (density 3) drop through everything but the ground; then no filter
at all.  A filter decides new pairs only: contacts that exist stay until
they are flagged for filtering.  Both filters answer alike for either order
of a pair and read only the fixtures' densities.
"""
DT = 1.0 / 60.0
VEL_ITERS, POS_ITERS = 8, 3
SNAPS = ("s0", "s1", "s40", "s41", "s80", "s120")


def same_team(fa, fb):
    """Dynamic fixtures of different densities pass through each other; the
    ground (density 0) meets every fixture."""
    return fa.density == 0.0 or fb.density == 0.0 or fa.density == fb.density


def heavy_ghosts(fa, fb):
    """The density-3 fixtures meet only the ground; the rest meet all."""
    if fa.density == 3.0 or fb.density == 3.0:
        return fa.density == 0.0 or fb.density == 0.0
    return True


def script(b2, snap, on_world=lambda world: None):
    world = b2.World((0, -10), True)
    on_world(world)
    world.contact_filter = same_team
    ground = world.create_static_body(position=(0, -0.5))
    ground.create_polygon_fixture(box=(20, 0.5), density=0.0, friction=0.6)
    boxes = []
    for i in range(6):
        for j in range(4):
            team = 1.0 if (i + j) % 2 == 0 else 2.0
            b = world.create_dynamic_body(position=(-5 + 2.0 * i + 0.3 * (j % 2), 1.0 + 1.1 * j))
            b.create_polygon_fixture(box=(0.5, 0.5), density=team, friction=0.5)
            boxes.append(b)
    balls = []
    for i in range(4):
        b = world.create_dynamic_body(position=(-4 + 2.5 * i, 8.0))
        b.create_circle_fixture(0.45, density=3.0, friction=0.3)
        balls.append(b)

    def run(n):
        for _ in range(n):
            world.step(DT, VEL_ITERS, POS_ITERS)

    snap("s0", world)
    run(1)
    snap("s1", world)
    run(39)
    snap("s40", world)
    world.contact_filter = heavy_ghosts
    run(1)
    snap("s41", world)
    run(39)
    snap("s80", world)
    world.contact_filter = None                    # the default rule again
    run(40)
    snap("s120", world)
    return world

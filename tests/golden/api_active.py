"""A scripted Body.active session of the World API (body.py:826-872), run on
the reference by make_golden.py (api_active.npz) and on pypybox2d_gb300 by
tests/test_world_active.py.

A box resting on the ground is made inactive (its one contact goes, it stops
moving and nothing collides with it: a falling box passes through it); a
body created inactive is activated later (its proxy is made at its
transform and the next step pairs it).  The script does not make the
deactivated box active again: in the reference that raises AssertionError
(Fixture._destroy_proxies clears each proxy's reference but not the
fixture's proxy list, and _create_proxies asserts the list is empty,
fixture.py:250-267) after the body's flag is already set, and its next step
fails moving the dead proxy (dynamictree.py:159).  The deactivated box has
a single contact: the
reference's own loop destroys only every second contact of a body
(body.py:865-869), and an inactive body left with a contact trips its
island search later, so sessions with more are not comparable.
"""
DT = 1.0 / 60.0
VEL_ITERS, POS_ITERS = 8, 3
SNAPS = ("s0", "s30", "s31", "s60", "s61", "s90", "s120")


def script(b2, snap, on_world=lambda world: None):
    world = b2.World((0, -10), True)
    on_world(world)
    ground = world.create_static_body(position=(0, -1))
    ground.create_polygon_fixture(box=(30, 1))
    a = world.create_dynamic_body(position=(0, 0.5))
    a.create_polygon_fixture(box=(1.0, 0.5), density=1.0, friction=0.6)
    b = world.create_dynamic_body(position=(0.3, 6.0), angle=0.1)
    b.create_polygon_fixture(box=(0.3, 0.3), density=1.0, friction=0.6)
    c = world.create_dynamic_body(position=(6, 3), active=False)
    c.create_circle_fixture(0.5, density=1.0, friction=0.4)
    d = world.create_dynamic_body(position=(-6, 0.5))
    d.create_circle_fixture(0.5, density=1.0, friction=0.4)

    def run(n):
        for _ in range(n):
            world.step(DT, VEL_ITERS, POS_ITERS)

    snap("s0", world)
    run(30)
    snap("s30", world)
    a.active = False
    run(1)
    snap("s31", world)
    run(29)
    snap("s60", world)
    c.active = True
    run(1)
    snap("s61", world)
    run(29)
    snap("s90", world)
    d.active = False
    run(30)
    snap("s120", world)
    return world

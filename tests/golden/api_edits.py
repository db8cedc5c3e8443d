"""A World-API session of host-side edits made between steps, on a world
with live contacts: run on the reference by make_golden_queries.py and on
pypybox2d_gb300 by tests/test_world_host_api.py (stepped by the CPU
restatement there, so the host logic is checked without a GPU).

Edits after 40 steps: fixture friction and filter changes (refiltering
touching contacts), a velocity, a mass-data override, fixed rotation, a
fixture destroyed while touching (end_contact), then 40 more steps; warm
starting switched off, then 20 more steps.  (A type change of a body that
touches a static one is left out: the reference asserts in
contact_manager.py:191 on the contact it leaves between two non-dynamic
bodies.)"""
DT = 1.0 / 60.0
SNAPS = ("s40", "s80", "s100")


def build(b2):
    world = b2.World(gravity=(0, -10), do_sleep=True)
    world.create_static_body(position=(0, -0.5)).create_polygon_fixture(box=(12, 0.5), friction=0.6)
    for i in range(8):
        b = world.create_dynamic_body(position=(-3.5 + i, 0.6 + 0.55 * (i % 3)), angle=0.1 * i)
        if i % 3 == 0:
            b.create_circle_fixture(radius=0.45, density=1.0, friction=0.4)
        else:
            b.create_polygon_fixture(box=(0.45, 0.3), density=1.5, friction=0.5)
        if i == 2:
            b.create_circle_fixture(radius=0.2, position=(0.3, 0.25), density=2.0)
    return world


def script(b2, snap, on_world=lambda world: None, log=None):
    log = [] if log is None else log
    world = build(b2)
    on_world(world)
    for _ in range(40):
        world.step(DT, 8, 3)
    snap("s40", world)
    bodies = world.bodies
    bodies[3].fixtures[0].friction = 0.05
    bodies[0].fixtures[0].group_index = -1
    bodies[4].fixtures[0].group_index = -1
    bodies[5].linear_velocity = (0.0, 4.0)
    bodies[6].mass_data = b2.shapes.MassData(mass=3.0, center=(0.05, -0.02), I=1.2)
    bodies[7].fixed_rotation = True
    world.contact_manager.end_contact = lambda c: log.append(
        (bodies.index(c.fixture_a.body), bodies.index(c.fixture_b.body)))
    bodies[3].destroy_fixture(bodies[3].fixtures[0])
    world.contact_manager.end_contact = None
    for _ in range(40):
        world.step(DT, 8, 3)
    snap("s80", world)
    world.warm_starting = False
    for _ in range(20):
        world.step(DT, 8, 3)
    snap("s100", world)
    return world, log

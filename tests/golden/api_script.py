"""A scripted World-API session, run on the reference by make_golden.py and
on pypybox2d_gb300 by tests/test_world_api.py.

Bodies are created through the API, stepped, edited between steps
(velocities, forces and impulses, a hand-set transform, a body created
after the first step with two fixtures, a destroyed body, new gravity, a
fast body that needs continuous collision) and stepped again.  The bodies
never touch each other, so every island holds one body and its ground
contacts and the solver order is the reference's whatever the GPU colouring.
"""
DT = 1.0 / 60.0
VEL_ITERS, POS_ITERS = 8, 3
SNAPS = ("s0", "s1", "s30", "s60", "s90", "s120", "s150", "s210")


def attach_listeners(world, log, step):
    """begin/end/post-solve listeners appending (kind, step, body a, fixture
    a, body b, fixture b, impulses) to `log`; step() gives the step number."""
    def ids(contact):   # fixtures carry (body tag, fixture slot) as user data
        return [*contact.fixture_a.user_data, *contact.fixture_b.user_data]

    world.contact_manager.begin_contact = lambda c: log.append(("begin", step(), *ids(c), ()))
    world.contact_manager.end_contact = lambda c: log.append(("end", step(), *ids(c), ()))
    world.contact_manager.post_solve = lambda c, imp: log.append(
        ("post", step(), *ids(c), tuple(float(x) for p in imp for x in p)))


def script(b2, snap, on_world=lambda world: None, log=None):
    world = b2.World((0, -10), True)
    on_world(world)
    counter = [0]
    if log is not None:
        attach_listeners(world, log, lambda: counter[0])
    ground = world.create_static_body(position=(0, -10))
    ground.create_polygon_fixture(box=(50, 10), user_data=(0, 0))
    a = world.create_dynamic_body(position=(0, 4))
    a.create_circle_fixture(1.0, density=1.0, user_data=(1, 0))
    b = world.create_dynamic_body(position=(-10, 2), angle=0.3)
    b.create_polygon_fixture(box=(0.5, 0.25), density=2.0, friction=0.4, user_data=(2, 0))
    c = world.create_dynamic_body(position=(10, 1))
    c.create_polygon_fixture(vertices=[(0, 0), (1, 0), (0.5, 1)], density=1.0, user_data=(3, 0))

    def run(n):
        for _ in range(n):
            counter[0] += 1
            world.step(DT, VEL_ITERS, POS_ITERS)

    snap("s0", world)
    run(1)
    snap("s1", world)
    run(29)
    snap("s30", world)
    a.linear_velocity = (3.0, 0.0)
    b.apply_force((50.0, 0.0), (-10.0, 0.3))
    c.angular_velocity = 2.0
    c.apply_linear_impulse((0.0, 4.0), (10.2, 0.5))
    run(30)
    snap("s60", world)
    d = world.create_dynamic_body(position=(20, 3), fixed_rotation=True)
    d.create_circle_fixture(0.5, density=3.0, user_data=(4, 0))
    d.create_circle_fixture(0.25, position=(0, 0.6), density=1.0, user_data=(4, 1))
    run(30)
    snap("s90", world)
    c.transform = ((14.0, 2.0), 0.5)
    world.destroy_body(a)
    world.gravity = (0, -5)
    run(30)
    snap("s120", world)
    e = world.create_dynamic_body(position=(-25, 6), linear_velocity=(0.0, -200.0))
    e.create_circle_fixture(0.2, density=5.0, user_data=(5, 0))
    run(30)
    snap("s150", world)
    b.awake = False
    d.apply_torque(3.0)
    run(60)
    snap("s210", world)
    return world

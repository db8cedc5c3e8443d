"""A scripted controller session of the World API (controllers.py,
world.py:923-957), run on the reference by make_golden.py
(api_controllers.npz) and on pypybox2d_gb300 by
tests/test_world_controllers.py.

A buoyancy pool and a gravity controller are made through
create_buoyancy_controller / create_gravity_controller and filled with
add_body (one box sits in both).  Between steps their parameters change
through the setters (density, offset, fluid velocity, G), bodies leave and
join the lists (remove_body, add_body), a body of the pool is destroyed
(it leaves its controller, body.py:342-344), the gravity controller is
destroyed (destroy_controller detaches its bodies) and a second buoyancy
controller is made with its bodies passed at creation and a zero gravity
vector (which takes the world's, controllers.py:177).  Every snapshot
records the bodies, contacts and each controller's body list.

The script destroys no body that sits in two controllers: the reference's
Body._detached_from_world removes a body from every second controller only
(it walks the list it removes from), and the one it stays in keeps acting
on the world's bodies through it: a gravity controller still pulls them
towards the dead body's last position.
"""
DT = 1.0 / 60.0
VEL_ITERS, POS_ITERS = 8, 3
SNAPS = ("s0", "s30", "s31", "s60", "s61", "s90", "s120")


def script(b2, snap, on_world=lambda world: None):
    world = b2.World((0, -10), True)
    on_world(world)
    world.create_static_body(shapes=b2.Edge((-20, 0), (20, 0)))
    pool = world.create_buoyancy_controller(offset=5, normal=(0, 1), density=2, linear_drag=2, angular_drag=1)
    grav = world.create_gravity_controller(G=2.0, inv_sqr=True)
    balls = []
    for i in range(4):
        b = world.create_dynamic_body(position=(-6 + 4 * i, 8),
                                      fixtures=b2.Fixture(shape=b2.Circle(radius=0.7), density=1.0))
        pool.add_body(b)
        balls.append(b)
    box = world.create_dynamic_body(position=(2, 9), angle=0.4)
    box.create_polygon_fixture(box=(0.6, 0.4), density=1.0, friction=0.4)
    pool.add_body(box)
    m1 = world.create_dynamic_body(position=(10, 12))
    m1.create_circle_fixture(0.5, density=3.0)
    m2 = world.create_dynamic_body(position=(13, 12))
    m2.create_circle_fixture(0.5, density=3.0)
    grav.add_body(m1)
    grav.add_body(m2)
    grav.add_body(box)

    def run(n):
        for _ in range(n):
            world.step(DT, VEL_ITERS, POS_ITERS)

    snap("s0", world)
    run(30)
    snap("s30", world)
    pool.density = 3.0
    pool.offset = 6.0
    pool.velocity = (1.0, 0.0)
    grav.G = 4.0
    run(1)
    snap("s31", world)
    run(29)
    snap("s60", world)
    pool.remove_body(balls[0])
    pool.add_body(m1)
    world.destroy_body(balls[2])
    run(1)
    snap("s61", world)
    run(29)
    snap("s90", world)
    world.destroy_controller(grav)
    world.create_buoyancy_controller(bodies=[balls[1], m2], offset=7, density=1, linear_drag=0.5, gravity=(0, 0))
    run(30)
    snap("s120", world)
    return world

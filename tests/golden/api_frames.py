"""Body frame helpers and World flags through the World API, run on the
reference by make_golden_queries.py and on pypybox2d_gb300 by
tests/test_world_batch.py (no step: host records only).

Returns one row per (body, probe point): the body's get_world_point,
get_world_vector, get_local_point, get_local_vector,
get_linear_velocity_from_world_point and
get_linear_velocity_from_local_point of the probe and its mass_data, and
the World flags."""

PROBES = ((0.0, 0.0), (1.25, -0.5), (-3.0, 2.75), (0.1, 0.3))


def build(b2):
    world = b2.World(gravity=(0, -10), do_sleep=True)
    world.create_static_body(position=(0, -1)).create_polygon_fixture(box=(10, 1))
    for i in range(5):
        b = world.create_dynamic_body(position=(-4.0 + 2.0 * i, 1.5 + 0.3 * i), angle=0.7 * i - 1.1,
                                      linear_velocity=(0.5 * i - 1.0, 0.25 * i), angular_velocity=0.4 * i - 0.9)
        if i % 2:
            b.create_circle_fixture(radius=0.4, density=1.0)
        else:
            b.create_polygon_fixture(box=(0.5, 0.25), density=2.0)
    return world


def rows(b2):
    world = build(b2)
    out = []
    for body in world.bodies:
        for p in PROBES:
            vals = (body.get_world_point(p), body.get_world_vector(p), body.get_local_point(p),
                    body.get_local_vector(p), body.get_linear_velocity_from_world_point(p),
                    body.get_linear_velocity_from_local_point(p))
            md = body.mass_data
            out.append([float(c) for v in vals for c in (v[0], v[1])] +
                       [float(md.mass), float(md.I), float(md.center[0]), float(md.center[1])])
    flags = [world.warm_starting, world.continuous_physics, world.allow_sleep, world.auto_clear_forces]
    return out, flags


def destroy_rows(b2, on_world=lambda world: None):
    """create_fixtures on a dynamic body, then destroy_fixture twice: the
    body's mass data and fixture count after each call (and the world)."""
    world = build(b2)
    on_world(world)
    body = world.bodies[2]
    body.create_fixtures([b2.Polygon(box=(0.3, 0.2)), b2.Circle(radius=0.25, position=(0.4, -0.1))], density=3.0,
                         friction=0.7)
    out = []

    def record():
        md = body.mass_data
        out.append([float(len(body.fixtures)), float(md.mass), float(md.I), float(md.center[0]),
                    float(md.center[1]), float(body.world_center[0]), float(body.world_center[1]),
                    float(body.linear_velocity[0]), float(body.linear_velocity[1])])

    record()
    body.destroy_fixture(body.fixtures[0])
    record()
    body.destroy_fixture(body.fixtures[1])
    record()
    return out, world


STEPS_AFTER_DESTROY = 40


def mass_rows(b2, on_world=lambda world: None):
    """mass_data overrides (a normal one, one with zero mass and inertia) and
    reset_mass_data: each body's mass data, centre and velocity after each
    call (and the world)."""
    world = build(b2)
    on_world(world)
    MassData = b2.shapes.MassData
    out = []

    def record(body):
        md = body.mass_data
        out.append([float(md.mass), float(md.I), float(md.center[0]), float(md.center[1]),
                    float(body.world_center[0]), float(body.world_center[1]),
                    float(body.linear_velocity[0]), float(body.linear_velocity[1])])

    a, b, c = world.bodies[2], world.bodies[3], world.bodies[0]
    a.mass_data = MassData(mass=2.5, center=(0.1, -0.2), I=0.8)
    record(a)
    b.mass_data = MassData(mass=0.0, center=(0.05, 0.05), I=0.0)
    record(b)
    c.mass_data = MassData(mass=3.0, center=(1.0, 1.0), I=2.0)     # static: unchanged
    record(c)
    b.reset_mass_data()
    record(b)
    return out, world


def type_rows(b2, on_world=lambda world: None):
    """fixed_rotation, sleeping and type setters: each changed body's type,
    mass data, velocity and sleep state afterwards (and the world)."""
    world = build(b2)
    on_world(world)
    bodies = world.bodies
    bodies[1].fixed_rotation = True
    bodies[2].sleeping = True
    bodies[3].type = b2.Body.STATIC
    bodies[4].type = b2.Body.KINEMATIC
    bodies[5].type = b2.Body.KINEMATIC
    bodies[5].type = b2.Body.DYNAMIC
    out = []
    for body in bodies:
        md = body.mass_data
        out.append([float(body.type), float(md.mass), float(md.I), float(md.center[0]), float(md.center[1]),
                    float(body.linear_velocity[0]), float(body.linear_velocity[1]), float(body.angular_velocity),
                    float(body.awake), float(body.fixed_rotation)])
    return out, world


def fixture_rows(b2, on_world=lambda world: None):
    """Fixture material and filter setters: friction, restitution, density
    (then reset_mass_data), sensor, group index and mask bits; each body's
    mass data afterwards (and the world)."""
    world = build(b2)
    on_world(world)
    bodies = world.bodies
    bodies[1].fixtures[0].friction = 0.95
    bodies[2].fixtures[0].restitution = 0.6
    bodies[3].fixtures[0].density = 4.0
    bodies[3].reset_mass_data()
    bodies[4].fixtures[0].sensor = True
    bodies[0].fixtures[0].group_index = -2
    bodies[5].fixtures[0].group_index = -2
    bodies[1].fixtures[0].mask_bits = 0xFFFE
    bodies[1].fixtures[0].category_bits = 0x0002
    out = []
    for body in bodies:
        md = body.mass_data
        f = body.fixtures[0]
        out.append([float(md.mass), float(md.I), float(f.friction), float(f.restitution), float(f.density),
                    float(f.sensor), float(f.group_index), float(f.mask_bits), float(f.category_bits),
                    float(body.awake)])
    return out, world

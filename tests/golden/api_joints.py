"""A scripted joint session of the World API, run on the reference by
make_golden.py (api_joints.npz) and on pypybox2d_gb300 by
tests/test_world_joints.py.

Joints are created through the World API (world.create_*_joint with world
anchors, an axis, limits, motors and springs), stepped, edited between steps
through their setters (motor speed and torque, limit switches and limits,
spring length and frequency), destroyed, created between two bodies whose
contact the joint then filters out, and removed with their body
(destroy_body, reporting each joint to joint_destruction_listener).  Every
snapshot records the bodies, fat boxes, contacts, joint records and the
joint getters (anchors, reaction force and torque, angle, translation,
speed, motor torque).  Apart from the two circles that touch before they
are joined, each island holds at most one joint beside contacts with the
static ground, so the float64 GPU step solves most islands in the
reference's order.
"""
DT = 1.0 / 60.0
VEL_ITERS, POS_ITERS = 8, 3
SNAPS = ("s0", "s1", "s30", "s60", "s90", "s120", "s150", "s200")
GETTERS = 14   # floats per joint in a getter row


def getter_row(j, inv_dt=60.0):
    """The joint getters of one joint, padded to GETTERS floats (NaN for a
    getter that raises IndexError: the reference's revolute
    get_reaction_force slices its Vec3 impulse, which Vec3.__getitem__
    refuses, revolute.py:208 and common.py:303-311)."""
    try:
        force = tuple(j.get_reaction_force(inv_dt))
    except IndexError:
        force = (float("nan"), float("nan"))
    row = [*j.anchor_a, *j.anchor_b, *force, j.get_reaction_torque(inv_dt)]
    name = type(j).__name__
    if name == "RevoluteJoint":
        row += [j.joint_angle, j.joint_speed, j.get_motor_torque(inv_dt), j.motor_speed, j.lower_angle, j.upper_angle]
    elif name == "PrismaticJoint":
        row += [j.joint_translation, j.joint_speed, *j.axis, j.lower_limit, j.upper_limit]
    elif name == "DistanceJoint":
        row += [j.length, j.frequency, j.damping_ratio]
    return [float(x) for x in row] + [0.0] * (GETTERS - len(row))


def script(b2, snap, on_world=lambda world: None, log=None):
    world = b2.World((0, -10), True)
    on_world(world)
    if log is not None:
        world.joint_destruction_listener = lambda j: log.append(type(j).__name__)
    ground = world.create_static_body(position=(0, -1))
    ground.create_polygon_fixture(box=(60, 1))
    # a motorised pendulum with an angle limit
    hub = world.create_static_body(position=(-20, 8))
    hub.create_circle_fixture(0.2)
    arm = world.create_dynamic_body(position=(-18.5, 8))
    arm.create_polygon_fixture(box=(1.5, 0.2), density=2.0, friction=0.4)
    rev = world.create_revolute_joint(hub, arm, anchor=(-20, 8), lower_angle=-1.0, upper_angle=0.5, limit_enabled=True,
                                      motor_speed=-1.0, max_motor_torque=60.0, motor_enabled=True)
    # a slider on the ground along x, with limits and a motor
    sled = world.create_dynamic_body(position=(-10, 0.3))
    sled.create_polygon_fixture(box=(0.6, 0.3), density=1.0, friction=0.3)
    pri = world.create_prismatic_joint(ground, sled, anchor=(-10, 0.3), axis=(1, 0), lower_limit=-2.0, upper_limit=3.0,
                                       limit_enabled=True, motor_speed=2.0, max_motor_force=20.0, motor_enabled=True)
    # two circles held apart by a rigid distance joint, a box on a soft spring
    c1 = world.create_dynamic_body(position=(0, 3))
    c1.create_circle_fixture(0.4, density=1.0, friction=0.5)
    c2 = world.create_dynamic_body(position=(2, 4))
    c2.create_circle_fixture(0.3, density=1.0, friction=0.5)
    dist = world.create_distance_joint(c1, c2, anchor_a=(0, 3), anchor_b=(2, 4))
    post = world.create_static_body(position=(8, 10))
    post.create_polygon_fixture(box=(0.2, 0.2))
    bob = world.create_dynamic_body(position=(8.5, 6))
    bob.create_polygon_fixture(box=(0.3, 0.3), density=2.0, friction=0.4)
    spring = world.create_distance_joint(post, bob, anchor_a=(8, 10), anchor_b=(8.5, 6.3), frequency=1.5,
                                         damping_ratio=0.2)
    # two boxes welded into an L, dropped on the ground
    w1 = world.create_dynamic_body(position=(15, 3))
    w1.create_polygon_fixture(box=(1.0, 0.2), density=1.0, friction=0.6)
    w2 = world.create_dynamic_body(position=(16.2, 3.8), angle=0.2)
    w2.create_polygon_fixture(box=(0.2, 1.0), density=1.0, friction=0.6)
    world.create_weld_joint(w1, w2, anchor=(16.0, 3.0))
    # two free circles that will touch and then be joined
    f1 = world.create_dynamic_body(position=(25, 0.5))
    f1.create_circle_fixture(0.5, density=1.0, friction=0.3)
    f2 = world.create_dynamic_body(position=(25.95, 0.5))
    f2.create_circle_fixture(0.5, density=1.0, friction=0.3)
    steps = [0]

    def run(n):
        for _ in range(n):
            steps[0] += 1
            world.step(DT, VEL_ITERS, POS_ITERS)

    snap("s0", world)
    run(1)
    snap("s1", world)
    run(29)
    snap("s30", world)
    rev.motor_speed = 1.5
    rev.max_motor_torque = 120.0
    pri.motor_speed = -3.0
    spring.frequency = 3.0
    spring.length = 3.0
    world.create_revolute_joint(f1, f2, anchor=(25.45, 0.5))   # filters the circles' contact out
    run(30)
    snap("s60", world)
    rev.limit_enabled = False
    pri.upper_limit = 1.0
    pri.motor_enabled = False
    dist.length = 1.5
    run(30)
    snap("s90", world)
    rev.limit_enabled = True
    rev.lower_angle = -0.3
    rev.upper_angle = 0.3
    pri.limit_enabled = False
    world.destroy_joint(spring)
    run(30)
    snap("s120", world)
    world.destroy_body(c2)
    rev.motor_enabled = False
    run(30)
    snap("s150", world)
    world.destroy_body(arm)
    run(50)
    snap("s200", world)
    return world

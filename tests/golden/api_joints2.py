"""A scripted session of the friction, rope, wheel, pulley and mouse joints through
the World API, run on the reference by make_golden.py (api_joints2.npz) and
on pypybox2d_gb300 by tests/test_world_joints.py.

The joints are created with world.create_*_joint, stepped, edited between
steps through their setters (friction force and torque limits; the wheel's
motor switch, speed and torque), and destroyed; every snapshot records the
bodies, contacts, joint records and the joint getters (anchors, reaction
force and torque, and per kind: friction limits; rope maximum length;
wheel translation, speed, motor torque and axis; pulley lengths, ground
anchors and ratio).
"""
DT = 1.0 / 60.0
VEL_ITERS, POS_ITERS = 8, 3
SNAPS = ("s0", "s1", "s30", "s60", "s90", "s120")
GETTERS = 12   # floats per joint in a getter row


def getter_row(j, inv_dt=60.0):
    """The getters of one joint, padded to GETTERS floats (the reference's
    rope and mouse joints have no anchor properties: zeros there)."""
    name = type(j).__name__
    anchors = [0.0] * 4 if name in ("RopeJoint", "MouseJoint") else [*j.anchor_a, *j.anchor_b]
    row = [*anchors, *j.get_reaction_force(inv_dt), j.get_reaction_torque(inv_dt)]
    if name == "FrictionJoint":
        row += [j.max_force, j.max_torque]
    elif name == "RopeJoint":
        row += [j.max_length]
    elif name == "WheelJoint":
        row += [j.joint_translation, j.joint_speed, j.motor_torque(inv_dt), j.motor_speed, j.max_motor_torque]
    elif name == "PulleyJoint":
        row += [j.length_a, j.length_b, j.ratio]
    elif name == "MouseJoint":
        row += [*j.target, j.max_force, j.frequency, j.damping_ratio]
    return [float(x) for x in row] + [0.0] * (GETTERS - len(row))


def script(b2, snap, on_world=lambda world: None):
    world = b2.World((0, -10), True)
    on_world(world)
    ground = world.create_static_body(position=(0, -1))
    ground.create_polygon_fixture(box=(40, 1))
    sled = world.create_dynamic_body(position=(-12, 0.5), linear_velocity=(3, 0))
    sled.create_polygon_fixture(box=(0.5, 0.5), density=1.0, friction=0.2)
    fr = world.create_friction_joint(ground, sled, local_anchor_a=(-12, 1.5), local_anchor_b=(0, 0), max_force=2.0,
                                     max_torque=0.5)
    post = world.create_static_body(position=(-4, 6))
    post.create_circle_fixture(0.2)
    bob = world.create_dynamic_body(position=(-2, 5))
    bob.create_circle_fixture(0.3, density=1.0)
    rope = world.create_rope_joint(post, bob, local_anchor_a=(0, 0), local_anchor_b=(0, 0), max_length=3.0)
    body = world.create_dynamic_body(position=(4, 1.2))
    body.create_polygon_fixture(box=(1.0, 0.25), density=1.0)
    wheel = world.create_dynamic_body(position=(4.6, 0.45))
    wheel.create_circle_fixture(0.45, density=1.0, friction=0.9)
    wj = world.create_wheel_joint(body, wheel, anchor=(4.6, 0.45), axis=(0, 1), frequency=3.0, damping_ratio=0.5,
                                  motor_enabled=False, max_motor_torque=10.0)
    left = world.create_dynamic_body(position=(10, 4))
    left.create_polygon_fixture(box=(0.3, 0.3), density=1.0)
    right = world.create_dynamic_body(position=(13, 3))
    right.create_polygon_fixture(box=(0.3, 0.3), density=2.0)
    world.create_pulley_joint(left, right, ground_anchor_a=(10, 9), ground_anchor_b=(13, 9), anchor_a=(10, 4.3),
                              anchor_b=(13, 3.3), ratio=1.0)
    crate = world.create_dynamic_body(position=(18, 0.3))
    crate.create_polygon_fixture(box=(0.4, 0.3), density=1.0, friction=0.6)
    mouse = world.create_mouse_joint(crate, target=(18.2, 0.4), max_force=30.0, frequency=4.0, damping_ratio=0.7)

    def run(n):
        for _ in range(n):
            world.step(DT, VEL_ITERS, POS_ITERS)

    snap("s0", world)
    run(1)
    snap("s1", world)
    run(29)
    snap("s30", world)
    fr.max_force = 6.0
    fr.max_torque = 0.0
    wj.motor_enabled = True
    wj.motor_speed = -5.0
    mouse.target = (20, 2.5)
    run(30)
    snap("s60", world)
    wj.max_motor_torque = 2.0
    mouse.max_force = 5.0
    mouse.frequency = 2.0
    world.destroy_joint(rope)
    run(30)
    snap("s90", world)
    wj.motor_enabled = False
    world.destroy_joint(fr)
    run(30)
    snap("s120", world)
    return world

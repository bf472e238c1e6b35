"""A second restatement of the reference's body update and frame loop, in
plain Python (TEST INFRASTRUCTURE: only tests/test_oracle_second_restatement.py
uses it).

RigidBody.Integrate and CalculateDerivedData (rigidbody.go:213-299) and the
frame of examples/cubedrop.go:29-75 (every body integrated, the ordered
narrowphase of oracle/colliders_ref.py, ResolveContacts of
oracle/contact_ref.py), written from the Go source independently of the C++
oracle.  Bodies are the dicts of those two modules plus acceleration, iit_body
(the body-space inverse inertia, column-major), linear_damping,
angular_damping, can_sleep and motion.
"""
import math

from oracle import colliders_ref, contact_ref
from oracle.contact_ref import add_scaled, dot, m3_mul_vector, mul_with, quat_add_scaled_vector, quat_normalize

SLEEP_EPSILON = 0.3  # rigidbody.go:14 (an untyped constant: 10 * it is exactly 3)


def transform_inertia_tensor(iit_body, t):  # rigidbody.go:275-299
    b = iit_body
    t4 = t[0] * b[0] + t[3] * b[1] + t[6] * b[2]
    t9 = t[0] * b[3] + t[3] * b[4] + t[6] * b[5]
    t14 = t[0] * b[6] + t[3] * b[7] + t[6] * b[8]
    t28 = t[1] * b[0] + t[4] * b[1] + t[7] * b[2]
    t33 = t[1] * b[3] + t[4] * b[4] + t[7] * b[5]
    t38 = t[1] * b[6] + t[4] * b[7] + t[7] * b[8]
    t52 = t[2] * b[0] + t[5] * b[1] + t[8] * b[2]
    t57 = t[2] * b[3] + t[5] * b[4] + t[8] * b[5]
    t62 = t[2] * b[6] + t[5] * b[7] + t[8] * b[8]
    w = [0.0] * 9
    w[0] = t4 * t[0] + t9 * t[3] + t14 * t[6]
    w[3] = t4 * t[1] + t9 * t[4] + t14 * t[7]
    w[6] = t4 * t[2] + t9 * t[5] + t14 * t[8]
    w[1] = t28 * t[0] + t33 * t[3] + t38 * t[6]
    w[4] = t28 * t[1] + t33 * t[4] + t38 * t[7]
    w[7] = t28 * t[2] + t33 * t[5] + t38 * t[8]
    w[2] = t52 * t[0] + t57 * t[3] + t62 * t[6]
    w[5] = t52 * t[1] + t57 * t[4] + t62 * t[7]
    w[8] = t52 * t[2] + t57 * t[5] + t62 * t[8]
    return w


def calculate_derived_data(b):  # rigidbody.go:268-272
    quat_normalize(b["orientation"])
    t = colliders_ref.set_as_transform(b["position"], b["orientation"])
    b["iit"] = transform_inertia_tensor(b["iit_body"], t)


def set_awake(b, awake):  # rigidbody.go:182-192
    if awake:
        b["awake"] = True
        b["motion"] = SLEEP_EPSILON * 2.0
    else:
        b["awake"] = False
        b["velocity"] = [0.0, 0.0, 0.0]
        b["rotation"] = [0.0, 0.0, 0.0]


def integrate(b, dt):  # rigidbody.go:213-259, no forces or torques accumulated
    if not b["awake"]:
        return
    force, torque = [0.0, 0.0, 0.0], [0.0, 0.0, 0.0]
    lfa = list(b["acceleration"])
    add_scaled(lfa, force, b["inverse_mass"])
    b["lfa"] = lfa
    ang_acc = m3_mul_vector(b["iit"], torque)
    add_scaled(b["velocity"], lfa, dt)
    add_scaled(b["rotation"], ang_acc, dt)
    mul_with(b["velocity"], math.pow(b["linear_damping"], dt))
    mul_with(b["rotation"], math.pow(b["angular_damping"], dt))
    add_scaled(b["position"], b["velocity"], dt)
    quat_add_scaled_vector(b["orientation"], b["rotation"], dt)
    calculate_derived_data(b)
    if b["can_sleep"]:
        current = dot(b["velocity"], b["velocity"]) + dot(b["rotation"], b["rotation"])
        bias = math.pow(0.5, dt)
        b["motion"] = bias * b["motion"] + (1.0 - bias) * current
        if b["motion"] < SLEEP_EPSILON:
            set_awake(b, False)
        elif b["motion"] > 10 * SLEEP_EPSILON:
            b["motion"] = 3.0


def step(bodies, plane, dt, iter_mult=4):
    """One frame of examples/cubedrop.go:69-75 (with the batch's iteration
    multiplier); returns (contacts, adjustPositions and adjustVelocities
    iterations)."""
    for b in bodies:
        integrate(b, dt)
    found = colliders_ref.generate_contacts(bodies, plane)
    contacts = [contact_ref.Contact(b0, b1, p, n, pen) for b0, b1, p, n, pen in found]
    pos_used, vel_used = contact_ref.resolve_contacts(len(contacts) * iter_mult, contacts, bodies, dt)
    return len(contacts), pos_used, vel_used

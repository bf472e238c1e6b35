"""A second restatement of the reference's body update and frame loop, in
plain Python (TEST INFRASTRUCTURE: only tests/test_oracle_second_restatement.py
uses it).

RigidBody.Integrate and CalculateDerivedData (rigidbody.go:213-299) and the
frame of examples/cubedrop.go:29-75 (every body integrated, the ordered
narrowphase of oracle/colliders_ref.py, ResolveContacts of
oracle/contact_ref.py), written from the Go source independently of the C++
oracle.  Bodies are the dicts of those two modules plus acceleration, iit_body
(the body-space inverse inertia, column-major), linear_damping,
angular_damping, can_sleep and motion.  With numpy float32 values it states
the precision form (see oracle/contact_ref.py): the quaternion
renormalisation is its float64 island here.
"""
import math

from oracle import colliders_ref, contact_ref
from oracle.contact_ref import (add_scaled, dot, m3_mul_vector, mul_with, quat_add_scaled_vector, quat_normalize,
                                quat_normalize_island,
                                real_type)

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
    q = b["orientation"]
    rt = real_type(*q)
    qw = [float(x) for x in q]  # the renormalisation in float64
    if rt is float:
        quat_normalize(qw)
    else:
        quat_normalize_island(qw)
    b["orientation"] = [rt(x) for x in qw]
    t = colliders_ref.set_as_transform(b["position"], b["orientation"])
    b["iit"] = transform_inertia_tensor(b["iit_body"], t)


def set_awake(b, awake):  # rigidbody.go:182-192
    rt = real_type(b["motion"])
    if awake:
        b["awake"] = True
        b["motion"] = rt(SLEEP_EPSILON * 2.0)
    else:
        b["awake"] = False
        b["velocity"] = [rt(0.0)] * 3
        b["rotation"] = [rt(0.0)] * 3


def integrate(b, dt):  # rigidbody.go:213-259, no forces or torques accumulated
    """dt is the float64 frame time; the damping powers pow(d, dt) and the
    sleep bias pow(0.5, dt) are taken in float64 and rounded to the bodies'
    type, as the batch computes them once on the host."""
    if not b["awake"]:
        return
    rt = real_type(b["inverse_mass"])
    duration = rt(dt)
    force, torque = [rt(0.0)] * 3, [rt(0.0)] * 3
    lfa = list(b["acceleration"])
    add_scaled(lfa, force, b["inverse_mass"])
    b["lfa"] = lfa
    ang_acc = m3_mul_vector(b["iit"], torque)
    add_scaled(b["velocity"], lfa, duration)
    add_scaled(b["rotation"], ang_acc, duration)
    mul_with(b["velocity"], rt(math.pow(b["linear_damping"], dt)))
    mul_with(b["rotation"], rt(math.pow(b["angular_damping"], dt)))
    add_scaled(b["position"], b["velocity"], duration)
    quat_add_scaled_vector(b["orientation"], b["rotation"], duration)
    calculate_derived_data(b)
    if b["can_sleep"]:
        current = dot(b["velocity"], b["velocity"]) + dot(b["rotation"], b["rotation"])
        bias = rt(math.pow(0.5, dt))
        b["motion"] = bias * b["motion"] + (rt(1.0) - bias) * current
        if b["motion"] < rt(SLEEP_EPSILON):
            set_awake(b, False)
        elif b["motion"] > rt(10 * SLEEP_EPSILON):
            b["motion"] = rt(10 * SLEEP_EPSILON)


def step(bodies, plane, dt, iter_mult=4, units=None, trace=None):
    """One frame of examples/cubedrop.go:69-75 (with the batch's iteration
    multiplier), or with `units` a caller's test list in place of the
    all-pairs order (examples/ballistic.go:47-104); returns (contacts,
    adjustPositions and adjustVelocities iterations).  `trace`: see
    contact_ref.resolve_contacts."""
    for b in bodies:
        integrate(b, dt)
    if units is None:
        found = colliders_ref.generate_contacts(bodies, plane)
    else:
        found = colliders_ref.collide_units(bodies, plane, units)
    contacts = [contact_ref.Contact(b0, b1, p, n, pen) for b0, b1, p, n, pen in found]
    pos_used, vel_used = contact_ref.resolve_contacts(len(contacts) * iter_mult, contacts, bodies, dt, trace)
    return len(contacts), pos_used, vel_used

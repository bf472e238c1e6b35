"""A second restatement of the reference's contact resolver, in plain Python
(TEST INFRASTRUCTURE: only tests/test_oracle_second_restatement.py uses it).

ResolveContacts and everything it calls (contact.go:59-616) with the math it
needs (math/math.go:64-78, math/vector.go, math/matrix.go:37-165,
math/quaternion.go:20-99), written from the Go source independently of the
C++ oracle (oracle/cubez_ref.hpp).  Python floats are IEEE doubles and Python
evaluates left to right without fused multiply-adds, so this is the
reference's float64 arithmetic; the test runs both restatements on the same
contact sets and compares every bit.  Pure-Python loops: small worlds only.

Vectors are lists of 3 floats, Matrix3 lists of 9 (column-major), Quat lists
(w, x, y, z).  Bodies are dicts (see oracle/rigidbody_ref.py); a sleeping body
needs its iit_body for the derived data that applyPositionChange refreshes.

The same code also states the precision form (float32 with float64 islands):
given numpy float32 values, every operation stays in float32 (Python float
constants convert to float32 first, NumPy's scalar rules), and the islands
convert to Python floats (float64) and back, where the precision form keeps
float64: the friction solve's inversion and product, and the position and
orientation accumulated across adjustPositions.
"""
import math

import numpy as np

EPSILON = 1e-7
EPSILON2 = EPSILON * EPSILON
MIN_NORMAL = 1.1754943508222875e-38
MAX_VALUE = 1.7976931348623157e308
POSITION_EPSILON = 0.01
VELOCITY_EPSILON = 0.01


def real_type(*xs):
    """np.float32 when any value is float32 (the precision form), else float."""
    return np.float32 if any(isinstance(x, np.float32) for x in xs) else float


def sqrt_(x):
    return np.sqrt(x) if isinstance(x, np.float32) else math.sqrt(x)


def real_equal(a, b):  # math/math.go:64-78, with the constants in the values' type
    t = real_type(a, b)
    eps = t(EPSILON)
    if a == b:
        return True
    diff = abs(a - b)
    if a * b == 0 or diff < t(MIN_NORMAL):
        return diff < eps * eps
    return diff / (abs(a) + abs(b)) < eps


# ---------------------------------------------------------------- vector.go
def cross(v, o):
    return [v[1] * o[2] - v[2] * o[1], v[2] * o[0] - v[0] * o[2], v[0] * o[1] - v[1] * o[0]]


def dot(v, o):
    return v[0] * o[0] + v[1] * o[1] + v[2] * o[2]


def magnitude(v):
    return sqrt_(v[0] * v[0] + v[1] * v[1] + v[2] * v[2])


def add(v, o):
    v[0] += o[0]
    v[1] += o[1]
    v[2] += o[2]


def add_scaled(v, o, s):
    v[0] += o[0] * s
    v[1] += o[1] * s
    v[2] += o[2] * s


def mul_with(v, s):
    for i in range(len(v)):
        v[i] *= s


# ---------------------------------------------------------------- matrix.go
def m3_mul_vector(m, v):
    return [m[0] * v[0] + m[3] * v[1] + m[6] * v[2],
            m[1] * v[0] + m[4] * v[1] + m[7] * v[2],
            m[2] * v[0] + m[5] * v[1] + m[8] * v[2]]


def m3_transform_transpose(m, v):
    return [v[0] * m[0] + v[1] * m[1] + v[2] * m[2],
            v[0] * m[3] + v[1] * m[4] + v[2] * m[5],
            v[0] * m[6] + v[1] * m[7] + v[2] * m[8]]


def m3_mul(a, b):
    out = []
    for c in range(3):
        for r in range(3):
            out.append(a[r] * b[3 * c] + a[3 + r] * b[3 * c + 1] + a[6 + r] * b[3 * c + 2])
    return out


def m3_transpose(m):
    return [m[0], m[3], m[6], m[1], m[4], m[7], m[2], m[5], m[8]]


def m3_invert(m):  # math/matrix.go:133-153
    det = m[0] * m[4] * m[8] + m[3] * m[7] * m[2] + m[6] * m[1] * m[5] - m[6] * m[4] * m[2] - \
        m[3] * m[1] * m[8] - m[0] * m[7] * m[5]
    if real_equal(det, 0.0):
        return [0.0] * 9
    r = [m[4] * m[8] - m[5] * m[7], m[2] * m[7] - m[1] * m[8], m[1] * m[5] - m[2] * m[4],
         m[5] * m[6] - m[3] * m[8], m[0] * m[8] - m[2] * m[6], m[2] * m[3] - m[0] * m[5],
         m[3] * m[7] - m[4] * m[6], m[1] * m[6] - m[0] * m[7], m[0] * m[4] - m[1] * m[3]]
    mul_with(r, 1 / det)
    return r


def skew(v):  # contact.go:612-616
    return [0.0, v[2], -v[1], -v[2], 0.0, v[0], v[1], -v[0], 0.0]


# ---------------------------------------------------------------- quaternion.go
def quat_scaled_increment(q, v, scale):  # quaternion.go:20-33 up to the sum
    t = [0.0, v[0] * scale, v[1] * scale, v[2] * scale]
    w = t[0] * q[0] - t[1] * q[1] - t[2] * q[2] - t[3] * q[3]
    x = t[0] * q[1] + t[1] * q[0] + t[2] * q[3] - t[3] * q[2]
    y = t[0] * q[2] + t[2] * q[0] + t[3] * q[1] - t[1] * q[3]
    z = t[0] * q[3] + t[3] * q[0] + t[1] * q[2] - t[2] * q[1]
    return [w * 0.5, x * 0.5, y * 0.5, z * 0.5]


def quat_add_scaled_vector(q, v, scale):  # quaternion.go:20-33
    inc = quat_scaled_increment(q, v, scale)
    for k in range(4):
        q[k] += inc[k]


def quat_normalize_island(q):
    """The precision form's float64 renormalisation of q (a list of floats):
    with s = |q|^2 and e = s - 1, nothing when |e| < 4e-7 (where
    RealEqual(1, |q|) holds), q * 1/sqrt(s) from its five-term Taylor series
    in e when |e| < 2^-11, else Normalize."""
    s = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]
    e = s - 1.0
    if abs(e) < 4e-7:
        return
    if abs(e) < 2.0 ** -11:
        inv = 1.0 + e * (-0.5 + e * (0.375 + e * (-0.3125 + e * 0.2734375)))
        for i in range(4):
            q[i] *= inv
        return
    quat_normalize(q)


def quat_normalize(q):  # quaternion.go:78-99
    length = math.sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3])
    if real_equal(1.0, length):
        return
    if length == 0.0:
        q[:] = [1.0, 0.0, 0.0, 0.0]
        return
    if length == math.inf:
        length = MAX_VALUE
    inv = 1.0 / length
    for i in range(4):
        q[i] *= inv


# ---------------------------------------------------------------- contact.go
class Contact:
    """The exported fields (contact.go:17-36) and the private ones
    (contact.go:38-50); bodies are indices into the body list or None."""

    def __init__(self, b0, b1, point, normal, penetration, friction=0.9, restitution=0.1):
        self.bodies = [b0, b1]
        self.point = list(point)
        self.normal = list(normal)
        self.penetration = penetration
        self.friction = friction
        self.restitution = restitution
        self.to_world = [0.0] * 9
        self.rel = [[0.0] * 3, [0.0] * 3]
        self.velocity = [0.0] * 3
        self.desired = 0.0


def _basis(c):  # contact.go:118-156
    n = c.normal
    if abs(n[0]) > abs(n[1]):
        s = 1.0 / sqrt_(n[2] * n[2] + n[0] * n[0])
        ty = [n[2] * s, 0.0, n[0] * -s]
        tz = [n[1] * ty[0], n[2] * ty[0] - n[0] * ty[2], -n[1] * ty[0]]
    else:
        s = 1.0 / sqrt_(n[2] * n[2] + n[1] * n[1])
        ty = [0.0, -n[2] * s, n[1] * s]
        tz = [n[1] * ty[2] - n[2] * ty[1], -n[0] * ty[2], n[0] * ty[1]]
    c.to_world = [n[0], n[1], n[2], ty[0], ty[1], ty[2], tz[0], tz[1], tz[2]]


def _local_velocity(c, k, bodies, dt):  # contact.go:159-182
    b = bodies[c.bodies[k]]
    v = cross(b["rotation"], c.rel[k])
    add(v, b["velocity"])
    cv = m3_transform_transpose(c.to_world, v)
    acc = list(b["lfa"])
    mul_with(acc, dt)
    acc = m3_transform_transpose(c.to_world, acc)
    acc[0] = 0.0
    add(cv, acc)
    return cv


def _desired(c, bodies, dt):  # contact.go:87-112
    from_acc = 0.0
    b0 = bodies[c.bodies[0]]
    if b0["awake"]:
        t = list(b0["lfa"])
        mul_with(t, dt)
        from_acc += dot(t, c.normal)
    if c.bodies[1] is not None and bodies[c.bodies[1]]["awake"]:
        t = list(bodies[c.bodies[1]]["lfa"])
        mul_with(t, dt)
        from_acc -= dot(t, c.normal)
    e = c.restitution
    if abs(c.velocity[0]) < 0.25:
        e = 0.0
    c.desired = -c.velocity[0] - e * (c.velocity[0] - from_acc)


def _internals(c, bodies, dt):  # contact.go:59-85
    if c.bodies[0] is None:
        mul_with(c.normal, -1.0)
        c.bodies[0], c.bodies[1] = c.bodies[1], None
    _basis(c)
    c.rel[0] = [c.point[i] - bodies[c.bodies[0]]["position"][i] for i in range(3)]
    c.velocity = _local_velocity(c, 0, bodies, dt)
    if c.bodies[1] is not None:
        c.rel[1] = [c.point[i] - bodies[c.bodies[1]]["position"][i] for i in range(3)]
        v1 = _local_velocity(c, 1, bodies, dt)
        c.velocity = [c.velocity[i] - v1[i] for i in range(3)]
    _desired(c, bodies, dt)


def _match_awake_state(c, bodies):  # contact.go:185-202
    if c.bodies[1] is None:
        return
    from oracle.rigidbody_ref import set_awake
    a0, a1 = bodies[c.bodies[0]]["awake"], bodies[c.bodies[1]]["awake"]
    if (a0 or a1) and not (a0 and a1):
        set_awake(bodies[c.bodies[1]] if a0 else bodies[c.bodies[0]], True)


def _apply_position_change(c, bodies, penetration):  # contact.go:286-386
    ang_i, lin_i = [0.0, 0.0], [0.0, 0.0]
    ang_m, lin_m = [0.0, 0.0], [0.0, 0.0]
    lin_change = [[0.0] * 3, [0.0] * 3]
    ang_change = [[0.0] * 3, [0.0] * 3]
    total = 0.0
    for i in range(2):
        if c.bodies[i] is None:
            continue
        b = bodies[c.bodies[i]]
        w = cross(c.rel[i], c.normal)
        w = m3_mul_vector(b["iit"], w)
        w = cross(w, c.rel[i])
        ang_i[i] = dot(w, c.normal)
        lin_i[i] = b["inverse_mass"]
        total += lin_i[i] + ang_i[i]
    for i in range(2):
        if c.bodies[i] is None:
            continue
        b = bodies[c.bodies[i]]
        sign = 1.0 if i == 0 else -1.0
        ang_m[i] = sign * penetration * (ang_i[i] / total)
        lin_m[i] = sign * penetration * (lin_i[i] / total)
        proj = list(c.rel[i])
        add_scaled(proj, c.normal, -dot(c.rel[i], c.normal))
        max_m = 0.2 * magnitude(proj)
        if ang_m[i] < -max_m:
            t = ang_m[i] + lin_m[i]
            ang_m[i] = -max_m
            lin_m[i] = t - ang_m[i]
        elif ang_m[i] > max_m:
            t = ang_m[i] + lin_m[i]
            ang_m[i] = max_m
            lin_m[i] = t - ang_m[i]
        if ang_m[i] == 0.0:
            ang_change[i] = [0.0, 0.0, 0.0]
        else:
            d = cross(c.rel[i], c.normal)
            ang_change[i] = m3_mul_vector(b["iit"], d)
            mul_with(ang_change[i], ang_m[i] / ang_i[i])
        lin_change[i] = list(c.normal)
        mul_with(lin_change[i], lin_m[i])
        # Position.AddScaled(normal, linearMove) and the orientation change,
        # accumulated in float64 across the iterations (the precision form's
        # island; plain float64 arithmetic in the float64 form)
        t = real_type(lin_m[i])
        pw, qw = b["position_w"], b["orientation_w"]
        for k in range(3):
            pw[k] += float(c.normal[k] * lin_m[i])
        if t is float:
            quat_add_scaled_vector(qw, ang_change[i], 1.0)
        else:
            # the increment in float32 from the orientation rounded to float32,
            # accumulated in float64
            inc = quat_scaled_increment([t(x) for x in qw], ang_change[i], t(1.0))
            for k in range(4):
                qw[k] += float(inc[k])
        if t is float:
            quat_normalize(qw)
        else:
            quat_normalize_island(qw)
        b["position"] = [t(x) for x in pw]
        b["orientation"] = [t(x) for x in qw]
        if not b["awake"]:
            from oracle.rigidbody_ref import calculate_derived_data
            calculate_derived_data(b)
            b["orientation_w"] = [float(x) for x in b["orientation"]]
    return lin_change, ang_change


def _friction_impulse(c, bodies, iits):  # contact.go:535-606
    inv_mass = bodies[c.bodies[0]]["inverse_mass"]
    itt = skew(c.rel[0])
    dvw = m3_mul(itt, iits[0])
    dvw = m3_mul(dvw, itt)
    mul_with(dvw, -1.0)
    if c.bodies[1] is not None:
        itt = skew(c.rel[1])
        d2 = m3_mul(itt, iits[1])
        d2 = m3_mul(d2, itt)
        mul_with(d2, -1.0)
        for i in range(9):
            dvw[i] += d2[i]
        inv_mass += bodies[c.bodies[1]]["inverse_mass"]
    dv = m3_transpose(c.to_world)
    dv = m3_mul(dv, dvw)
    dv = m3_mul(dv, c.to_world)
    dv[0] += inv_mass
    dv[4] += inv_mass
    dv[8] += inv_mass
    # the inversion in float64 (the precision form's island), the product in
    # the bulk type
    t = real_type(dv[0])
    k = [t(x) for x in m3_invert([float(x) for x in dv])]
    kill = [c.desired, -c.velocity[1], -c.velocity[2]]
    ic = m3_mul_vector(k, kill)
    planar = sqrt_(ic[1] * ic[1] + ic[2] * ic[2])
    if planar > ic[0] * c.friction:
        ic[1] /= planar
        ic[2] /= planar
        ic[0] = dv[0] + dv[3] * c.friction * ic[1] + dv[6] * c.friction * ic[2]
        ic[0] = c.desired / ic[0]
        ic[1] *= c.friction * ic[0]
        ic[2] *= c.friction * ic[0]
    return ic


class NilBody(Exception):
    """calculateFrictionlessImpulse on a single-body contact: the reference's
    inverted nil test (contact.go:512) dereferences the missing body."""


def _frictionless_impulse(c, bodies, iits):  # contact.go:496-531
    d = cross(c.rel[0], c.normal)
    d = m3_mul_vector(iits[0], d)
    d = cross(d, c.rel[0])
    dv = dot(d, c.normal)
    dv += bodies[c.bodies[0]]["inverse_mass"]
    if c.bodies[1] is None:  # sic: the second body is added only when there is none
        raise NilBody()
    return [c.desired / dv, 0.0, 0.0]


def _apply_velocity_change(c, bodies):  # contact.go:447-494
    iits = [bodies[c.bodies[0]]["iit"], [0.0] * 9]
    if c.bodies[1] is not None:
        iits[1] = bodies[c.bodies[1]]["iit"]
    if c.friction == 0.0:
        ic = _frictionless_impulse(c, bodies, iits)
    else:
        ic = _friction_impulse(c, bodies, iits)
    impulse = m3_mul_vector(c.to_world, ic)
    vel = [[0.0] * 3, [0.0] * 3]
    rot = [[0.0] * 3, [0.0] * 3]
    b0 = bodies[c.bodies[0]]
    rot[0] = m3_mul_vector(iits[0], cross(c.rel[0], impulse))
    vel[0] = [0.0, 0.0, 0.0]
    add_scaled(vel[0], impulse, b0["inverse_mass"])
    add(b0["velocity"], vel[0])
    add(b0["rotation"], rot[0])
    if c.bodies[1] is not None:
        b1 = bodies[c.bodies[1]]
        rot[1] = m3_mul_vector(iits[1], cross(impulse, c.rel[1]))
        vel[1] = [0.0, 0.0, 0.0]
        add_scaled(vel[1], impulse, -b1["inverse_mass"])
        add(b1["velocity"], vel[1])
        add(b1["rotation"], rot[1])
    return vel, rot


def resolve_contacts(max_iterations, contacts, bodies, dt, trace=None):
    """ResolveContacts (contact.go:208-222); returns the iterations used by
    adjustPositions and adjustVelocities.  `trace` (a list), when given,
    receives ("p", index) / ("v", index) for every contact resolved."""
    if dt <= 0.0 or not contacts:
        return 0, 0
    for b in bodies:
        b["position_w"] = [float(x) for x in b["position"]]
        b["orientation_w"] = [float(x) for x in b["orientation"]]
    for c in contacts:  # prepareContacts, contact.go:225-229
        _internals(c, bodies, dt)
    pos_used = 0  # adjustPositions, contact.go:233-283
    while pos_used < max_iterations:
        best, index = POSITION_EPSILON, len(contacts)
        for i, c in enumerate(contacts):
            if c.penetration > best:
                best, index = c.penetration, i
        if index == len(contacts):
            break
        ct = contacts[index]
        if trace is not None:
            trace.append(("p", index))
        _match_awake_state(ct, bodies)
        lin, ang = _apply_position_change(ct, bodies, best)
        for c in contacts:
            for b in range(2):
                if c.bodies[b] is None:
                    continue
                for d in range(2):
                    if c.bodies[b] == ct.bodies[d]:
                        dp = cross(ang[d], c.rel[b])
                        add(dp, lin[d])
                        sign = -1.0 if b == 0 else 1.0
                        c.penetration += dot(dp, c.normal) * sign
        pos_used += 1
    vel_used = 0  # adjustVelocities, contact.go:388-445
    while vel_used < max_iterations:
        best, index = VELOCITY_EPSILON, len(contacts)
        for i, c in enumerate(contacts):
            if c.desired > best:
                best, index = c.desired, i
        if index == len(contacts):
            break
        ct = contacts[index]
        if trace is not None:
            trace.append(("v", index))
        _match_awake_state(ct, bodies)
        vel, rot = _apply_velocity_change(ct, bodies)
        for c in contacts:
            for b in range(2):
                if c.bodies[b] is None:
                    continue
                for d in range(2):
                    if c.bodies[b] == ct.bodies[d]:
                        dv = cross(rot[d], c.rel[b])
                        add(dv, vel[d])
                        sign = -1.0 if b == 1 else 1.0
                        t = m3_transform_transpose(c.to_world, dv)
                        mul_with(t, sign)
                        add(c.velocity, t)
                        _desired(c, bodies, dt)
        vel_used += 1
    return pos_used, vel_used

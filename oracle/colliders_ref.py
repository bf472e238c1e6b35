"""A second restatement of the reference's narrowphase, in plain Python
(TEST INFRASTRUCTURE: only tests/test_oracle_second_restatement.py uses it).

The colliders (colliders.go:173-770), the Matrix3x4 helpers they use
(math/matrix.go:165-250) and the cubedrop test order (examples/cubedrop.go:
41-67), written from the Go source independently of the C++ oracle.  Python
floats are IEEE doubles evaluated left to right without fused multiply-adds,
so this is the reference's float64 arithmetic.  Pure-Python loops: small
worlds only.

A body is a dict with shape (0 sphere, 1 cube), half (3), radius, position
(3), orientation (w, x, y, z), velocity (3) and offset (12, column-major,
the collider's Offset).  A contact is (body0, body1 or None, point, normal,
penetration).  With numpy float32 values (and a float32 plane) it states the
precision form's narrowphase, which is float32 throughout.
"""
import numpy as np

from oracle.contact_ref import EPSILON, MAX_VALUE, cross, dot, magnitude, mul_with, real_equal, real_type, sqrt_

SPHERE, CUBE = 0, 1

# CheckAgainstHalfSpace's vertex order (colliders.go:318-327)
MULTS = [(1.0, 1.0, 1.0), (-1.0, 1.0, 1.0), (1.0, -1.0, 1.0), (-1.0, -1.0, 1.0),
         (1.0, 1.0, -1.0), (-1.0, 1.0, -1.0), (1.0, -1.0, -1.0), (-1.0, -1.0, -1.0)]


class NoAxis(Exception):
    """The box-box test accepted no axis (only with non-finite transforms);
    the reference indexes HalfSize out of range there."""


# ---------------------------------------------------------------- matrix.go (Matrix3x4)
def set_as_transform(p, q):  # matrix.go:165-185
    w, x, y, z = q
    return [1 - 2 * y * y - 2 * z * z, 2 * x * y + 2 * w * z, 2 * x * z - 2 * w * y,
            2 * x * y - 2 * w * z, 1 - 2 * x * x - 2 * z * z, 2 * y * z + 2 * w * x,
            2 * x * z + 2 * w * y, 2 * y * z - 2 * w * x, 1 - 2 * x * x - 2 * y * y,
            p[0], p[1], p[2]]


def mul3x4(m, o):  # matrix.go:196-217
    r = []
    for c in range(3):
        for i in range(3):
            r.append(m[i] * o[3 * c] + m[3 + i] * o[3 * c + 1] + m[6 + i] * o[3 * c + 2])
    for i in range(3):
        r.append(m[i] * o[9] + m[3 + i] * o[10] + m[6 + i] * o[11] + m[9 + i])
    return r


def mul_vector(m, v):  # matrix.go:187-194
    return [v[0] * m[0] + v[1] * m[3] + v[2] * m[6] + m[9],
            v[0] * m[1] + v[1] * m[4] + v[2] * m[7] + m[10],
            v[0] * m[2] + v[1] * m[5] + v[2] * m[8] + m[11]]


def transform_inverse(m, v):  # matrix.go:222-233
    t = [v[0] - m[9], v[1] - m[10], v[2] - m[11]]
    return [t[0] * m[0] + t[1] * m[1] + t[2] * m[2],
            t[0] * m[3] + t[1] * m[4] + t[2] * m[5],
            t[0] * m[6] + t[1] * m[7] + t[2] * m[8]]


def get_axis(m, col):  # matrix.go:235-247
    i = 3 if col > 3 else col
    return [m[3 * i], m[3 * i + 1], m[3 * i + 2]]


def vec_normalize(v):  # vector.go:64-72
    mg = magnitude(v)
    if not real_equal(mg, 0.0):
        mul_with(v, 1.0 / mg)


# ---------------------------------------------------------------- colliders.go
def collider_transform(b):  # colliders.go:173-176, 302-304 (after CalculateDerivedData)
    return mul3x4(set_as_transform(b["position"], b["orientation"]), b["offset"])


def _transform_to_axis(b, axis):  # colliders.go:762-770
    t, h = b["T"], b["half"]
    return h[0] * abs(dot(axis, get_axis(t, 0))) + h[1] * abs(dot(axis, get_axis(t, 1))) + \
        h[2] * abs(dot(axis, get_axis(t, 2)))


def sphere_half_space(b, i, plane, out):  # colliders.go:180-207
    n, off = plane[:3], plane[3]
    pos = get_axis(b["T"], 3)
    distance = dot(n, pos) - b["radius"]
    if not distance <= off:
        return
    p = list(n)
    mul_with(p, distance + b["radius"] * -1.0)
    p = [p[k] + pos[k] for k in range(3)]
    out.append((i, None, p, list(n), -distance))


def cube_half_space(b, i, plane, out):  # colliders.go:308-366, 750-760
    n, off = plane[:3], plane[3]
    proj = _transform_to_axis(b, n)
    if not dot(n, get_axis(b["T"], 3)) - proj <= off:
        return
    for mult in MULTS:
        v = [mult[k] * b["half"][k] for k in range(3)]
        vp = mul_vector(b["T"], v)
        vd = dot(vp, n)
        if vd <= off:
            p = list(n)
            mul_with(p, vd - off)
            p = [p[k] + vp[k] for k in range(3)]
            out.append((i, None, p, list(n), off - vd))


def sphere_sphere(s, i, t, j, out):  # colliders.go:216-254
    one, two = get_axis(s["T"], 3), get_axis(t["T"], 3)
    mid = [one[k] - two[k] for k in range(3)]
    size = magnitude(mid)
    if size <= 0.0 or size >= s["radius"] + t["radius"]:
        return
    p = list(mid)
    mul_with(p, 0.5)
    p = [p[k] + one[k] for k in range(3)]
    nrm = list(mid)
    mul_with(nrm, 1.0 / size)
    out.append((i, j, p, nrm, s["radius"] + t["radius"] - size))


def cube_sphere(c, i, s, j, out):  # colliders.go:369-441
    pos = get_axis(s["T"], 3)
    rel = transform_inverse(c["T"], pos)
    h, r = c["half"], s["radius"]
    if abs(rel[0]) - r > h[0] or abs(rel[1]) - r > h[1] or abs(rel[2]) - r > h[2]:
        return
    closest = [0.0, 0.0, 0.0]
    for k in range(3):
        d = rel[k]
        if d > h[k]:
            d = h[k]
        elif d < -h[k]:
            d = -h[k]
        closest[k] = d
    dc = [closest[k] - rel[k] for k in range(3)]
    dist = dc[0] * dc[0] + dc[1] * dc[1] + dc[2] * dc[2]
    if dist > r * r:
        return
    cw = mul_vector(c["T"], closest)
    nrm = [cw[k] - pos[k] for k in range(3)]
    # colliders.go:417-421; with float32 values (the precision form) also when
    # the centre needed no clamping: the reference's absolute 1e-14 is below
    # float32's rounding of the world-space round trip
    if real_equal(magnitude(nrm), 0.0) or (real_type(dist) is np.float32 and dist == 0.0):
        nrm = list(s["velocity"])
    vec_normalize(nrm)
    pen = r
    if not real_equal(dist, 0.0):
        pen -= sqrt_(dist)
    else:
        pen = 0.0
    out.append((i, j, cw, nrm, pen))


def _try_axis(one, two, axis, to_center, index, smallest, case):  # colliders.go:445-477
    if axis[0] * axis[0] + axis[1] * axis[1] + axis[2] * axis[2] < real_type(*axis)(EPSILON):
        return True, smallest, case
    axis = list(axis)
    vec_normalize(axis)
    pen = _transform_to_axis(one, axis) + _transform_to_axis(two, axis) - abs(dot(to_center, axis))
    if pen < 0:
        return False, smallest, case
    if pen < smallest:
        return True, pen, index
    return True, smallest, case


def _point_face(one, i, two, j, to_center, best, pen, out):  # colliders.go:481-517
    nrm = get_axis(one["T"], best)
    if dot(nrm, to_center) > 0:
        mul_with(nrm, -1.0)
    v = list(two["half"])
    for k in range(3):
        if dot(get_axis(two["T"], k), nrm) < 0:
            v[k] = -v[k]
    out.append((i, j, mul_vector(two["T"], v), nrm, pen))


def _contact_point(p_one, d_one, one_size, p_two, d_two, two_size, use_one):  # colliders.go:519-573
    sm_one = d_one[0] * d_one[0] + d_one[1] * d_one[1] + d_one[2] * d_one[2]
    sm_two = d_two[0] * d_two[0] + d_two[1] * d_two[1] + d_two[2] * d_two[2]
    dp_one_two = dot(d_two, d_one)
    to_st = [p_one[k] - p_two[k] for k in range(3)]
    dp_sta_one = dot(d_one, to_st)
    dp_sta_two = dot(d_two, to_st)
    denom = sm_one * sm_two - dp_one_two * dp_one_two
    if abs(denom) < real_type(denom)(EPSILON):
        return list(p_one) if use_one else list(p_two)
    mua = (dp_one_two * dp_sta_two - sm_two * dp_sta_one) / denom
    mub = (sm_one * dp_sta_two - dp_one_two * dp_sta_one) / denom
    if mua > one_size or mua < -one_size or mub > two_size or mub < -two_size:
        return list(p_one) if use_one else list(p_two)
    c_one = [d_one[k] * mua + p_one[k] for k in range(3)]
    c_two = [d_two[k] * mub + p_two[k] for k in range(3)]
    return [c_one[k] * 0.5 + c_two[k] * 0.5 for k in range(3)]


def cube_cube(one, i, two, j, out):  # colliders.go:576-710
    c2, c1 = get_axis(two["T"], 3), get_axis(one["T"], 3)
    to_center = [c2[k] - c1[k] for k in range(3)]
    rt = real_type(*to_center)
    pen, best = (np.finfo(np.float32).max if rt is np.float32 else MAX_VALUE), 0xffffff
    for k in range(3):
        ok, pen, best = _try_axis(one, two, get_axis(one["T"], k), to_center, k, pen, best)
        if not ok:
            return
    for k in range(3):
        ok, pen, best = _try_axis(one, two, get_axis(two["T"], k), to_center, k + 3, pen, best)
        if not ok:
            return
    best_single = best
    for a in range(3):
        for b in range(3):
            axis = cross(get_axis(one["T"], a), get_axis(two["T"], b))
            ok, pen, best = _try_axis(one, two, axis, to_center, a * 3 + b + 6, pen, best)
            if not ok:
                return
    if best < 3:
        _point_face(one, i, two, j, to_center, best, pen, out)
        return
    if best < 6:
        nc = list(to_center)
        mul_with(nc, -1.0)
        # the contact's bodies follow fillPointFaceBoxBox's argument order
        _point_face(two, j, one, i, nc, best - 3, pen, out)
        return
    if best == 0xffffff:
        raise NoAxis()
    best -= 6
    ia, ib = best // 3, best % 3
    one_axis, two_axis = get_axis(one["T"], ia), get_axis(two["T"], ib)
    axis = cross(one_axis, two_axis)
    vec_normalize(axis)
    if dot(axis, to_center) > 0:
        mul_with(axis, -1.0)
    p1, p2 = list(one["half"]), list(two["half"])
    for k in range(3):
        if k == ia:
            p1[k] = 0
        elif dot(get_axis(one["T"], k), axis) > 0:
            p1[k] = -p1[k]
        if k == ib:
            p2[k] = 0
        elif dot(get_axis(two["T"], k), axis) < 0:
            p2[k] = -p2[k]
    p1 = mul_vector(one["T"], p1)
    p2 = mul_vector(two["T"], p2)
    point = _contact_point(p1, one_axis, one["half"][ia], p2, two_axis, two["half"][ib], best_single > 2)
    out.append((i, j, point, axis, pen))


def check_for_collisions(one, i, two, j, out):  # colliders.go:720-747 (+ 209-213)
    if two["shape"] == SPHERE:
        if one["shape"] == SPHERE:
            sphere_sphere(one, i, two, j, out)
        else:
            cube_sphere(one, i, two, j, out)
    elif one["shape"] == SPHERE:
        cube_sphere(two, j, one, i, out)  # CollisionSphere.CheckAgainstCube forwards
    else:
        cube_cube(one, i, two, j, out)


def collide_units(bodies, plane, units):
    """A caller's test list in its order: (i, -1) is body i's
    CheckAgainstHalfSpace, (i, j) CheckForCollisions(i, j)."""
    for b in bodies:
        b["T"] = collider_transform(b)
    out = []
    for i, j in units:
        if j < 0:
            if bodies[i]["shape"] == SPHERE:
                sphere_half_space(bodies[i], i, plane, out)
            else:
                cube_half_space(bodies[i], i, plane, out)
        else:
            check_for_collisions(bodies[i], i, bodies[j], j, out)
    return out


def generate_contacts(bodies, plane):
    """examples/cubedrop.go:41-67: for each body the half-space test, then
    every other body in list order."""
    for b in bodies:
        b["T"] = collider_transform(b)
    out = []
    for i, b in enumerate(bodies):
        if b["shape"] == SPHERE:
            sphere_half_space(b, i, plane, out)
        else:
            cube_half_space(b, i, plane, out)
        for j, o in enumerate(bodies):
            if j != i:
                check_for_collisions(b, i, o, j, out)
    return out

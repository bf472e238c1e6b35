"""The narrowphase's float32 culls (k_narrowphase, pair_test) are
conservative: on random pairs placed just past each cull's threshold, with
elongated boxes, arbitrary and nearly parallel orientations and scaled
positions, the reference's own tests (the second restatement,
oracle/colliders_ref.py) report no contact in either order.  CPU only; the
cull formulas are restated here in float32 as the kernel evaluates them."""
import numpy as np
import pytest

from oracle import colliders_ref as cr
from cubez_gb300 import scenes

F = np.float32


def _cull_radii(body):
    if body["shape"] == cr.SPHERE:
        r = F(body["radius"])
        return r, r
    h = [F(x) for x in body["half"]]
    rb = np.sqrt(h[0] * h[0] + h[1] * h[1] + h[2] * h[2]) * F(1.0001)
    rl = (h[0] + h[1] + h[2]) * F(1.0001)
    return rb, rl


def _rejects(a, b):
    """The cull of pair_test for (a, b): True when it skips the full test."""
    ca = [F(x) for x in cr.get_axis(a["T"], 3)]
    cb = [F(x) for x in cr.get_axis(b["T"], 3)]
    d = [cb[k] - ca[k] for k in range(3)]
    sc = F(1) + abs(ca[0]) + abs(ca[1]) + abs(ca[2]) + abs(cb[0]) + abs(cb[1]) + abs(cb[2])
    d2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2]
    (rba, rla), (rbb, rlb) = _cull_radii(a), _cull_radii(b)
    if a["shape"] == cr.SPHERE and b["shape"] == cr.SPHERE:
        t = rba + rbb + F(1e-3) + F(1e-5) * sc
    elif a["shape"] == cr.CUBE and b["shape"] == cr.CUBE:
        t = (rba + rbb) * F(1.1) + F(1e-3) + F(1e-5) * sc
    else:
        box_rl, sph_rb = (rla, rbb) if a["shape"] == cr.CUBE else (rlb, rba)
        t = box_rl + F(3) * sph_rb + F(1e-3) + F(1e-5) * sc
    return bool(d2 > t * t), float(t)


def _body(rng, shape, centre, q):
    b = {"shape": shape, "half": [0.0] * 3, "radius": 0.0, "position": list(centre), "orientation": list(q),
         "velocity": rng.normal(0, 1, 3).tolist(), "offset": scenes.IDENTITY_OFFSET.tolist()}
    if shape == cr.CUBE:
        b["half"] = (rng.uniform(0.02, 2.0, 3) * np.array([1.0, rng.choice([1.0, 0.05]), 1.0])).tolist()
    else:
        b["radius"] = float(rng.uniform(0.02, 1.5))
    b["T"] = cr.collider_transform(b)
    return b


def _quat(rng):
    q = rng.normal(0, 1, 4)
    return q / np.linalg.norm(q)


def _near(q, rng, angle):
    a = rng.normal(0, 1, 3)
    a /= np.linalg.norm(a)
    s = np.sin(angle / 2)
    dq = np.array([np.cos(angle / 2), a[0] * s, a[1] * s, a[2] * s])
    w1, x1, y1, z1 = dq
    w2, x2, y2, z2 = q
    r = np.array([w1 * w2 - x1 * x2 - y1 * y2 - z1 * z2, w1 * x2 + x1 * w2 + y1 * z2 - z1 * y2,
                  w1 * y2 - x1 * z2 + y1 * w2 + z1 * x2, w1 * z2 + x1 * y2 - y1 * x2 + z1 * w2])
    return r / np.linalg.norm(r)


@pytest.mark.parametrize("kinds", [(cr.CUBE, cr.CUBE), (cr.CUBE, cr.SPHERE), (cr.SPHERE, cr.SPHERE)])
def test_culled_pairs_have_no_contact(kinds):
    rng = np.random.default_rng(17 + kinds[0] * 2 + kinds[1])
    culled = 0
    for trial in range(1500):
        qa = _quat(rng)
        # a third of the pairs nearly parallel (edge-cross axes the reference skips)
        qb = _near(qa, rng, rng.uniform(1e-5, 1e-3)) if trial % 3 == 0 else _quat(rng)
        offset = rng.uniform(-50, 50, 3) * (trial % 2)  # far from the origin too
        a = _body(rng, kinds[0], offset, qa)
        b = _body(rng, kinds[1], offset, qb)
        _, t = _rejects(a, b)
        direction = rng.normal(0, 1, 3)
        direction /= np.linalg.norm(direction)
        dist = t * (1.0 + rng.uniform(1e-7, 2e-3))
        b["position"] = (np.asarray(offset) + direction * dist).tolist()
        b["T"] = cr.collider_transform(b)
        rej, _ = _rejects(a, b)
        if not rej:
            continue
        culled += 1
        out = []
        cr.check_for_collisions(a, 0, b, 1, out)
        cr.check_for_collisions(b, 1, a, 0, out)
        assert not out, "trial %d: a culled pair has %d contacts" % (trial, len(out))
    assert culled > 1000


def _plane_rejects(b, plane):
    """The half-space cull of k_narrowphase (plane_culled) for body b."""
    n = [F(x) for x in plane[:3]]
    off = F(plane[3])
    c = [F(x) for x in cr.get_axis(b["T"], 3)]
    d = n[0] * c[0] + n[1] * c[1] + n[2] * c[2]
    nlen = np.sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]) * F(1.0001)
    rb, _ = _cull_radii(b)
    r = rb if b["shape"] == cr.SPHERE else rb * nlen
    scale = F(1) + (abs(c[0]) + abs(c[1]) + abs(c[2])) * nlen + abs(off)
    return bool(d - r > off + F(1e-3) + F(1e-5) * scale), float(r)


@pytest.mark.parametrize("shape", [cr.CUBE, cr.SPHERE])
def test_culled_plane_units_have_no_contact(shape):
    """Bodies just above the half-space cull's threshold, for tilted planes
    with non-unit normals and offsets too: the reference's
    CheckAgainstHalfSpace (colliders.go:180-207, 308-366) finds no contact."""
    rng = np.random.default_rng(23 + shape)
    culled = 0
    for trial in range(2000):
        nrm = rng.normal(0, 1, 3)
        nrm *= rng.uniform(0.5, 2.0) / np.linalg.norm(nrm)
        plane = [float(nrm[0]), float(nrm[1]), float(nrm[2]), float(rng.uniform(-30, 30))]
        b = _body(rng, shape, [0.0, 0.0, 0.0], _quat(rng))
        _, r = _plane_rejects(b, plane)
        # centre at a height just past the threshold along the normal, far off the origin sideways
        side = rng.normal(0, 1, 3) * rng.uniform(0, 40)
        side -= nrm * (side @ nrm) / (nrm @ nrm)
        height = (plane[3] + r + 1e-3) * (1.0 + rng.uniform(1e-6, 3e-3)) + rng.uniform(0, 2e-3)
        centre = nrm / (nrm @ nrm) * height + side
        b["position"] = centre.tolist()
        b["T"] = cr.collider_transform(b)
        rej, _ = _plane_rejects(b, plane)
        if not rej:
            continue
        culled += 1
        out = []
        if shape == cr.SPHERE:
            cr.sphere_half_space(b, 0, plane, out)
        else:
            cr.cube_half_space(b, 0, plane, out)
        assert not out, "trial %d: a culled half-space test has %d contacts" % (trial, len(out))
    assert culled > 1000

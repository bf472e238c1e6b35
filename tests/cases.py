"""Hand-built single-world scenes, one per narrowphase branch, with the
contacts the reference's formulas give for them (worked out by hand from
colliders.go, including its quirks).  Shared by the CPU oracle tests and the
GPU parity tests."""
import math

import numpy as np

from cubez_gb300 import scenes


def quat_axis(angle, axis):
    a = np.asarray(axis, float)
    a = a / np.linalg.norm(a)
    s = math.sin(angle / 2.0)
    return np.array([math.cos(angle / 2.0), a[0] * s, a[1] * s, a[2] * s])


def world(bodies, plane=(0.0, 1.0, 0.0, 0.0)):
    """bodies: list of dicts with shape ('cube'|'sphere'), pos, half or r, and
    optional quat, vel, rot, inv_mass."""
    n = len(bodies)
    shape = np.array([scenes.CUBE if b["shape"] == "cube" else scenes.SPHERE for b in bodies])
    half = np.array([b.get("half", (0.0, 0.0, 0.0)) for b in bodies], float)
    radius = np.array([b.get("r", 0.0) for b in bodies], float)
    pos = np.array([b["pos"] for b in bodies], float)
    quat = np.array([b.get("quat", (1.0, 0.0, 0.0, 0.0)) for b in bodies], float)
    vel = np.array([b.get("vel", (0.0, 0.0, 0.0)) for b in bodies], float)
    rot = np.array([b.get("rot", (0.0, 0.0, 0.0)) for b in bodies], float)
    sc = scenes._assemble(np.array([n], np.int32), shape, half, radius, pos, quat, vel, rot, "case")
    sc.plane = np.asarray(plane, float)
    return sc


FAR_PLANE = (0.0, 1.0, 0.0, -100.0)


def cube_resting():
    # h = 0.5 at y = 0.49: the four lower vertices are 0.01 below the plane
    return world([dict(shape="cube", pos=(0.0, 0.49, 0.0), half=(0.5, 0.5, 0.5))])


def sphere_resting():
    return world([dict(shape="sphere", pos=(2.0, 0.4, -1.0), r=0.5)])


def sphere_pair():
    return world([dict(shape="sphere", pos=(0.0, 5.0, 0.0), r=1.0),
                  dict(shape="sphere", pos=(1.5, 5.0, 0.0), r=1.0)], FAR_PLANE)


def cube_sphere():
    return world([dict(shape="cube", pos=(0.0, 5.0, 0.0), half=(1.0, 1.0, 1.0)),
                  dict(shape="sphere", pos=(1.3, 5.0, 0.0), r=0.5)], FAR_PLANE)


def sphere_inside_cube():
    return world([dict(shape="cube", pos=(0.0, 5.0, 0.0), half=(1.0, 1.0, 1.0)),
                  dict(shape="sphere", pos=(0.2, 5.0, 0.0), r=0.5, vel=(0.0, -2.0, 0.0))], FAR_PLANE)


def sphere_inside_turned_cube_far():
    """A sphere centre inside a turned box 20 m from the origin: the world-space
    round trip of the centre is off by float32 rounding (about 1e-6), far above
    RealEqual's absolute 1e-14, so the precision form decides the fallback by
    the clamp (colliders.go:414-421)."""
    q = quat_axis(0.7, (0.3, 1.0, -0.4))
    return world([dict(shape="cube", pos=(4.98, 19.37, -1.04), half=(0.93, 0.52, 0.89), quat=q),
                  dict(shape="sphere", pos=(5.3, 19.45, -0.72), r=0.48, vel=(-1.7, -2.13, 0.81))], FAR_PLANE)


def cube_on_cube():
    # B (h=0.5) rotated 45 deg about z, resting a vertex... an edge into A's top face
    return world([dict(shape="cube", pos=(0.0, 5.0, 0.0), half=(1.0, 1.0, 1.0)),
                  dict(shape="cube", pos=(0.1, 6.6, 0.05), half=(0.5, 0.5, 0.5),
                       quat=quat_axis(0.3, (0.2, 0.1, 1.0)))], FAR_PLANE)


def cube_edge_edge():
    # two long boxes crossing edge to edge: A along x, B along z, both rolled 45 deg
    qa = quat_axis(math.pi / 4, (1.0, 0.0, 0.0))
    qb = quat_axis(math.pi / 4, (0.0, 0.0, 1.0))
    d = 0.5 * math.sqrt(2.0)  # half-diagonal of a 1x1 square section
    return world([dict(shape="cube", pos=(0.0, 5.0, 0.0), half=(2.0, 0.5, 0.5), quat=qa),
                  dict(shape="cube", pos=(0.05, 5.0 + 2 * d - 0.04, -0.03), half=(0.5, 0.5, 2.0), quat=qb)],
                 FAR_PLANE)


def _qmul(a, b):
    w1, x1, y1, z1 = a
    w2, x2, y2, z2 = b
    return np.array([w1 * w2 - x1 * x2 - y1 * y2 - z1 * z2, w1 * x2 + x1 * w2 + y1 * z2 - z1 * y2,
                     w1 * y2 - x1 * z2 + y1 * w2 + z1 * x2, w1 * z2 + x1 * y2 - y1 * x2 + z1 * w2])


def cube_edge_edge_near_parallel(twist, yaw):
    """Two unit cubes turned 45 deg about z, one on the other edge to edge
    (0.03 deep), the upper one twisted by `twist` about the vertical and both
    turned by `yaw` about it: the cross product of the two edges is tiny, so
    the edge-edge axis is the best one while the edges are almost parallel
    and contactPoint (colliders.go:519-573) meets a denominator near its
    epsilon.  Whether it takes the parallel or the out-of-range fallback, or
    crosses the edges, depends on the rounding of the form's arithmetic."""
    spin = quat_axis(math.pi / 4, (0.0, 0.0, 1.0))
    turn = quat_axis(yaw, (0.0, 1.0, 0.0))
    qa = _qmul(turn, spin)
    qb = _qmul(turn, _qmul(quat_axis(twist, (0.0, 1.0, 0.0)), spin))
    d = math.sqrt(2.0)
    return world([dict(shape="cube", pos=(0.0, 5.0, 0.0), half=(0.5, 0.5, 0.5), quat=qa),
                  dict(shape="cube", pos=(0.0, 5.0 + d - 0.03, 0.0), half=(0.5, 0.5, 0.5), quat=qb)], FAR_PLANE)


def edge_parallel_fallback():
    # in the precision form, |denom| < epsilon: contactPoint returns an edge's midpoint
    return cube_edge_edge_near_parallel(0.0005068890466341242, 3.143832173958728)


def edge_range_fallback():
    # in the precision form, the closest points fall outside the edges: an edge's midpoint again
    return cube_edge_edge_near_parallel(0.000588497158099136, 4.553989506659829)


def tilted_cube_on_plane():
    # one vertex down: a single plane contact
    q = quat_axis(math.atan(math.sqrt(2.0)), (1.0, 0.0, -1.0))
    return world([dict(shape="cube", pos=(0.0, 0.85, 0.0), half=(0.5, 0.5, 0.5), quat=q)])


def cube_edge_down():
    # turned 45 deg about z, one edge 0.01 under the plane: two vertex contacts
    q = quat_axis(math.pi / 4, (0.0, 0.0, 1.0))
    return world([dict(shape="cube", pos=(0.0, 0.5 * math.sqrt(2.0) - 0.01, 0.0), half=(0.5, 0.5, 0.5), quat=q)])


def cube_below_plane():
    # entirely under the plane: all eight vertices are contacts
    return world([dict(shape="cube", pos=(0.0, -1.0, 0.0), half=(0.5, 0.5, 0.5))])


def static_cube_singular_friction():
    """A cube of infinite mass and zero inverse inertia moving down at 1 m/s,
    0.005 into the plane: the friction solve's response matrix is zero, so
    Invert returns the zero matrix (math/matrix.go:135-137), every impulse is
    zero and adjustVelocities spends its whole budget on the same contact."""
    sc = world([dict(shape="cube", pos=(0.0, 0.495, 0.0), half=(0.5, 0.5, 0.5), vel=(0.0, -1.0, 0.0))])
    sc.inverse_mass[:] = 0.0
    sc.inverse_inertia[:] = 0.0
    sc.acceleration[:] = 0.0
    return sc


ALL = {"cube_resting": cube_resting, "sphere_resting": sphere_resting, "sphere_pair": sphere_pair,
       "cube_sphere": cube_sphere, "sphere_inside_cube": sphere_inside_cube,
       "sphere_inside_turned_cube_far": sphere_inside_turned_cube_far, "cube_on_cube": cube_on_cube,
       "cube_edge_edge": cube_edge_edge, "tilted_cube_on_plane": tilted_cube_on_plane,
       "cube_edge_down": cube_edge_down, "cube_below_plane": cube_below_plane,
       "static_cube_singular_friction": static_cube_singular_friction,
       "edge_parallel_fallback": edge_parallel_fallback, "edge_range_fallback": edge_range_fallback}

"""Seeded synthetic scenes for the rigid-body step.

Every random number is a pure function of (seed, world, body, field) through the
splitmix64 finaliser, and every float operation below is an IEEE-exact
elementwise operation (+, -, *, /, sqrt), so a scene is bit-identical on any
host and does not depend on generation order.

Body setup follows the reference's own helpers:
  * cube mass 8*hx*hy*hz (density 1), inertia from Matrix3.SetBlockInertiaTensor
    (math/matrix.go:68-77, note its 0.3 factor) inverted by Matrix3.Invert
    (math/matrix.go:131-153) as RigidBody.SetInertiaTensor does
    (rigidbody.go:176-178);
  * sphere mass 4/3*pi*r^3, inertia 0.4*m*r^2 on the diagonal
    (examples/ballistic.go:217-220);
  * SetMass stores 1/m (rigidbody.go:124-127); SetAwake(true) sets motion to
    2*sleepEpsilon (rigidbody.go:182-187).

The workloads:
  cubedrop      1 world, 20 cubes (examples/cubedrop.go scene)
  mixed         many worlds of U{8..64} spheres/cubes
  precision     many worlds x 32 bodies, 16 spheres + 16 cubes
  piles         worlds x 1024 cubes on a 16x16x4 lattice
  offsets       mixed-type worlds whose colliders carry Offsets
  ballistic     examples/ballistic.go's scene: a cube, a static backboard and
                bullets (its test order: ballistic_units)
"""
import math

import numpy as np

SPHERE = 0
CUBE = 1
# the collider Offset NewCollisionCube / NewCollisionSphere set (colliders.go:138, 267)
IDENTITY_OFFSET = np.array([1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0])

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _mix(z):
    """splitmix64 finaliser on a uint64 array (wrapping arithmetic)."""
    z = z + np.uint64(0x9E3779B97F4A7C15)
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def _u01(seed, world, body, field):
    """Uniform doubles in [0, 1) for broadcastable integer arrays."""
    with np.errstate(over="ignore"):
        w = np.asarray(world, dtype=np.uint64)
        b = np.asarray(body, dtype=np.uint64)
        f = np.asarray(field, dtype=np.uint64)
        x = _mix(np.uint64(seed) * np.uint64(0xD1B54A32D192ED03) + w)
        x = _mix(x ^ (b * np.uint64(0x100) + f))
    return (x >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def _uniform(seed, world, body, field, lo, hi):
    return lo + (hi - lo) * _u01(seed, world, body, field)


def _unit_quaternions(seed, world, body, field0):
    """Uniform random unit quaternions by rejection sampling in the 4-ball
    (16 candidates; the first with 1e-6 < |q|^2 <= 1 is normalised)."""
    world = np.asarray(world)
    body = np.asarray(body)
    k = np.arange(16)
    cand = np.stack([2.0 * _u01(seed, world[:, None], body[:, None], field0 + 4 * k[None, :] + c) - 1.0
                     for c in range(4)], axis=-1)  # (N, 16, 4)
    s = ((cand[..., 0] * cand[..., 0] + cand[..., 1] * cand[..., 1]) + cand[..., 2] * cand[..., 2]) + \
        cand[..., 3] * cand[..., 3]
    ok = (s <= 1.0) & (s > 1e-6)
    first = np.argmax(ok, axis=1)
    rows = np.arange(len(world))
    q = cand[rows, first]
    inv = 1.0 / np.sqrt(s[rows, first])
    q = q * inv[:, None]
    q[~ok.any(axis=1)] = np.array([1.0, 0.0, 0.0, 0.0])
    return q


def _invert3(m):
    """Matrix3.Invert (math/matrix.go:131-153), vectorised over rows of 9."""
    m0, m1, m2, m3, m4, m5, m6, m7, m8 = [m[:, i] for i in range(9)]
    det = (((((m0 * m4) * m8 + (m3 * m7) * m2) + (m6 * m1) * m5) - (m6 * m4) * m2) - (m3 * m1) * m8) - \
        (m0 * m7) * m5
    r = np.stack([m4 * m8 - m5 * m7, m2 * m7 - m1 * m8, m1 * m5 - m2 * m4,
                  m5 * m6 - m3 * m8, m0 * m8 - m2 * m6, m2 * m3 - m0 * m5,
                  m3 * m7 - m4 * m6, m1 * m6 - m0 * m7, m0 * m4 - m1 * m3], axis=1)
    with np.errstate(divide="ignore"):
        inv_det = 1.0 / det
    r = r * inv_det[:, None]
    # RealEqual(det, 0) with b == 0 reduces to |det| < Epsilon*Epsilon
    r[np.abs(det) < 1e-7 * 1e-7] = 0.0
    return r


def _coeffs(ix, iy, iz):
    """Matrix3.SetInertiaTensorCoeffs(ix, iy, iz, 0, 0, 0) (math/matrix.go:59-63)."""
    z = np.zeros_like(ix)
    nz = -z
    return np.stack([ix, nz, nz, nz, iy, nz, nz, nz, iz], axis=1)


class Scene:
    """Host body arrays in world-major order (float64 unless noted)."""

    FIELDS = ("position", "orientation", "velocity", "rotation", "acceleration", "inverse_inertia",
              "inverse_mass", "linear_damping", "angular_damping", "motion", "is_awake", "can_sleep",
              "shape", "half_size", "radius")

    def __init__(self, counts, plane=(0.0, 1.0, 0.0, 0.0), **arrays):
        self.counts = np.ascontiguousarray(counts, dtype=np.int32)
        self.plane = np.ascontiguousarray(plane, dtype=np.float64)
        for name in self.FIELDS:
            setattr(self, name, arrays[name])
        # [n, 12] collider Offsets (column-major 3x4, colliders.go:44,62); None = the identity
        self.collider_offset = arrays.get("collider_offset")
        self.name = arrays.get("name", "scene")

    def _optional(self, idx=None):
        if self.collider_offset is None:
            return {}
        off = self.collider_offset if idx is None else self.collider_offset[idx]
        return {"collider_offset": np.array(off, dtype=np.float64, copy=True)}

    @property
    def num_worlds(self):
        return int(self.counts.shape[0])

    @property
    def num_bodies(self):
        return int(self.counts.sum())

    def world_slice(self, w):
        start = int(self.counts[:w].sum())
        return slice(start, start + int(self.counts[w]))

    def copy(self):
        arrays = {k: np.array(getattr(self, k), copy=True) for k in self.FIELDS}
        arrays.update(self._optional())
        return Scene(self.counts.copy(), self.plane.copy(), name=self.name, **arrays)

    @staticmethod
    def concat(parts, counts=None):
        """The worlds of several scenes (same plane) in one scene; `counts`
        may insert empty worlds: a list of per-world body counts whose
        non-zero entries consume the parts' worlds in order."""
        arrays = {k: np.concatenate([getattr(p, k) for p in parts]) for k in Scene.FIELDS}
        if any(p.collider_offset is not None for p in parts):
            arrays["collider_offset"] = np.concatenate([
                p.collider_offset if p.collider_offset is not None else np.tile(IDENTITY_OFFSET, (p.num_bodies, 1))
                for p in parts])
        all_counts = np.concatenate([p.counts for p in parts])
        if counts is not None:
            nz = [c for c in counts if c > 0]
            assert list(all_counts) == nz, "non-zero counts must match the parts' worlds"
            all_counts = np.asarray(counts, np.int32)
        return Scene(all_counts, parts[0].plane.copy(), name="concat", **arrays)

    def subset(self, worlds):
        """A scene holding only the listed worlds (same bodies, same order)."""
        idx = np.concatenate([np.arange(self.world_slice(w).start, self.world_slice(w).stop) for w in worlds])
        arrays = {k: np.ascontiguousarray(getattr(self, k)[idx]) for k in self.FIELDS}
        arrays.update(self._optional(idx))
        return Scene(self.counts[list(worlds)], self.plane.copy(), name=self.name, **arrays)


def _assemble(counts, shape, half, radius, pos, quat, vel, rot, name, gravity=-9.8, lin_damp=0.95,
              ang_damp=0.8):
    n = len(shape)
    is_cube = shape == CUBE
    # cube: m = 8*hx*hy*hz ; sphere: m = 4/3*pi*r^3 (density 1)
    m_cube = ((8.0 * half[:, 0]) * half[:, 1]) * half[:, 2]
    m_sph = (((4.0 / 3.0) * math.pi) * radius * radius) * radius
    mass = np.where(is_cube, m_cube, m_sph)
    sq = half * half
    ic = _coeffs((0.3 * mass) * (sq[:, 1] + sq[:, 2]), (0.3 * mass) * (sq[:, 0] + sq[:, 2]),
                 (0.3 * mass) * (sq[:, 0] + sq[:, 1]))
    c = ((0.4 * mass) * radius) * radius
    isph = _coeffs(c, c, c)
    inertia = np.where(is_cube[:, None], ic, isph)
    acc = np.zeros((n, 3))
    acc[:, 1] = gravity
    return Scene(counts, (0.0, 1.0, 0.0, 0.0), name=name,
                 position=np.ascontiguousarray(pos), orientation=np.ascontiguousarray(quat),
                 velocity=np.ascontiguousarray(vel), rotation=np.ascontiguousarray(rot),
                 acceleration=acc, inverse_inertia=np.ascontiguousarray(_invert3(inertia)),
                 inverse_mass=1.0 / mass, linear_damping=np.full(n, lin_damp),
                 angular_damping=np.full(n, ang_damp), motion=np.full(n, 0.3 * 2.0),
                 is_awake=np.ones(n, np.uint8), can_sleep=np.zeros(n, np.uint8),
                 shape=shape.astype(np.int32), half_size=np.ascontiguousarray(half),
                 radius=np.ascontiguousarray(radius))


def _ids(counts):
    counts = np.asarray(counts, dtype=np.int64)
    world = np.repeat(np.arange(len(counts)), counts)
    starts = np.concatenate([[0], np.cumsum(counts)[:-1]])
    body = np.arange(int(counts.sum())) - np.repeat(starts, counts)
    return world, body


def cubedrop(seed=1):
    """1 world, 20 cubes: h ~ U[0.5,1]^3, centres U([-5,5]x[1,20]x[-5,5]),
    uniform orientations, at rest."""
    counts = np.array([20], np.int32)
    w, b = _ids(counts)
    half = np.stack([_uniform(seed, w, b, 1 + k, 0.5, 1.0) for k in range(3)], axis=1)
    pos = np.stack([_uniform(seed, w, b, 4, -5.0, 5.0), _uniform(seed, w, b, 5, 1.0, 20.0),
                    _uniform(seed, w, b, 6, -5.0, 5.0)], axis=1)
    quat = _unit_quaternions(seed, w, b, 64)
    n = len(w)
    return _assemble(counts, np.full(n, CUBE), half, np.zeros(n), pos, quat, np.zeros((n, 3)),
                     np.zeros((n, 3)), "cubedrop")


def _mixed_bodies(seed, counts, shape):
    w, b = _ids(counts)
    half = np.stack([_uniform(seed, w, b, 1 + k, 0.25, 1.0) for k in range(3)], axis=1)
    radius = _uniform(seed, w, b, 4, 0.25, 1.0)
    is_cube = shape == CUBE
    half = np.where(is_cube[:, None], half, 0.0)
    radius = np.where(is_cube, 0.0, radius)
    pos = np.stack([_uniform(seed, w, b, 5, -6.0, 6.0), _uniform(seed, w, b, 6, 0.5, 25.0),
                    _uniform(seed, w, b, 7, -6.0, 6.0)], axis=1)
    vel = np.stack([_uniform(seed, w, b, 8 + k, -2.0, 2.0) for k in range(3)], axis=1)
    rot = np.stack([_uniform(seed, w, b, 11 + k, -1.0, 1.0) for k in range(3)], axis=1)
    quat = _unit_quaternions(seed, w, b, 64)
    return half, radius, pos, quat, vel, rot


def mixed(num_worlds=4096, seed=2, min_bodies=8, max_bodies=64):
    """Worlds of U{min..max} bodies; each a sphere (r ~ U[0.25,1]) with p=0.5,
    else a cube (h ~ U[0.25,1]^3); positions U([-6,6]x[0.5,25]x[-6,6]),
    velocities U[-2,2]^3, angular velocities U[-1,1]^3."""
    wid = np.arange(num_worlds)
    counts = (min_bodies + np.floor(_u01(seed, wid, 0xFFFFFF, 0) * (max_bodies - min_bodies + 1))).astype(np.int32)
    w, b = _ids(counts)
    shape = np.where(_u01(seed, w, b, 0) < 0.5, SPHERE, CUBE)
    half, radius, pos, quat, vel, rot = _mixed_bodies(seed, counts, shape)
    return _assemble(counts, shape, half, radius, pos, quat, vel, rot, "mixed")


def precision(num_worlds=16384, bodies=32, seed=3):
    """Worlds of `bodies` bodies, exactly half spheres and half cubes in a
    seeded random order, distributions as in mixed()."""
    counts = np.full(num_worlds, bodies, np.int32)
    w, b = _ids(counts)
    key = _u01(seed, w, b, 0).reshape(num_worlds, bodies)
    rank = np.argsort(np.argsort(key, axis=1, kind="stable"), axis=1, kind="stable").reshape(-1)
    shape = np.where(rank < bodies // 2, SPHERE, CUBE)
    half, radius, pos, quat, vel, rot = _mixed_bodies(seed, counts, shape)
    return _assemble(counts, shape, half, radius, pos, quat, vel, rot, "precision")


def piles(num_worlds=256, seed=5, nx=16, nz=16, ny=4, spacing=1.3):
    """Worlds of nx*nz*ny cubes (h ~ U[0.3,0.6]^3) on a lattice with the given
    spacing, jitter U[-0.1,0.1]^3 and a small tilt, the lowest layer's centres
    0.5 m + 0.6 m above the plane, at rest.  The tilt quaternion is
    normalise(1, t*a) with a a uniform unit axis and t ~ U[0, 0.1], i.e. a tilt
    angle 2*atan(t) in [0, 0.1993] rad (exact arithmetic, no libm)."""
    per = nx * nz * ny
    counts = np.full(num_worlds, per, np.int32)
    w, b = _ids(counts)
    half = np.stack([_uniform(seed, w, b, 1 + k, 0.3, 0.6) for k in range(3)], axis=1)
    ix = b % nx
    iz = (b // nx) % nz
    iy = b // (nx * nz)
    base = np.stack([(ix - (nx - 1) / 2.0) * spacing, 0.5 + 0.6 + iy * spacing, (iz - (nz - 1) / 2.0) * spacing],
                    axis=1)
    jitter = np.stack([_uniform(seed, w, b, 4 + k, -0.1, 0.1) for k in range(3)], axis=1)
    pos = base + jitter
    axis = _unit_quaternions(seed, w, b, 64)[:, 1:]
    alen = np.sqrt((axis[:, 0] * axis[:, 0] + axis[:, 1] * axis[:, 1]) + axis[:, 2] * axis[:, 2])
    alen = np.where(alen > 1e-12, alen, 1.0)
    t = _uniform(seed, w, b, 7, 0.0, 0.1)
    q = np.concatenate([np.ones((len(w), 1)), axis * (t / alen)[:, None]], axis=1)
    qn = np.sqrt(((q[:, 0] * q[:, 0] + q[:, 1] * q[:, 1]) + q[:, 2] * q[:, 2]) + q[:, 3] * q[:, 3])
    q = q * (1.0 / qn)[:, None]
    n = len(w)
    return _assemble(counts, np.full(n, CUBE), half, np.zeros(n), pos, q, np.zeros((n, 3)), np.zeros((n, 3)),
                     "piles")


def _rotation_columns(q):
    """The rotation part of Matrix3x4.SetAsTransform (math/matrix.go:167-180)
    of rows of quaternions (w, x, y, z): column-major rows of 9."""
    w, x, y, z = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    return np.stack([1 - 2 * y * y - 2 * z * z, 2 * x * y + 2 * w * z, 2 * x * z - 2 * w * y,
                     2 * x * y - 2 * w * z, 1 - 2 * x * x - 2 * z * z, 2 * y * z + 2 * w * x,
                     2 * x * z + 2 * w * y, 2 * y * z - 2 * w * x, 1 - 2 * x * x - 2 * y * y], axis=1)


def offsets(num_worlds=64, bodies=24, seed=9, nonrigid=0.125):
    """mixed()-type worlds of `bodies` bodies whose colliders carry an Offset
    (CollisionCube/CollisionSphere.Offset, colliders.go:44,62): a uniform
    rotation and a translation U[-0.3,0.3]^3.  A fraction `nonrigid` of the
    Offsets also scale their three axes by U[0.7,1.3] (the reference applies
    any 3x4 Offset; such a collider is not a rigid image of its box)."""
    counts = np.full(num_worlds, bodies, np.int32)
    w, b = _ids(counts)
    shape = np.where(_u01(seed, w, b, 0) < 0.5, SPHERE, CUBE)
    half, radius, pos, quat, vel, rot = _mixed_bodies(seed, counts, shape)
    sc = _assemble(counts, shape, half, radius, pos, quat, vel, rot, "offsets")
    r = _rotation_columns(_unit_quaternions(seed, w, b, 160))
    scaled = _u01(seed, w, b, 20) < nonrigid
    scale = np.stack([_uniform(seed, w, b, 21 + k, 0.7, 1.3) for k in range(3)], axis=1)
    scale = np.where(scaled[:, None], scale, 1.0)
    r = r * np.repeat(scale, 3, axis=1)
    t = np.stack([_uniform(seed, w, b, 24 + k, -0.3, 0.3) for k in range(3)], axis=1)
    sc.collider_offset = np.ascontiguousarray(np.concatenate([r, t], axis=1))
    return sc


def ballistic(num_worlds=16, bullets=8, seed=13):
    """The scene of examples/ballistic.go:149-231 as a batch of worlds.
    Body 0: the cube (half size 1, mass 8, block inertia, at (x0, 5, 0) with
    x0 ~ U[-0.5, 0.5]).  Body 1: the backboard (half size (0.5, 2, 0.25) at
    (0, 2, -10), SetInfiniteMass, zero inverse inertia).  Bodies 2..: the
    bullets of fire() (spheres r = 0.2, mass 1.5, inertia 0.4 m r^2, velocity
    (0, 0, -40), acceleration (0, -2.5, 0)), bullet k starting at
    (U[-0.3, 0.3], 1.5 + U[-0.2, 0.2], 20 + 4k).  The cube and bullets keep
    NewRigidBody's defaults (rigidbody.go:104-114: both dampings 0.95, gravity
    -9.78 on the cube, CanSleep).

    The example never integrates the backboard.  A batch integrates every
    body, so the backboard is made static: zero acceleration, velocity and
    rotation and CanSleep false.  Integrate then leaves its state unchanged
    bit for bit, and the contact impulses move it by inverse mass and inverse
    inertia zero, so every frame equals the example's."""
    n = 2 + bullets
    counts = np.full(num_worlds, n, np.int32)
    w, b = _ids(counts)
    N = len(w)
    shape = np.where(b < 2, CUBE, SPHERE).astype(np.int32)
    half = np.zeros((N, 3))
    half[b == 0] = (1.0, 1.0, 1.0)
    half[b == 1] = (0.5, 2.0, 0.25)
    radius = np.where(b >= 2, 0.2, 0.0)
    pos = np.zeros((N, 3))
    cube, board, bullet = b == 0, b == 1, b >= 2
    pos[cube, 0] = _uniform(seed, w[cube], b[cube], 1, -0.5, 0.5)
    pos[cube, 1] = 5.0
    pos[board] = (0.0, 2.0, -10.0)
    k = (b - 2).astype(np.float64)
    pos[bullet, 0] = _uniform(seed, w[bullet], b[bullet], 2, -0.3, 0.3)
    pos[bullet, 1] = 1.5 + _uniform(seed, w[bullet], b[bullet], 3, -0.2, 0.2)
    pos[bullet, 2] = 20.0 + 4.0 * k[bullet]
    quat = np.tile([1.0, 0.0, 0.0, 0.0], (N, 1))
    vel = np.zeros((N, 3))
    vel[bullet, 2] = -40.0
    acc = np.zeros((N, 3))
    acc[cube, 1] = -9.78
    acc[bullet, 1] = -2.5
    inv_mass = np.where(cube, 1.0 / 8.0, np.where(bullet, 1.0 / 1.5, 0.0))
    # SetBlockInertiaTensor(h = 1, m = 8) and SetInertiaTensorCoeffs(0.4 m r^2), inverted
    ic = 0.3 * 8.0 * (1.0 + 1.0)
    c = ((0.4 * 1.5) * 0.2) * 0.2
    inertia = np.where(cube[:, None], _coeffs(np.full(N, ic), np.full(N, ic), np.full(N, ic)),
                       _coeffs(np.full(N, c), np.full(N, c), np.full(N, c)))
    inv_inertia = _invert3(inertia)
    inv_inertia[board] = 0.0
    return Scene(counts, (0.0, 1.0, 0.0, 0.0), name="ballistic", position=pos, orientation=quat, velocity=vel,
                 rotation=np.zeros((N, 3)), acceleration=acc, inverse_inertia=np.ascontiguousarray(inv_inertia),
                 inverse_mass=inv_mass, linear_damping=np.full(N, 0.95), angular_damping=np.full(N, 0.95),
                 motion=np.full(N, 0.3 * 2.0), is_awake=np.ones(N, np.uint8),
                 can_sleep=np.where(board, 0, 1).astype(np.uint8), shape=shape, half_size=half,
                 radius=np.ascontiguousarray(radius))


def ballistic_units(bodies):
    """generateContacts of examples/ballistic.go:47-98 as a unit list for a
    world of `bodies` bodies laid out as ballistic() does: (i, -1) is i's
    half-space test, (i, j) CheckForCollisions(i, j)."""
    units = [(0, -1), (0, 1)]
    bl = range(2, bodies)
    for k in bl:
        units += [(k, -1), (0, k), (1, k)]
        units += [(k2, k) for k2 in bl if k2 != k]
    return np.asarray(units, np.int32)


WORKLOADS = {"cubedrop": cubedrop, "mixed": mixed, "precision": precision, "piles": piles, "offsets": offsets,
             "ballistic": ballistic}

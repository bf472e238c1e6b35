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

The five workloads:
  cubedrop      1 world, 20 cubes (examples/cubedrop.go scene)
  mixed         many worlds of U{8..64} spheres/cubes
  precision     many worlds x 32 bodies, 16 spheres + 16 cubes
  piles         worlds x 1024 cubes on a 16x16x4 lattice
"""
import math

import numpy as np

SPHERE = 0
CUBE = 1

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
        self.name = arrays.get("name", "scene")

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
        return Scene(self.counts.copy(), self.plane.copy(), name=self.name, **arrays)

    @staticmethod
    def concat(parts, counts=None):
        """The worlds of several scenes (same plane) in one scene; `counts`
        may insert empty worlds: a list of per-world body counts whose
        non-zero entries consume the parts' worlds in order."""
        arrays = {k: np.concatenate([getattr(p, k) for p in parts]) for k in Scene.FIELDS}
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


WORKLOADS = {"cubedrop": cubedrop, "mixed": mixed, "precision": precision, "piles": piles}

"""ctypes front end of the oracle (TEST INFRASTRUCTURE).

Only the tests, __graft_entry__.smoke() and the CPU-baseline leg of bench.py
import this module; it is the checker, never the thing measured or shipped.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None

FP64 = 0
FP32 = 1


class OrcBodies(C.Structure):
    _fields_ = [(name, C.c_void_p) for name in (
        "position", "orientation", "velocity", "rotation", "acceleration", "inverse_inertia", "inverse_mass",
        "linear_damping", "angular_damping", "motion", "is_awake", "can_sleep", "shape", "half_size", "radius",
        "collider_offset", "last_frame_acceleration")]


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.c_int, C.c_int, C.c_void_p, C.POINTER(OrcBodies), C.c_void_p]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_step.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_int, C.c_int]
        L.orc_integrate.argtypes = [C.c_void_p, C.c_double]
        L.orc_narrowphase.argtypes = [C.c_void_p]
        L.orc_collide.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int]
        L.orc_resolve.argtypes = [C.c_void_p, C.c_double, C.c_int]
        L.orc_get_bodies.argtypes = [C.c_void_p, C.POINTER(OrcBodies)]
        L.orc_contact_count.argtypes = [C.c_void_p, C.c_int]
        L.orc_get_contacts.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        L.orc_get_stats.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_set_contacts.argtypes = [C.c_void_p, C.c_int] + [C.c_void_p] * 6 + [C.c_int]
        L.orc_resolve_fixed.argtypes = [C.c_void_p, C.c_double, C.c_int]
        L.orc_get_resolved.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        L.orc_real_equal.argtypes = [C.c_double, C.c_double]
        L.orc_quat_len.restype = C.c_double
        L.orc_quat_len.argtypes = [C.c_void_p]
        L.orc_quat_normalize.argtypes = [C.c_void_p]
        L.orc_quat_mul.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_quat_from_axis.argtypes = [C.c_double, C.c_double, C.c_double, C.c_double, C.c_void_p]
        L.orc_quat_rotate.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_quat_add_scaled_vector.argtypes = [C.c_void_p, C.c_void_p, C.c_double]
        L.orc_m3_mul.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_m3_invert.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_m34_mul.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_set_as_transform.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_v3_op.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_double]
        L.orc_v3_dot.restype = C.c_double
        L.orc_v3_dot.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_v3_magnitude.restype = C.c_double
        L.orc_v3_magnitude.argtypes = [C.c_void_p]
        L.orc_v3_square_magnitude.restype = C.c_double
        L.orc_v3_square_magnitude.argtypes = [C.c_void_p]
        L.orc_block_inverse_inertia.argtypes = [C.c_void_p, C.c_double, C.c_void_p]
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


_DTYPES = {"is_awake": np.uint8, "can_sleep": np.uint8, "shape": np.int32}


def _bodies_struct(arrays):
    s = OrcBodies()
    for name, _ in OrcBodies._fields_:
        setattr(s, name, _ptr(arrays.get(name)))
    return s


class OracleBatch:
    """A batch of independent worlds stepped on the CPU by the oracle."""

    def __init__(self, scene, form=FP64, last_frame_acceleration=None):
        """`last_frame_acceleration` ([n, 3]): the bodies' lastFrameAccelleration
        at setup (default zero, as NewRigidBody leaves it)."""
        self.L = lib()
        self.scene = scene
        self.form = form
        self._keep = {k: np.ascontiguousarray(getattr(scene, k), dtype=_DTYPES.get(k, np.float64))
                      for k in scene.FIELDS}
        if getattr(scene, "collider_offset", None) is not None:
            self._keep["collider_offset"] = np.ascontiguousarray(scene.collider_offset, dtype=np.float64)
        if last_frame_acceleration is not None:
            self._keep["last_frame_acceleration"] = np.ascontiguousarray(last_frame_acceleration, dtype=np.float64)
        s = _bodies_struct(self._keep)
        self.h = self.L.orc_create(form, scene.num_worlds, _ptr(scene.counts), C.byref(s), _ptr(scene.plane))

    def __del__(self):
        if getattr(self, "h", None):
            self.L.orc_destroy(self.h)
            self.h = None

    def step(self, nsteps, dt=1.0 / 60.0, iter_mult=4, threads=1):
        return self.L.orc_step(self.h, nsteps, dt, iter_mult, threads)

    def integrate(self, dt=1.0 / 60.0):
        self.L.orc_integrate(self.h, dt)

    def narrowphase(self):
        return self.L.orc_narrowphase(self.h)

    def collide(self, world, units):
        """The narrowphase tests of `units` ((i, j), j = -1 for the half-space)
        of one world, in list order; replaces the world's contacts."""
        u = np.ascontiguousarray(np.asarray(units, dtype=np.int32).reshape(-1, 2))
        return self.L.orc_collide(self.h, int(world), _ptr(u), int(u.shape[0]))

    def resolve(self, dt=1.0 / 60.0, iter_mult=4):
        return self.L.orc_resolve(self.h, dt, iter_mult)

    def bodies(self):
        n = self.scene.num_bodies
        out = {"position": np.zeros((n, 3)), "orientation": np.zeros((n, 4)), "velocity": np.zeros((n, 3)),
               "rotation": np.zeros((n, 3)), "inverse_inertia": np.zeros((n, 9)), "motion": np.zeros(n),
               "is_awake": np.zeros(n, np.uint8)}
        s = _bodies_struct(out)
        self.L.orc_get_bodies(self.h, C.byref(s))
        out["iit_world"] = out.pop("inverse_inertia")
        return out

    def contacts(self, world):
        n = self.L.orc_contact_count(self.h, world)
        b = np.zeros((n, 2), np.int32)
        p = np.zeros((n, 3))
        nn = np.zeros((n, 3))
        pen = np.zeros(n)
        self.L.orc_get_contacts(self.h, world, _ptr(b), _ptr(p), _ptr(nn), _ptr(pen), n)
        return {"bodies": b, "point": p, "normal": nn, "penetration": pen}

    def set_contacts(self, world, c):
        """Replace world's contact list (dict of bodies, point, normal,
        penetration, friction, restitution arrays)."""
        n = len(c["penetration"])
        self._c = {k: np.ascontiguousarray(c[k], dtype=np.int32 if k == "bodies" else np.float64)
                   for k in ("bodies", "point", "normal", "penetration", "friction", "restitution")}
        k = self._c
        self.L.orc_set_contacts(self.h, world, _ptr(k["bodies"]), _ptr(k["point"]), _ptr(k["normal"]),
                                _ptr(k["penetration"]), _ptr(k["friction"]), _ptr(k["restitution"]), n)

    def resolve_fixed(self, max_iterations, dt=1.0 / 60.0):
        return self.L.orc_resolve_fixed(self.h, dt, max_iterations)

    def resolved_contacts(self, world):
        n = self.L.orc_contact_count(self.h, world)
        b = np.zeros((n, 2), np.int32)
        nn = np.zeros((n, 3))
        pen = np.zeros(n)
        self.L.orc_get_resolved(self.h, world, _ptr(b), _ptr(nn), _ptr(pen), n)
        return {"bodies": b, "normal": nn, "penetration": pen}

    def stats(self):
        W = self.scene.num_worlds
        c = np.zeros(W, np.int32)
        pi = np.zeros(W, np.int32)
        vi = np.zeros(W, np.int32)
        self.L.orc_get_stats(self.h, _ptr(c), _ptr(pi), _ptr(vi))
        return {"contacts": c, "pos_iterations": pi, "vel_iterations": vi}


def hardware_threads():
    return lib().orc_hardware_threads()

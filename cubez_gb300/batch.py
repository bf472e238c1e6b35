"""WorldBatch: many independent cubez worlds stepped on one GPU.

A thin host wrapper over the C ABI: bodies are numpy arrays in the layout of
cubez's value types (m.Vector3 = 3 doubles, m.Quat = (w, x, y, z),
m.Matrix3 = 9 doubles column-major), world-major.
"""
import ctypes as C

import numpy as np

from . import _lib
from ._lib import FORM_FP32, FORM_FP64, check  # noqa: F401

_DT = {"is_awake": np.uint8, "can_sleep": np.uint8, "shape": np.int32}
_WIDTH = {"position": 3, "orientation": 4, "velocity": 3, "rotation": 3, "acceleration": 3, "inverse_inertia": 9,
          "inverse_mass": 1, "linear_damping": 1, "angular_damping": 1, "motion": 1, "is_awake": 1, "can_sleep": 1,
          "shape": 1, "half_size": 3, "radius": 1, "inverse_inertia_world": 9, "last_frame_acceleration": 3,
          "collider_offset": 12}


# the collider Offset NewCollisionCube / NewCollisionSphere set (colliders.go:138, 267)
_IDENTITY_OFFSET = np.array([1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0])


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def bodies_struct(arrays):
    s = _lib.Bodies()
    for name in _lib.BODY_FIELDS:
        setattr(s, name, _ptr(arrays.get(name)))
    return s


class WorldBatch:
    """Device-resident batch of worlds (cz_batch_create .. cz_batch_destroy)."""

    def __init__(self, counts, form=FORM_FP64, plane=(0.0, 1.0, 0.0, 0.0), contact_capacity=0,
                 iteration_multiplier=4, max_iterations=0, device=0):
        self.L = _lib.load()
        self.counts = np.ascontiguousarray(counts, dtype=np.int32)
        self.num_worlds = int(self.counts.shape[0])
        self.num_bodies = int(self.counts.sum())
        self.form = form
        self.warm_start = False  # set by learned.set_warm_start
        self.desc = {"plane": [float(x) for x in plane], "contact_capacity": int(contact_capacity),
                     "iteration_multiplier": int(iteration_multiplier), "max_iterations": int(max_iterations)}
        d = _lib.BatchDesc()
        d.form = form
        d.num_worlds = self.num_worlds
        d.body_counts = _ptr(self.counts)
        d.contact_capacity = contact_capacity
        for i in range(4):
            d.plane[i] = float(plane[i])
        d.iteration_multiplier = iteration_multiplier
        d.max_iterations = max_iterations
        d.device = device
        h = C.c_void_p()
        check(self.L.cz_batch_create(C.byref(d), C.byref(h)))
        self.h = h

    @classmethod
    def from_scene(cls, scene, form=FORM_FP64, **kw):
        b = cls(scene.counts, form=form, plane=scene.plane, **kw)
        b.upload(scene)
        return b

    def close(self):
        if getattr(self, "h", None):
            self.L.cz_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---------------------------------------------------------------- bodies
    def upload(self, scene=None, **arrays):
        if scene is not None:
            for k in scene.FIELDS:
                arrays.setdefault(k, getattr(scene, k))
            arrays.setdefault("collider_offset", scene.collider_offset)
        keep = {k: np.ascontiguousarray(v, dtype=_DT.get(k, np.float64)) for k, v in arrays.items() if v is not None}
        s = bodies_struct(keep)
        check(self.L.cz_upload_bodies(self.h, C.byref(s)))

    def download(self, fields=None):
        n = self.num_bodies
        fields = fields or ("position", "orientation", "velocity", "rotation", "inverse_inertia_world", "motion",
                            "is_awake", "last_frame_acceleration")
        out = {}
        for f in fields:
            w = _WIDTH[f]
            out[f] = np.zeros((n, w) if w > 1 else n, dtype=_DT.get(f, np.float64))
        s = bodies_struct(out)
        check(self.L.cz_download_bodies(self.h, C.byref(s)))
        return out

    # ---------------------------------------------------------------- checkpoint
    def save(self, path):
        """Write the batch's description and full body state (derived data,
        motion, awake flags and collider Offsets included) to an .npz file."""
        state = self.download(tuple(_WIDTH))
        if np.array_equal(state["collider_offset"], np.tile(_IDENTITY_OFFSET, (self.num_bodies, 1))):
            del state["collider_offset"]
        np.savez(path, counts=self.counts, form=np.int32(self.form), plane=np.array(self.desc["plane"]),
                 contact_capacity=np.int32(self.desc["contact_capacity"]),
                 iteration_multiplier=np.int32(self.desc["iteration_multiplier"]),
                 max_iterations=np.int32(self.desc["max_iterations"]), **state)

    @classmethod
    def load(cls, path, device=0):
        """A new batch holding the state `save` wrote; it steps on exactly as
        the saved batch would (tuning is not saved: it changes no result)."""
        z = np.load(path)
        b = cls(z["counts"], form=int(z["form"]), plane=z["plane"], contact_capacity=int(z["contact_capacity"]),
                iteration_multiplier=int(z["iteration_multiplier"]), max_iterations=int(z["max_iterations"]),
                device=device)
        b.upload(**{k: z[k] for k in _WIDTH if k in z.files})
        return b

    # ---------------------------------------------------------------- stepping
    def step(self, nsteps=1, dt=1.0 / 60.0):
        check(self.L.cz_step(self.h, int(nsteps), float(dt)))

    def integrate(self, dt=1.0 / 60.0):
        check(self.L.cz_integrate(self.h, float(dt)))

    def narrowphase(self):
        check(self.L.cz_narrowphase(self.h))

    def collide(self, world, units, plane=None):
        """The narrowphase for a list of (i, j) tests of one world, j = -1 for
        the half-space (cz_collide); the world's contact list is replaced."""
        u = np.ascontiguousarray(np.asarray(units, dtype=np.int32).reshape(-1, 2))
        p = None if plane is None else np.ascontiguousarray(plane, dtype=np.float64)
        check(self.L.cz_collide(self.h, int(world), None if p is None else _ptr(p), _ptr(u), len(u)))

    def resolve(self, dt=1.0 / 60.0):
        check(self.L.cz_resolve(self.h, float(dt)))

    def prepare_rollout(self, nsteps, dt=1.0 / 60.0):
        check(self.L.cz_prepare_rollout(self.h, int(nsteps), float(dt)))

    def snapshot(self):
        check(self.L.cz_snapshot(self.h))

    def restore(self):
        check(self.L.cz_restore(self.h))

    def step_timed(self, nsteps, dt=1.0 / 60.0):
        """Run a captured rollout; returns (total_ms, [integrate, narrowphase, resolve] ms)."""
        tot = C.c_double(0.0)
        ph = np.zeros(3)
        check(self.L.cz_step_timed(self.h, int(nsteps), float(dt), C.byref(tot), _ptr(ph)))
        return tot.value, ph

    def counters(self, reset=False):
        a = np.zeros(8, np.int64)
        check(self.L.cz_counters(self.h, _ptr(a), 1 if reset else 0))
        return {"contacts": int(a[0]), "pos_iterations": int(a[1]), "vel_iterations": int(a[2]),
                "contacts_resolved": int(a[3]), "warm_fallbacks": int(a[4]), "warm_worlds": int(a[5]),
                "warm_scale_sum": int(a[6]) * 1e-6, "warm_bodies": int(a[7])}

    def info(self):
        a = np.zeros(9, np.int64)
        check(self.L.cz_batch_info(self.h, _ptr(a)))
        keys = ("bodies", "padded_bodies", "contact_slots", "real_bytes", "sms", "narrowphase_ctas", "resolver_ctas",
                "narrowphase_smem", "resolver_smem")
        return dict(zip(keys, (int(x) for x in a)))

    # ---------------------------------------------------------------- results
    def contact_counts(self):
        c = np.zeros(self.num_worlds, np.int32)
        check(self.L.cz_contact_counts(self.h, _ptr(c)))
        return c

    def contacts(self, world):
        n = C.c_int32(0)
        check(self.L.cz_download_contacts(self.h, int(world), None, 0, C.byref(n)))
        m = n.value
        arr = (_lib.Contact * max(m, 1))()
        check(self.L.cz_download_contacts(self.h, int(world), C.cast(arr, C.c_void_p), m, C.byref(n)))
        raw = np.frombuffer(arr, dtype=np.dtype([("body", "<i4", 2), ("friction", "<f8"), ("restitution", "<f8"),
                                                 ("point", "<f8", 3), ("normal", "<f8", 3),
                                                 ("penetration", "<f8")]))[:m]
        return {"bodies": raw["body"].copy(), "point": raw["point"].copy(), "normal": raw["normal"].copy(),
                "penetration": raw["penetration"].copy(), "friction": raw["friction"].copy(),
                "restitution": raw["restitution"].copy()}

    def stats(self):
        W = self.num_worlds
        pi = np.zeros(W, np.int32)
        vi = np.zeros(W, np.int32)
        st = np.zeros(W, np.uint32)
        check(self.L.cz_world_stats(self.h, _ptr(pi), _ptr(vi), _ptr(st)))
        return {"pos_iterations": pi, "vel_iterations": vi, "status": st}

    # ---------------------------------------------------------------- tuning
    def set_tuning(self, narrowphase_threads=0, resolver_contacts=0, resolver_ctas_per_sm=0, integrate_threads=0,
                   resolver_lanes=0, warm_start_budget_shift=0, large_world_lanes=0, broadphase_min_bodies=0,
                   fused_frame=0):
        t = _lib.Tuning(narrowphase_threads, resolver_contacts, resolver_ctas_per_sm, integrate_threads, resolver_lanes,
                        warm_start_budget_shift, large_world_lanes, broadphase_min_bodies, fused_frame)
        check(self.L.cz_set_tuning(self.h, C.byref(t)))

    def get_tuning(self):
        t = _lib.Tuning()
        check(self.L.cz_get_tuning(self.h, C.byref(t)))
        return {"narrowphase_threads": t.narrowphase_threads, "resolver_contacts": t.resolver_contacts,
                "resolver_ctas_per_sm": t.resolver_ctas_per_sm, "integrate_threads": t.integrate_threads,
                "resolver_lanes": t.resolver_lanes, "warm_start_budget_shift": t.warm_start_budget_shift,
                "large_world_lanes": t.large_world_lanes, "broadphase_min_bodies": t.broadphase_min_bodies,
                "fused_frame": t.fused_frame}

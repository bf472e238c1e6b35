"""ctypes binding of libcubez_gb300.so (the C ABI in include/cubez_gpu.h).

There is no CPU fallback: if the library has not been built, loading fails
with an error that says how to build it.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libcubez_gb300.so")

CZ_OK = 0
STATUS_NAMES = {0: "CZ_OK", 1: "CZ_ERR_BAD_ARG", 2: "CZ_ERR_CUDA", 3: "CZ_ERR_NO_DEVICE", 4: "CZ_ERR_NONFINITE",
                5: "CZ_ERR_CAPACITY", 6: "CZ_ERR_TIMEOUT", 7: "CZ_ERR_FRICTIONLESS", 8: "CZ_ERR_BODY_LIMIT"}
FORM_FP64 = 0
FORM_FP32 = 1


class CubezError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s (%d): %s" % (STATUS_NAMES.get(status, "?"), status, message))
        self.status = status


class BatchDesc(C.Structure):
    _fields_ = [("form", C.c_int32), ("num_worlds", C.c_int32), ("body_counts", C.c_void_p),
                ("contact_capacity", C.c_int32), ("plane", C.c_double * 4), ("iteration_multiplier", C.c_int32),
                ("max_iterations", C.c_int32), ("device", C.c_int32)]


BODY_FIELDS = ("position", "orientation", "velocity", "rotation", "acceleration", "inverse_inertia", "inverse_mass",
               "linear_damping", "angular_damping", "motion", "is_awake", "can_sleep", "shape", "half_size", "radius",
               "inverse_inertia_world", "last_frame_acceleration", "collider_offset")


class Bodies(C.Structure):
    _fields_ = [(name, C.c_void_p) for name in BODY_FIELDS]


class Contact(C.Structure):
    _fields_ = [("body", C.c_int32 * 2), ("friction", C.c_double), ("restitution", C.c_double),
                ("point", C.c_double * 3), ("normal", C.c_double * 3), ("penetration", C.c_double)]


class Tuning(C.Structure):
    _fields_ = [("narrowphase_threads", C.c_int32), ("resolver_contacts", C.c_int32),
                ("resolver_ctas_per_sm", C.c_int32), ("integrate_threads", C.c_int32), ("resolver_lanes", C.c_int32),
                ("warm_start_budget_shift", C.c_int32), ("large_world_lanes", C.c_int32),
                ("broadphase_min_bodies", C.c_int32), ("fused_frame", C.c_int32)]


# every symbol include/cubez_gpu.h declares, with (restype, argtypes)
SIGNATURES = {
    "cz_batch_create": (C.c_int, [C.POINTER(BatchDesc), C.POINTER(C.c_void_p)]),
    "cz_batch_destroy": (C.c_int, [C.c_void_p]),
    "cz_upload_bodies": (C.c_int, [C.c_void_p, C.POINTER(Bodies)]),
    "cz_download_bodies": (C.c_int, [C.c_void_p, C.POINTER(Bodies)]),
    "cz_step": (C.c_int, [C.c_void_p, C.c_int32, C.c_double]),
    "cz_integrate": (C.c_int, [C.c_void_p, C.c_double]),
    "cz_narrowphase": (C.c_int, [C.c_void_p]),
    "cz_resolve": (C.c_int, [C.c_void_p, C.c_double]),
    "cz_contact_counts": (C.c_int, [C.c_void_p, C.c_void_p]),
    "cz_download_contacts": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.POINTER(C.c_int32)]),
    "cz_world_stats": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "cz_resolve_contacts": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_double,
                                      C.POINTER(Bodies)]),
    "cz_resolve_contacts_static": (C.c_int, [C.c_int32, C.c_int32, C.c_void_p, C.c_int32, C.c_double,
                                             C.POINTER(Bodies), C.c_int32, C.c_void_p]),
    "cz_set_warm_start": (C.c_int, [C.c_void_p, C.c_void_p]),
    "cz_harvest": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, C.c_int32, C.c_void_p, C.c_void_p, C.c_int64,
                             C.POINTER(C.c_int64)]),
    "cz_mlp_create": (C.c_int, [C.c_int32, C.c_uint64, C.POINTER(C.c_void_p)]),
    "cz_mlp_destroy": (C.c_int, [C.c_void_p]),
    "cz_mlp_get_params": (C.c_int, [C.c_void_p, C.c_void_p]),
    "cz_mlp_set_params": (C.c_int, [C.c_void_p, C.c_void_p]),
    "cz_mlp_set_data": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int32]),
    "cz_mlp_train": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_float, C.c_uint64, C.c_void_p]),
    "cz_mlp_loss_and_grad": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_float), C.c_void_p]),
    "cz_mlp_predict": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]),
    "cz_set_tuning": (C.c_int, [C.c_void_p, C.POINTER(Tuning)]),
    "cz_get_tuning": (C.c_int, [C.c_void_p, C.POINTER(Tuning)]),
    "cz_prepare_rollout": (C.c_int, [C.c_void_p, C.c_int32, C.c_double]),
    "cz_snapshot": (C.c_int, [C.c_void_p]),
    "cz_restore": (C.c_int, [C.c_void_p]),
    "cz_step_timed": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, C.POINTER(C.c_double), C.c_void_p]),
    "cz_batch_info": (C.c_int, [C.c_void_p, C.c_void_p]),
    "cz_counters": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32]),
    "cz_collide": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_int32]),
    "cz_set_wait_test": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "cz_status_string": (C.c_char_p, [C.c_int]),
    "cz_last_error": (C.c_char_p, []),
    "cz_kernel_launches": (C.c_int64, []),
}

_lib = None


def load():
    """Load the CUDA library (built by cubez_gb300.build); raises if absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("libcubez_gb300.so is not built (run `python -c \"import __graft_entry__ as g; g.build()\"` "
                          "or `python cubez_gb300/build.py`); there is no CPU fallback")
    L = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(status):
    if status != CZ_OK:
        L = load()
        raise CubezError(status, L.cz_last_error().decode(errors="replace"))
    return status


def kernel_launches():
    return int(load().cz_kernel_launches())

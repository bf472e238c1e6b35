"""cubez_gb300: cubez's rigid-body step (integrate, narrowphase, contact
resolution) as hand-written CUDA for GB300 (sm_103a), behind a C ABI
(include/cubez_gpu.h).  The CUDA library is the only compute path; importing
the batch API without the built library raises.
"""
from . import scenes  # noqa: F401

__all__ = ["scenes", "WorldBatch", "FORM_FP64", "FORM_FP32", "CubezError"]


def __getattr__(name):
    if name in ("WorldBatch", "FORM_FP64", "FORM_FP32", "CubezError"):
        from . import batch, _lib
        return {"WorldBatch": batch.WorldBatch, "FORM_FP64": _lib.FORM_FP64, "FORM_FP32": _lib.FORM_FP32,
                "CubezError": _lib.CubezError}[name]
    raise AttributeError(name)

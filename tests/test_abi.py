"""The C ABI boundary without a GPU: the library builds for sm_103a, loads,
and exports every function include/*.h declares; the ctypes binding covers
the same set; argument validation runs on the host."""
import ctypes as C
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s*(cz_[A-Za-z0-9_]+)\s*\(", text, re.M):
            names.add(m.group(1))
    return names


def test_header_declares_the_boundary():
    names = declared_functions()
    for required in ("cz_batch_create", "cz_batch_destroy", "cz_upload_bodies", "cz_download_bodies", "cz_step",
                     "cz_integrate", "cz_narrowphase", "cz_resolve", "cz_resolve_contacts",
                     "cz_download_contacts"):
        assert required in names


def test_library_exports_every_declared_symbol(cuda_lib):
    from cubez_gb300 import _lib
    missing = [n for n in sorted(declared_functions()) if not hasattr(cuda_lib, n)]
    assert not missing, "not exported: %s" % missing
    # the ctypes binding declares a signature for each of them
    assert declared_functions() <= set(_lib.SIGNATURES), sorted(declared_functions() - set(_lib.SIGNATURES))


def test_status_strings(cuda_lib):
    for s in range(9):
        assert cuda_lib.cz_status_string(s)
    assert cuda_lib.cz_status_string(99) == b"unknown status"


def test_null_arguments_rejected_on_host(cuda_lib):
    from cubez_gb300 import _lib
    assert cuda_lib.cz_batch_create(None, None) == 1
    assert cuda_lib.cz_step(None, 1, 1.0 / 60) == 1
    assert cuda_lib.cz_upload_bodies(None, None) == 1
    assert cuda_lib.cz_download_bodies(None, None) == 1
    assert cuda_lib.cz_batch_destroy(None) == 1
    assert b"null" in cuda_lib.cz_last_error()


def test_bad_descriptor_rejected(cuda_lib):
    from cubez_gb300 import _lib
    d = _lib.BatchDesc()
    d.form = 7
    d.num_worlds = 1
    h = C.c_void_p()
    assert cuda_lib.cz_batch_create(C.byref(d), C.byref(h)) == 1


def test_no_device_reported_without_gpu(cuda_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import numpy as np
    from cubez_gb300 import _lib
    counts = np.array([4], np.int32)
    d = _lib.BatchDesc()
    d.form = 0
    d.num_worlds = 1
    d.body_counts = counts.ctypes.data_as(C.c_void_p)
    h = C.c_void_p()
    st = cuda_lib.cz_batch_create(C.byref(d), C.byref(h))
    assert st in (2, 3)  # CZ_ERR_CUDA or CZ_ERR_NO_DEVICE, never a crash


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    from cubez_gb300 import _lib
    monkeypatch.setattr(_lib, "_lib", None)
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "absent.so"))
    with pytest.raises(ImportError, match="no CPU fallback"):
        _lib.load()

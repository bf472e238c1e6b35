"""The C++ mirror's host-side setup math (include/cubez.hpp) against the
oracle, bit for bit, on random and edge-case inputs.  CPU only: the program
makes no GPU call (it links the library because the header's classes do)."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "host_math.cpp")
LIBDIR = os.path.join(ROOT, "cubez_gb300", "_build")
REC = 12 + 12 + 9 + 3 + 1 + 2 + 3 + 4
OUT = 12 + 9 + 9 + 1 + 12


def _records(rng, n):
    r = rng.normal(0.0, 2.0, (n, REC))
    r[:, 33:36] = np.abs(r[:, 33:36]) + 0.05     # half sizes
    r[:, 36] = np.abs(r[:, 36]) + 0.1            # mass
    q = r[:, 42:46]
    r[:, 42:46] = q / np.linalg.norm(q, axis=1)[:, None]
    # edge cases: a singular matrix, equal and nearly equal reals, zeros
    r[0, 24:33] = [1, 2, 3, 2, 4, 6, 0, 1, 0]
    r[1, 37:39] = [1.0, 1.0 + 1e-8]
    r[2, 37:39] = [0.0, 1e-15]
    r[3, 37:39] = [1e-40, 0.0]
    r[4, 37:39] = [3.0, 3.0]
    r[5, 24:33] = 0.0
    return r


def test_host_math_matches_oracle(tmp_path, oracle_lib):
    gxx = shutil.which("g++")
    if gxx is None or not os.path.exists(os.path.join(LIBDIR, "libcubez_gb300.so")):
        pytest.skip("g++ or the built library is missing")
    exe = os.path.join(str(tmp_path), "host_math")
    r = subprocess.run([gxx, "-std=c++17", "-O2", "-ffp-contract=off", "-Wall", "-I", os.path.join(ROOT, "include"),
                        SRC, "-L", LIBDIR, "-lcubez_gb300", "-Wl,-rpath," + LIBDIR, "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    rec = _records(np.random.default_rng(7), 256)
    inp, out = os.path.join(str(tmp_path), "in.bin"), os.path.join(str(tmp_path), "out.bin")
    rec.astype(np.float64).tofile(inp)
    r = subprocess.run([exe, inp, out], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = np.fromfile(out, np.float64).reshape(len(rec), OUT)
    L = oracle_lib
    p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    for i, x in enumerate(rec):
        a, b, m = np.ascontiguousarray(x[0:12]), np.ascontiguousarray(x[12:24]), np.ascontiguousarray(x[24:33])
        half, mass = np.ascontiguousarray(x[33:36]), float(x[36])
        pos, q = np.ascontiguousarray(x[39:42]), np.ascontiguousarray(x[42:46])
        ab, mi, bi, t = np.zeros(12), np.zeros(9), np.zeros(9), np.zeros(12)
        L.orc_m34_mul(p(a), p(b), p(ab))
        L.orc_m3_invert(p(m), p(mi))
        L.orc_block_inverse_inertia(p(half), mass, p(bi))
        L.orc_set_as_transform(p(pos), p(q), p(t))
        eq = 1.0 if L.orc_real_equal(float(x[37]), float(x[38])) else 0.0
        want = np.concatenate([ab, mi, bi, [eq], t])
        assert np.array_equal(got[i], want), "record %d differs at %s" % (i, np.flatnonzero(got[i] != want))
    assert not got[0, 12:21].any()                 # singular: the zero matrix (math/matrix.go:135-137)
    assert got[1:5, 30].tolist() == [1.0, 1.0, 1.0, 1.0]  # within 1e-7 relative; both near zero; equal

"""Build the oracle shared library (TEST INFRASTRUCTURE).

The oracle is the CPU restatement of the reference's rigid-body step used by the
tests and by the CPU-baseline leg of bench.py.  It is compiled with
-ffp-contract=off so that no multiply-add is fused, matching the GPU kernels,
which are compiled with --fmad=false.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SOURCES = [os.path.join(HERE, "oracle_capi.cpp")]
HEADERS = [os.path.join(HERE, "cubez_ref.hpp")]


def build(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    newest = max(os.path.getmtime(p) for p in SOURCES + HEADERS + [__file__])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-pthread", "-o", LIB + ".tmp"] + SOURCES
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))

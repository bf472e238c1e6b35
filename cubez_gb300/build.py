"""Build the CUDA library libcubez_gb300.so in-tree for sm_103a.

Three translation units compiled in parallel (one per arithmetic form plus the
C ABI), one -gencode, no CMake.  --fmad=false keeps every multiply and add
separately rounded, as the reference's Go arithmetic is.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libcubez_gb300.so")
UNITS = ["cz_fp64.cu", "cz_fp32.cu", "cz_api.cu", "cz_static.cu", "cz_mlp.cu"]
HEADERS = ["cz_math.cuh", "cz_layout.cuh", "cz_kernels.cuh", "cz_resolve.cuh", "cz_resolve_big.cuh",
           "cz_form_impl.cuh", "cz_forms.h", "cz_mlp.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fno-fast-math"]


def _nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _sources():
    inc = os.path.join(os.path.dirname(HERE), "include", "cubez_gpu.h")
    return [os.path.join(CSRC, u) for u in UNITS] + [os.path.join(CSRC, h) for h in HEADERS] + [inc, __file__]


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(p) <= t for p in _sources())


def build(force=False, verbose=False, ptxas_info=False):
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    extra = ["-Xptxas", "-v"] if ptxas_info else []

    def compile_unit(u):
        obj = os.path.join(OUT, u.replace(".cu", ".o"))
        cmd = [nvcc] + ARCH + FLAGS + extra + ["-c", os.path.join(CSRC, u), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (u, r.stdout, r.stderr))
        return obj, r.stderr

    with cf.ThreadPoolExecutor(len(UNITS)) as ex:
        results = list(ex.map(compile_unit, UNITS))
    if verbose or ptxas_info:
        for _, err in results:
            sys.stderr.write(err)
    tmp = LIB + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + [o for o, _ in results]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv))

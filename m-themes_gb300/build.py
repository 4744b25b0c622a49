"""Build libmth.so (CUDA kernels for sm_103a + C-ABI + host readers) and the
`forge` driver, in tree, with nvcc and gcc only.

    python m-themes_gb300/build.py [--force]

Outputs m-themes_gb300/lib/libmth.so and m-themes_gb300/lib/forge.  Objects go
to m-themes_gb300/_build/.  Translation units compile in parallel.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(HERE, "host")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "lib")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-I" + os.path.join(REPO, "include")]
CU_SOURCES = ["fft_green.cu", "fft_tma.cu", "newton.cu", "drx.cu", "dd.cu", "adjoint.cu", "book.cu", "capi.cu", "capi_iout.cu",
              "capi_arrays.cu", "capi_batch.cu", "capi_adjoint.cu"]
# sources compiled without FMA contraction (bit-exact FP64 restatement)
NO_FMAD = {"drx.cu", "book.cu"}
# sources whose host code is compiled without FMA contraction: the FP64 host
# bookkeeping gives the same doubles on x86 and Arm (gcc contracts by default
# on aarch64), and host-side tensor conversions match the device's rounded,
# uncontracted ones
NO_HOST_CONTRACT = {"capi.cu", "capi_iout.cu", "capi_arrays.cu", "capi_batch.cu", "capi_adjoint.cu"}
C_SOURCES = ["mth_io.c"]


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIB, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    headers.append(os.path.join(REPO, "include", "mth.h"))
    jobs = []
    objs = []
    for s in CU_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            extra = ["-fmad=false"] if s in NO_FMAD else []
            if s in NO_HOST_CONTRACT:
                extra += ["-Xcompiler", "-ffp-contract=off"]
            jobs.append([nvcc()] + NVCC_FLAGS + extra + ["-c", src, "-o", obj])
    for s in C_SOURCES:
        src = os.path.join(HOST, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append(["gcc", "-O2", "-fPIC", "-Wall", "-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    so = os.path.join(LIB, "libmth.so")
    if force or _stale(so, objs):
        _run([nvcc()] + ARCH + ["-shared", "-o", so] + objs + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"])
    forge = os.path.join(LIB, "forge")
    fsrc = os.path.join(HOST, "forge.c")
    if force or _stale(forge, [fsrc, so]):
        _run(["gcc", "-O2", "-Wall", "-o", forge, fsrc, "-L" + LIB, "-lmth", "-Wl,-rpath,$ORIGIN"])
    return so


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))

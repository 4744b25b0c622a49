"""CPU check of the per-voxel transposed Jacobians of the calibration
adjoint (m-themes_gb300/csrc/adj_local.cuh): the same header the adjoint
kernels use is compiled with the host compiler and its adj_pre / adj_post /
tangent_stiffness are compared with central finite differences of the
end-of-step map (flow rule, Voce hardening, lattice rotation)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def _cuda_include():
    for d in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if d and os.path.exists(os.path.join(d, "include", "cuda_runtime.h")):
            return os.path.join(d, "include")
    return None


def test_local_vjp_against_finite_differences(tmp_path):
    cxx = shutil.which("g++")
    inc = _cuda_include()
    if cxx is None or inc is None:
        pytest.skip("needs g++ and the CUDA headers")
    exe = str(tmp_path / "adjchk")
    r = subprocess.run([cxx, "-O2", "-std=c++17", "-I" + inc, "-I" + os.path.join(REPO, "m-themes_gb300", "csrc"),
                        os.path.join(HERE, "adj_local_check.cpp"), "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe, "12"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    worst = float(r.stdout.strip().splitlines()[-1].split()[1])
    assert worst < 2e-5

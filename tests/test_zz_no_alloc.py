"""Allocation-free batch local solve, mth_local_solve_noalloc, through the C-ABI.

Some callers hand out all device memory from their own preallocated pool and
cannot let a library call cudaMalloc behind their back (it would bypass the
pool and may fail on a GPU the pool has filled, or synchronise the device).
For them the local solve takes device pointers for every input and output and
keeps its only scratch in a fixed array in the library's device image.  This
test allocates the buffers itself, as such a caller would, and checks the
result against the allocating entry point mth_local_solve and against the
oracle's restatement of the reference's UpdateStress on the same inputs, on
two calls in a row (the scratch keeps the previous call's contents), and that
repeated calls leave the device's free memory unchanged.
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

from mth import capi, synth

pytestmark = pytest.mark.gpu
REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    subprocess.check_call([sys.executable, os.path.join(REPO, "m-themes_gb300", "build.py")])
    return capi.load()


def states(n, seed):
    from scipy.spatial.transform import Rotation
    rng = np.random.default_rng(seed)
    rot = Rotation.random(n, random_state=seed).as_matrix().reshape(n, 9)
    sig = rng.standard_normal((n, 6)) * 30.0
    sig[:, 5] *= 0.1
    strain = rng.standard_normal((n, 6)) * 1e-3
    epsp = rng.standard_normal((n, 6)) * 3e-4
    epsp[:, 5] = 0.0
    crss = 16.0 + rng.random((n, 12)) * 10.0
    return sig, epsp, strain, rot, crss


def c066_of(cfg):
    """Reference stiffness of a small polycrystal: the average of the grains'
    rotated cubic stiffness (uniform weights), built in the LT basis."""
    from mth.capi import MthParams  # noqa: F401
    m = cfg.material
    ev = np.array([m.c11 - m.c12, m.c11 - m.c12, 2 * m.c44, 2 * m.c44, 2 * m.c44, m.c11 + 2 * m.c12])
    # isotropic-like average of the 5 deviatoric eigenvalues; hydrostatic apart
    c = np.zeros((6, 6))
    c[:5, :5] = np.eye(5) * ev[:5].mean()
    c[5, 5] = ev[5]
    return c


def solve_noalloc(lib, par, c066, st):
    import torch
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in st]
    n = st[0].shape[0]
    d_edot = torch.zeros((n, 6), dtype=torch.float64, device="cuda")
    d_err = torch.zeros((n, 2), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    it = C.c_longlong(-1)
    c = np.ascontiguousarray(c066, dtype=np.float64)
    capi.check(lib, lib.mth_local_solve_noalloc(C.byref(par), capi._dptr(c), n, dev[0].data_ptr(),
                                                dev[1].data_ptr(), dev[2].data_ptr(), dev[3].data_ptr(),
                                                dev[4].data_ptr(), d_edot.data_ptr(), d_err.data_ptr(),
                                                C.byref(it), None))
    torch.cuda.synchronize()
    return dev[0].cpu().numpy(), d_edot.cpu().numpy(), d_err.cpu().numpy(), it.value


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def test_noalloc_matches_allocating_entry_point(lib):
    import pyoracle
    from mth import local_solve
    cfg = synth.Config(cell_dim=(8, 8, 8), n_grains=4)
    par = capi.params_from_config(cfg)
    c066 = c066_of(cfg)
    # two calls in a row; the first uses more blocks than the second, so the
    # second sees stale partial sums beyond its own blocks
    for n, seed in ((3000, 21), (700, 22)):
        st = states(n, seed)
        s_ref, e_ref, err_ref, it_ref = local_solve(par, c066, *st)
        s, e, err, it = solve_noalloc(lib, par, c066, st)
        assert rel(s, s_ref) < 1e-8
        assert rel(e, e_ref) < 1e-6
        assert rel(err[:, 0], err_ref[:, 0]) < 1e-6
        assert it > 0 and abs(it - it_ref) <= max(1, it_ref // 100)
        # and the reference's own algorithm (Newton with line search on |R|^2)
        s_orc, e_orc, _, _ = pyoracle.local_solve(par, c066, *st)
        assert rel(s, s_orc) < 1e-8
        assert rel(e, e_orc) < 1e-6


def test_noalloc_leaves_device_memory_and_current_device_alone(lib):
    import torch
    cfg = synth.Config(cell_dim=(8, 8, 8), n_grains=4)
    par = capi.params_from_config(cfg)
    c066 = np.ascontiguousarray(c066_of(cfg))
    n = 1 << 20
    st = states(n, 5)
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in st]
    d_edot = torch.zeros((n, 6), dtype=torch.float64, device="cuda")
    d_err = torch.zeros((n, 2), dtype=torch.float64, device="cuda")
    it = C.c_longlong(0)

    def call():
        capi.check(lib, lib.mth_local_solve_noalloc(C.byref(par), capi._dptr(c066), n, dev[0].data_ptr(),
                                                    dev[1].data_ptr(), dev[2].data_ptr(), dev[3].data_ptr(),
                                                    dev[4].data_ptr(), d_edot.data_ptr(), d_err.data_ptr(),
                                                    C.byref(it), None))
    call()                       # loads the module and looks up the scratch address
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        call()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert torch.cuda.current_device() == par.device


def test_noalloc_rejects_oversize(lib):
    cfg = synth.Config(cell_dim=(8, 8, 8), n_grains=4)
    par = capi.params_from_config(cfg)
    c = np.ascontiguousarray(c066_of(cfg))
    it = C.c_longlong(0)
    fake = C.c_void_p(16)   # never dereferenced: the size check comes first
    st = lib.mth_local_solve_noalloc(C.byref(par), capi._dptr(c), (1 << 20) + 1, fake, fake, fake, fake, fake,
                                     fake, fake, C.byref(it), None)
    assert st == 1
    assert b"allocation-free limit" in lib.mth_last_error()

"""C-ABI checks that need no GPU: the library loads, exports every entry
point include/mth.h declares, the input readers parse the reference's file
formats, and argument validation returns status codes before any device
call."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from mth import capi, synth

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    import subprocess
    import sys
    subprocess.check_call([sys.executable, os.path.join(REPO, "m-themes_gb300", "build.py")])
    return capi.load()


def declared_symbols():
    txt = open(os.path.join(REPO, "include", "mth.h")).read()
    return sorted(set(re.findall(r"\b(mth_[a-z_0-9]+)\s*\(", txt)))


def test_exports_every_declared_symbol(lib):
    syms = declared_symbols()
    assert len(syms) >= 11
    for s in syms:
        assert hasattr(lib, s), s
    assert lib.mth_version().decode().startswith("mth-gb300")


def test_readers_roundtrip(lib, tmp_path):
    cfg = synth.Config(cell_dim=(8, 6, 4), n_grains=5, n_pores=1, pore_radius=1, seed=3)
    g, p, e = synth.write_case(str(tmp_path), cfg)
    par = capi.MthParams()
    s1, s2, ms = C.create_string_buffer(256), C.create_string_buffer(256), C.create_string_buffer(256)
    capi.check(lib, lib.mth_read_namelist(str(tmp_path / "input.in").encode(), C.byref(par), s1, s2, ms, 256))
    assert list(par.cell_dim) == [8, 6, 4]
    assert par.n_phases == 2
    assert s1.value == b"cu.sx" and ms.value == b"ms.txt"
    assert par.time_step == cfg.time_step and par.iter_max == cfg.iter_max and par.err == cfg.err
    assert list(par.velgrad_bc_flag) == list(cfg.velgrad_bc_flag)
    assert list(par.velgrad_bc) == list(cfg.velgrad_bc)
    assert par.phase[0].c11 == cfg.material.c11 and par.phase[1].type == 1
    capi.check(lib, lib.mth_read_sx(str(tmp_path / "cu.sx").encode(), C.byref(par), 0))
    ref = capi.params_from_config(cfg)
    for k in ("nsys", "nrs", "gamd0", "tau0f", "tau0b", "tau1", "thet0", "thet1", "hself", "hlat"):
        assert getattr(par.phase[0], k) == getattr(ref.phase[0], k), k
    assert np.array_equal(np.ctypeslib.as_array(par.phase[0].bn), np.ctypeslib.as_array(ref.phase[0].bn))
    assert np.array_equal(np.ctypeslib.as_array(par.phase[0].bb), np.ctypeslib.as_array(ref.phase[0].bb))
    nv = 8 * 6 * 4
    gg = np.zeros(nv, np.int32)
    pp = np.zeros(nv, np.int32)
    ee = np.zeros(3 * nv)
    dims = (C.c_int * 3)(8, 6, 4)
    capi.check(lib, lib.mth_read_microstructure(str(tmp_path / "ms.txt").encode(), dims, capi._iptr(gg),
                                                capi._iptr(pp), capi._dptr(ee)))
    assert np.array_equal(gg, g) and np.array_equal(pp, p) and np.array_equal(ee.reshape(-1, 3), e)


def test_reader_errors(lib, tmp_path):
    par = capi.MthParams()
    assert lib.mth_read_namelist(b"/nonexistent/input.in", C.byref(par), None, None, None, 0) == 6
    assert lib.mth_read_sx(b"/nonexistent.sx", C.byref(par), 0) == 6
    bad = tmp_path / "ms.txt"
    bad.write_text("0 0 0 1 1 2 1 1\n")     # index out of order
    dims = (C.c_int * 3)(1, 1, 1)
    g = np.zeros(1, np.int32)
    e = np.zeros(3)
    assert lib.mth_read_microstructure(str(bad).encode(), dims, capi._iptr(g), capi._iptr(g), capi._dptr(e)) == 6


@pytest.mark.parametrize("mutate,status", [
    (lambda p: p.cell_dim.__setitem__(0, 10), 10),         # 10 = 2*5: not a 2^a 3^b edge
    (lambda p: p.cell_dim.__setitem__(1, 7), 10),          # odd edge
    (lambda p: setattr(p, "iter_max", 0), 1),
    (lambda p: setattr(p, "n_phases", 3), 1),
    (lambda p: p.velgrad_bc_flag.__setitem__(0, 1), 1),   # two deviatoric components
    (lambda p: p.stress_bc_flag.__setitem__(2, 1), 1),    # stress and velocity both set
    (lambda p: setattr(p.phase[0], "thet1", 1e4), 1),     # thet0 < thet1 (src/init.c:127)
    (lambda p: setattr(p, "precision", 7), 1),
])
def test_create_validation(lib, mutate, status):
    p = capi.params_from_config(synth.Config(cell_dim=(8, 8, 8)))
    mutate(p)
    ctx = C.c_void_p()
    assert lib.mth_create(C.byref(p), C.byref(ctx)) == status
    assert not ctx.value
    assert lib.mth_last_error()


def test_null_arguments(lib):
    assert lib.mth_create(None, None) == 1
    assert lib.mth_step(None, None) == 1
    assert lib.mth_destroy(None) == 1


def test_batch_argument_checks(lib):
    """Batch arguments are checked before any device call."""
    out = C.c_void_p()
    assert lib.mth_batch_create(None, 1, C.byref(out)) == 1
    p = (capi.MthParams * 2)(capi.params_from_config(synth.Config(cell_dim=(8, 8, 8))),
                             capi.params_from_config(synth.Config(cell_dim=(16, 16, 16))))
    assert lib.mth_batch_create(p, 0, C.byref(out)) == 1
    p[1].device = 1                                   # members on different devices
    assert lib.mth_batch_create(p, 2, C.byref(out)) == 1
    p[1].device = 0
    p[1].pf_substeps = 10                             # recrystallisation in a member
    assert lib.mth_batch_create(p, 2, C.byref(out)) == 10
    assert not out.value
    assert lib.mth_batch_step(None, None) == 1
    assert lib.mth_batch_destroy(None) == 1
    assert lib.mth_batch_upload(None, 0, None, None, None, 0) == 1
    t = C.c_int()
    assert lib.mth_batch_passes(None, 0, C.byref(t), C.byref(t), C.byref(t)) == 1


def test_iout_argument_checks(lib):
    assert lib.mth_write_iout(None, 0, b"x", 0) == 1
    assert lib.mth_iout_wait(None) == 1
    assert lib.mth_track_disgrad(None, 1) == 1


def test_namelist_dislocation_density_block(lib, tmp_path):
    """The DD keys of the namelist (a0, L0, T__K, Q_slip, Q_bulk, C_1..C_8,
    the six junction strengths, rho_SSD_initial, D_0, the Poisson ratio of
    ElastConst_PhaseI) land in mth_params as params_from_config puts them."""
    cfg = synth.Config(cell_dim=(8, 8, 8), n_grains=3, seed=5,
                       dd=synth.DD(T=293.0, q_slip=0.31, c=(0.5, 3.1, 2.9, 810.0, 15.0, 1000.0, 1.2e-8, 0.3),
                                   chi=(0.12, 0.13, 0.7, 0.11, 0.06, 0.2), rho_ssd0=0.07, nu=0.34))
    synth.write_case(str(tmp_path), cfg)
    par = capi.MthParams()
    capi.check(lib, lib.mth_read_namelist(str(tmp_path / "input.in").encode(), C.byref(par), None, None, None, 0))
    ref = capi.params_from_config(cfg)
    for k in ("dd_a0", "dd_L0", "dd_T", "dd_q_slip", "dd_q_bulk", "dd_rho_ssd0", "dd_d0", "dd_nu"):
        assert getattr(par, k) == getattr(ref, k), k
    assert list(par.dd_c) == list(ref.dd_c)
    assert list(par.dd_chi) == list(ref.dd_chi)
    assert ref.flow_law == 1 and par.flow_law == 0   # the law is chosen by the caller (forge --dd)


def test_local_solve_rejects_dislocation_density_law(lib):
    """The array-level local solve has no per-voxel density state: it runs the
    power law and refuses flow_law = 1 before touching the device."""
    par = capi.params_from_config(synth.Config(cell_dim=(8, 8, 8), n_grains=2, dd=synth.DD()))
    a = np.zeros(64)
    assert lib.mth_local_solve(C.byref(par), capi._dptr(a), 1, capi._dptr(a), capi._dptr(a), capi._dptr(a),
                               capi._dptr(a), capi._dptr(a), capi._dptr(a), capi._dptr(a), None) == 10
    assert b"power law" in lib.mth_last_error()

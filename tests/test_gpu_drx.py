"""GPU dynamic recrystallisation against the oracle and the reference.

The oracle restates the reference's phase-field sweep literally and matches
the reference's own PF_XRX bit for bit (tests/test_drx_oracle.py); the GPU
computes the same sweep in parallel passes.  FP64: order parameters (in
stored order), grain maps, the rho_avg table and nucleation sites must be
bit-identical to the oracle's, and to the reference fixtures directly.  Mixed
precision (FP32 order parameters) must agree on at least 99% of the grain
map."""
import ctypes as C
import os

import numpy as np
import pytest

import pyoracle
from helpers import rel
from mth import capi, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def lib():
    import os
    import subprocess
    import sys
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    subprocess.check_call([sys.executable, os.path.join(repo, "m-themes_gb300", "build.py")])
    return capi.load()


def pf_case(dims=(24, 24, 24), seed=3):
    cfg = synth.Config(cell_dim=dims, n_grains=8, seed=seed, drx=synth.Drx(stored_energy_scale=50.0))
    g, _, _ = synth.microstructure(cfg)
    rng = np.random.default_rng(seed)
    base = 100.0 + 400.0 * rng.random(9)
    rho = base[g] + 20.0 * rng.random(g.size)
    # three dislocation-free nuclei on grain boundaries
    ax = [np.arange(n) for n in dims]
    X, Y, Z = np.meshgrid(*ax, indexing="ij")
    for k, c in enumerate(((4, 5, 6), (15, 10, 18), (20, 20, 3))):
        m = ((X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2 <= 4).ravel()
        g[m] = 9 + k
        rho[m] = 1.0
    return cfg, g.astype(np.int32), rho


def gpu_pf(lib, par, dims, g, rho, substeps, init_gid, table):
    nv = g.size
    d = (C.c_int * 3)(*dims)
    go = np.zeros(nv, np.int32)
    K = capi.PF_K
    ids = np.zeros(nv * K, np.int32)
    phi = np.zeros(nv * K)
    cnt = np.zeros(nv, np.int32)
    t = np.array(table, dtype=np.float64)
    capi.check(lib, lib.mth_pf_relax(C.byref(par), d, capi._iptr(np.ascontiguousarray(g, np.int32)),
                                     capi._dptr(np.ascontiguousarray(rho, np.float64)), substeps, init_gid,
                                     capi._dptr(t), len(t), capi._iptr(go), capi._iptr(ids), capi._dptr(phi),
                                     capi._iptr(cnt)))
    return go, ids.reshape(nv, K), phi.reshape(nv, K), cnt, t


def test_pf_relax_fp64_bit_exact(lib):
    cfg, g, rho = pf_case()
    par = capi.params_from_config(cfg, precision=capi.MTH_FP64)
    table = np.zeros(12)
    for steps in (1, 2, 8):
        o = pyoracle.pf_relax(par, cfg.cell_dim, g, rho, steps, 8, table, kmax=capi.PF_K)
        r = gpu_pf(lib, par, cfg.cell_dim, g, rho, steps, 8, table)
        assert np.array_equal(r[0], o[0]), steps                 # grain map
        assert np.array_equal(r[3], o[3]), steps                 # counts
        assert np.array_equal(r[1], o[1]), steps                 # ids, in stored order
        assert np.array_equal(r[2].view(np.int64), o[2].view(np.int64)), steps   # values, bit for bit
        assert np.array_equal(r[4], o[4]), steps                 # rho_avg table
    assert (r[0] >= 9).sum() > 0
    # a second call continues from the table the first one left
    g2 = np.where(r[0] == 0, g, r[0]).astype(np.int32)
    o2 = pyoracle.pf_relax(par, cfg.cell_dim, g2, rho, 4, 8, r[4], kmax=capi.PF_K)
    r2 = gpu_pf(lib, par, cfg.cell_dim, g2, rho, 4, 8, r[4])
    assert np.array_equal(r2[0], o2[0]) and np.array_equal(r2[4], o2[4])
    assert np.array_equal(r2[2].view(np.int64), o2[2].view(np.int64))


GOLDEN = __import__("os").path.join(__import__("os").path.dirname(__import__("os").path.abspath(__file__)), "golden")


@pytest.mark.parametrize("name", sorted(f[:-4] for f in __import__("os").listdir(GOLDEN) if f.startswith("pf_")))
def test_pf_relax_matches_reference_fixtures(lib, name):
    """The GPU against the reference's own PF_XRX run on the same inputs."""
    import json
    from test_drx_oracle import coef_params, golden_lists
    z = np.load(__import__("os").path.join(GOLDEN, name + ".npz"))
    dims = tuple(int(d) for d in z["dims"])
    par = coef_params(json.loads(str(z["coef"])))
    steps, init_gid = int(z["steps"]), int(z["init_gid"])
    table0 = np.zeros(int(z["grain"].max()) + 1)
    for s in (1, 2, steps):
        go, ids, phi, cnt, tab = gpu_pf(lib, par, dims, z["grain"], z["rho"], s, init_gid, table0)
        gc, gi, gv = golden_lists(z, s)
        assert np.array_equal(cnt, gc), s
        k = np.arange(capi.PF_K)[None, :] < cnt[:, None]
        assert np.array_equal(ids[k], gi), s
        assert np.array_equal(phi[k], gv), s
    assert np.array_equal(go, z["gnew"]) and np.array_equal(tab, z["table"])


def test_pf_relax_mixed_close(lib):
    cfg, g, rho = pf_case(seed=5)
    par64 = capi.params_from_config(cfg, precision=capi.MTH_FP64)
    par32 = capi.params_from_config(cfg, precision=capi.MTH_MIXED)
    o = pyoracle.pf_relax(par64, cfg.cell_dim, g, rho, 8, 8, np.zeros(12))
    r = gpu_pf(lib, par32, cfg.cell_dim, g, rho, 8, 8, np.zeros(12))
    assert (r[0] == o[0]).mean() >= 0.99


def test_nucleation_bit_exact(lib):
    dims = (20, 20, 20)
    cfg = synth.Config(cell_dim=dims, n_grains=9, seed=8,
                       drx=synth.Drx(rho_nucleation=50.0, nucleation_prob=0.03, seed=777))
    g, ph, _ = synth.microstructure(cfg)
    rho = 100.0 * np.random.default_rng(1).random(g.size)
    par = capi.params_from_config(cfg)
    og, osites = pyoracle.nucleate(par, dims, g, np.ones(g.size, np.int32), rho, step=7, first_id=10)
    gg = g.astype(np.int32).copy()
    sites = np.zeros(65536, np.int64)
    n = C.c_int(0)
    capi.check(lib, lib.mth_nucleate(C.byref(par), (C.c_int * 3)(*dims), capi._iptr(gg), capi._iptr(ph),
                                     capi._dptr(rho), 7, 10, sites.ctypes.data_as(C.POINTER(C.c_longlong)), 65536,
                                     C.byref(n)))
    assert n.value == osites.size > 0
    assert np.array_equal(sites[:n.value], osites)
    assert np.array_equal(gg, og)


@pytest.mark.parametrize("name", ["nucl_voronoi", "nucl_edges"])
def test_nucleation_matches_reference_fixtures(lib, name):
    """NucleationCheckDRX of the reference (static threshold) is mth_nucleate
    with nucleation_prob = 1: same sites, ids and painted map."""
    z = np.load(__import__("os").path.join(GOLDEN, name + ".npz"))
    dims = tuple(int(d) for d in z["dims"])
    par = capi.params_from_config(synth.Config(cell_dim=dims, drx=synth.Drx()))
    par.rho_nucleation = float(z["kappa"])
    par.nucleation_prob = 1.0
    par.nucleus_radius = int(z["radius"])
    par.n_phases = 2
    par.phase[1].type = 1
    gg = np.ascontiguousarray(z["grain"], np.int32).copy()
    ph = np.ascontiguousarray(z["phase"], np.int32)
    sites = np.zeros(4096, np.int64)
    n = C.c_int(0)
    ng = int(z["n_grains"])
    capi.check(lib, lib.mth_nucleate(C.byref(par), (C.c_int * 3)(*dims), capi._iptr(gg), capi._iptr(ph),
                                     capi._dptr(np.ascontiguousarray(z["diff_rho"])), 3, ng + 1,
                                     sites.ctypes.data_as(C.POINTER(C.c_longlong)), 4096, C.byref(n)))
    assert n.value == int(z["n_new"])
    assert np.array_equal(gg, z["grain_out"])


def test_coupled_drx_matches_oracle():
    cfg = synth.Config(cell_dim=(16, 16, 16), n_grains=6, n_steps=6, seed=5, iter_max=8,
                       drx=synth.Drx(rho_k=4000.0, rho_nucleation=30.0, nucleation_prob=0.005))
    g, p, e = synth.microstructure(cfg)
    par = capi.params_from_config(cfg, precision=capi.MTH_FP64)
    from mth import Solver
    s = Solver(par, g, p, e)
    o = pyoracle.Oracle(par, g, p, e, nthreads=4)
    total_new = 0
    for k in range(cfg.n_steps):
        a, b = s.step(), o.step()
        assert a["n_new_grains"] == b["n_new_grains"], k
        total_new += a["n_new_grains"]
        assert np.array_equal(s.field("grain"), o.field("grain")), k
        assert rel(a["sig_avg"], b["sig_avg"]) < 1e-6, k
    assert total_new > 0
    assert rel(s.field("sig"), o.field("sig")) < 1e-5


@pytest.mark.parametrize("pf_dims", [(32, 32, 32), (24, 16, 20)])
def test_coupled_drx_on_its_own_pf_grid(pf_dims):
    """CellDim_pf != CellDim: grain ids and rho carried to the PF grid and the
    relaxed ids back (InterpolateGrid / Update_microstructure), FP64 grain
    maps identical to the oracle's at every step."""
    cfg = synth.Config(cell_dim=(16, 16, 16), n_grains=6, n_steps=4, seed=5, iter_max=8,
                       drx=synth.Drx(rho_k=4000.0, rho_nucleation=30.0, nucleation_prob=0.02, pf_cell_dim=pf_dims))
    g, p, e = synth.microstructure(cfg)
    par = capi.params_from_config(cfg, precision=capi.MTH_FP64)
    from mth import Solver
    s = Solver(par, g, p, e)
    o = pyoracle.Oracle(par, g, p, e, nthreads=4)
    total_new = 0
    for k in range(cfg.n_steps):
        a, b = s.step(), o.step()
        assert a["n_new_grains"] == b["n_new_grains"], k
        total_new += a["n_new_grains"]
        assert np.array_equal(s.field("grain"), o.field("grain")), k
        assert rel(a["sig_avg"], b["sig_avg"]) < 1e-6, k
    assert total_new > 0
    s.close()


@pytest.mark.parametrize("radius2", [36, 9])
def test_coupled_drx_growth_rule_matches_oracle(radius2):
    """The "< 1 % grew" rule (src/integrated.c:1537-1582) on the GPU: runs in
    which grown recrystallised grains gain under 1 % of their voxels in a
    step (radius-6 nuclei) and some percent (radius-3 nuclei), FP64 grain
    maps identical to the oracle's and its orientation, slip and stress
    fields at every step."""
    from test_drx_oracle import rollback_case
    cfg = rollback_case(radius2)
    g, p, e = synth.microstructure(cfg)
    par = capi.params_from_config(cfg, precision=capi.MTH_FP64)
    from mth import Solver
    s = Solver(par, g, p, e)
    o = pyoracle.Oracle(par, g, p, e, nthreads=os.cpu_count())
    for k in range(cfg.n_steps):
        a, b = s.step(), o.step()
        assert a["n_new_grains"] == b["n_new_grains"], k
        assert np.array_equal(s.field("grain"), o.field("grain")), k
        assert rel(s.field("rot"), o.field("rot")) < 1e-8, k
        assert rel(s.field("gamacum"), o.field("gamacum")) < 1e-6, k
        assert rel(a["sig_avg"], b["sig_avg"]) < 1e-6, k
    s.close()
    o.close()

"""Dislocation-density law on the GPU (flow_law = 1): against the reference
built with its shipped DD path (golden traces of tests/golden/dd8_*.npz) and
the oracle; mixed precision against FP64; the forge driver's dd.out; the
set-ups the law does not take.

Tolerances as the power-law parity tests: FP64 1e-6 relative on the
macroscopic stress and the dd.out averages, 1e-6 relative on the densities;
mixed 1e-4 on the stress, 1e-3 on the averages."""
import os
import subprocess

import numpy as np
import pytest

from helpers import DD_GOLDEN_CASES, T_DG, T_DD, T_ITER, T_SIG, load_golden, rel, rel_l2, run_gpu, run_oracle
from mth import MthError, Solver, capi, synth

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("name", DD_GOLDEN_CASES)
def test_fp64_matches_reference_dd(name):
    cfg, trace, fields = load_golden(name)
    s, reps = run_gpu(cfg, capi.MTH_FP64)
    for k, r in enumerate(reps):
        row = trace[k]
        assert r["iterations"] == int(row[T_ITER]), (k, r["iterations"], row[T_ITER])
        assert rel(r["sig_avg"], row[T_SIG].reshape(3, 3)) < 1e-6, k
        assert rel(r["disgrad_avg"], row[T_DG].reshape(3, 3)) < 1e-6, k
        ref = row[T_DD]
        for j in range(7):
            assert abs(r["dd_avg"][j] - ref[j]) <= 1e-6 * abs(ref[j]) + 1e-300, (k, j, r["dd_avg"], ref)
        assert r["newton_failed"] == 0
    assert rel_l2(s.field("sig"), fields["sig"]) < 1e-6
    assert rel(s.field("rho_ssd"), fields["rho_ssd"]) < 1e-6
    if np.abs(fields["rho_gnd"]).max() > 0:
        assert rel(s.field("rho_gnd"), fields["rho_gnd"]) < 1e-6
    s.close()


def test_fp64_matches_oracle_dd_16cube():
    """A larger polycrystal with pores and GNDs from the third step on."""
    cfg = synth.Config(cell_dim=(16, 16, 16), n_grains=10, n_pores=2, pore_radius=2, n_steps=5, seed=211,
                       iter_max=40, dd=synth.DD())
    o, ro = run_oracle(cfg, nthreads=8)
    s, rg = run_gpu(cfg, capi.MTH_FP64)
    for k in range(cfg.n_steps):
        assert rg[k]["iterations"] == ro[k]["iterations"]
        assert rel(rg[k]["sig_avg"], ro[k]["sig_avg"]) < 1e-6, k
        assert np.all(np.abs(rg[k]["dd_avg"] - ro[k]["dd_avg"]) <= 1e-6 * np.abs(ro[k]["dd_avg"])), k
    assert ro[-1]["dd_avg"][4] > 0          # GNDs grew
    assert rel(s.field("rho_ssd"), o.field("rho_ssd")) < 1e-6
    assert rel(s.field("rho_gnd"), o.field("rho_gnd")) < 1e-6
    cry = synth.microstructure(cfg)[1] == 1   # gas voxels carry no orientation (0 in the oracle, I here)
    assert rel_l2(s.field("rot")[cry], o.field("rot")[cry]) < 1e-9
    s.close()


@pytest.mark.parametrize("precision", [capi.MTH_MIXED, capi.MTH_MIXED_FAST, capi.MTH_MIXED_ROOT64])
def test_mixed_dd_within_tolerance(precision):
    """Every mixed mode runs the dislocation-density law with the FP64
    Jacobian solve at each Newton step."""
    cfg = synth.Config(cell_dim=(16, 16, 16), n_grains=10, n_steps=5, seed=212, iter_max=40, dd=synth.DD())
    _, r64 = run_gpu(cfg, capi.MTH_FP64)
    s, rm = run_gpu(cfg, precision)
    for k in range(cfg.n_steps):
        assert rel(rm[k]["sig_avg"], r64[k]["sig_avg"]) < 1e-4, k
        assert np.all(np.abs(rm[k]["dd_avg"] - r64[k]["dd_avg"]) <= 1e-3 * np.abs(r64[k]["dd_avg"]) + 1e-9), k
    s.close()


def test_forge_dd_writes_dd_out(tmp_path):
    cfg = synth.Config(cell_dim=(8, 8, 8), n_grains=4, n_steps=3, seed=213, iter_max=30, dd=synth.DD())
    synth.write_case(str(tmp_path), cfg)
    forge = os.path.join(REPO, "m-themes_gb300", "lib", "forge")
    subprocess.run([forge, "input.in", "--dd"], cwd=tmp_path, check=True, capture_output=True)
    rows = np.loadtxt(tmp_path / "dd.out", skiprows=1, ndmin=2)
    assert rows.shape == (3, 9)
    _, reps = run_gpu(cfg, capi.MTH_FP64)
    for k, r in enumerate(reps):
        assert rows[k, 1] == pytest.approx(r["e_vm"], rel=2e-6)   # %e: 7 digits
        np.testing.assert_allclose(rows[k, 2:], r["dd_avg"], rtol=2e-6)


def test_dd_rejected_setups():
    dd = synth.DD()
    with pytest.raises(MthError, match="UNSUPPORTED"):
        run_gpu(synth.Config(cell_dim=(8, 8, 8), n_grains=3, n_steps=1, dd=dd, drx=synth.Drx()))
    cfg = synth.Config(cell_dim=(8, 8, 8), n_grains=3, n_steps=1, dd=dd)
    with Solver(capi.params_from_config(cfg), *synth.microstructure(cfg)) as s:
        with pytest.raises(MthError, match="UNSUPPORTED"):
            s.adjoint(np.zeros(1))
    plain = synth.Config(cell_dim=(8, 8, 8), n_grains=3)
    with Solver(capi.params_from_config(plain), *synth.microstructure(plain)) as s:
        with pytest.raises(MthError, match="STATE"):
            s.field("rho_ssd")


def test_reference_test_run_unmodified():
    """The reference's own test_run/ inputs (32^3 single crystal with a pore,
    the shipped DD parameters, DD_CU elastic constants, Err 5e-5, two steps),
    parsed by this project's readers, against both steps of the reference's
    run."""
    from helpers import GOLDEN
    z = np.load(os.path.join(GOLDEN, "tr_dd_test_run.npz"))
    par = capi.MthParams.from_buffer_copy(z["params"].tobytes())
    par.phase[0].c11, par.phase[0].c12, par.phase[0].c44 = (float(x) for x in z["dd_cu"])
    par.flow_law = 1
    par.precision = capi.MTH_FP64
    par.device = 0
    assert z["trace"].shape[0] == 2
    with Solver(par, z["grain"], z["phase"], z["euler"]) as s:
        for k, row in enumerate(z["trace"]):
            r = s.step()
            assert abs(r["iterations"] - int(row[T_ITER])) <= 2, (k, r["iterations"], row[T_ITER])
            assert rel(r["sig_avg"], row[T_SIG].reshape(3, 3)) < 1e-6, k
            assert rel(r["disgrad_avg"], row[T_DG].reshape(3, 3)) < 1e-6, k
            ref = row[T_DD]
            for j in range(7):
                assert abs(r["dd_avg"][j] - ref[j]) <= 1e-6 * abs(ref[j]), (k, j, r["dd_avg"], ref)

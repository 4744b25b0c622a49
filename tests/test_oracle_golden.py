"""The oracle against the reference's own outputs.

The golden fixtures come from the reference M-THEMES sources compiled here
with single-rank stand-ins (tests/golden/make_golden.py); the oracle must
reproduce their per-step trace and final fields to round-off.
"""
import numpy as np
import pytest

from helpers import (DD_GOLDEN_CASES, GOLDEN_CASES, T_DD, T_DG, T_EDOT, T_EPS, T_ERRE, T_ERRS, T_ITER, T_SIG, T_SVM,
                     T_SVM1, load_golden, rel, run_oracle)


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_oracle_matches_reference_trace(name):
    cfg, trace, fields = load_golden(name)
    o, reps = run_oracle(cfg, nthreads=4)
    for s, r in enumerate(reps):
        row = trace[s]
        assert r["iterations"] == int(row[T_ITER]), (s, r["iterations"], row[T_ITER])
        assert rel(r["sig_avg"], row[T_SIG].reshape(3, 3)) < 1e-11
        assert rel(r["disgrad_avg"], row[T_DG].reshape(3, 3)) < 1e-11
        assert rel(r["eps_avg"], row[T_EPS].reshape(3, 3)) < 1e-9
        assert rel(r["edot_avg"], row[T_EDOT].reshape(3, 3)) < 1e-9
        assert abs(r["s_vm"] - row[T_SVM]) <= 1e-11 * abs(row[T_SVM])
        assert abs(r["s_vm1"] - row[T_SVM1]) <= 1e-11 * abs(row[T_SVM1])
        assert abs(r["err_s"] - row[T_ERRS]) <= 1e-7 * abs(row[T_ERRS])
        assert abs(r["err_e"] - row[T_ERRE]) <= 1e-7 * abs(row[T_ERRE]) + 1e-18
    if fields:
        assert rel(o.field("sig"), fields["sig"]) < 1e-10
        assert rel(o.field("eps"), fields["eps"]) < 1e-9
        assert rel(o.field("rot"), fields["rot"]) < 1e-12
        assert rel(o.field("crss"), fields["crss"]) < 1e-12
        assert rel(o.field("gamacum")[:, 0], fields["gamacum"][:, 0]) < 1e-9
        dg = fields["disgrad"].reshape(-1, 3, 3)
        strain = 0.5 * (dg + dg.transpose(0, 2, 1))
        assert rel(o.field("strain"), strain.reshape(-1, 9)) < 1e-10
        # the full displacement gradient, whose antisymmetric part (the local
        # rotation) varies from voxel to voxel
        assert rel(o.field("disgrad"), dg.reshape(-1, 9)) < 1e-10
    assert o.second_backtracks() == 0


@pytest.mark.parametrize("name", DD_GOLDEN_CASES)
def test_oracle_matches_reference_dd_trace(name):
    """Dislocation-density law: the reference built with its shipped
    DD_BASED_FLAG path (StrainRate_Orowan, DislocationEvolution with
    first-order GNDs, AvgDislocation) against the oracle's restatement."""
    cfg, trace, fields = load_golden(name)
    o, reps = run_oracle(cfg, nthreads=4)
    for s, r in enumerate(reps):
        row = trace[s]
        assert r["iterations"] == int(row[T_ITER]), (s, r["iterations"], row[T_ITER])
        assert rel(r["sig_avg"], row[T_SIG].reshape(3, 3)) < 1e-11
        assert rel(r["disgrad_avg"], row[T_DG].reshape(3, 3)) < 1e-11
        assert rel(r["eps_avg"], row[T_EPS].reshape(3, 3)) < 1e-9
        ref_dd = row[T_DD]
        for k in range(7):
            assert abs(r["dd_avg"][k] - ref_dd[k]) <= 1e-11 * abs(ref_dd[k]) + 1e-300, (s, k, r["dd_avg"], ref_dd)
    assert rel(o.field("sig"), fields["sig"]) < 1e-10
    assert rel(o.field("rot"), fields["rot"]) < 1e-12
    assert rel(o.field("rho_ssd"), fields["rho_ssd"]) < 1e-11
    if np.abs(fields["rho_gnd"]).max() > 0:
        assert rel(o.field("rho_gnd"), fields["rho_gnd"]) < 1e-10


def test_oracle_matches_reference_at_32cube_size():
    """The 32^3 FP64 workload as stated: 64 grains, 10 steps, IterMax 100, Err 1e-5
    (every step runs its 100 Green iterations); per-step trace and a summary
    of the final stress field (component norms and 64 sampled voxels)."""
    import json
    import os
    from helpers import GOLDEN
    from mth import synth
    z = np.load(os.path.join(GOLDEN, "fp64_32cube_trace.npz"))
    d = json.loads(str(z["config"]))
    d["material"] = synth.Material(**d["material"])
    for k in ("cell_dim", "velgrad_bc_flag", "velgrad_bc", "stress_bc_flag", "stress_bc"):
        d[k] = tuple(d[k])
    cfg = synth.Config(**d)
    o, reps = run_oracle(cfg, nthreads=os.cpu_count() or 4)
    trace = z["trace"]
    for s, r in enumerate(reps):
        row = trace[s]
        assert r["iterations"] == int(row[T_ITER]) == 100
        assert rel(r["sig_avg"], row[T_SIG].reshape(3, 3)) < 1e-10
        assert rel(r["disgrad_avg"], row[T_DG].reshape(3, 3)) < 1e-10
        assert abs(r["s_vm"] - row[T_SVM]) <= 1e-10 * abs(row[T_SVM])
        assert abs(r["err_s"] - row[T_ERRS]) <= 1e-6 * abs(row[T_ERRS])
    sig = o.field("sig")
    assert rel(np.linalg.norm(sig, axis=0), z["sig_norm"]) < 1e-10
    assert rel(sig[z["sample_voxels"]], z["sig_sample"]) < 1e-9


def test_oracle_matches_reference_at_128cube_benchmark_grid():
    """The 128^3 benchmark workload on its stated grid (512 grains, 40
    radius-3 pores as the gas phase), 2 steps of 5 Green iterations, against
    the reference's own run: per-step trace and a summary of the final stress
    field.  tests/test_gpu_configs.py holds the GPU to the oracle on the same
    case in FP64 and mixed precision."""
    import json
    import os
    from helpers import GOLDEN
    from mth import synth
    z = np.load(os.path.join(GOLDEN, "rve128_2x5_trace.npz"))
    d = json.loads(str(z["config"]))
    d["material"] = synth.Material(**d["material"])
    for k in ("cell_dim", "velgrad_bc_flag", "velgrad_bc", "stress_bc_flag", "stress_bc"):
        d[k] = tuple(d[k])
    cfg = synth.Config(**d)
    ref = synth.workload("rve128")
    assert (cfg.cell_dim, cfg.n_grains, cfg.n_pores, cfg.seed) == (ref.cell_dim, ref.n_grains, ref.n_pores, ref.seed)
    o, reps = run_oracle(cfg, nthreads=os.cpu_count() or 4)
    trace = z["trace"]
    for s, r in enumerate(reps):
        row = trace[s]
        assert r["iterations"] == int(row[T_ITER]) == 5
        assert rel(r["sig_avg"], row[T_SIG].reshape(3, 3)) < 1e-10
        assert rel(r["disgrad_avg"], row[T_DG].reshape(3, 3)) < 1e-10
        assert abs(r["s_vm"] - row[T_SVM]) <= 1e-10 * abs(row[T_SVM])
        assert abs(r["err_s"] - row[T_ERRS]) <= 1e-6 * abs(row[T_ERRS])
    sig = o.field("sig")
    assert rel(np.linalg.norm(sig, axis=0), z["sig_norm"]) < 1e-10
    assert rel(sig[z["sample_voxels"]], z["sig_sample"]) < 1e-9
    o.close()

"""The per-iteration bookkeeping of the Green iteration (book.cuh: error
norms, get_smacro's volume averages and mixed-boundary strain correction,
the next iteration's strain increment, the convergence test) runs in a
one-warp kernel in mth_step, so that iterations follow one another
without a host round trip.  With MTH_HOST_BOOK=1 the same code runs on the
host after every iteration.  Both must give the same doubles: equal
reports and bit-identical fields, in FP64 and mixed precision, for steps
that run to IterMax and steps that meet Err early (iterations queued after
the last one must change nothing)."""
import os

import numpy as np
import pytest

from mth import Solver, capi, synth

pytestmark = pytest.mark.gpu

CASES = [
    # uniaxial tension with stress-free lateral faces, to IterMax
    synth.Config(cell_dim=(16, 16, 16), n_grains=7, n_steps=3, seed=4101, iter_max=12),
    # Err met after a few iterations; a pore
    synth.Config(cell_dim=(32, 16, 16), n_grains=9, n_steps=3, seed=4102, iter_max=60, err=2e-3, n_pores=1,
                 pore_radius=2),
]


def _run(cfg, precision, host):
    par = capi.params_from_config(cfg, precision=precision)
    if host:
        os.environ["MTH_HOST_BOOK"] = "1"
    try:
        with Solver(par, *synth.microstructure(cfg)) as s:
            reps = [s.step() for _ in range(cfg.n_steps)]
            return reps, s.field("sig"), s.field("strain")
    finally:
        os.environ.pop("MTH_HOST_BOOK", None)


@pytest.mark.parametrize("precision", [capi.MTH_FP64, capi.MTH_MIXED])
@pytest.mark.parametrize("case", range(len(CASES)))
def test_device_bookkeeping_equals_host(case, precision):
    cfg = CASES[case]
    rh, sh, eh = _run(cfg, precision, True)
    rd, sd, ed = _run(cfg, precision, False)
    for k, (a, b) in enumerate(zip(rd, rh)):
        for key in ("iterations", "newton_iters", "newton_failed"):
            assert a[key] == b[key], (k, key)
        for key in ("sig_avg", "disgrad_avg", "s_vm", "e_vm", "err_s", "err_e"):
            assert np.array_equal(np.asarray(a[key]), np.asarray(b[key])), (k, key)
    assert np.array_equal(sd, sh) and np.array_equal(ed, eh)
    if case == 1:
        assert all(r["iterations"] < cfg.iter_max for r in rd[1:])   # Err met before IterMax

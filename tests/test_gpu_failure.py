"""Failure paths, exercised without a GPU fault.

* The local Newton's iteration cap (newton_itmax): solves that hit it are
  counted in the step report and the step goes on, as UpdateStress does when
  its loop ends unconverged (src/evolution.c:110-288).
* The bounded tile-copy waits of the TMA passes: with the library's test hook
  (MTH_TEST_FAIL_TILE_WAIT=1 at context creation) every block's first wait
  reports a time-out at once, while the drain wait still waits for the real
  copies, so nothing stays in flight.  The step must return MTH_ERR_TIMEOUT,
  and a context created afterwards on the same GPU must run normally.
"""
import os

import numpy as np
import pytest

from mth import Solver, capi, synth

pytestmark = pytest.mark.gpu


def case(**kw):
    cfg = synth.Config(cell_dim=(16, 16, 16), n_grains=6, n_steps=3, seed=31, iter_max=6, **kw)
    g, p, e = synth.microstructure(cfg)
    return cfg, g, p, e


def test_newton_iteration_cap_is_reported():
    cfg, g, p, e = case()
    par = capi.params_from_config(cfg, precision=capi.MTH_FP64)
    with Solver(par, g, p, e) as s:
        base = [s.step() for _ in range(3)]
    assert all(r["newton_failed"] == 0 for r in base)
    par.newton_itmax = 1
    with Solver(par, g, p, e) as s:
        capped = [s.step() for _ in range(3)]
    # step 0 runs with the flow rule off; plastic steps hit the cap of 1
    assert capped[1]["newton_failed"] > 0 and capped[2]["newton_failed"] > 0
    assert np.all(np.isfinite(capped[2]["sig_avg"]))


def test_tile_wait_timeout_returns_status_and_gpu_stays_usable():
    cfg, g, p, e = case()
    par = capi.params_from_config(cfg, precision=capi.MTH_MIXED)
    os.environ["MTH_TEST_FAIL_TILE_WAIT"] = "1"
    try:
        with Solver(par, g, p, e) as s:
            with pytest.raises(capi.MthError, match="TIMEOUT"):
                s.step()
    finally:
        del os.environ["MTH_TEST_FAIL_TILE_WAIT"]
    # a new context clears the hook; the GPU answers and the results are the usual ones
    with Solver(par, g, p, e) as s:
        a = [s.step() for _ in range(2)]
    with Solver(par, g, p, e) as s:
        b = [s.step() for _ in range(2)]
    assert a[1]["iterations"] == b[1]["iterations"]
    assert np.array_equal(a[1]["sig_avg"], b[1]["sig_avg"])

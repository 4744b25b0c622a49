"""Batched RVEs (mth_batch_*) against one Solver per member: uneven grid
sizes, per-member material and precision, members converging at different
Green iterations; the FFT tile widths the batch tunes per grid, each checked
against the default widths."""
from __future__ import annotations

import os

import numpy as np
import pytest

from helpers import rel
from mth import Batch, Solver, capi, synth

pytestmark = pytest.mark.gpu


def _members(precision):
    cfgs = [
        synth.Config(cell_dim=(16, 16, 16), n_grains=6, n_steps=3, seed=301, iter_max=40),
        synth.Config(cell_dim=(32, 16, 48), n_grains=9, n_steps=3, seed=302, iter_max=40,
                     material=synth.Material(tau0f=12.5, tau0b=12.5, nrs=20.0)),
        synth.Config(cell_dim=(8, 8, 8), n_grains=3, n_steps=3, seed=303, iter_max=40, n_pores=1, pore_radius=1,
                     material=synth.Material(tau0f=19.0, tau0b=19.0, nrs=8.0)),
        # nearly elastic: converges before IterMax
        synth.Config(cell_dim=(24, 24, 24), n_grains=5, n_steps=3, seed=304, iter_max=40, err=1e-4,
                     material=synth.Material(tau0f=400.0, tau0b=400.0)),
        # single crystal: equilibrium after one Green iteration
        synth.Config(cell_dim=(16, 32, 16), n_grains=1, n_steps=3, seed=305, iter_max=40, err=2e-3),
    ]
    params = [capi.params_from_config(c, precision=precision) for c in cfgs]
    micro = [synth.microstructure(c) for c in cfgs]
    return cfgs, params, micro


@pytest.mark.parametrize("precision,tol", [(capi.MTH_FP64, 1e-9), (capi.MTH_MIXED, 2e-5)])
def test_batch_matches_single_solvers(precision, tol):
    cfgs, params, micro = _members(precision)
    ref = []
    for p, m in zip(params, micro):
        s = Solver(p, *m)
        ref.append(([s.step() for _ in range(3)], s.field("sig")))
        s.close()
    with Batch(params, micro) as b:
        reps = [b.step() for _ in range(3)]
        sig = [b.field(i, "sig") for i in range(len(cfgs))]
        chosen = [b.passes(i) for i in range(len(cfgs))]
    wide = {capi.MTH_FP64: ((2, 4, 8), (1, 2, 4)), capi.MTH_MIXED: ((8, 16, 32), (2, 4, 8))}[precision]
    for c in chosen:
        assert c["tma"] in (0, 1)
        if c["tma"]:
            assert c["kz_strided"] in wide[0] and c["kz_green"] in wide[1], c
    its = set()
    for i in range(len(cfgs)):
        for k in range(3):
            a, r = reps[k][i], ref[i][0][k]
            assert a["iterations"] == r["iterations"], (i, k)
            assert rel(a["sig_avg"], r["sig_avg"]) < tol, (i, k)
            assert rel(a["disgrad_avg"], r["disgrad_avg"]) < tol, (i, k)
            its.add(a["iterations"])
        assert rel(sig[i], ref[i][1]) < 100 * tol
    assert len(its) > 1   # members stopped at different Green iterations


def test_batch_workload_small():
    """The 6-member slice of the 64-RVE workload: steps run, reports finite,
    the imposed strain rate reached by every member."""
    cfgs = synth.batch_workload("batch6")
    params = [capi.params_from_config(c, precision=capi.MTH_MIXED) for c in cfgs]
    micro = [synth.microstructure(c) for c in cfgs]
    with Batch(params, micro) as b:
        for k in range(2):
            reps = b.step()
            for c, r in zip(cfgs, reps):
                assert np.all(np.isfinite(r["sig_avg"]))
                assert abs(r["disgrad_avg"][2, 2] - (k + 1) * c.time_step) < 1e-12
                assert 1 <= r["iterations"] <= c.iter_max


def test_batch_members_match_the_oracle():
    """One member of each grid size of the 64-RVE workload (32^3, 48^3, 64^3),
    with their own grain counts, tau0 and n, stepped together in FP64, against
    the oracle (the reference's algorithm restated) run on each alone."""
    import os
    import pyoracle
    cfgs = synth.batch_workload("batch64")
    pick = {}
    for c in cfgs:
        pick.setdefault(c.cell_dim, c)
    members = [pick[d] for d in sorted(pick)]
    assert sorted(m.cell_dim[0] for m in members) == [32, 48, 64]
    import dataclasses
    members = [dataclasses.replace(m, n_steps=2, iter_max=8) for m in members]
    params = [capi.params_from_config(c, precision=capi.MTH_FP64) for c in members]
    micro = [synth.microstructure(c) for c in members]
    with Batch(params, micro) as b:
        reps = [b.step() for _ in range(2)]
        sig = [b.field(i, "sig") for i in range(len(members))]
    for i, (p, m) in enumerate(zip(params, micro)):
        o = pyoracle.Oracle(p, *m, nthreads=os.cpu_count())
        orep = [o.step() for _ in range(2)]
        for k in range(2):
            assert reps[k][i]["iterations"] == orep[k]["iterations"], (i, k)
            assert rel(reps[k][i]["sig_avg"], orep[k]["sig_avg"]) < 1e-6, (i, k)
            assert rel(reps[k][i]["disgrad_avg"], orep[k]["disgrad_avg"]) < 1e-6, (i, k)
        assert rel(sig[i], o.field("sig")) < 1e-5
        o.close()


@pytest.mark.parametrize("precision", [capi.MTH_FP64, capi.MTH_MIXED])
def test_every_tile_width_gives_the_default_result(precision):
    """Each compiled tile width of the strided and the Green TMA passes (kz
    columns per block; the batch picks among them by timing) against the
    default widths, on a 32x48x64 grid whose 34 kz columns leave a partial
    last tile for every width above 2."""
    cfg = synth.Config(cell_dim=(32, 48, 64), n_grains=7, n_steps=2, seed=311, iter_max=6)
    par = capi.params_from_config(cfg, precision=precision)
    micro = synth.microstructure(cfg)

    def run(tiles):
        if tiles:
            os.environ["MTH_FFT_TILES"] = tiles
        try:
            with Solver(par, *micro) as s:
                reps = [s.step() for _ in range(2)]
                return reps, s.field("sig")
        finally:
            os.environ.pop("MTH_FFT_TILES", None)

    ref, sig0 = run(None)
    tol = 1e-12 if precision == capi.MTH_FP64 else 1e-5
    ks_list, kg_list = {capi.MTH_FP64: ((2, 4, 8), (1, 2, 4)), capi.MTH_MIXED: ((8, 16, 32), (2, 4, 8))}[precision]
    for ks in ks_list:
        for kg in kg_list:
            reps, sig = run(f"{ks},{kg}")
            for a, r in zip(reps, ref):
                assert a["iterations"] == r["iterations"], (ks, kg)
                assert rel(a["sig_avg"], r["sig_avg"]) < tol, (ks, kg)
            assert rel(sig, sig0) < 10 * tol, (ks, kg)

"""Per-step field files in the reference's .iout format (mth_write_iout):
contents against the downloaded fields, file names, and the write running
in the background while the next step proceeds."""
from __future__ import annotations

import os

import numpy as np
import pytest

from helpers import run_gpu
from mth import capi, synth

pytestmark = pytest.mark.gpu

COMP = [(0, 0), (1, 1), (2, 2), (1, 2), (0, 2), (0, 1)]
TEX = np.dtype([("angle", "<f8", 3), ("coord", "<i4", 3), ("jgr", "<i4"), ("jph", "<i4"), ("buff", "<i4")])


def _components(prefix, step, nv):
    out = []
    for c in range(6):
        name = f"{prefix}_{c + 1}_S{step:06d}.iout"
        a = np.fromfile(name, dtype="<f8")
        assert a.size == nv
        out.append(a)
    return np.stack(out, axis=1)


def _bunge(rot):
    """EulerToTransMatrix opt 1 on the sample->crystal matrix (transpose of rot)."""
    a = rot.reshape(-1, 3, 3).transpose(0, 2, 1)
    ph = np.arccos(a[:, 2, 2])
    sph = np.sin(ph)
    special = np.abs(a[:, 2, 2]) > 0.9999
    with np.errstate(divide="ignore", invalid="ignore"):
        t1 = np.where(special, np.arctan2(a[:, 0, 1], a[:, 0, 0]), np.arctan2(a[:, 2, 0] / sph, -a[:, 2, 1] / sph))
        t2 = np.where(special, 0.0, np.arctan2(a[:, 0, 2] / sph, a[:, 1, 2] / sph))
    return np.degrees(np.stack([t1, ph, t2], axis=1))


@pytest.mark.parametrize("precision", [capi.MTH_FP64, capi.MTH_MIXED])
def test_iout_files(tmp_path, precision):
    cfg = synth.Config(cell_dim=(16, 8, 12), n_grains=5, n_pores=1, pore_radius=2, n_steps=2, seed=61, iter_max=15)
    s, _ = run_gpu(cfg, precision)
    nv = 16 * 8 * 12
    pre = str(tmp_path / "f")
    for kind in ("sig", "els", "eps", "grain", "texture"):
        s.write_iout(kind, f"{pre}_{kind}", 2)
    s.wait_iout()
    sig = s.field("sig").reshape(nv, 3, 3)
    got = _components(f"{pre}_sig", 2, nv)
    for c, (i, j) in enumerate(COMP):
        assert np.array_equal(got[:, c], sig[:, i, j])
    els = (s.field("strain") - s.field("eps")).reshape(nv, 3, 3)
    got = _components(f"{pre}_els", 2, nv)
    for c, (i, j) in enumerate(COMP):
        np.testing.assert_allclose(got[:, c], els[:, i, j], rtol=1e-12, atol=1e-15)
    eps = s.field("eps").reshape(nv, 3, 3)
    got = _components(f"{pre}_eps", 2, nv)
    for c, (i, j) in enumerate(COMP):
        assert np.array_equal(got[:, c], eps[:, i, j])
    g = np.fromfile(f"{pre}_grain_S000002.iout", dtype="<i4")
    assert np.array_equal(g, s.field("grain")[:, 0].astype(np.int32))
    t = np.fromfile(f"{pre}_texture_S000002.iout", dtype=TEX)
    assert t.size == nv
    grain, phase, _ = synth.microstructure(cfg)
    X, Y, Z = np.meshgrid(np.arange(16), np.arange(8), np.arange(12), indexing="ij")
    assert np.array_equal(t["coord"], np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1) + 1)
    assert np.array_equal(t["jgr"], grain)
    assert np.array_equal(t["jph"], phase)
    assert np.all(t["buff"] == 0)
    np.testing.assert_allclose(t["angle"], _bunge(s.field("rot")), rtol=0, atol=1e-9)
    s.close()


@pytest.mark.parametrize("precision", [capi.MTH_FP64, capi.MTH_MIXED])
def test_iout_disgrad(tmp_path, precision):
    """WriteDisgradMPI's files (src/io.c:283-320): entries 11, 22, 33, 23,
    13, 12 of the full displacement gradient, whose off-diagonal pairs differ
    by the local rotation, against the downloaded field."""
    from mth import Solver
    cfg = synth.Config(cell_dim=(16, 8, 12), n_grains=5, n_pores=1, pore_radius=2, n_steps=2, seed=61, iter_max=15)
    s = Solver(capi.params_from_config(cfg, precision=precision), *synth.microstructure(cfg))
    s.track_disgrad()
    for _ in range(cfg.n_steps):
        s.step()
    nv = 16 * 8 * 12
    pre = str(tmp_path / "disg")
    s.write_iout("disgrad", pre, 2)
    s.wait_iout()
    dg = s.field("disgrad").reshape(nv, 3, 3)
    got = _components(pre, 2, nv)
    for c, (i, j) in enumerate(COMP):
        np.testing.assert_allclose(got[:, c], dg[:, i, j], rtol=1e-12, atol=1e-15)
    strain = s.field("strain").reshape(nv, 3, 3)
    np.testing.assert_allclose(0.5 * (dg + dg.transpose(0, 2, 1)), strain, rtol=1e-12, atol=1e-15)
    w = 0.5 * (dg - dg.transpose(0, 2, 1))
    assert np.abs(w).max() > 1e-2 * np.abs(dg).max()
    assert sorted(os.listdir(tmp_path)) == [f"disg_{c}_S000002.iout" for c in range(1, 7)]
    s.close()


def test_disgrad_needs_tracking(tmp_path):
    """Without mth_track_disgrad the full gradient is not kept: its download
    and its files are refused, and tracking cannot start after a step."""
    cfg = synth.Config(cell_dim=(8, 8, 8), n_grains=2, n_steps=1, seed=63, iter_max=5)
    s, _ = run_gpu(cfg)
    with pytest.raises(capi.MthError):
        s.field("disgrad")
    with pytest.raises(capi.MthError):
        s.write_iout("disgrad", str(tmp_path / "d"), 0)
    with pytest.raises(capi.MthError):
        s.track_disgrad()
    s.close()


def test_iout_overlaps_next_step(tmp_path):
    """The snapshot is taken at the call: files hold the state before the
    step that runs while they are written."""
    cfg = synth.Config(cell_dim=(32, 32, 32), n_grains=8, n_steps=1, seed=62, iter_max=10)
    s, _ = run_gpu(cfg, capi.MTH_MIXED)
    before = s.field("sig").reshape(-1, 3, 3)
    pre = str(tmp_path / "sig")
    s.write_iout("sig", pre, 7)
    s.step()
    s.wait_iout()
    got = _components(pre, 7, 32 ** 3)
    assert np.array_equal(got[:, 0], before[:, 0, 0])
    assert not np.array_equal(before, s.field("sig").reshape(-1, 3, 3))
    assert sorted(os.listdir(tmp_path)) == [f"sig_{c}_S000007.iout" for c in range(1, 7)]
    s.close()


def test_iout_errors(tmp_path):
    cfg = synth.Config(cell_dim=(8, 8, 8), n_grains=2, n_steps=1, seed=63, iter_max=5)
    s, _ = run_gpu(cfg)
    assert s.lib.mth_write_iout(s.ctx, 9, b"x", 0) == 1   # unknown kind
    s.write_iout("sig", str(tmp_path / "missing_dir" / "sig"), 0)
    with pytest.raises(capi.MthError):
        s.wait_iout()
    s.close()


def test_iout_against_the_reference_writers(tmp_path):
    """The files the reference itself wrote at the end of step 0 (WriteElsMPI
    "els" and WriteSigMPI "sig_afterDRX", src/io.c:322-437, with PrintControl
    1) against mth_write_iout after the same step in FP64: the same file
    names and sizes, values within the FP64 parity tolerance."""
    import json
    from helpers import GOLDEN
    z = np.load(os.path.join(GOLDEN, "iout_g8.npz"))
    d = json.loads(str(z["config"]))
    d["material"] = synth.Material(**d["material"])
    for k in ("cell_dim", "velgrad_bc_flag", "velgrad_bc", "stress_bc_flag", "stress_bc"):
        d[k] = tuple(d[k])
    d.pop("dd", None)
    d.pop("drx", None)
    cfg = synth.Config(**d)
    s, _ = run_gpu(cfg, capi.MTH_FP64)
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        s.write_iout("els", "els", 0)
        s.write_iout("sig", "sig_afterDRX", 0)
        s.wait_iout()
        names = sorted(f for f in os.listdir(tmp_path) if f.endswith(".iout"))
        assert names == [str(n) for n in z["names"]]
        for i, n in enumerate(names):
            ref = z["f%02d" % i].view("<f8")
            got = np.fromfile(n, dtype="<f8")
            assert got.nbytes == z["f%02d" % i].size
            assert np.abs(got - ref).max() <= 1e-6 * np.abs(ref).max(), n
    finally:
        os.chdir(cwd)
        s.close()

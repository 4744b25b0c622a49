"""The DRX restatement (oracle/drx_oracle.c) on its own: invariants of the
sparse order parameters and the physics the reference's phase-field step
encodes (stored-energy-driven growth of a recrystallised nucleus)."""
import numpy as np

import pyoracle
from mth import capi, synth


def pf_params(**kw):
    cfg = synth.Config(cell_dim=(16, 16, 16), drx=synth.Drx(**kw))
    return capi.params_from_config(cfg, precision=capi.MTH_FP64)


def sphere(dims, c, r):
    ax = [np.arange(n) for n in dims]
    X, Y, Z = np.meshgrid(*ax, indexing="ij")
    return ((X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2 <= r * r).ravel()


def test_single_grain_is_stationary():
    dims = (12, 12, 12)
    g = np.full(int(np.prod(dims)), 3, np.int32)
    rho = np.full(g.size, 200.0)
    go, ids, phi, cnt = pyoracle.pf_relax(pf_params(), dims, g, rho, 5)
    assert np.array_equal(go, g)
    assert np.all(cnt == 1) and np.all(ids[:, 0] == 3) and np.all(phi[:, 0] == 1.0)


def test_nucleus_grows_into_deformed_grain():
    """A dislocation-free nucleus (rho=1) in a grain at rho=500 expands: the
    stored-energy driving force of src/pf_xrx.c:1184-1233."""
    dims = (24, 24, 24)
    nv = int(np.prod(dims))
    g = np.full(nv, 1, np.int32)
    nuc = sphere(dims, (12, 12, 12), 3)
    g[nuc] = 2
    rho = np.where(nuc, 1.0, 500.0)
    p = pf_params()
    go, ids, phi, cnt = pyoracle.pf_relax(p, dims, g, rho, 30)
    assert (go == 2).sum() > nuc.sum()
    # without the stored-energy difference the nucleus does not grow
    go2, *_ = pyoracle.pf_relax(p, dims, g, np.full(nv, 500.0), 30)
    assert (go2 == 2).sum() <= nuc.sum()


def test_sparse_invariants():
    dims = (16, 16, 16)
    cfg = synth.Config(cell_dim=dims, n_grains=10, seed=4)
    g, _, _ = synth.microstructure(cfg)
    rng = np.random.default_rng(0)
    rho = 50.0 + 400.0 * rng.random(g.size)
    go, ids, phi, cnt = pyoracle.pf_relax(pf_params(), dims, g, rho, 8)
    assert cnt.min() >= 1 and cnt.max() <= 8
    for v in range(0, g.size, 7):
        k = cnt[v]
        assert np.all(np.diff(ids[v, :k]) > 0)          # sorted, unique
        assert np.all(phi[v, :k] > 1e-4)                 # kept values
        assert go[v] == ids[v, np.argmax(phi[v, :k])]    # argmax, ties to the smaller id


def test_nucleation_counter_rng():
    dims = (16, 16, 16)
    cfg = synth.Config(cell_dim=dims, n_grains=8, seed=2)
    g, ph, _ = synth.microstructure(cfg)
    p = pf_params(rho_nucleation=10.0, nucleation_prob=0.05, seed=99)
    rho = np.full(g.size, 100.0)
    cry = np.ones(g.size, np.int32)
    g1, s1 = pyoracle.nucleate(p, dims, g, cry, rho, step=3, first_id=100)
    g2, s2 = pyoracle.nucleate(p, dims, g, cry, rho, step=3, first_id=100)
    assert np.array_equal(s1, s2) and np.array_equal(g1, g2)
    assert np.all(np.diff(s1) > 0)
    g3, s3 = pyoracle.nucleate(p, dims, g, cry, rho, step=4, first_id=100)
    assert not np.array_equal(s1, s3)
    # below the threshold nothing nucleates
    g4, s4 = pyoracle.nucleate(p, dims, g, cry, np.full(g.size, 5.0), step=3, first_id=100)
    assert s4.size == 0 and np.array_equal(g4, g)
    # every site is a grain-boundary voxel, painted with consecutive ids
    assert set(np.unique(g1[g1 >= 100])) <= set(range(100, 100 + s1.size))


def test_grid_transfer_properties():
    """Phase-field grid transfer (InterpolateGrid): identity on equal grids,
    up-then-down recovers integer maps, trilinear is exact on affine fields."""
    import pyoracle
    rng = np.random.default_rng(7)
    ns = (8, 6, 10)
    g = rng.integers(1, 20, size=int(np.prod(ns))).astype(np.int32)
    assert np.array_equal(pyoracle.resample(g, ns, ns), g)
    for r in (2, 3):
        nd = tuple(r * n for n in ns)
        up = pyoracle.resample(g, ns, nd)
        assert set(np.unique(up)) <= set(np.unique(g))
        assert np.array_equal(pyoracle.resample(up, nd, ns), g)
    X, Y, Z = np.meshgrid(*[np.arange(n) / (n - 1) for n in ns], indexing="ij")
    f = (1.5 + 2.0 * X - 0.5 * Y + 3.0 * Z).ravel()
    nd = (13, 11, 17)
    Xd, Yd, Zd = np.meshgrid(*[np.arange(n) / (n - 1) for n in nd], indexing="ij")
    want = (1.5 + 2.0 * Xd - 0.5 * Yd + 3.0 * Zd).ravel()
    np.testing.assert_allclose(pyoracle.resample(f, ns, nd), want, rtol=0, atol=1e-12)

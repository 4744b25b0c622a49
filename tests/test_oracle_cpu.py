"""Oracle building blocks: its FFT against numpy, the seeded synthetic
inputs, and the local Newton's convergence."""
import numpy as np
import pytest

import pyoracle
from mth import capi, synth


@pytest.mark.parametrize("shape", [(8, 8, 8), (12, 8, 6), (24, 4, 2), (48, 2, 2)])
def test_oracle_fft_matches_numpy(shape):
    rng = np.random.default_rng(1)
    a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    f = pyoracle.fft3d(a, -1)
    assert np.abs(f - np.fft.fftn(a)).max() < 1e-12 * np.abs(f).max()
    b = pyoracle.fft3d(f, +1)
    assert np.abs(b / a.size - a).max() < 1e-13


def test_synth_is_seeded_and_periodic():
    cfg = synth.Config(cell_dim=(16, 16, 16), n_grains=10, n_pores=3, pore_radius=2, seed=5)
    g1, p1, e1 = synth.microstructure(cfg)
    g2, p2, e2 = synth.microstructure(cfg)
    assert np.array_equal(g1, g2) and np.array_equal(e1, e2)
    assert set(np.unique(g1[p1 == 1])) <= set(range(1, 11))
    assert (p1 == 2).sum() > 0 and np.all(g1[p1 == 2] == 11)
    assert np.all(e1[p1 == 2] == 0)
    # orientations are per grain
    for gid in np.unique(g1[p1 == 1]):
        assert np.all(e1[(g1 == gid) & (p1 == 1)] == e1[(g1 == gid) & (p1 == 1)][0])


def random_states(n, rng, cfg):
    """Voxel states around yield: random orientation, strain increments of
    ~1e-3 and stresses near the CRSS."""
    from scipy.spatial.transform import Rotation
    rot = Rotation.random(n, random_state=int(rng.integers(1 << 30))).as_matrix().reshape(n, 9)
    sig = rng.standard_normal((n, 6)) * 30.0
    sig[:, 5] *= 0.1
    strain = rng.standard_normal((n, 6)) * 1e-3
    epsp = rng.standard_normal((n, 6)) * 3e-4
    epsp[:, 5] = 0.0
    crss = 16.0 + rng.random((n, 12)) * 10.0
    return sig, epsp, strain, rot, crss


def test_oracle_local_solve_converges():
    cfg = synth.Config(cell_dim=(8, 8, 8), n_grains=4)
    p = capi.params_from_config(cfg)
    o = pyoracle.Oracle(p, *synth.microstructure(cfg), nthreads=2)
    c066 = o.c066()
    rng = np.random.default_rng(7)
    sig, epsp, strain, rot, crss = random_states(64, rng, cfg)
    s, ed, err, it = pyoracle.local_solve(p, c066, sig, epsp, strain, rot, crss)
    assert np.all(np.isfinite(s)) and it > 0
    assert np.all(ed[:, 5] == 0.0)

"""The C driver (m-themes_gb300/host/forge.c, the shape of the reference's
evp.c) end to end on the reference's three input files: it must reproduce the
oracle's per-step vm.out columns and macroscopic curve."""
import os
import subprocess
import sys

import numpy as np
import pytest

from helpers import run_oracle
from mth import synth

pytestmark = pytest.mark.gpu
REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module", autouse=True)
def built():
    subprocess.check_call([sys.executable, os.path.join(REPO, "m-themes_gb300", "build.py")])


def test_forge_driver_matches_oracle(tmp_path):
    cfg = synth.Config(cell_dim=(16, 16, 16), n_grains=6, n_pores=1, pore_radius=2, n_steps=4, seed=61,
                       iter_max=15)
    synth.write_case(str(tmp_path), cfg)
    forge = os.path.join(REPO, "m-themes_gb300", "lib", "forge")
    r = subprocess.run([forge, "input.in"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    vm = np.loadtxt(tmp_path / "vm.out", skiprows=1)
    ss = np.loadtxt(tmp_path / "ss.out", skiprows=1)
    _, reps = run_oracle(cfg)
    assert vm.shape == (4, 7) and ss.shape == (4, 11)
    for k, rep in enumerate(reps):
        ref = [rep["time"], rep["e_vm"], rep["evmp"], rep["d_vm"], rep["dvmp"], rep["s_vm"], rep["s_vm1"]]
        # vm.out is printed with %e (7 significant digits)
        assert np.allclose(vm[k], ref, rtol=2e-6, atol=1e-12), (k, vm[k], ref)
        assert int(ss[k, 1]) == rep["iterations"]
        assert abs(ss[k, 8] - rep["sig_avg"][2, 2]) <= 1e-6 * abs(rep["sig_avg"][2, 2])


def test_forge_writes_field_files(tmp_path):
    cfg = synth.Config(cell_dim=(8, 8, 8), n_grains=3, n_steps=3, seed=64, iter_max=10)
    synth.write_case(str(tmp_path), cfg)
    forge = os.path.join(REPO, "m-themes_gb300", "lib", "forge")
    r = subprocess.run([forge, "input.in", "--iout-every", "2"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    for pre in ("els", "sig"):
        for step in (0, 2):
            for c in range(1, 7):
                f = tmp_path / f"{pre}_{c}_S{step:06d}.iout"
                assert f.stat().st_size == 8 * 8 ** 3
    assert not (tmp_path / "sig_1_S000001.iout").exists()

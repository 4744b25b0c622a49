"""Generate the golden fixtures of tests/golden/ by running the reference.

The reference M-THEMES `forge` is compiled from its own sources by
oracle/build_ref.sh (single-rank MPI/FFTW/GSL stand-ins, power-law flow rule
and Voce hardening wired in through the build's hooks) and run on small seeded
synthetic inputs written in the reference's file formats.  Each fixture holds
the configuration, the per-step trace (Green iterations, <sigma>,
<grad u>, <eps_p>, <edot_p>, s_vm, s_vm1, e_vm, d_vm, Err_s, Err_e) and the
final fields.

Needs the reference sources (MTH_REFERENCE, default /root/reference) and a
C++ compiler; it is not run by the tests.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import dataclasses
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "m-themes_gb300"))
from mth import synth  # noqa: E402

CASES = {
    # name: Config
    "g8_poly": synth.Config(cell_dim=(8, 8, 8), n_grains=4, n_steps=4, seed=101, iter_max=30),
    "g12_radix3": synth.Config(cell_dim=(12, 12, 12), n_grains=6, n_steps=3, seed=102, iter_max=25),
    "g16_pores": synth.Config(cell_dim=(16, 16, 16), n_grains=8, n_pores=2, pore_radius=2, n_steps=3, seed=103,
                              iter_max=25),
    "g8_elastbc0": synth.Config(cell_dim=(8, 8, 8), n_grains=3, n_steps=3, seed=104, elast_bc=0, iter_max=25),
    "g8_shear": synth.Config(cell_dim=(8, 8, 8), n_grains=4, n_steps=4, seed=105, iter_max=25,
                             velgrad_bc_flag=(0, 0, 1, 1, 1, 0), velgrad_bc=(0.0, 0.0, 1.0, 0.0, 0.0, 0.0),
                             stress_bc_flag=(1, 1, 0, 0, 0, 1), stress_bc=(0.0, 0.0, 0.0, 0.0, 0.0, 20.0)),
    "g8_stiff_n20": synth.Config(cell_dim=(8, 8, 8), n_grains=4, n_steps=3, seed=106, iter_max=25,
                                 material=synth.Material(nrs=20.0, tau0f=12.0, tau0b=12.0)),
    # nearly elastic polycrystal: the Green loop converges before IterMax
    "g8_elastic": synth.Config(cell_dim=(8, 8, 8), n_grains=4, n_steps=3, seed=107, iter_max=60, err=1e-4,
                               material=synth.Material(tau0f=400.0, tau0b=400.0)),
    # homogeneous single crystal: equilibrium holds after one Green iteration
    "g8_single": synth.Config(cell_dim=(8, 8, 8), n_grains=1, n_steps=3, seed=108, iter_max=40, err=2e-3),
}


# dislocation-density law (the reference's shipped DD_BASED_FLAG path, built as
# oracle/_ref/forge_ref_dd): per-step trace with the dd.out averages and the
# final SSD / GND densities
DD_CASES = {
    "dd8_poly": synth.Config(cell_dim=(8, 8, 8), n_grains=4, n_steps=4, seed=201, iter_max=40, dd=synth.DD()),
    "dd8_pores": synth.Config(cell_dim=(8, 8, 8), n_grains=4, n_pores=1, pore_radius=1, n_steps=4, seed=202,
                              iter_max=30, dd=synth.DD(q_slip=0.22, L0=0.002)),
    # test_run/input.in's DD values: thermally activated slip switched off
    "dd8_test_run_values": synth.Config(cell_dim=(8, 8, 8), n_grains=4, n_steps=3, seed=203, iter_max=30,
                                        dd=synth.DD(T=30.0, q_slip=20000000000.0, q_bulk=300000000000.51)),
}


def cfg_to_json(cfg):
    d = dataclasses.asdict(cfg)
    return json.dumps(d)


def main():
    ref = os.path.join(REPO, "oracle", "_ref", "forge_ref")
    subprocess.check_call([os.path.join(REPO, "oracle", "build_ref.sh")])
    for name, cfg in CASES.items():
        d = os.path.join("/tmp", "mth_golden_" + name)
        grain, phase, euler = synth.write_case(d, cfg)
        env = dict(os.environ, MTH_REF_TRACE=os.path.join(d, "trace.txt"), MTH_REF_DUMP=d, MTH_REF_SEED="1")
        subprocess.run(["bash", "-c", f"ulimit -s unlimited; {ref} input.in > ref.log 2>&1"], cwd=d, env=env,
                       check=True)
        trace = np.atleast_2d(np.loadtxt(os.path.join(d, "trace.txt")))
        nv = int(np.prod(cfg.cell_dim))
        fields = {}
        if nv > 12 ** 3:   # keep the fixtures small: traces only for larger grids
            np.savez_compressed(os.path.join(HERE, name + ".npz"), config=cfg_to_json(cfg), trace=trace)
            print(name, trace.shape, "iters", trace[:, 1].astype(int).tolist())
            continue
        for fn, nc in [("sig", 9), ("eps", 9), ("edot", 9), ("disgrad", 9), ("rot", 9), ("crss", 12),
                       ("gamacum", 1)]:
            fields[fn] = np.fromfile(os.path.join(d, fn + ".bin")).reshape(nv, nc)
        out = os.path.join(HERE, name + ".npz")
        np.savez_compressed(out, config=cfg_to_json(cfg), trace=trace, **fields)
        print(name, trace.shape, "iters", trace[:, 1].astype(int).tolist(), "->", os.path.relpath(out, REPO))


def main_dd():
    ref = os.path.join(REPO, "oracle", "_ref", "forge_ref_dd")
    for name, cfg in DD_CASES.items():
        d = os.path.join("/tmp", "mth_golden_" + name)
        synth.write_case(d, cfg)
        env = dict(os.environ, MTH_REF_TRACE=os.path.join(d, "trace.txt"), MTH_REF_DUMP=d, MTH_REF_SEED="1",
                   MTH_REF_DD="1")
        subprocess.run(["bash", "-c", f"ulimit -s unlimited; {ref} input.in > ref.log 2>&1"], cwd=d, env=env,
                       check=True)
        trace = np.atleast_2d(np.loadtxt(os.path.join(d, "trace.txt")))
        nv = int(np.prod(cfg.cell_dim))
        fields = {fn: np.fromfile(os.path.join(d, fn + ".bin")).reshape(nv, nc)
                  for fn, nc in [("sig", 9), ("rot", 9)]}
        rho = np.fromfile(os.path.join(d, "rho.bin")).reshape(nv, 4, 12)
        fields["rho_ssd"] = rho[:, 0]
        fields["rho_gnd"] = rho[:, 1:].reshape(nv, 36)
        out = os.path.join(HERE, name + ".npz")
        np.savez_compressed(out, config=cfg_to_json(cfg), trace=trace, **fields)
        print(name, trace.shape, "iters", trace[:, 1].astype(int).tolist(), "->", os.path.relpath(out, REPO))


# The elastic constants that the DD_CU switch of the shipped flags writes over
# input.in's (src/init.c:821-825), MPa.
DD_CU_ELASTIC = (241.1674 * 1000, 89.1989 * 1000, 151.9685 * 1000)


def main_test_run():
    """The reference's own test_run/ inputs, unmodified, through the build with
    the shipped flags (DD law, DD_CU).  That build stops with a segmentation
    fault during the second mechanical step of this input; the first step's
    trace is kept, with the parameters and microstructure as this project's
    readers parse them."""
    import ctypes as C
    import shutil
    from mth import capi
    src = os.path.join(os.environ.get("MTH_REFERENCE", "/root/reference"), "test_run")
    d = "/tmp/mth_golden_test_run"
    shutil.rmtree(d, ignore_errors=True)
    shutil.copytree(src, d)
    for f in os.listdir(d):
        os.chmod(os.path.join(d, f), 0o644)
    ref = os.path.join(REPO, "oracle", "_ref", "forge_ref_dd_cu")
    env = dict(os.environ, MTH_REF_TRACE=os.path.join(d, "trace.txt"), MTH_REF_SEED="1")
    subprocess.run(["bash", "-c", f"ulimit -s unlimited; {ref} input.in > ref.log 2>&1"], cwd=d, env=env)
    trace = np.atleast_2d(np.loadtxt(os.path.join(d, "trace.txt")))[:1]
    lib = capi.load()
    par = capi.MthParams()
    s1, s2, ms = C.create_string_buffer(256), C.create_string_buffer(256), C.create_string_buffer(256)
    capi.check(lib, lib.mth_read_namelist(os.path.join(d, "input.in").encode(), C.byref(par), s1, s2, ms, 256))
    capi.check(lib, lib.mth_read_sx(os.path.join(d, s1.value.decode()).encode(), C.byref(par), 0))
    nv = int(np.prod(list(par.cell_dim)))
    g = np.zeros(nv, np.int32)
    ph = np.zeros(nv, np.int32)
    e = np.zeros(3 * nv)
    capi.check(lib, lib.mth_read_microstructure(os.path.join(d, ms.value.decode()).encode(), par.cell_dim,
                                                capi._iptr(g), capi._iptr(ph), capi._dptr(e)))
    out = os.path.join(HERE, "tr_dd_step0.npz")
    np.savez_compressed(out, params=np.frombuffer(bytes(par), dtype=np.uint8), dd_cu=np.array(DD_CU_ELASTIC),
                        grain=g, phase=ph, euler=e.reshape(nv, 3), trace=trace)
    print("test_run step 0: iterations", int(trace[0, 1]), "->", os.path.relpath(out, REPO))


if __name__ == "__main__":
    main()
    main_dd()
    main_test_run()

"""Generate the golden fixtures of tests/golden/ by running the reference.

The reference M-THEMES `forge` is compiled from its own sources by
oracle/build_ref.sh (single-rank MPI/FFTW/GSL stand-ins, power-law flow rule
and Voce hardening wired in through the build's hooks) and run on small seeded
synthetic inputs written in the reference's file formats.  Each fixture holds
the configuration, the per-step trace (Green iterations, <sigma>,
<grad u>, <eps_p>, <edot_p>, s_vm, s_vm1, e_vm, d_vm, Err_s, Err_e) and the
final fields.

Needs the reference sources (the directory named by MTH_REFERENCE) and a
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
    the shipped flags (DD law, DD_CU): both mechanical steps' trace, with the
    parameters and microstructure as this project's readers parse them.  (The
    FFT buffers carry slack for the reference's out-of-range write at
    src/evolution.c:1598-1599, which otherwise crashes the second step.)"""
    import ctypes as C
    import shutil
    from mth import capi
    src = os.path.join(os.environ["MTH_REFERENCE"], "test_run")
    d = "/tmp/mth_golden_test_run"
    shutil.rmtree(d, ignore_errors=True)
    shutil.copytree(src, d)
    for f in os.listdir(d):
        os.chmod(os.path.join(d, f), 0o644)
    ref = os.path.join(REPO, "oracle", "_ref", "forge_ref_dd_cu")
    env = dict(os.environ, MTH_REF_TRACE=os.path.join(d, "trace.txt"), MTH_REF_SEED="1")
    subprocess.run(["bash", "-c", f"ulimit -s unlimited; {ref} input.in > ref.log 2>&1"], cwd=d, env=env)
    trace = np.atleast_2d(np.loadtxt(os.path.join(d, "trace.txt")))
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
    out = os.path.join(HERE, "tr_dd_test_run.npz")
    np.savez_compressed(out, params=np.frombuffer(bytes(par), dtype=np.uint8), dd_cu=np.array(DD_CU_ELASTIC),
                        grain=g, phase=ph, euler=e.reshape(nv, 3), trace=trace)
    print("test_run: iterations", trace[:, 1].astype(int).tolist(), "->", os.path.relpath(out, REPO))


# The 32^3 FP64 workload at its stated size: 64 seeded Voronoi grains,
# Cu power law + Voce, uniaxial tension, 10 steps, IterMax 100, Err 1e-5.
# The input declares two phases (the second unused): with N_phases 1 the
# reference reads nSYS[1] past its one-element allocation in SetupJob
# (src/init.c:806-807 against the NPHMAX loop at :1104-1108), which crashes
# this 64-grain case; with no voxel of phase 2 the traces are identical (checked
# on an 8^3 case).  Trace plus a summary of the final stress field.
SAMPLE_VOXELS = np.arange(0, 32 ** 3, 32 ** 3 // 64)


def main_configs():
    ref = os.path.join(REPO, "oracle", "_ref", "forge_ref")
    cfg = synth.workload("fp64_32cube")
    d = "/tmp/mth_golden_fp64_32cube"
    synth.write_case(d, cfg)
    inp = os.path.join(d, "input.in")
    txt = open(inp).read().replace("N_phases\t1\n", "N_phases\t2\n")
    open(inp, "w").write(txt)
    env = dict(os.environ, MTH_REF_TRACE=os.path.join(d, "trace.txt"), MTH_REF_DUMP=d, MTH_REF_SEED="1")
    subprocess.run(["bash", "-c", f"ulimit -s unlimited; {ref} input.in > ref.log 2>&1"], cwd=d, env=env, check=True)
    trace = np.atleast_2d(np.loadtxt(os.path.join(d, "trace.txt")))
    nv = int(np.prod(cfg.cell_dim))
    sig = np.fromfile(os.path.join(d, "sig.bin")).reshape(nv, 9)
    out = os.path.join(HERE, "fp64_32cube_trace.npz")
    np.savez_compressed(out, config=cfg_to_json(cfg), trace=trace, sig_norm=np.linalg.norm(sig, axis=0),
                        sample_voxels=SAMPLE_VOXELS, sig_sample=sig[SAMPLE_VOXELS])
    print("fp64_32cube_trace", trace.shape, "iters", trace[:, 1].astype(int).tolist(), "->", os.path.relpath(out, REPO))


# The 128^3 benchmark workload at its stated grid (512 grains, 40 radius-3
# pores as the gas phase), 2 steps of 5 Green iterations: the trace plus a
# summary of the final stress field (column norms, 64 sampled voxels).
def main_rve128():
    ref = os.path.join(REPO, "oracle", "_ref", "forge_ref")
    cfg = synth.workload("rve128")
    cfg = dataclasses.replace(cfg, n_steps=2, iter_max=5)
    d = "/tmp/mth_golden_rve128"
    import shutil
    shutil.rmtree(d, ignore_errors=True)
    synth.write_case(d, cfg)
    env = dict(os.environ, MTH_REF_TRACE=os.path.join(d, "trace.txt"), MTH_REF_DUMP=d, MTH_REF_SEED="1")
    subprocess.run(["bash", "-c", f"ulimit -s unlimited; {ref} input.in > ref.log 2>&1"], cwd=d, env=env, check=True)
    trace = np.atleast_2d(np.loadtxt(os.path.join(d, "trace.txt")))
    nv = int(np.prod(cfg.cell_dim))
    sig = np.fromfile(os.path.join(d, "sig.bin")).reshape(nv, 9)
    samples = np.arange(0, nv, nv // 64)
    out = os.path.join(HERE, "rve128_2x5_trace.npz")
    np.savez_compressed(out, config=cfg_to_json(cfg), trace=trace, sig_norm=np.linalg.norm(sig, axis=0),
                        sample_voxels=samples, sig_sample=sig[samples])
    print("rve128_2x5_trace", trace.shape, "iters", trace[:, 1].astype(int).tolist(), "->", os.path.relpath(out, REPO))


# The reference's own field files: with PrintControl 1 it writes, at the end
# of step 0, the elastic strain and the stress (WriteElsMPI "els",
# WriteSigMPI "sig_afterDRX", src/evolution.c:1632-1652, src/io.c:322-437)
# through MPI-IO (here the single-rank shim: the same bytes at offset 0).
def main_iout():
    ref = os.path.join(REPO, "oracle", "_ref", "forge_ref")
    cfg = CASES["g8_poly"]
    cfg = dataclasses.replace(cfg, n_steps=1)
    d = "/tmp/mth_golden_iout"
    import shutil
    shutil.rmtree(d, ignore_errors=True)
    synth.write_case(d, cfg)
    inp = os.path.join(d, "input.in")
    txt = open(inp).read()
    assert "PrintControl 0 2000" in txt
    open(inp, "w").write(txt.replace("PrintControl 0 2000", "PrintControl 1 2000"))
    env = dict(os.environ, MTH_REF_TRACE=os.path.join(d, "trace.txt"), MTH_REF_SEED="1")
    subprocess.run(["bash", "-c", f"ulimit -s unlimited; {ref} input.in > ref.log 2>&1"], cwd=d, env=env, check=True)
    names = sorted(f for f in os.listdir(d) if f.endswith(".iout"))
    assert len(names) == 12, names
    files = {n: np.frombuffer(open(os.path.join(d, n), "rb").read(), dtype=np.uint8) for n in names}
    out = os.path.join(HERE, "iout_g8.npz")
    np.savez_compressed(out, config=cfg_to_json(cfg), names=np.array(names), **{"f%02d" % i: files[n] for i, n in enumerate(names)})
    print("iout_g8", names, "->", os.path.relpath(out, REPO))


# ------------------------------------------------------------------ DRX
# The reference's own PF_XRX, NucleationCheckDRX (with Gradient_ExchangeGrainID
# and the GB indicator of src/evolution.c:816-829) and InterpolateGrid, run on
# crafted inputs through oracle/refshim/drx_harness.cc (oracle/_ref/drx_ref),
# one case per process.  File layouts are those documented in the harness.

DRX_REF = os.path.join(REPO, "oracle", "_ref", "drx_ref")
# test_run/input.in's PF constants; stored-energy scale 0.5 and a 500x one
# (a driving force that moves boundaries within a few substeps)
PF_COEF = dict(E_gb=0.625, M_gb=1e-10, mu=48.0, bb=0.256, alpha=0.5, dx=2.5e-6, dt=0.004)
PF_COEF_STRONG = dict(PF_COEF, alpha=1000.0)


def _run_drx_ref(mode, blob, d):
    fi, fo = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
    with open(fi, "wb") as f:
        f.write(blob)
    subprocess.run(["bash", "-c", f"ulimit -s unlimited; {DRX_REF} {mode} in.bin out.bin > ref.log 2>&1"], cwd=d,
                   check=True)
    return open(fo, "rb").read()


def ref_pf(d, dims, gid, rho, steps, coef, init_gid, table):
    """PF_XRX: per-substep (cnt, ids, vals), gID_new, rho_avg table."""
    n = int(np.prod(dims))
    blob = (np.array([*dims, steps, init_gid, len(table), 1], np.int32).tobytes() +
            np.array([coef[k] for k in ("E_gb", "M_gb", "mu", "bb", "alpha", "dx", "dt")], np.float64).tobytes() +
            np.asarray(gid, np.int32).tobytes() + np.asarray(rho, np.float64).tobytes() +
            np.asarray(table, np.float64).tobytes())
    b = _run_drx_ref("pf", blob, d)
    off, subs = 0, []
    for _ in range(steps):
        cnt = np.frombuffer(b, np.int32, n, off); off += 4 * n
        tot = int(np.frombuffer(b, np.int32, 1, off)[0]); off += 4
        ids = np.frombuffer(b, np.int32, tot, off); off += 4 * tot
        val = np.frombuffer(b, np.float64, tot, off); off += 8 * tot
        subs.append((cnt.copy(), ids.copy(), val.copy()))
    gnew = np.frombuffer(b, np.int32, n, off).copy(); off += 4 * n
    tab = np.frombuffer(b, np.float64, len(table), off).copy(); off += 8 * len(table)
    assert off == len(b)
    return subs, gnew, tab


def voronoi(dims, ng, rng):
    pts = rng.uniform(0, 1, size=(ng, 3)) * np.array(dims)
    pos = np.indices(dims).reshape(3, -1).T + 0.5
    best = np.full(pos.shape[0], np.inf)
    g = np.zeros(pos.shape[0], np.int32)
    for k, c in enumerate(pts):
        dd = pos - c
        dd -= np.round(dd / np.array(dims)) * np.array(dims)
        r = (dd ** 2).sum(1)
        m = r < best
        best[m] = r[m]
        g[m] = k + 1
    return g


def pf_cases():
    rng = np.random.default_rng(2024)
    dims = (10, 10, 10)
    ix = np.indices(dims)
    cases = {}
    for ax, nm in ((0, "x"), (2, "z")):
        g = np.where(ix[ax] < 5, 1, 2).astype(np.int32).ravel()
        cases[f"pf_bicrystal_{nm}"] = (dims, g, np.where(g == 1, 100.0, 600.0), 8, PF_COEF, 2)
    r2 = ((ix - 5) ** 2).sum(0).ravel()
    g = np.where(r2 <= 9, 2, 1).astype(np.int32)
    cases["pf_nucleus"] = (dims, g, np.where(g == 1, 600.0, 1.0), 8, PF_COEF, 1)
    cases["pf_nucleus_growing"] = (dims, g, np.where(g == 1, 600.0, 1.0), 10, PF_COEF_STRONG, 1)
    g = np.ones(dims, np.int32)
    g[ix[0] >= 5] = 2
    g[(ix[0] < 5) & (ix[1] >= 5)] = 3
    g = g.ravel()
    cases["pf_triple"] = (dims, g, np.array([0.0, 100.0, 300.0, 600.0])[g], 8, PF_COEF, 3)
    d2 = (12, 10, 8)
    g = voronoi(d2, 9, rng)
    cases["pf_voronoi"] = (d2, g, rng.uniform(50.0, 600.0, g.size), 10, PF_COEF_STRONG, 5)
    return cases


def main_drx():
    subprocess.check_call([os.path.join(REPO, "oracle", "build_ref.sh")])
    d = "/tmp/mth_golden_drx"
    os.makedirs(d, exist_ok=True)
    for name, (dims, g, rho, steps, coef, init_gid) in pf_cases().items():
        table = np.zeros(int(g.max()) + 1)
        subs, gnew, tab = ref_pf(d, dims, g, rho, steps, coef, init_gid, table)
        extra = {}
        if name == "pf_voronoi":   # a second call on the relaxed map, with the table the first one left
            rho2 = np.where(gnew > init_gid, 1.0, rho)
            subs2, gnew2, tab2 = ref_pf(d, dims, gnew, rho2, 4, coef, init_gid, tab)
            extra = dict(rho2=rho2, gnew2=gnew2, table2=tab2, cnt2=subs2[-1][0], ids2=subs2[-1][1], val2=subs2[-1][2])
        out = os.path.join(HERE, name + ".npz")
        np.savez_compressed(out, dims=np.array(dims), grain=g, rho=rho, steps=steps, init_gid=init_gid,
                            coef=json.dumps(coef), gnew=gnew, table=tab,
                            cnt=np.concatenate([s[0] for s in subs]), ntot=np.array([len(s[1]) for s in subs]),
                            ids=np.concatenate([s[1] for s in subs]), val=np.concatenate([s[2] for s in subs]),
                            **extra)
        print(name, "substeps", steps, "entries", [len(s[1]) for s in subs], "->", os.path.relpath(out, REPO))
    # nucleation: static branch (threshold kappa_drx), nucleus_radius compared with |d|^2
    rng = np.random.default_rng(77)
    for name, dims, ng, kap, rad in (("nucl_voronoi", (10, 9, 8), 7, 47.0, 4), ("nucl_edges", (8, 8, 8), 5, 48.0, 2)):
        n = int(np.prod(dims))
        g = voronoi(dims, ng, rng)
        phase = np.ones(n, np.int32)
        phase[rng.uniform(size=n) < 0.05] = 2
        rs = rng.uniform(0.0, 600.0, n)
        kappa = np.full(n, kap)
        rot = np.stack([_rand_rot(rng) for _ in range(ng)])[g - 1].reshape(n, 9)
        blob = (np.array([*dims, ng, rad, 3], np.int32).tobytes() + g.tobytes() + phase.tobytes() + rs.tobytes() +
                kappa.tobytes() + rot.tobytes())
        b = _run_drx_ref("nucl", blob, d)
        nn = int(np.frombuffer(b, np.int32, 1, 0)[0])
        off = 4
        gout = np.frombuffer(b, np.int32, n, off).copy(); off += 4 * n
        gb = np.frombuffer(b, np.int32, n, off).copy(); off += 4 * n
        diff = np.frombuffer(b, np.float64, n, off).copy(); off += 8 * n
        rec = np.frombuffer(b, np.dtype([("id", "<i4"), ("t1", "<f8"), ("Phi", "<f8"), ("t2", "<f8")]), nn, off)
        out = os.path.join(HERE, name + ".npz")
        np.savez_compressed(out, dims=np.array(dims), grain=g, phase=phase, rho_s0=rs, kappa=kap, radius=rad,
                            n_grains=ng, rot=rot, n_new=nn, grain_out=gout, gb=gb, diff_rho=diff,
                            new_id=rec["id"].copy(), new_euler_deg=np.stack([rec["t1"], rec["Phi"], rec["t2"]], 1))
        print(name, "nuclei", nn, "->", os.path.relpath(out, REPO))
    # grid transfer, integer refinement in x (InterpolateGrid's slab rule)
    for name, ns, nd in (("interp_refine", (8, 8, 8), (16, 12, 10)), ("interp_mixed", (6, 9, 12), (18, 6, 8))):
        n, npf = int(np.prod(ns)), int(np.prod(nd))
        g = rng.integers(1, 40, n).astype(np.int32)
        rt = rng.uniform(0.0, 700.0, n)
        b = _run_drx_ref("interp", np.array([*ns, *nd], np.int32).tobytes() + g.tobytes() + rt.tobytes(), d)
        gpf = np.frombuffer(b, np.int32, npf, 0).copy()
        rpf = np.frombuffer(b, np.float64, npf, 4 * npf).copy()
        out = os.path.join(HERE, name + ".npz")
        np.savez_compressed(out, ns=np.array(ns), nd=np.array(nd), grain=g, rho=rt, grain_pf=gpf, rho_pf=rpf)
        print(name, ns, "->", nd, "->", os.path.relpath(out, REPO))


# Update_microstructure (src/integrated.c:801-1807) over crafted sequences of
# relaxed grain maps on a 10^3 grid of three deformed x slabs (ids 1-3,
# init_gid 3): the grain map and the membership counters after each call.
# The reference resets the voxels whose counter `growth` is 1 after the call
# (src/evolution.c:1132-1145).
def upd_sequences():
    dims = (10, 10, 10)
    X, Y, Z = np.meshgrid(*[np.arange(d) for d in dims], indexing="ij")
    base = np.where(X < 4, 1, np.where(X < 7, 2, 3)).astype(np.int32).ravel()

    def box(x0, x1, y0, y1, z0, z1):
        return ((X >= x0) & (X < x1) & (Y >= y0) & (Y < y1) & (Z >= z0) & (Z < z1)).ravel()

    zero = np.zeros(base.size, np.int32)
    seq = {}
    # one recrystallised grain: painted, grows, grows by 16 %, by one voxel
    # (under 1 %: rolled back), then by 19 voxels
    paint = np.where(box(2, 5, 4, 7, 4, 7), 4, 0).astype(np.int32)
    g0 = np.where(box(1, 6, 3, 8, 3, 8), 4, base).astype(np.int32)
    g1 = np.where(box(1, 6, 3, 8, 3, 9), 4, g0).astype(np.int32)
    g2 = g1.copy()
    g2[np.flatnonzero((g1 != 4) & box(6, 7, 3, 4, 3, 4))[:1]] = 4
    g3 = np.where(box(6, 7, 3, 8, 3, 7), 4, g2).astype(np.int32)
    seq["upd_growth_rollback"] = ([1, 2, 3, 4], [(paint, g0), (zero, g1), (zero, g2), (zero, g3)])
    # two recrystallised grains: voxels of the older (4) go to the younger
    # (5), voxels of the younger go to the older, and some go back to a
    # deformed grain
    p4 = np.where(box(1, 3, 1, 3, 1, 3), 4, 0)
    p5 = np.where(box(6, 8, 6, 8, 6, 8), 5, 0)
    paint = (p4 + p5).astype(np.int32)
    h0 = np.where(box(0, 4, 0, 4, 0, 4), 4, np.where(box(5, 9, 5, 9, 5, 9), 5, base)).astype(np.int32)
    h1 = h0.copy()
    h1[box(3, 4, 0, 4, 0, 4)] = 5          # older -> younger
    h1[box(5, 6, 5, 9, 5, 9)] = 4          # younger -> older
    h1[box(0, 1, 0, 4, 0, 1)] = 1          # recrystallised -> deformed
    h2 = np.where(box(0, 4, 4, 6, 0, 4), 4, h1).astype(np.int32)
    seq["upd_two_grains"] = ([1, 2, 3, 4, 5], [(paint, h0), (zero, h1), (zero, h2)])
    return dims, base, seq


def main_upd():
    exe = os.path.join(REPO, "oracle", "_ref", "drx_ref")
    d = "/tmp/mth_golden_upd"
    os.makedirs(d, exist_ok=True)
    dims, base, seq = upd_sequences()
    n = int(np.prod(dims))
    for name, (ids, calls) in seq.items():
        blob = np.array([*dims, len(ids), len(calls)], np.int32).tobytes() + np.array(ids, np.int32).tobytes()
        blob += base.tobytes() + np.zeros(n, np.int32).tobytes() + np.zeros(n, np.int32).tobytes()
        for paint, gnew in calls:
            blob += paint.astype(np.int32).tobytes() + gnew.astype(np.int32).tobytes()
        fin, fout = os.path.join(d, name + ".in"), os.path.join(d, name + ".out")
        open(fin, "wb").write(blob)
        subprocess.check_call([exe, "upd", fin, fout], stdout=subprocess.DEVNULL)
        out = np.fromfile(fout, np.int32).reshape(len(calls), 3, n)
        dst = os.path.join(HERE, name + ".npz")
        np.savez_compressed(dst, dims=np.array(dims), ids=np.array(ids), base=base,
                            paint=np.stack([c[0] for c in calls]), gnew=np.stack([c[1] for c in calls]),
                            grain=out[:, 0], gid_rex=out[:, 1], growth=out[:, 2])
        print(name, "reset per call", [(out[k, 2] == 1).sum() for k in range(len(calls))], "->",
              os.path.relpath(dst, REPO))


def _rand_rot(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


if __name__ == "__main__":
    which = sys.argv[1:] or ["evp", "dd", "test_run", "drx", "upd", "configs", "rve128", "iout"]
    if "evp" in which:
        main()
    if "dd" in which:
        main_dd()
    if "test_run" in which:
        main_test_run()
    if "drx" in which:
        main_drx()
    if "upd" in which:
        main_upd()
    if "configs" in which:
        main_configs()
    if "rve128" in which:
        main_rve128()
    if "iout" in which:
        main_iout()

#!/usr/bin/env python3
"""Benchmark of the EVPFFT Green iteration on GB300.

Metric: voxel-iterations/s = voxels x Green iterations / time, on the
128^3 workload (512 periodic Voronoi grains, uniform SO(3) orientations, 40
non-overlapping radius-3 pores as gas, FCC Cu power law n=10 with Voce
hardening, uniaxial tension eps33_dot = 1/s with stress-free lateral mixed
boundary conditions, dt = 1e-3, IterMax 100 Green iterations per step).  A
"step" is one mechanical step.  Inputs are seeded synthetic data of those
shapes (the reference ships no dataset).  The fields (~0.5 GB in mixed
precision) are larger than L2, so no L2 flush is done between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]

--impl reference times the CPU implementation of the same path: the oracle
(a C restatement of the reference's algorithm, oracle/evpfft_oracle.c) on
all host cores, one Green iteration of the same workload per step.  The
reference's own build needs its sources, which do not travel with the repo.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "m-themes_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))

import numpy as np  # noqa: E402

METRIC = "voxel-iterations/s at 128³: mixed vs FP64 GPU at ≤1e-4 rel stress error"
UNIT = "voxel-iterations/s"
THROTTLE_BAD = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gpu", "reference"], default="gpu")
    ap.add_argument("--precision", choices=["mixed", "fp64", "mixed_fast", "mixed_root64"], default="mixed")
    ap.add_argument("--workload", default="rve128")
    ap.add_argument("--iter-max", type=int, default=0, help="override IterMax (default: the workload's 100)")
    ap.add_argument("--err", type=float, default=0.0, help="override Err (calib64_fd only; default: the workload's 1e-5)")
    ap.add_argument("--fd-steps", type=int, default=0, help="override the mechanical steps (calib64_fd only; default 50)")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 comparison run")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint calibration measurement")
    ap.add_argument("--no-dd", action="store_true", help="skip the dislocation-density law measurement")
    ap.add_argument("--no-drx", action="store_true", help="skip the coupled recrystallisation measurement")
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-RVE batch measurement")
    return ap.parse_args()


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi samples every 200 ms during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                          "-i", str(self.index), "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"),
                                 f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# --------------------------------------------------------------- helpers
def measured_peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def fp64_peak_tflops(dev):
    """FP64 throughput of this GPU, measured here: cuBLAS DGEMM
    (torch.matmul in float64, 4096^3, best of 5 after 2 warm-up calls, CUDA
    events on the current stream), in TFLOP/s."""
    import torch
    n = 4096
    g = torch.Generator(device=dev).manual_seed(0)
    a = torch.randn(n, n, dtype=torch.float64, device=dev, generator=g)
    b = torch.randn(n, n, dtype=torch.float64, device=dev, generator=g)
    for _ in range(2):
        torch.matmul(a, b)
    best = None
    for _ in range(5):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        t = e0.elapsed_time(e1)
        best = t if best is None else min(best, t)
    del a, b
    return 2.0 * n ** 3 / (best / 1e3) / 1e12


# FP64 flops of the mixed mode's Jacobian solve per local Newton step, counted
# algorithmically (a fused multiply-add is two flops, a reciprocal one): the
# LDL^T factorisation of the 5x5 Hessian (20 + 20 from the two update sums, 10
# scalings, 5 pivot reciprocals) and the two triangular solves (20 + 25)
SOLVE_FP64_FLOPS = 100


def traffic_per_launch(kernel):
    """DRAM bytes per launch of a kernel from the committed ncu summary,
    scaled to the 128^3 workload (profiles/traffic.json), or None."""
    p = os.path.join(REPO, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    v = d.get(kernel)
    return None if v is None else float(v)


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    lrank = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, lrank


def workload_cfg(args):
    from mth import synth
    cfg = synth.workload(args.workload)
    if args.iter_max:
        cfg.iter_max = args.iter_max
    return cfg


def describe(cfg):
    """(data, workload) strings of a synth.Config."""
    g = "x".join(str(n) for n in cfg.cell_dim)
    pores = ", %d radius-%d pores" % (cfg.n_pores, cfg.pore_radius) if cfg.n_pores else ""
    data = "synthetic: seeded periodic Voronoi, %d grains, uniform SO(3) orientations%s" % (cfg.n_grains, pores)
    e = cfg.velgrad_bc[2]
    load = "uniaxial %s eps33_dot=%g/s" % ("tension" if e > 0 else "compression", e)
    m = cfg.material
    wl = "%s RVE, %d grains%s, FCC Cu power law n=%g + Voce, %s, dt=%g, IterMax=%d" % (
        g, cfg.n_grains, pores, m.nrs, load, cfg.time_step, cfg.iter_max)
    if cfg.drx is not None:
        from mth import capi
        wl += ", coupled DRX (%d PF substeps, K=%d)" % (cfg.drx.pf_substeps, capi.PF_K)
    return data, wl


# ------------------------------------------------------------ GPU arm
def run_gpu(args):
    import torch
    from mth import Solver, capi, synth
    ws, rank, lrank = dist_init()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(lrank)
        dist.init_process_group("nccl")
    dev_index = lrank if ws > 1 else 0
    from mth import replicas
    cfg = replicas.replica_config(workload_cfg(args), rank)   # replicas: each rank its own RVE
    grain, phase, euler = synth.microstructure(cfg)
    nv = int(np.prod(cfg.cell_dim))
    prec = {"mixed": capi.MTH_MIXED, "fp64": capi.MTH_FP64, "mixed_fast": capi.MTH_MIXED_FAST,
            "mixed_root64": capi.MTH_MIXED_ROOT64}[args.precision]

    def barrier_sync():
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    def reduce_max(x):
        if ws == 1:
            return x
        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        return float(t.item())

    def reduce_sum(x):
        if ws == 1:
            return x
        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        torch.distributed.all_reduce(t)
        return float(t.item())

    def timed_run(precision, steps, warmup, profile=False, clocks=False):
        par = capi.params_from_config(cfg, precision=precision)
        par.device = dev_index
        s = Solver(par, grain, phase, euler)
        for _ in range(warmup):
            s.step()
        s.profile(enable=profile, reset=True)
        barrier_sync()
        cs = ClockSampler(dev_index) if clocks else None
        if cs:
            cs.start()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        reps = [s.step() for _ in range(steps)]
        e1.record()
        barrier_sync()
        ms = e0.elapsed_time(e1)
        clk = cs.stop() if cs else None
        prof, launches = s.profile(reset=True)
        iters = sum(r["iterations"] for r in reps)
        s.close()
        return ms, iters, reps, prof, launches, clk

    # main (device-resident) measurement, without the library's per-launch
    # events; then the same steps again with them, for the kernel table and
    # the roofline (the events sit between the kernels and cost time)
    ms, iters, reps, _, _, clk = timed_run(prec, args.steps, args.warmup, clocks=True)
    ms_prof, iters_prof, reps_prof, prof, launches, _ = timed_run(prec, args.steps, args.warmup, profile=True)
    ms_max = reduce_max(ms)
    vox_it = reduce_sum(float(nv) * iters)
    value = vox_it / (ms_max / 1e3)

    fb = nv * 55 * (8 if prec == capi.MTH_FP64 else 4) / 1e9   # field planes + half spectra
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": {capi.MTH_MIXED: "f32 fields + f64 Newton solve", capi.MTH_FP64: "f64",
                     capi.MTH_MIXED_FAST: "f32", capi.MTH_MIXED_ROOT64: "f32 fields + f64 Newton solve near the root"}[prec],
           "data": describe(cfg)[0],
           "config": {"workload": describe(cfg)[1],
                      "grid": list(cfg.cell_dim), "voxels": nv, "green_iterations": iters,
                      "precision": args.precision, "parallelism": "replicas" if ws > 1 else "single GPU",
                      "l2": ("fields (%.2f GB) larger than the 129 MB L2; no flush" % fb if fb > 0.129 else
                             "fields (%.3f GB) fit in the 129 MB L2: a profiling case, not an HBM measurement" % fb)}}

    # roofline of the dominant kernel (device time from CUDA events on the library stream)
    dom = max(((k, v) for k, v in prof.items() if v["bytes"] > 0), key=lambda kv: kv[1]["ms"])
    dname, d = dom
    peak, peak_kind = measured_peaks()
    per_launch_s = (d["ms"] / 1e3) / max(d["launches"], 1)
    per_launch_bytes = d["bytes"] / max(d["launches"], 1)
    achieved = per_launch_bytes / per_launch_s / 1e9
    tr = traffic_per_launch(dname)
    out["roofline"] = {"bound": "hbm", "kernel": dname, "achieved": achieved, "peak": peak, "unit": "GB/s",
                       "frac": achieved / peak, "peak_source": peak_kind, "traffic": tr,
                       "algorithmic_bytes_per_launch": per_launch_bytes, "ms_per_launch": per_launch_s * 1e3,
                       "note": "the local Newton is ALU-bound (FP64 solve, FP32 flow rule); its HBM fraction is low "
                               "by construction"}
    if prec == capi.MTH_MIXED and dname == "newton":
        # the local Newton is bound by GB300's FP64 pipe: its FP64 solve flops
        # against the FP64 throughput measured in this run
        p64 = fp64_peak_tflops("cuda:%d" % dev_index)
        steps = float(sum(r["newton_iters"] for r in reps_prof))
        a64 = SOLVE_FP64_FLOPS * steps / (d["ms"] / 1e3) / 1e12
        out["roofline"]["fp64"] = {"achieved": a64, "peak": p64, "unit": "TFLOP/s", "frac": a64 / p64,
                                   "peak_source": "cuBLAS DGEMM 4096^3 measured in this run",
                                   "flops_per_newton_step": SOLVE_FP64_FLOPS, "newton_steps": steps,
                                   "note": "algorithmic FP64 flops of the Jacobian solves; the kernel also "
                                           "runs the FP32 flow rule, residual and Hessian assembly"}
    tot_ms = sum(v["ms"] for v in prof.values())
    out["kernels"] = {k: {"ms": round(v["ms"], 3), "share": round(v["ms"] / tot_ms, 4) if tot_ms else None,
                          "launches": v["launches"],
                          "gbs": (v["bytes"] / (v["ms"] / 1e3) / 1e9) if v["ms"] > 0 else None,
                          "hbm_frac": ((v["bytes"] / (v["ms"] / 1e3) / 1e9) / peak) if v["ms"] > 0 else None}
                      for k, v in prof.items() if v["launches"]}
    out["gpu_launches"] = launches
    out["profiled_run"] = {"ms_per_step": reduce_max(ms_prof) / args.steps, "green_iterations": iters_prof,
                           "note": "the same steps with the library's per-launch CUDA events, which give kernels, "
                                   "roofline and gpu_launches"}
    out["clocks"] = clk
    nvc = float(nv) * (1.0 - float(np.mean(phase == 2)))   # crystal voxels
    out["newton_iterations_per_voxel_solve"] = float(sum(r["newton_iters"] for r in reps)) / (nvc * iters)

    # FP64 comparison: same warm-up and steps, last-step macroscopic stress
    if not args.no_fp64 and prec == capi.MTH_MIXED:
        ms64, it64, reps64, _, _, _ = timed_run(capi.MTH_FP64, args.steps, args.warmup)
        ms64 = reduce_max(ms64)
        v64 = reduce_sum(float(nv) * it64) / (ms64 / 1e3)
        a, b = reps[-1]["sig_avg"], reps64[-1]["sig_avg"]
        err = float(np.abs(a - b).max() / np.abs(b).max())
        out["fp64"] = {"value": v64, "ms_per_step": ms64 / args.steps, "green_iterations": it64}
        out["mixed_over_fp64"] = value / v64
        out["rel_stress_err_vs_fp64"] = err
        # opt-in variant with the 5x5 Jacobian solve in FP32 as well
        msf, itf, repsf, _, _, _ = timed_run(capi.MTH_MIXED_FAST, args.steps, args.warmup)
        msf = reduce_max(msf)
        vf = reduce_sum(float(nv) * itf) / (msf / 1e3)
        ef = float(np.abs(repsf[-1]["sig_avg"] - b).max() / np.abs(b).max())
        out["mixed_fast"] = {"value": vf, "ms_per_step": msf / args.steps, "rel_stress_err_vs_fp64": ef,
                             "note": "MTH_MIXED_FAST: Jacobian solve in FP32 too"}
        # opt-in variant with the FP64 solve only near the root
        msr, itr, repsr, _, _, _ = timed_run(capi.MTH_MIXED_ROOT64, args.steps, args.warmup)
        msr = reduce_max(msr)
        vr = reduce_sum(float(nv) * itr) / (msr / 1e3)
        er = float(np.abs(repsr[-1]["sig_avg"] - b).max() / np.abs(b).max())
        out["mixed_root64"] = {"value": vr, "ms_per_step": msr / args.steps, "rel_stress_err_vs_fp64": er,
                               "note": "MTH_MIXED_ROOT64: FP64 Jacobian solve only within 1e-3|lambda| of the root"}

    # end to end through the C-ABI with host buffers: create + upload (H2D of
    # the microstructure from pinned memory), K steps each returning the
    # report and the full stress field to the host
    if not args.no_e2e:
        import ctypes as C
        lib = capi.load()
        pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()  # noqa: E731
        g_h, p_h, e_h = pin(grain), pin(phase), pin(euler)
        sig_h = torch.empty(9 * nv, dtype=torch.float64).pin_memory().numpy()
        par = capi.params_from_config(cfg, precision=prec)
        par.device = dev_index
        barrier_sync()
        t0 = time.perf_counter()
        ctx = C.c_void_p()
        capi.check(lib, lib.mth_create(C.byref(par), C.byref(ctx)))
        capi.check(lib, lib.mth_upload_microstructure(ctx, capi._iptr(g_h), capi._iptr(p_h), capi._dptr(e_h), nv))
        rep = capi.MthStepReport()
        it_e2e = 0
        for _ in range(args.steps):
            capi.check(lib, lib.mth_step(ctx, C.byref(rep)))
            it_e2e += rep.iterations
            capi.check(lib, lib.mth_download_field(ctx, 0, capi._dptr(sig_h), sig_h.size))
        barrier_sync()
        dt = time.perf_counter() - t0
        lib.mth_destroy(ctx)
        dt = reduce_max(dt)
        h2d = (g_h.nbytes + p_h.nbytes + e_h.nbytes) / args.steps
        out["e2e"] = {"value": reduce_sum(float(nv) * it_e2e) / dt, "unit": UNIT,
                      "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(sig_h.nbytes + C.sizeof(rep)),
                      "note": "create + microstructure upload amortised over the steps; the stress field is "
                              "returned to the host after every step"}

    if rank == 0 and not args.no_cpu:
        out["cpu_baseline"] = cpu_sample(cfg)
    if not args.no_adjoint and args.workload == "rve128":
        out["adjoint"] = adjoint_measure(dev_index)
    if not args.no_dd and args.workload == "rve128":
        out["dislocation_density"] = dd_measure(dev_index, args)
    if not args.no_drx and args.workload == "rve128":
        out["drx"] = drx_measure(dev_index, args)
    if not args.no_batch and args.workload == "rve128" and ws == 1:
        out["batch"] = batch_measure(dev_index)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


# ------------------------------------------------- dislocation-density law
def dd_measure(dev_index, args):
    """The same 128^3 workload with the reference's shipped dislocation-density
    law instead of the power law + Voce (flow_law = 1, mixed precision):
    voxel-iterations/s over the timed steps, with the per-step density
    update (SSD/GND evolution and averages) inside the timed region."""
    import dataclasses
    import torch
    from mth import Solver, capi, synth
    cfg = dataclasses.replace(synth.workload("rve128"), dd=synth.DD())
    par = capi.params_from_config(cfg, precision=capi.MTH_MIXED)
    par.device = dev_index
    nv = int(np.prod(cfg.cell_dim))
    with Solver(par, *synth.microstructure(cfg)) as s:
        for _ in range(2):
            s.step()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        its = 0
        reps = []
        for _ in range(max(2, args.steps // 2)):
            r = s.step()
            its += r["iterations"]
            reps.append(r)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
    return {"workload": "128x128x128 RVE, 512 grains, 40 radius-3 pores, dislocation-density law (sinh slip, "
                        "SSD + first-order GND evolution), tension eps33_dot=1/s, dt=0.001, IterMax=100, mixed",
            "value": nv * its / dt, "unit": UNIT, "ms_per_step": dt * 1e3 / len(reps), "green_iterations": its,
            "dd_avg_last_step": [float(x) for x in reps[-1]["dd_avg"]]}


# ------------------------------------------- coupled recrystallisation (drx128)
def drx_measure(dev_index, args):
    """The coupled EVPFFT + sparse phase-field workload at 128^3 (1000 grains,
    compression, 10 PF substeps per mechanical step, nucleation every step
    from the second on), mixed precision: timed mechanical steps with the
    whole DRX step (density, nucleation, phase field, grain adoption, new
    reference medium) inside the timed region, after two warm-up steps."""
    import torch
    from mth import Solver, capi, synth
    cfg = synth.workload("drx128_each")
    par = capi.params_from_config(cfg, precision=capi.MTH_MIXED)
    par.device = dev_index
    nv = int(np.prod(cfg.cell_dim))
    nsteps = 3
    with Solver(par, *synth.microstructure(cfg)) as s:
        for _ in range(2):
            s.step()
        s.profile(enable=True, reset=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        reps = [s.step() for _ in range(nsteps)]
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        prof, launches = s.profile(reset=True)
        grains = s.field("grain")
    its = sum(r["iterations"] for r in reps)
    pf = prof.get("pf_relax", {"ms": 0.0, "bytes": 0.0, "launches": 0})
    sub = nsteps * cfg.drx.pf_substeps
    peak, _ = measured_peaks()
    pf_gbs = pf["bytes"] / (pf["ms"] / 1e3) / 1e9 if pf["ms"] > 0 else None
    return {"workload": "128x128x128 RVE, 1000 grains, compression eps33_dot=-1/s, dt=0.001, IterMax=100, "
                        "coupled DRX: 10 PF substeps per step, nucleation every step, mixed precision",
            "value": nv * its / dt, "unit": UNIT, "ms_per_step": dt * 1e3 / nsteps, "green_iterations": its,
            "nuclei_per_step": [r["n_new_grains"] for r in reps], "recrystallised_voxels": int((grains > 1000).sum()),
            "pf_ms_per_mechanical_step": pf["ms"] / nsteps, "pf_substeps_per_s": sub / (pf["ms"] / 1e3) if pf["ms"] else None,
            "pf_voxel_substeps_per_s": nv * sub / (pf["ms"] / 1e3) if pf["ms"] else None,
            "pf_bytes_per_voxel_substep": pf["bytes"] / (nv * sub) if sub else None,
            "pf_gbs": pf_gbs, "pf_hbm_frac": pf_gbs / peak if pf_gbs else None, "pf_launches": pf["launches"],
            "kernels": {k: {"ms": round(v["ms"], 3), "launches": v["launches"]} for k, v in prof.items() if v["launches"]},
            "gpu_launches": launches}


# ------------------------------------------------------ calibration adjoint
def adjoint_measure(dev_index, name="calib64"):
    """Cost of the calibration gradient (mth_adjoint: forward sweep with
    stored states every 10 steps, recomputation, reverse sweep) against a
    plain forward run of the same 64^3 / 256-grain, 50-step tension, mixed
    precision with the FP64 Jacobian solve.  The target curve comes from the
    forward model at tau0 = 18, thet0 = 280, tau1 = 160, n = 12."""
    import dataclasses
    import torch
    from mth import Solver, capi, synth
    cfg = synth.workload(name)
    micro = synth.microstructure(cfg)

    def params(c):
        p = capi.params_from_config(c, precision=capi.MTH_MIXED)
        p.device = dev_index
        return p

    tcfg = dataclasses.replace(cfg, material=synth.calibration_target_material())
    with Solver(params(tcfg), *micro) as s:
        target = np.array([s.step()["sig_avg"][2][2] for _ in range(cfg.n_steps)])
    with Solver(params(cfg), *micro) as s:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        its = 0
        for _ in range(cfg.n_steps):
            its += s.step()["iterations"]
        torch.cuda.synchronize()
        fwd_ms = (time.perf_counter() - t0) * 1e3
    with Solver(params(cfg), *micro) as s:
        J, g, s33, info = s.adjoint(target, checkpoint_every=10)
    with Solver(params(cfg), *micro) as s:   # again with per-kernel events, for the breakdown only
        s.profile(enable=True)
        s.adjoint(target, checkpoint_every=10)
        prof, launches = s.profile()
    grad_ms = info["forward_ms"] + info["reverse_ms"]
    classes = {k: {"ms": round(v["ms"], 3), "launches": v["launches"],
                   "gbs": (v["bytes"] / (v["ms"] * 1e-3) / 1e9) if v["ms"] > 0 else None}
               for k, v in prof.items() if v["launches"]}
    return {"workload": "64x64x64 RVE, 256 grains, tension eps33_dot=1/s, 50 steps of 1e-3, mixed precision, "
                        "misfit of <sigma_33> against the curve of (tau0, thet0, tau1, n) = (18, 280, 160, 12)",
            "forward_ms": fwd_ms, "green_iterations": its, "gradient_ms": grad_ms,
            "gradient_over_forward": grad_ms / fwd_ms, "reverse_over_forward": info["reverse_ms"] / fwd_ms,
            "checkpoint_every": 10, "recomputed_steps": info["recomputed_steps"],
            "cg_iterations": info["cg_iterations"], "cg_iterations_max_step": info["cg_iterations_max"],
            "misfit": J, "grad": dict(zip(capi.ADJOINT_PARAMS, g.tolist())),
            "kernels_during_gradient": classes, "gpu_launches_during_gradient": launches}


def adjoint_fd_check(dev_index, err=None, iter_max=None, n_steps=None):
    """The calibration gradient of the 64^3 calibration workload (256 grains, 50 steps)
    against central finite differences with relative step 1e-4 of the FP64
    forward, for all five parameters: the FP64 adjoint and the mixed one.
    err / iter_max override the workload's Err 1e-5 / IterMax 100 (the
    adjoint is that of the converged fixed point; the finite differences see
    the forward as it stops)."""
    import dataclasses
    from mth import Solver, capi, synth
    cfg = synth.workload("calib64")
    if err is not None:
        cfg = dataclasses.replace(cfg, err=err)
    if iter_max is not None:
        cfg = dataclasses.replace(cfg, iter_max=iter_max)
    if n_steps is not None:
        cfg = dataclasses.replace(cfg, n_steps=n_steps)
    micro = synth.microstructure(cfg)

    def params(c, prec):
        p = capi.params_from_config(c, precision=prec)
        p.device = dev_index
        return p

    def forward(c, prec):
        with Solver(params(c, prec), *micro) as s:
            reps = [s.step() for _ in range(c.n_steps)]
        return np.array([r["sig_avg"][2][2] for r in reps]), sum(r["iterations"] for r in reps)

    t0 = time.perf_counter()
    target, _ = forward(dataclasses.replace(cfg, material=synth.calibration_target_material()), capi.MTH_FP64)
    base = cfg.material
    out = {"workload": "64x64x64 RVE, 256 grains, tension, %d steps of 1e-3, Err %g, IterMax %d" % (
               cfg.n_steps, cfg.err, cfg.iter_max),
           "params": list(capi.ADJOINT_PARAMS)}
    grads = {}
    for name, prec in (("fp64", capi.MTH_FP64), ("mixed", capi.MTH_MIXED)):
        with Solver(params(cfg, prec), *micro) as s:
            J, g, s33, info = s.adjoint(target, checkpoint_every=10)
        grads[name] = np.asarray(g)
        out["adjoint_" + name] = {"misfit": J, "grad": [float(x) for x in g]}
    vals = synth.calibration_values(base)
    fd, its = [], 0
    for k in range(5):
        h = 1e-4 * vals[k]
        sp, ip = forward(dataclasses.replace(cfg, material=synth.perturb_material(base, k, h)), capi.MTH_FP64)
        sm, im = forward(dataclasses.replace(cfg, material=synth.perturb_material(base, k, -h)), capi.MTH_FP64)
        its += ip + im
        fd.append((np.sum((sp - target) ** 2) - np.sum((sm - target) ** 2)) / (2 * h))
    fd = np.array(fd)
    out["central_fd_fp64"] = [float(x) for x in fd]
    out["rel_err_fp64_adjoint_vs_fd"] = [float(abs(a - b) / abs(b)) for a, b in zip(grads["fp64"], fd)]
    out["rel_err_mixed_adjoint_vs_fd"] = [float(abs(a - b) / abs(b)) for a, b in zip(grads["mixed"], fd)]
    out["rel_err_mixed_vs_fp64_adjoint"] = [float(abs(a - b) / abs(b)) for a, b in zip(grads["mixed"], grads["fp64"])]
    out["fd_green_iterations_per_forward"] = its / 10
    out["seconds"] = time.perf_counter() - t0
    return out


# ------------------------------------------------------------ CPU (oracle)
def cpu_sample(cfg, iterations=1):
    """Oracle (C port of the reference algorithm, OpenMP over all host cores)
    on one mechanical step limited to `iterations` Green iterations of the
    full 128^3 workload."""
    import pyoracle
    from mth import capi, synth
    c = synth.Config(**{**cfg.__dict__})
    c.iter_max = iterations
    grain, phase, euler = synth.microstructure(c)
    cores = os.cpu_count() or 1
    o = pyoracle.Oracle(capi.params_from_config(c), grain, phase, euler, nthreads=cores)
    t0 = time.perf_counter()
    r = o.step()
    dt = time.perf_counter() - t0
    o.close()
    nv = int(np.prod(c.cell_dim))
    return {"value": nv * r["iterations"] / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "%d Green iteration(s) of mechanical step 0 of the 128^3 workload (%d voxel-iterations), "
                      "%.1f s" % (r["iterations"], nv * r["iterations"], dt)}


def run_reference(args):
    ws, rank, _ = dist_init()
    if rank != 0:
        return
    import pyoracle
    from mth import capi, synth
    cfg = workload_cfg(args)
    c = synth.Config(**{**cfg.__dict__})
    c.iter_max = 1
    grain, phase, euler = synth.microstructure(c)
    cores = os.cpu_count() or 1
    o = pyoracle.Oracle(capi.params_from_config(c), grain, phase, euler, nthreads=cores)
    for _ in range(args.warmup):
        o.step()
    nv = int(np.prod(c.cell_dim))
    t0 = time.perf_counter()
    its = 0
    for _ in range(args.steps):
        its += o.step()["iterations"]
    dt = time.perf_counter() - t0
    o.close()
    value = nv * its / dt
    sample = "one Green iteration per step of the 128^3 workload (%d voxel-iterations per step)" % nv
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "impl": "reference",
           "data": describe(c)[0],
           "config": {"workload": describe(cfg)[1] + " (one Green iteration per step timed)", "grid": list(c.cell_dim),
                      "parallelism": "OpenMP %d threads" % cores},
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def batch_measure(dev_index, steps=2, warmup=3):
    """The 64-RVE batch (the batch64 workload) on this GPU, mixed precision:
    whole-batch voxel-iterations/s over `steps` mechanical steps after
    `warmup`, the tile widths the batch chose per grid, and one Solver per
    RVE stepped in turn on the same steps."""
    import torch
    from mth import Batch, Solver, capi, synth
    cfgs = synth.batch_workload("batch64")
    params = [capi.params_from_config(c, precision=capi.MTH_MIXED) for c in cfgs]
    for p in params:
        p.device = dev_index
    micro = [synth.microstructure(c) for c in cfgs]
    nvs = [int(np.prod(c.cell_dim)) for c in cfgs]

    def timed(step_all):
        for _ in range(warmup):
            step_all()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        vi = sum(step_all() for _ in range(steps))
        torch.cuda.synchronize()
        return vi / (time.perf_counter() - t0)

    with Batch(params, micro) as b:
        batched = timed(lambda: sum(n * r["iterations"] for n, r in zip(nvs, b.step())))
        passes = {}
        for i, c in enumerate(cfgs):
            passes.setdefault("x".join(str(n) for n in c.cell_dim), b.passes(i))
    sols = [Solver(p, *m) for p, m in zip(params, micro)]
    try:
        single = timed(lambda: sum(n * s.step()["iterations"] for n, s in zip(nvs, sols)))
    finally:
        for s in sols:
            s.close()
    return {"workload": "64 RVEs (24x32^3, 24x48^3, 16x64^3), per-RVE seed, grains ~U[32,256], tau0 ~U[12,20] "
                        "MPa, n in {8,10,15,20}, tension, dt=1e-3, mixed",
            "value": batched, "unit": UNIT, "steps": steps, "warmup": warmup, "fft_passes": passes,
            "one_solver_per_rve": single, "batched_over_one_solver_per_rve": batched / single}


def run_batch(args):
    """Batched-RVE workload (64 RVEs of 32^3, 48^3 and 64^3 with their own
    seeds, grain counts, tau0 and n): whole-batch voxel-iterations/s over K
    mechanical steps after W warm-up steps, plus the single-Solver-per-RVE
    baseline on the same steps."""
    import torch
    from mth import Batch, Solver, capi, replicas, synth
    ws, rank, lrank = dist_init()
    if ws > 1:
        # the members are partitioned over the ranks; no data-path collective
        import torch.distributed as dist
        torch.cuda.set_device(lrank)
        dist.init_process_group("nccl")
    dev_index = lrank if ws > 1 else 0
    cfgs_all = synth.batch_workload(args.workload)
    mine = replicas.batch_share([int(np.prod(c.cell_dim)) for c in cfgs_all], rank, ws)
    cfgs = [cfgs_all[i] for i in mine]
    prec = {"mixed": capi.MTH_MIXED, "fp64": capi.MTH_FP64, "mixed_fast": capi.MTH_MIXED_FAST,
            "mixed_root64": capi.MTH_MIXED_ROOT64}[args.precision]
    params = [capi.params_from_config(c, precision=prec) for c in cfgs]
    for p in params:
        p.device = dev_index
    micro = [synth.microstructure(c) for c in cfgs]
    nvs = [int(np.prod(c.cell_dim)) for c in cfgs]
    t0 = time.perf_counter()
    b = Batch(params, micro)
    t_create = time.perf_counter() - t0
    for _ in range(args.warmup):
        b.step()
    cs = ClockSampler(dev_index)
    cs.start()
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    vox_it = 0
    for _ in range(args.steps):
        reps = b.step()
        vox_it += sum(n * r["iterations"] for n, r in zip(nvs, reps))
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    if ws > 1:
        torch.distributed.barrier()
    clk = cs.stop()
    passes = {}
    for i, c in enumerate(cfgs):
        passes.setdefault("x".join(str(n) for n in c.cell_dim), b.passes(i))
    b.close()
    vox_it, dt, value = replicas.aggregate(float(vox_it), dt, device="cuda:%d" % dev_index)
    if rank != 0:
        return
    out = {"metric": "voxel-iterations/s, 64 batched RVEs (24x32^3, 24x48^3, 16x64^3)", "value": value,
           "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": dt * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": {capi.MTH_MIXED: "f32 fields + f64 Newton solve", capi.MTH_FP64: "f64",
                     capi.MTH_MIXED_FAST: "f32", capi.MTH_MIXED_ROOT64: "f32 fields + f64 Newton solve near the root"}[prec],
           "data": "synthetic: per-RVE seeded periodic Voronoi, grains ~U[32,256], uniform SO(3), "
                   "tau0 ~U[12,20] MPa, n in {8,10,15,20}",
           "config": {"workload": "%d RVEs, uniaxial tension, dt=1e-3" % len(cfgs_all), "rves": len(cfgs_all),
                      "voxels": int(sum(np.prod(c.cell_dim) for c in cfgs_all)), "batch_create_s": t_create,
                      "parallelism": ("members dealt over %d ranks by voxel count, one batch per rank, no "
                                      "data-path collective" % ws) if ws > 1 else "single GPU",
                      "timing": "host wall clock around whole batch steps (one graph launch per step + host "
                                "bookkeeping), device synchronised on both sides",
                      "fft_passes": passes},
           "clocks": clk}
    if not args.no_fp64 and ws == 1:
        # one Solver per RVE, stepped one after the other: the unbatched baseline
        sols = [Solver(p, *m) for p, m in zip(params, micro)]
        for _ in range(args.warmup):
            for s in sols:
                s.step()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        vi = 0
        for _ in range(args.steps):
            for n, s in zip(nvs, sols):
                vi += n * s.step()["iterations"]
        torch.cuda.synchronize()
        dts = time.perf_counter() - t0
        for s in sols:
            s.close()
        out["unbatched"] = {"value": vi / dts, "ms_per_step": dts * 1e3 / args.steps,
                            "note": "one Solver per RVE, stepped in turn"}
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload in ("batch64", "batch6"):
        run_batch(args)
    elif args.workload == "calib64":
        # the calibration gradient alone (the adjoint block of the default line)
        print(json.dumps({"workload": "calib64", "adjoint": adjoint_measure(0)}), flush=True)
    elif args.workload == "calib64_fd":
        # the calibration gradient against central finite differences (64^3 calibration workload, all five parameters)
        print(json.dumps({"workload": "calib64_fd", "adjoint_fd": adjoint_fd_check(
            0, err=args.err or None, iter_max=args.iter_max or None, n_steps=args.fd_steps or None)}), flush=True)
    elif args.workload == "dd128":
        # the dislocation-density law alone (the dislocation_density block of the default line)
        print(json.dumps({"workload": "dd128", "dislocation_density": dd_measure(0, args)}), flush=True)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()

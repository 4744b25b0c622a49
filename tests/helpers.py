"""Shared helpers of the test suite: golden fixtures, oracle and GPU runs."""
from __future__ import annotations

import json
import os

import numpy as np

from mth import capi, synth

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
GOLDEN_CASES = sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz") and f.startswith("g"))
# dislocation-density law: the trace rows end with the 7 dd.out averages
DD_GOLDEN_CASES = sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz") and f.startswith("dd"))
T_DD = slice(45, 52)

# trace columns written by the reference hook (oracle/refshim/refshim.cc)
T_ITER, T_SIG, T_DG, T_EPS, T_EDOT = 1, slice(2, 11), slice(11, 20), slice(20, 29), slice(29, 38)
T_SVM, T_SVM1, T_EVM, T_DVM, T_ERRS, T_ERRE = 38, 39, 40, 41, 42, 43


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    d = json.loads(str(z["config"]))
    mat = synth.Material(**d.pop("material"))
    for k in ("cell_dim", "velgrad_bc_flag", "velgrad_bc", "stress_bc_flag", "stress_bc"):
        d[k] = tuple(d[k])
    dd = d.pop("dd", None)
    if dd is not None:
        dd = synth.DD(**{k: (tuple(v) if isinstance(v, list) else v) for k, v in dd.items()})
    cfg = synth.Config(material=mat, dd=dd, **d)
    fields = {k: z[k] for k in z.files if k not in ("config", "trace")}
    return cfg, z["trace"], fields


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    s = max(np.abs(b).max(), 1e-300)
    return float(np.abs(a - b).max() / s)


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def run_oracle(cfg, nthreads=None):
    import pyoracle
    g, p, e = synth.microstructure(cfg)
    o = pyoracle.Oracle(capi.params_from_config(cfg), g, p, e, nthreads=nthreads)
    reps = [o.step() for _ in range(cfg.n_steps)]
    return o, reps


def run_gpu(cfg, precision=capi.MTH_FP64, steps=None, **kw):
    from mth import Solver
    g, p, e = synth.microstructure(cfg)
    s = Solver(capi.params_from_config(cfg, precision=precision, **kw), g, p, e)
    reps = [s.step() for _ in range(cfg.n_steps if steps is None else steps)]
    return s, reps

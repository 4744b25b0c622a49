"""CPU check of the per-iteration bookkeeping of the Green iteration
(m-themes_gb300/csrc/book.cuh, which mth_step runs on the device and the
batch and the adjoint on the host): the header is compiled with the host
compiler (tests/book_check.cpp) and its results on pseudo-random step
constants and reduced sums are compared with a restatement of the
reference's formulas written here: get_smacro (src/evolution.c:473-547:
volume averages, the mixed-boundary strain correction dDisGradAvg, the von
Mises measures, including the out-of-bounds SigDevAvg[3][3] word that holds
SigAvg1[0][0]), the error normalisation (src/evolution.c:1430-1455) and the
next iteration's uniform strain increment (src/evolution.c:1319-1332)."""
import json
import math
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)

R2, R3, R6 = 1.0 / math.sqrt(2.0), 1.0 / math.sqrt(3.0), 1.0 / math.sqrt(6.0)
# Lebensohn-Tome basis B_i (chg_basis, src/kinematics.c:27-53)
B = np.zeros((6, 3, 3))
B[0, 0, 0], B[0, 1, 1] = -R2, R2
B[1, 0, 0], B[1, 1, 1], B[1, 2, 2] = -R6, -R6, 2.0 * R6
B[2, 1, 2] = B[2, 2, 1] = R2
B[3, 0, 2] = B[3, 2, 0] = R2
B[4, 0, 1] = B[4, 1, 0] = R2
B[5, 0, 0] = B[5, 1, 1] = B[5, 2, 2] = R3
IJV = [(0, 0), (1, 1), (2, 2), (1, 2), (0, 2), (0, 1)]


def t2v(t, n=6):
    return np.array([np.sum(t * B[i]) for i in range(n)])


def v2t(v, n=6):
    return sum(v[i] * B[i] for i in range(n))


def expected(c):
    """The reference's bookkeeping of one iteration, from the case's inputs."""
    red = np.array(c["red"])
    if not np.all(np.isfinite(red)):
        return None
    wgt, wgt1 = c["wgt"], c["wgt_ph1"]
    sig = v2t(red[2:8] * wgt)
    sig1 = v2t(red[8:14] * (wgt / wgt1))
    s0 = np.array(c["s0_4"]).reshape(3, 3, 3, 3)
    sc = np.array(c["scauchy"]).reshape(3, 3)
    ddg = np.array(c["ddg0"]).reshape(3, 3).copy()
    for a, (i, j) in enumerate(IJV):
        ddg[i, j] = 0.0
        if c["vbc"][a] == 0:
            ddg[i, j] = sum(s0[i, j, k, l] * c["sbc"][q] * (sc[k, l] - sig[k, l]) for q, (k, l) in enumerate(IJV))
    acum = np.array(c["ddg_acum0"]).reshape(3, 3) + ddg
    dev = v2t(t2v(sig)[:5], 5)
    mean = (dev[1, 1] + dev[2, 2] + sig1[0, 0]) / 3.0      # SigDevAvg[3][3] reads SigAvg1[0][0]
    svm = math.sqrt(1.5 * sum((dev[i, j] - (mean if i == j else 0.0)) ** 2 for i in range(3) for j in range(3)))
    dev1 = v2t(t2v(sig1)[:5], 5)
    svm1 = math.sqrt(1.5 * float(np.sum(dev1 * dev1)))
    err_s = red[0] * wgt / svm
    err_e = 0.0 if abs(c["e_vm"]) < 1e-5 else red[1] * wgt / c["e_vm"]
    out = {"sig_avg": sig, "sig_avg1": sig1, "ddg": ddg, "ddg_acum": acum, "s_vm": svm, "s_vm1": svm1,
           "err_s": err_s, "err_e": err_e, "it_nit": c["it_nit"] + int(red[14]), "it_nbad": c["it_nbad"] + int(red[15])}
    more = c["it_iter"] < c["iter_max"] and max(abs(err_s), abs(err_e)) > c["err"]
    out["more"] = more
    applied = np.array(c["ddg_applied0"]).reshape(3, 3)
    add = np.zeros(6)
    it = c["it_iter"]
    if more:
        it += 1
        u = ddg + (np.array(c["udot"]).reshape(3, 3) * c["dt"] if it == 1 else 0.0)
        applied = applied + ddg
        add = t2v(u)
    out.update({"it_iter": it, "ddg_applied": applied, "add": add})
    return out


def close(a, b, tol=1e-13):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return np.all(np.abs(a - b) <= tol * (np.abs(b).max() + 1e-300))


def test_bookkeeping_matches_the_reference_formulas(tmp_path):
    cxx = shutil.which("g++")
    inc = next((os.path.join(d, "include") for d in (os.environ.get("CUDA_HOME"), "/usr/local/cuda")
                if d and os.path.exists(os.path.join(d, "include", "cuda_runtime.h"))), None)
    if cxx is None or inc is None:
        pytest.skip("needs g++ and the CUDA headers")
    exe = str(tmp_path / "bookchk")
    r = subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I" + inc,
                        "-I" + os.path.join(REPO, "m-themes_gb300", "csrc"), os.path.join(HERE, "book_check.cpp"),
                        "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    cases = [json.loads(line) for line in r.stdout.splitlines() if line.strip()]
    assert len(cases) == 12
    seen = {"nan": 0, "err_e0": 0, "stop": 0, "first": 0}
    for k, c in enumerate(cases):
        e = expected(c)
        if e is None:
            assert c["ok"] == 0 and c["nan"] == 1, k
            seen["nan"] += 1
            continue
        assert c["ok"] == 1 and c["nan"] == 0, k
        for key in ("sig_avg", "sig_avg1", "ddg", "ddg_acum", "ddg_applied", "add"):
            assert close(c[key], np.ravel(e[key])), (k, key)
        for key in ("s_vm", "s_vm1", "err_s", "err_e"):
            assert close([c[key]], [e[key]]), (k, key)
        assert c["out_it_nit"] == e["it_nit"] and c["out_it_nbad"] == e["it_nbad"], k
        assert bool(c["more"]) == e["more"] and c["out_it_iter"] == e["it_iter"], k
        seen["err_e0"] += e["err_e"] == 0.0
        seen["stop"] += not e["more"]
        seen["first"] += e["more"] and e["it_iter"] == 1
    assert all(v > 0 for v in seen.values()), seen

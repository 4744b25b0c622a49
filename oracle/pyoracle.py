"""ctypes binding of the oracle library (oracle/_build/liborc.so).

ORACLE - test infrastructure only.  tests/, __graft_entry__.smoke() and the
CPU legs of bench.py load it as the checker; the product never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(REPO, "m-themes_gb300"))
from mth import capi  # noqa: E402  (struct layouts shared with include/mth.h)

LIB = os.path.join(HERE, "_build", "liborc.so")
SVM_OOB_ZERO, SVM_OOB_EPSAVG10, SVM_OOB_SIGAVG1_00 = 0, 1, 2


def build(force=False):
    """Compile oracle/evpfft_oracle.c into oracle/_build/liborc.so."""
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    srcs = [os.path.join(HERE, f) for f in ("evpfft_oracle.c", "drx_oracle.c")]
    deps = srcs + [os.path.join(HERE, "oracle.h"), os.path.join(REPO, "include", "mth.h")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    # no FMA contraction: every operation separately rounded, on x86 and Arm alike
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-o", LIB] + srcs + ["-lm"]
    subprocess.check_call(cmd)
    return LIB


_lib = None


def load():
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(LIB)
        lib.orc_create.restype = C.c_void_p
        lib.orc_create.argtypes = [C.POINTER(capi.MthParams), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                   C.POINTER(C.c_double), C.c_int, C.c_int, C.POINTER(C.c_int)]
        lib.orc_step.argtypes = [C.c_void_p, C.POINTER(capi.MthStepReport)]
        lib.orc_get_field.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double)]
        lib.orc_get_c066.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        lib.orc_second_backtracks.argtypes = [C.c_void_p]
        lib.orc_second_backtracks.restype = C.c_longlong
        lib.orc_destroy.argtypes = [C.c_void_p]
        lib.orc_local_solve.argtypes = [C.POINTER(capi.MthParams), C.POINTER(C.c_double), C.c_size_t,
                                        C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double),
                                        C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double),
                                        C.POINTER(C.c_double), C.POINTER(C.c_longlong)]
        lib.orc_fft3d.argtypes = [C.POINTER(C.c_double), C.c_int, C.c_int, C.c_int, C.c_int]
        lib.orc_uniform.restype = C.c_double
        lib.orc_uniform.argtypes = [C.c_uint64, C.c_uint64]
        lib.orc_nucleation_sites.restype = C.c_longlong
        lib.orc_nucleation_sites.argtypes = [C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                             C.POINTER(C.c_double), C.c_double, C.c_double, C.c_uint64,
                                             C.c_longlong, C.POINTER(C.c_longlong), C.c_longlong]
        lib.orc_paint_nuclei.argtypes = [C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_longlong), C.c_int,
                                         C.c_int, C.c_int]
        lib.orc_pf_relax.argtypes = [C.POINTER(capi.MthParams), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                     C.POINTER(C.c_double), C.c_int, C.c_int, C.POINTER(C.c_double), C.c_int,
                                     C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                     C.POINTER(C.c_double), C.c_int]
        lib.orc_resample_nearest.argtypes = [C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                             C.POINTER(C.c_int)]
        lib.orc_resample_trilinear.argtypes = [C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_int),
                                               C.POINTER(C.c_double)]
        _lib = lib
    return _lib


class Oracle:
    """FP64 CPU restatement of the reference EVPFFT step."""

    def __init__(self, params, grain, phase, euler, nthreads=None, svm_oob=SVM_OOB_SIGAVG1_00):
        lib = load()
        self.lib = lib
        self.nv = int(np.prod(list(params.cell_dim)))
        g = np.ascontiguousarray(grain, dtype=np.int32)
        p = np.ascontiguousarray(phase, dtype=np.int32)
        e = np.ascontiguousarray(euler, dtype=np.float64)
        st = C.c_int(0)
        nt = nthreads or os.cpu_count() or 1
        self.ctx = lib.orc_create(C.byref(params), capi._iptr(g), capi._iptr(p), capi._dptr(e), nt, svm_oob,
                                  C.byref(st))
        if not self.ctx:
            raise RuntimeError(f"orc_create failed: {capi.STATUS.get(st.value, st.value)}")

    def step(self):
        rep = capi.MthStepReport()
        st = self.lib.orc_step(self.ctx, C.byref(rep))
        if st != 0:
            raise RuntimeError(f"orc_step failed: {capi.STATUS.get(st, st)}")
        return rep.to_dict()

    def field(self, name):
        f = capi.FIELD[name]
        out = np.zeros(self.nv * capi.FIELD_NCOMP[f])
        if self.lib.orc_get_field(self.ctx, f, capi._dptr(out)) != 0:
            raise RuntimeError("orc_get_field")
        return out.reshape(self.nv, -1)

    def c066(self):
        out = np.zeros(36)
        self.lib.orc_get_c066(self.ctx, capi._dptr(out))
        return out.reshape(6, 6)

    def second_backtracks(self):
        return self.lib.orc_second_backtracks(self.ctx)

    def close(self):
        if self.ctx:
            self.lib.orc_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def local_solve(params, c066, sig, eps_p, strain, rot, crss):
    lib = load()
    n = sig.shape[0]
    sig = np.ascontiguousarray(sig, dtype=np.float64).copy()
    edot = np.zeros((n, 6))
    err = np.zeros((n, 2))
    it = C.c_longlong(0)
    args = [np.ascontiguousarray(a, dtype=np.float64) for a in (c066, eps_p, strain, rot, crss)]
    st = lib.orc_local_solve(C.byref(params), capi._dptr(args[0]), n, capi._dptr(sig), capi._dptr(args[1]),
                             capi._dptr(args[2]), capi._dptr(args[3]), capi._dptr(args[4]), capi._dptr(edot),
                             capi._dptr(err), C.byref(it))
    if st != 0:
        raise RuntimeError(f"orc_local_solve: {capi.STATUS.get(st, st)}")
    return sig, edot, err, it.value


def fft3d(data, sign):
    """In-place complex 3-D FFT of a (n0,n1,n2) complex128 array (copy returned)."""
    lib = load()
    a = np.ascontiguousarray(data, dtype=np.complex128).copy()
    n0, n1, n2 = a.shape
    lib.orc_fft3d(a.ctypes.data_as(C.POINTER(C.c_double)), n0, n1, n2, sign)
    return a


def pf_relax(params, dims, grain, rho, substeps, init_gid=None, table=None, kmax=24):
    """Oracle PF_XRX: (grain_out, ids[N,kmax], phi[N,kmax], cnt[N], table).
    init_gid defaults to the largest id of grain (no recrystallised ids);
    table is the rho_avg table (zeros of max id + 1 entries by default),
    returned as left by the call."""
    lib = load()
    nv = int(np.prod(dims))
    d = (C.c_int * 3)(*dims)
    g = np.ascontiguousarray(grain, dtype=np.int32)
    r = np.ascontiguousarray(rho, dtype=np.float64)
    if init_gid is None:
        init_gid = int(g.max())
    t = np.zeros(int(g.max()) + 1) if table is None else np.array(table, dtype=np.float64)
    go = np.zeros(nv, np.int32)
    ids = np.zeros(nv * kmax, np.int32)
    phi = np.zeros(nv * kmax)
    cnt = np.zeros(nv, np.int32)
    st = lib.orc_pf_relax(C.byref(params), d, capi._iptr(g), capi._dptr(r), substeps, init_gid, capi._dptr(t), len(t),
                          capi._iptr(go), capi._iptr(cnt), capi._iptr(ids), capi._dptr(phi), kmax)
    if st != 0:
        raise RuntimeError(f"orc_pf_relax failed: {capi.STATUS.get(st, st)}")
    return go, ids.reshape(nv, kmax), phi.reshape(nv, kmax), cnt, t


def nucleate(params, dims, grain, crystal, rho, step, first_id, cap=65536):
    """Oracle nucleation: (painted grain, sites)."""
    lib = load()
    d = (C.c_int * 3)(*dims)
    g = np.ascontiguousarray(grain, dtype=np.int32).copy()
    cr = np.ascontiguousarray(crystal, dtype=np.int32)
    r = np.ascontiguousarray(rho, dtype=np.float64)
    sites = np.zeros(cap, np.int64)
    n = lib.orc_nucleation_sites(d, capi._iptr(g), capi._iptr(cr), capi._dptr(r), params.rho_nucleation,
                                 params.nucleation_prob, params.seed, step,
                                 sites.ctypes.data_as(C.POINTER(C.c_longlong)), cap)
    nn = int(min(n, cap))
    lib.orc_paint_nuclei(d, capi._iptr(g), sites.ctypes.data_as(C.POINTER(C.c_longlong)), nn, first_id,
                         params.nucleus_radius)
    return g, sites[:nn]


def resample(src, ns, nd):
    """Oracle grid transfer: nearest corner for integer arrays, trilinear for
    floating-point arrays (flattened, z fastest)."""
    lib = load()
    a = (C.c_int * 3)(*ns)
    b = (C.c_int * 3)(*nd)
    n = int(np.prod(nd))
    if np.issubdtype(np.asarray(src).dtype, np.integer):
        x = np.ascontiguousarray(src, dtype=np.int32)
        out = np.zeros(n, np.int32)
        lib.orc_resample_nearest(a, capi._iptr(x), b, capi._iptr(out))
    else:
        x = np.ascontiguousarray(src, dtype=np.float64)
        out = np.zeros(n)
        lib.orc_resample_trilinear(a, capi._dptr(x), b, capi._dptr(out))
    return out

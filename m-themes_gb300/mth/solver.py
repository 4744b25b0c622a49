"""High-level wrapper over the C-ABI (include/mth.h)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi


class Solver:
    """One RVE on the GPU: mth_create + mth_upload_microstructure, then
    `step()` per mechanical step (the loop body of Evolution,
    src/evolution.c:1319-1693)."""

    def __init__(self, params: capi.MthParams, grain, phase, euler):
        self.lib = capi.load()
        self.params = params
        self.nv = int(np.prod(list(params.cell_dim)))
        ctx = C.c_void_p()
        capi.check(self.lib, self.lib.mth_create(C.byref(params), C.byref(ctx)))
        self.ctx = ctx
        g = np.ascontiguousarray(grain, dtype=np.int32)
        p = np.ascontiguousarray(phase, dtype=np.int32)
        e = np.ascontiguousarray(euler, dtype=np.float64)
        if g.size != self.nv or p.size != self.nv or e.size != 3 * self.nv:
            self.close()
            raise ValueError("microstructure arrays do not match cell_dim")
        capi.check(self.lib, self.lib.mth_upload_microstructure(self.ctx, capi._iptr(g), capi._iptr(p),
                                                                capi._dptr(e), self.nv))

    def step(self) -> dict:
        rep = capi.MthStepReport()
        capi.check(self.lib, self.lib.mth_step(self.ctx, C.byref(rep)))
        return rep.to_dict()

    def field(self, name: str) -> np.ndarray:
        f = capi.FIELD[name]
        out = np.zeros(self.nv * capi.FIELD_NCOMP[f])
        capi.check(self.lib, self.lib.mth_download_field(self.ctx, f, capi._dptr(out), out.size))
        return out.reshape(self.nv, -1)

    def track_disgrad(self, on: bool = True):
        """Keep the full displacement gradient (field "disgrad", iout kind
        "disgrad"); before the first step (mth_track_disgrad)."""
        capi.check(self.lib, self.lib.mth_track_disgrad(self.ctx, 1 if on else 0))

    def write_iout(self, kind: str, prefix: str, step: int):
        """Start writing a field in the reference's .iout format (mth_write_iout);
        the files are complete after wait_iout()."""
        capi.check(self.lib, self.lib.mth_write_iout(self.ctx, capi.IOUT[kind], prefix.encode(), step))

    def wait_iout(self):
        capi.check(self.lib, self.lib.mth_iout_wait(self.ctx))

    def adjoint(self, target, checkpoint_every=10, cg_tol=0.0, cg_itmax=0):
        """Misfit J = sum_n (<sigma_33>_n - target_n)^2 of a forward run of
        len(target) steps from this (fresh) context and dJ/d(tau0, tau1,
        thet0, thet1, nrs) by the adjoint (mth_adjoint).  Returns
        (J, grad, s33, info)."""
        t = np.ascontiguousarray(target, dtype=np.float64)
        opts = capi.MthAdjointOpts()
        opts.n_steps = t.size
        opts.checkpoint_every = checkpoint_every
        opts.target = capi._dptr(t)
        opts.cg_tol = cg_tol
        opts.cg_itmax = cg_itmax
        s33 = np.zeros(t.size)
        res = capi.MthAdjointResult()
        capi.check(self.lib, self.lib.mth_adjoint(self.ctx, C.byref(opts), capi._dptr(s33), C.byref(res)))
        info = res.to_dict()
        return info["misfit"], np.array(info["grad"]), s33, info

    def profile(self, enable=None, reset=False):
        """Per-kernel device times (CUDA events on the context's stream),
        launch counts and algorithmic bytes; optionally switch timing on/off."""
        if enable is not None:
            capi.check(self.lib, self.lib.mth_profile_enable(self.ctx, 1 if enable else 0))
        pr = capi.MthProfile()
        capi.check(self.lib, self.lib.mth_profile_read(self.ctx, C.byref(pr), 1 if reset else 0))
        return pr.to_dict(), pr.total_launches

    def close(self):
        if getattr(self, "ctx", None):
            self.lib.mth_destroy(self.ctx)
            self.ctx = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def local_solve(params, c066, sig, eps_p, strain, rot, crss):
    """Batch local Newton (mth_local_solve); arrays as in include/mth.h."""
    lib = capi.load()
    n = sig.shape[0]
    sig = np.ascontiguousarray(sig, dtype=np.float64).copy()
    edot = np.zeros((n, 6))
    err = np.zeros((n, 2))
    it = C.c_longlong(0)
    a = [np.ascontiguousarray(x, dtype=np.float64) for x in (c066, eps_p, strain, rot, crss)]
    capi.check(lib, lib.mth_local_solve(C.byref(params), capi._dptr(a[0]), n, capi._dptr(sig), capi._dptr(a[1]),
                                        capi._dptr(a[2]), capi._dptr(a[3]), capi._dptr(a[4]), capi._dptr(edot),
                                        capi._dptr(err), C.byref(it)))
    return sig, edot, err, it.value


class Batch:
    """Independent RVEs advanced together on one GPU (mth_batch_*): members
    may differ in grid size, material and loading.  `step()` returns one
    report per member; results equal those of a `Solver` per member."""

    def __init__(self, params_list, microstructures):
        self.lib = capi.load()
        self.n = len(params_list)
        arr = (capi.MthParams * self.n)(*params_list)
        self.nv = [int(np.prod(list(p.cell_dim))) for p in params_list]
        b = C.c_void_p()
        capi.check(self.lib, self.lib.mth_batch_create(arr, self.n, C.byref(b)))
        self.b = b
        for i, (grain, phase, euler) in enumerate(microstructures):
            g = np.ascontiguousarray(grain, dtype=np.int32)
            p = np.ascontiguousarray(phase, dtype=np.int32)
            e = np.ascontiguousarray(euler, dtype=np.float64)
            if g.size != self.nv[i] or p.size != self.nv[i] or e.size != 3 * self.nv[i]:
                self.close()
                raise ValueError(f"microstructure {i} does not match its cell_dim")
            capi.check(self.lib, self.lib.mth_batch_upload(self.b, i, capi._iptr(g), capi._iptr(p), capi._dptr(e),
                                                           self.nv[i]))

    def step(self) -> list:
        reps = (capi.MthStepReport * self.n)()
        capi.check(self.lib, self.lib.mth_batch_step(self.b, reps))
        return [r.to_dict() for r in reps]

    def passes(self, i: int) -> dict:
        """The FFT passes chosen for member i: {"tma": 0/1, "kz_strided": w,
        "kz_green": w} (tile widths in kz columns; 0 without TMA)."""
        t, ks, kg = C.c_int(), C.c_int(), C.c_int()
        capi.check(self.lib, self.lib.mth_batch_passes(self.b, i, C.byref(t), C.byref(ks), C.byref(kg)))
        return {"tma": t.value, "kz_strided": ks.value, "kz_green": kg.value}

    def field(self, i: int, name: str) -> np.ndarray:
        f = capi.FIELD[name]
        out = np.zeros(self.nv[i] * capi.FIELD_NCOMP[f])
        capi.check(self.lib, self.lib.mth_batch_download_field(self.b, i, f, capi._dptr(out), out.size))
        return out.reshape(self.nv[i], -1)

    def close(self):
        if getattr(self, "b", None):
            self.lib.mth_batch_destroy(self.b)
            self.b = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

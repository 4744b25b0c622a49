"""ctypes mirror of include/mth.h and loader of the in-tree libmth.so.

The C-ABI is the product boundary; this module only marshals Python values
into the structs it declares.  Loading fails loudly when the shared library
has not been built: there is no Python fallback for any compute entry point.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

NSYS = 12
NPH = 2
HERE = os.path.dirname(os.path.abspath(__file__))
PKG_ROOT = os.path.dirname(HERE)
REPO_ROOT = os.path.dirname(PKG_ROOT)
LIB_PATH = os.path.join(PKG_ROOT, "lib", "libmth.so")

MTH_FP64 = 0
MTH_MIXED = 1
MTH_MIXED_FAST = 2
MTH_MIXED_ROOT64 = 3

FIELD = {"sig": 0, "eps": 1, "edot": 2, "strain": 3, "rot": 4, "crss": 5, "gamacum": 6, "grain": 7, "rho": 8,
         "rho_ssd": 9, "rho_gnd": 10, "disgrad": 11}
FIELD_NCOMP = {0: 9, 1: 9, 2: 9, 3: 9, 4: 9, 5: 12, 6: 1, 7: 1, 8: 1, 9: 12, 10: 36, 11: 9}

STATUS = {0: "MTH_OK", 1: "MTH_ERR_ARG", 2: "MTH_ERR_CUDA", 3: "MTH_ERR_NOMEM", 4: "MTH_ERR_SINGULAR",
          5: "MTH_ERR_NOT_CONVERGED", 6: "MTH_ERR_IO", 7: "MTH_ERR_STATE", 8: "MTH_ERR_TIMEOUT",
          9: "MTH_ERR_NAN", 10: "MTH_ERR_UNSUPPORTED"}


class MthPhase(C.Structure):
    _fields_ = [("type", C.c_int), ("c11", C.c_double), ("c12", C.c_double), ("c44", C.c_double),
                ("nsys", C.c_int), ("bn", (C.c_double * 3) * NSYS), ("bb", (C.c_double * 3) * NSYS),
                ("nrs", C.c_double), ("gamd0", C.c_double), ("tau0f", C.c_double), ("tau0b", C.c_double),
                ("tau1", C.c_double), ("thet0", C.c_double), ("thet1", C.c_double),
                ("hself", C.c_double), ("hlat", C.c_double)]


class MthParams(C.Structure):
    _fields_ = [("cell_dim", C.c_int * 3), ("n_phases", C.c_int), ("phase", MthPhase * NPH),
                ("time_step", C.c_double), ("n_steps", C.c_int), ("err", C.c_double), ("iter_max", C.c_int),
                ("velgrad_bc_flag", C.c_int * 6), ("velgrad_bc", C.c_double * 6),
                ("stress_bc_flag", C.c_int * 6), ("stress_bc", C.c_double * 6),
                ("elast_bc", C.c_int), ("update_flag", C.c_int), ("hard_flag", C.c_int),
                ("precision", C.c_int), ("newton_tol", C.c_double), ("newton_itmax", C.c_int),
                ("pf_length_scale", C.c_double), ("pf_time_step", C.c_double), ("e_gb", C.c_double),
                ("m_gb", C.c_double), ("pf_width_cells", C.c_double), ("stored_energy_scale", C.c_double),
                ("shear_modulus", C.c_double), ("burgers", C.c_double), ("nucleus_radius", C.c_int),
                ("rho_nucleation", C.c_double), ("rho0", C.c_double), ("rho_k", C.c_double),
                ("pf_substeps", C.c_int), ("seed", C.c_uint64), ("nucleation_prob", C.c_double),
                ("device", C.c_int), ("pf_cell_dim", C.c_int * 3),
                ("flow_law", C.c_int), ("dd_a0", C.c_double), ("dd_L0", C.c_double), ("dd_T", C.c_double),
                ("dd_q_slip", C.c_double), ("dd_q_bulk", C.c_double), ("dd_c", C.c_double * 8),
                ("dd_chi", C.c_double * 6), ("dd_rho_ssd0", C.c_double), ("dd_d0", C.c_double),
                ("dd_nu", C.c_double)]


T33 = (C.c_double * 3) * 3
PF_K = 16   # MTH_PF_K: list entries per voxel mth_pf_relax returns


class MthStepReport(C.Structure):
    _fields_ = [("step", C.c_int), ("iterations", C.c_int), ("time", C.c_double),
                ("sig_avg", T33), ("sig_avg_ph1", T33), ("disgrad_avg", T33), ("eps_avg", T33),
                ("edot_avg", T33), ("e_vm", C.c_double), ("evmp", C.c_double), ("d_vm", C.c_double),
                ("dvmp", C.c_double), ("s_vm", C.c_double), ("s_vm1", C.c_double),
                ("err_s", C.c_double), ("err_e", C.c_double), ("newton_iters", C.c_longlong),
                ("newton_failed", C.c_longlong), ("n_new_grains", C.c_int), ("dd_avg", C.c_double * 7)]

    def to_dict(self):
        d = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            if name == "dd_avg":
                v = np.array([v[i] for i in range(7)])
            elif isinstance(v, C.Array):
                v = np.array([[v[i][j] for j in range(3)] for i in range(3)])
            d[name] = v
        return d


class MthProfile(C.Structure):
    _fields_ = [("n_kernels", C.c_int), ("name", (C.c_char * 32) * 16), ("ms", C.c_double * 16),
                ("launches", C.c_longlong * 16), ("bytes", C.c_double * 16), ("total_launches", C.c_longlong)]

    def to_dict(self):
        out = {}
        for k in range(self.n_kernels):
            out[bytes(self.name[k]).split(b"\0")[0].decode()] = {
                "ms": self.ms[k], "launches": self.launches[k], "bytes": self.bytes[k]}
        return out


class MthAdjointOpts(C.Structure):
    _fields_ = [("n_steps", C.c_int), ("checkpoint_every", C.c_int), ("target", C.POINTER(C.c_double)),
                ("cg_tol", C.c_double), ("cg_itmax", C.c_int)]


class MthAdjointResult(C.Structure):
    _fields_ = [("misfit", C.c_double), ("grad", C.c_double * 5), ("cg_iterations", C.c_longlong),
                ("cg_iterations_max", C.c_int), ("recomputed_steps", C.c_int), ("forward_ms", C.c_double),
                ("reverse_ms", C.c_double)]

    def to_dict(self):
        return {"misfit": self.misfit, "grad": [self.grad[i] for i in range(5)],
                "cg_iterations": self.cg_iterations, "cg_iterations_max": self.cg_iterations_max,
                "recomputed_steps": self.recomputed_steps, "forward_ms": self.forward_ms,
                "reverse_ms": self.reverse_ms}


# order of the calibration parameters of mth_adjoint's gradient
ADJOINT_PARAMS = ("tau0", "tau1", "thet0", "thet1", "nrs")


def params_from_config(cfg, precision=MTH_FP64, newton_tol=0.0, newton_itmax=0) -> MthParams:
    """Fill MthParams from a synth.Config (power-law/Voce FCC, optional gas phase)."""
    from . import synth
    p = MthParams()
    p.cell_dim[:] = list(cfg.cell_dim)
    p.n_phases = 2 if cfg.n_pores else 1
    m = cfg.material
    for k in range(NPH):
        ph = p.phase[k]
        ph.type = 0 if k == 0 else 1
        if k == 0:
            ph.c11, ph.c12, ph.c44 = m.c11, m.c12, m.c44
            ph.nsys = len(synth.FCC_SLIP)
            for i, (n, b) in enumerate(synth.FCC_SLIP):
                ph.bn[i][:] = [float(x) for x in n]
                ph.bb[i][:] = [float(x) for x in b]
            ph.nrs, ph.gamd0 = m.nrs, m.gamd0
            ph.tau0f, ph.tau0b, ph.tau1, ph.thet0, ph.thet1 = m.tau0f, m.tau0b, m.tau1, m.thet0, m.thet1
            ph.hself, ph.hlat = m.hself, m.hlat
    p.time_step = cfg.time_step
    p.n_steps = cfg.n_steps
    p.err = cfg.err
    p.iter_max = cfg.iter_max
    p.velgrad_bc_flag[:] = list(cfg.velgrad_bc_flag)
    p.velgrad_bc[:] = [float(x) for x in cfg.velgrad_bc]
    p.stress_bc_flag[:] = list(cfg.stress_bc_flag)
    p.stress_bc[:] = [float(x) for x in cfg.stress_bc]
    p.elast_bc = cfg.elast_bc
    p.update_flag = cfg.update_flag
    p.hard_flag = cfg.hard_flag
    p.precision = precision
    p.newton_tol = newton_tol
    p.newton_itmax = newton_itmax
    dd = getattr(cfg, "dd", None)
    if dd is not None:
        p.flow_law = 1
        p.dd_a0, p.dd_L0, p.dd_T, p.dd_q_slip, p.dd_q_bulk = dd.a0, dd.L0, dd.T, dd.q_slip, dd.q_bulk
        p.dd_c[:] = [float(x) for x in dd.c]
        p.dd_chi[:] = [float(x) for x in dd.chi]
        p.dd_rho_ssd0, p.dd_d0, p.dd_nu = dd.rho_ssd0, dd.d0, dd.nu
    d = getattr(cfg, "drx", None)
    if d is not None:
        p.pf_substeps = d.pf_substeps
        p.pf_time_step = d.pf_time_step
        p.pf_length_scale = d.pf_length_scale
        p.e_gb = d.e_gb
        p.m_gb = d.m_gb
        p.pf_width_cells = d.pf_width_cells
        p.stored_energy_scale = d.stored_energy_scale
        p.shear_modulus = synth.shear_modulus(m)
        p.burgers = d.burgers
        p.rho0 = d.rho0
        p.rho_k = d.rho_k
        p.rho_nucleation = d.rho_nucleation
        p.nucleation_prob = d.nucleation_prob
        p.nucleus_radius = d.nucleus_radius
        p.seed = d.seed
        if d.pf_cell_dim:
            for i in range(3):
                p.pf_cell_dim[i] = d.pf_cell_dim[i]
    return p


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _iptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


IOUT = {"sig": 0, "eps": 1, "edot": 2, "els": 3, "grain": 4, "texture": 5, "disgrad": 6}


class MthError(RuntimeError):
    pass


_lib = None


def load(path: str | None = None):
    """Load libmth.so (built by build.py).  Raises if it is missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise MthError(f"{p} not found: build the CUDA library first (python -c 'import __graft_entry__ as g; g.build()')")
    lib = C.CDLL(p)
    lib.mth_version.restype = C.c_char_p
    lib.mth_last_error.restype = C.c_char_p
    lib.mth_create.argtypes = [C.POINTER(MthParams), C.POINTER(C.c_void_p)]
    lib.mth_upload_microstructure.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                              C.POINTER(C.c_double), C.c_size_t]
    lib.mth_step.argtypes = [C.c_void_p, C.POINTER(MthStepReport)]
    lib.mth_download_field.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double), C.c_size_t]
    lib.mth_track_disgrad.argtypes = [C.c_void_p, C.c_int]
    lib.mth_destroy.argtypes = [C.c_void_p]
    lib.mth_local_solve.argtypes = [C.POINTER(MthParams), C.POINTER(C.c_double), C.c_size_t,
                                    C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double),
                                    C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double),
                                    C.POINTER(C.c_double), C.POINTER(C.c_longlong)]
    lib.mth_local_solve_noalloc.argtypes = [C.POINTER(MthParams), C.POINTER(C.c_double), C.c_size_t,
                                            C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                            C.c_void_p, C.c_void_p, C.POINTER(C.c_longlong), C.c_void_p]
    lib.mth_pf_relax.argtypes = [C.POINTER(MthParams), C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_double),
                                 C.c_int, C.c_int, C.POINTER(C.c_double), C.c_int, C.POINTER(C.c_int),
                                 C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_int)]
    lib.mth_nucleate.argtypes = [C.POINTER(MthParams), C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                 C.POINTER(C.c_double), C.c_longlong, C.c_int, C.POINTER(C.c_longlong), C.c_longlong,
                                 C.POINTER(C.c_int)]
    lib.mth_profile_enable.argtypes = [C.c_void_p, C.c_int]
    lib.mth_profile_read.argtypes = [C.c_void_p, C.POINTER(MthProfile), C.c_int]
    lib.mth_read_namelist.argtypes = [C.c_char_p, C.POINTER(MthParams), C.c_char_p, C.c_char_p, C.c_char_p,
                                      C.c_size_t]
    lib.mth_read_sx.argtypes = [C.c_char_p, C.POINTER(MthParams), C.c_int]
    lib.mth_read_microstructure.argtypes = [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                            C.POINTER(C.c_double)]
    lib.mth_write_iout.argtypes = [C.c_void_p, C.c_int, C.c_char_p, C.c_int]
    lib.mth_iout_wait.argtypes = [C.c_void_p]
    lib.mth_batch_create.argtypes = [C.POINTER(MthParams), C.c_int, C.POINTER(C.c_void_p)]
    lib.mth_batch_upload.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                     C.POINTER(C.c_double), C.c_size_t]
    lib.mth_batch_step.argtypes = [C.c_void_p, C.POINTER(MthStepReport)]
    lib.mth_batch_download_field.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_double), C.c_size_t]
    lib.mth_batch_destroy.argtypes = [C.c_void_p]
    lib.mth_batch_passes.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]
    lib.mth_adjoint.argtypes = [C.c_void_p, C.POINTER(MthAdjointOpts), C.POINTER(C.c_double),
                                C.POINTER(MthAdjointResult)]
    if path is None:
        _lib = lib
    return lib


def check(lib, st):
    if st != 0:
        msg = lib.mth_last_error().decode(errors="replace")
        raise MthError(f"{STATUS.get(st, st)}: {msg}")

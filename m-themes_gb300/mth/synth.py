"""Seeded synthetic inputs in the reference's own file formats.

The reference reads three files: the ``input.in`` namelist (src/io.c:25-164),
a single-crystal ``.sx`` slip file (src/init.c:52-231) and a voxel
microstructure text with one line ``phi1 Phi phi2 i j k grain phase`` per voxel,
Bunge angles in degrees, 1-based indices, x slowest and z fastest
(src/init.c:255-270).  This module generates periodic Voronoi polycrystals with
orientations uniform on SO(3), optional spherical pores (phase 2 = gas), and the
FCC copper parameter sets of the benchmark workloads, and writes all three
files.  Values are rounded to what the text holds, so a run that reads the
files and a run that takes the arrays directly see identical doubles.
"""
from __future__ import annotations

import dataclasses
import os

import numpy as np

# FCC {111}<110>: the 12 systems of test_run/Cu_p.sx mode 1 (plane normal, direction)
FCC_SLIP = [
    ((1, 1, -1), (0, 1, 1)), ((1, 1, -1), (1, 0, 1)), ((1, 1, -1), (1, -1, 0)),
    ((1, -1, -1), (0, 1, -1)), ((1, -1, -1), (1, 0, 1)), ((1, -1, -1), (1, 1, 0)),
    ((1, -1, 1), (0, 1, 1)), ((1, -1, 1), (1, 0, -1)), ((1, -1, 1), (1, 1, 0)),
    ((1, 1, 1), (0, 1, -1)), ((1, 1, 1), (1, 0, -1)), ((1, 1, 1), (1, -1, 0)),
]


@dataclasses.dataclass
class Material:
    """Cubic elastic constants (MPa) and one power-law/Voce slip mode."""
    c11: float = 168400.0
    c12: float = 121400.0
    c44: float = 75400.0
    nrs: float = 10.0
    gamd0: float = 1.0
    tau0f: float = 16.0
    tau0b: float = 16.0
    tau1: float = 148.0
    thet0: float = 250.0
    thet1: float = 2.0
    hself: float = 1.0
    hlat: float = 1.0


@dataclasses.dataclass
class Drx:
    """Dynamic-recrystallisation parameters.  Defaults follow the reference's
    test_run/input.in (pf_length_scale, pf_time_step, E_gb, Scale_Fdeform)
    and the coupled DRX workload (mobility 1e-10 m^4/(J s), interface width 4
    cells, 10 substeps, nucleus radius 2 cells -- nucleus_radius = 4, as the
    reference compares the key with the squared distance -- nucleation at
    5e14 m^-2).  rho is
    rho0 + rho_k * accumulated slip in units of 1e12 m^-2."""
    pf_substeps: int = 10
    pf_time_step: float = 0.004
    pf_length_scale: float = 2.5e-6
    e_gb: float = 0.625
    m_gb: float = 1e-10
    pf_width_cells: float = 4.0
    stored_energy_scale: float = 0.5
    burgers: float = 0.362 / 2 ** 0.5      # nm, a0/sqrt(2) (src/init.c:172)
    rho0: float = 1.0
    rho_k: float = 600.0
    rho_nucleation: float = 500.0
    nucleation_prob: float = 2e-5
    nucleus_radius: int = 4     # bound on |d|^2 (the reference's key): radius 2 cells
    seed: int = 12345
    pf_cell_dim: tuple = None   # CellDim_pf; None: the mechanical grid


def shear_modulus(m: "Material") -> float:
    """Shear_G of src/init.c:826 from the cubic constants (MPa)."""
    c11, c12, c44 = m.c11, m.c12, m.c44
    return 0.1 * (c11 - c12 + 3 * c44) + 0.5 * (5 * (c11 - c12) * c44) / (4 * c44 + 3 * (c11 - c12))


@dataclasses.dataclass
class DD:
    """Parameters of the dislocation-density law (the namelist keys a0, L0,
    T__K, Q_slip, Q_bulk, C_1..C_8, the six interaction strengths,
    rho_SSD_initial, D_0 and the Poisson ratio of ElastConst_PhaseI).  The
    defaults are test_run/input.in's except T__K, Q_slip and Q_bulk, which
    there switch thermally activated slip and climb off (T = 30 K with
    activation energies of 2e10 and 3e11 x 1e-19 J); here slip is active at
    the workloads' strain rate of 1/s."""
    a0: float = 0.362
    L0: float = 0.003
    T: float = 300.0
    q_slip: float = 0.25
    q_bulk: float = 1.0
    c: tuple = (0.48, 3.0, 3.0, 800.0, 16.0, 1100.0, 1.25e-8, 0.24)
    chi: tuple = (0.125, 0.125, 0.725, 0.125, 0.05, 0.18)   # self, coplanar, cross, glissile, Hirth, Lomer
    rho_ssd0: float = 0.05
    d0: float = 4e-5
    nu: float = 0.35


@dataclasses.dataclass
class Config:
    """One run: grid, loading and control parameters (namelist keys)."""
    cell_dim: tuple = (32, 32, 32)
    n_grains: int = 64
    n_pores: int = 0
    pore_radius: int = 3
    seed: int = 1234
    material: Material = dataclasses.field(default_factory=Material)
    time_step: float = 1e-3
    n_steps: int = 10
    err: float = 1e-5
    iter_max: int = 100
    velgrad_bc_flag: tuple = (0, 0, 1, 1, 1, 1)
    velgrad_bc: tuple = (-0.5, -0.5, 1.0, 0.0, 0.0, 0.0)
    stress_bc_flag: tuple = (1, 1, 0, 0, 0, 0)
    stress_bc: tuple = (0.0, 0.0, 0.0, 0.0, 0.0, 0.0)
    elast_bc: int = 1
    update_flag: int = 1
    hard_flag: int = 1
    drx: Drx = None
    dd: DD = None           # dislocation-density law instead of the power law + Voce


def voronoi(cell_dim, n_grains, rng):
    """Periodic Voronoi tessellation: 1-based grain id of every voxel centre,
    flattened with z fastest."""
    from scipy.spatial import cKDTree
    dims = np.asarray(cell_dim, dtype=np.float64)
    seeds = rng.random((n_grains, 3)) * dims
    tree = cKDTree(seeds, boxsize=dims)
    ax = [np.arange(n, dtype=np.float64) + 0.5 for n in cell_dim]
    X, Y, Z = np.meshgrid(*ax, indexing="ij")
    pts = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    _, idx = tree.query(pts, k=1)
    return idx.astype(np.int32) + 1


def uniform_orientations(n, rng):
    """Bunge angles (degrees) uniform on SO(3): phi1, phi2 ~ U[0, 360),
    cos(Phi) ~ U[-1, 1]."""
    phi1 = rng.random(n) * 360.0
    phi2 = rng.random(n) * 360.0
    Phi = np.degrees(np.arccos(rng.random(n) * 2.0 - 1.0))
    eul = np.stack([phi1, Phi, phi2], axis=1)
    return np.round(eul, 6)


def spherical_pores(cell_dim, n_pores, radius, rng, max_tries=100000):
    """Boolean gas mask of non-overlapping periodic spheres of the given radius
    (cells) at seeded random centres."""
    dims = np.asarray(cell_dim)
    centres = []
    tries = 0
    while len(centres) < n_pores:
        tries += 1
        if tries > max_tries:
            raise RuntimeError("could not place non-overlapping pores")
        c = rng.random(3) * dims
        ok = True
        for o in centres:
            d = np.abs(c - o)
            d = np.minimum(d, dims - d)
            if np.sqrt((d * d).sum()) < 2 * radius + 1:
                ok = False
                break
        if ok:
            centres.append(c)
    mask = np.zeros(tuple(cell_dim), dtype=bool)
    ax = [np.arange(n, dtype=np.float64) + 0.5 for n in cell_dim]
    X, Y, Z = np.meshgrid(*ax, indexing="ij")
    for c in centres:
        d = [np.abs(A - ci) for A, ci in zip((X, Y, Z), c)]
        d = [np.minimum(di, n - di) for di, n in zip(d, cell_dim)]
        mask |= (d[0] ** 2 + d[1] ** 2 + d[2] ** 2) <= radius * radius
    return mask.ravel()


def microstructure(cfg: Config):
    """(grain, phase, euler_deg) arrays of one configuration, z fastest."""
    rng = np.random.default_rng(cfg.seed)
    grain = voronoi(cfg.cell_dim, cfg.n_grains, rng)
    eul_g = uniform_orientations(cfg.n_grains, rng)
    euler = eul_g[grain - 1].copy()
    phase = np.ones(grain.shape, dtype=np.int32)
    if cfg.n_pores:
        gas = spherical_pores(cfg.cell_dim, cfg.n_pores, cfg.pore_radius, rng)
        phase[gas] = 2
        grain[gas] = cfg.n_grains + 1
        euler[gas] = 0.0
    return grain.astype(np.int32), phase, np.ascontiguousarray(euler)


# ---------------------------------------------------------------- writers
def write_microstructure(path, cfg: Config, grain, phase, euler):
    nx, ny, nz = cfg.cell_dim
    ii, jj, kk = np.meshgrid(np.arange(1, nx + 1), np.arange(1, ny + 1), np.arange(1, nz + 1), indexing="ij")
    with open(path, "w") as f:
        for v, (i, j, k) in enumerate(zip(ii.ravel(), jj.ravel(), kk.ravel())):
            e = euler[v]
            f.write("%.6f %.6f %.6f %d %d %d %d %d\n" % (e[0], e[1], e[2], i, j, k, grain[v], phase[v]))


def write_sx(path, m: Material):
    """One-mode FCC file in the line layout PlasticInit reads (src/init.c:66-176)."""
    lines = ["# Crystal system (XtalSys):", "CUBIC", "",
             "# Crystal axes (XtalAxis):", "1.0 1.0 1.0", "",
             "# Total number of modes listed in the file (N_modes_max):", "1", "",
             "# Number of modes to be used in the calculation (N_modes):", "1", "",
             "# Labels of the modes to be used (iMode):", "1", "",
             "# Mode# 1 -- <110>(111) SLIP",
             "\tnsmx\tnrsx\tgamd0x\ttwshx\tisectwx",
             "\t12\t\t%r\t\t%r\t\t0.0\t\t0" % (float(m.nrs), float(m.gamd0)),
             "\ttau0xf\ttau0xb\ttau1x\tthet0\tthet1",
             "\t%r\t\t%r\t\t%r\t\t%r\t\t%r" % (float(m.tau0f), float(m.tau0b), float(m.tau1),
                                                float(m.thet0), float(m.thet1)),
             "\thselfx\thlatex",
             "\t%r\t\t%r" % (float(m.hself), float(m.hlat)),
             "\tSlip (n-b)"]
    for n, b in FCC_SLIP:
        lines.append("\t%d %d %d\t\t%d %d %d" % (n + b))
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def write_input(path, cfg: Config, ms_name="ms.txt", sx_name="cu.sx"):
    m = cfg.material
    pfd = cfg.drx.pf_cell_dim if (cfg.drx is not None and cfg.drx.pf_cell_dim) else cfg.cell_dim
    n_phases = 2 if cfg.n_pores else 1
    dd = cfg.dd if cfg.dd is not None else DD(T=30.0, q_slip=20000000000.0, q_bulk=300000000000.51)
    c = dd.c
    x = dd.chi

    def vec(v):
        return " ".join(repr(float(x)) if isinstance(x, float) else str(x) for x in v)

    txt = f"""# generated input (reference namelist layout)
N_phases\t{n_phases}
CellDim {cfg.cell_dim[0]} {cfg.cell_dim[1]} {cfg.cell_dim[2]}
initial_ms {ms_name}
Type_phases 0 1
ElastConst_PhaseI {m.c11!r} {m.c12!r} {m.c44!r} {dd.nu!r}
Slip_PhaseI {sx_name}
ElastConst_PhaseII 0.0 0.0 0.0 0.0
Slip_PhaseII {sx_name}
VelGrad_BC_Flag {vec(cfg.velgrad_bc_flag)}
VelGrad_BC {vec(cfg.velgrad_bc)}
Stress_BC_Flag {vec(cfg.stress_bc_flag)}
Stress_BC {vec(cfg.stress_bc)}
ElastBC {cfg.elast_bc}
TimeStep {cfg.time_step!r}
N_steps {cfg.n_steps}
Err {cfg.err!r}
IterMax {cfg.iter_max}
PrintControl 0 2000
Update_Flag {cfg.update_flag}
Hard_Flag {cfg.hard_flag}
Tex_Flag 0
a0 {dd.a0!r} 0.0
L0 {dd.L0!r}
GND_ScaleRatio 6000.0
Q_slip {dd.q_slip!r} 0.0
Q_bulk {dd.q_bulk!r} 0.0
rho_SSD_initial {dd.rho_ssd0!r}
T__K {dd.T!r}
C_1 {c[0]!r} 0.0
C_2 {c[1]!r} 0.0
C_3 {c[2]!r} 0.0
C_4 {c[3]!r} 0.0
C_5 {c[4]!r} 0.0
C_6 {c[5]!r} 0.0
C_7 {c[6]!r} 0.0
C_8 {c[7]!r} 0.0
Selfinter {x[0]!r} 0.0
Coplanar {x[1]!r} 0.0
CrossSlip {x[2]!r} 0.0
GlissileJunction {x[3]!r} 0.0
HirthLock {x[4]!r} 0.0
LomerCottrellLock {x[5]!r} 0.0
D_0 {dd.d0!r}
nucleus_radius {cfg.drx.nucleus_radius if cfg.drx is not None else 4}
CellDim_pf {pfd[0]} {pfd[1]} {pfd[2]}
RandSeed 123
E_gb 0.625
M_gb 7.4E-11
Scale_Fdeform 0.5
k_c 320000.0
alpha 8.5
zeta_kc 1.0
age_drx 1E0
ssdScaler_DRX 0.74
gndScaler_DRX 0.66
sigScaler_DRX 0.66
Nucl_Static_Flag 1
tau_DRX 1000.0
DeltaQ_DRX 0.0
DeltaTau_DRX 0.0
pf_length_scale 2.5E-06
pf_time_step 0.004
"""
    with open(path, "w") as f:
        f.write(txt)


def write_case(directory, cfg: Config):
    """Write input.in, cu.sx and ms.txt of one configuration; returns the
    microstructure arrays."""
    os.makedirs(directory, exist_ok=True)
    grain, phase, euler = microstructure(cfg)
    write_microstructure(os.path.join(directory, "ms.txt"), cfg, grain, phase, euler)
    write_sx(os.path.join(directory, "cu.sx"), cfg.material)
    write_input(os.path.join(directory, "input.in"), cfg)
    return grain, phase, euler


# ------------------------------------------------------ named workloads
def workload(name: str) -> Config:
    """Benchmark workloads: 'fp64_32cube' = 32^3 / 64 grains FP64 plain EVPFFT, 10 steps;
    'rve128' = 128^3 / 512 grains + 40 radius-3 pores, 100 steps; 'rve96' = the same at 96^3
    (216 grains, 17 pores) for profiler captures."""
    if name == "fp64_32cube":
        return Config(cell_dim=(32, 32, 32), n_grains=64, n_steps=10, seed=20240101)
    if name == "rve128":
        return Config(cell_dim=(128, 128, 128), n_grains=512, n_pores=40, pore_radius=3,
                      n_steps=100, seed=20240102)
    if name == "drx128":    # coupled EVPFFT + sparse phase-field DRX, compression to true strain 0.5
        return Config(cell_dim=(128, 128, 128), n_grains=1000, n_steps=500, seed=20240104,
                      velgrad_bc=(0.5, 0.5, -1.0, 0.0, 0.0, 0.0), drx=Drx())
    if name == "drx64":   # 64^3 profiling case of drx128: nucleation from the second step on
        return Config(cell_dim=(64, 64, 64), n_grains=125, n_steps=10, seed=20240105, iter_max=10,
                      velgrad_bc=(0.5, 0.5, -1.0, 0.0, 0.0, 0.0),
                      drx=Drx(rho_k=40000.0, nucleation_prob=2e-3))
    if name == "drx128_each":   # drx128 with nucleation from the second step on: the DRX step at 128^3 every step
        return Config(cell_dim=(128, 128, 128), n_grains=1000, n_steps=500, seed=20240104,
                      velgrad_bc=(0.5, 0.5, -1.0, 0.0, 0.0, 0.0), drx=Drx(rho_k=40000.0, nucleation_prob=2e-4))
    if name == "calib64":    # adjoint calibration: 64^3, 256 grains, tension for 50 steps of 1e-3
        return Config(cell_dim=(64, 64, 64), n_grains=256, n_steps=50, seed=20240107)
    if name == "calib16":   # small case of calib64 for tests: 16^3, 8 grains, 5 steps
        return Config(cell_dim=(16, 16, 16), n_grains=8, n_steps=5, seed=777)
    if name == "rve96":   # 96^3 profiling case of rve128: fields still larger than L2
        return Config(cell_dim=(96, 96, 96), n_grains=216, n_pores=17, pore_radius=3,
                      n_steps=100, seed=20240103)
    raise KeyError(name)


def batch_workload(name: str = "batch64", master_seed: int = 20240106) -> list:
    """Batched-RVE workloads.  'batch64': 64 independent RVEs, 24 x 32^3, 24 x 48^3
    and 16 x 64^3; RVE i has seed master + i, a grain count drawn uniformly
    from [32, 256], uniform orientations, tau0 ~ U[12, 20] MPa (forward and
    backward CRSS) and n drawn from {8, 10, 15, 20}; uniaxial tension for 50
    steps of 1e-3.  'batch6': the first 2 RVEs of each size (6), for tests."""
    sizes = [32] * 24 + [48] * 24 + [64] * 16
    if name == "batch6":
        sizes = [32, 32, 48, 48, 64, 64]
    elif name != "batch64":
        raise KeyError(name)
    out = []
    for i, n in enumerate(sizes):
        seed = master_seed + i
        rng = np.random.default_rng(seed)
        n_grains = int(rng.integers(32, 257))
        tau0 = float(rng.uniform(12.0, 20.0))
        nrs = float(rng.choice([8.0, 10.0, 15.0, 20.0]))
        mat = Material(tau0f=tau0, tau0b=tau0, nrs=nrs)
        out.append(Config(cell_dim=(n, n, n), n_grains=n_grains, n_steps=50, seed=seed, material=mat))
    return out


def calibration_target_material() -> Material:
    """Parameters that generate the target stress-strain curve of the
    adjoint calibration workload: tau0 = 18 MPa, thet0 = 280 MPa,
    tau1 = 160 MPa, n = 12 (the other Cu values as Material())."""
    return Material(tau0f=18.0, tau0b=18.0, thet0=280.0, tau1=160.0, nrs=12.0)


def perturb_material(m: Material, k: int, h: float) -> Material:
    """Copy of m with calibration parameter k (tau0, tau1, thet0, thet1, nrs
    in that order; tau0 moves the forward and backward CRSS together)
    shifted by h."""
    r = dataclasses.replace(m)
    if k == 0:
        r.tau0f += h
        r.tau0b += h
    elif k == 1:
        r.tau1 += h
    elif k == 2:
        r.thet0 += h
    elif k == 3:
        r.thet1 += h
    elif k == 4:
        r.nrs += h
    else:
        raise IndexError(k)
    return r


def calibration_values(m: Material) -> list:
    """(tau0, tau1, thet0, thet1, nrs) of m."""
    return [m.tau0f, m.tau1, m.thet0, m.thet1, m.nrs]

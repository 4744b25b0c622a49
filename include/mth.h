/*
 * mth.h -- C-ABI of the GB300 EVPFFT / sparse phase-field solve.
 *
 * The reference (M-THEMES, `forge`) has no plugin layer: `main` calls
 * `SetupJob()`, `Evolution()` and `DestroyJob()` over global state
 * (src/evp.c:18-25, src/evp.h:595-615).  This header replaces that trio with
 * a context object; every entry point returns an `mth_status` instead of
 * aborting (the reference calls `PError` -> `MPI_Abort`, src/evp.h:62-63).
 *
 * Plain C types only: no CUDA or torch types cross this boundary.  All host
 * buffers belong to the caller and are never retained after a call returns.
 * One context per host thread; contexts are independent.
 */
#ifndef MTH_H
#define MTH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MTH_NSYS_MAX 12   /* NSYSMX, src/evpFlags.h:5 */
#define MTH_NPH_MAX 2     /* NPHMAX, src/evpFlags.h:4 */

typedef enum {
  MTH_OK = 0,
  MTH_ERR_ARG = 1,          /* bad argument or inconsistent input */
  MTH_ERR_CUDA = 2,         /* CUDA runtime error (message in mth_last_error) */
  MTH_ERR_NOMEM = 3,        /* device or host allocation failed */
  MTH_ERR_SINGULAR = 4,     /* singular matrix (reference: exit(35), src/kinematics.c:306-313) */
  MTH_ERR_NOT_CONVERGED = 5,/* local Newton hit its iteration cap in some voxel */
  MTH_ERR_IO = 6,           /* input file missing or malformed */
  MTH_ERR_STATE = 7,        /* call out of order (e.g. step before upload) */
  MTH_ERR_TIMEOUT = 8,      /* a bounded device wait gave up */
  MTH_ERR_NAN = 9,          /* non-finite value in a field or a report */
  MTH_ERR_UNSUPPORTED = 10  /* grid size / option not supported by this build */
} mth_status;

typedef enum {
  MTH_FP64 = 0,       /* all fields, FFTs and the local Newton in FP64 */
  MTH_MIXED = 1,      /* FP32 fields/FFT/Green operator/flow rule; FP64 Jacobian solve of the
                         local Newton, FP64 error norms and volume averages */
  MTH_MIXED_FAST = 2, /* as MTH_MIXED but the 5x5 Jacobian solve in FP32 too */
  MTH_MIXED_ROOT64 = 3 /* as MTH_MIXED but the Jacobian solve in FP64 only for the Newton steps
                          within 1e-3 |lambda| of the root, in FP32 for the large early steps */
} mth_precision;

/* One phase: elastic constants plus the active slip mode of its .sx file
 * (src/init.c:52-231).  Slip normals/directions are given as read (not
 * normalised); the library normalises them as PlasticInit does. */
typedef struct {
  int    type;               /* Type_phases: 0 crystal, 1 gas */
  double c11, c12, c44;      /* MPa (ElastConst_Phase*, src/io.c:42-43) */
  int    nsys;               /* nsmx */
  double bn[MTH_NSYS_MAX][3];/* slip-plane normals */
  double bb[MTH_NSYS_MAX][3];/* slip directions */
  double nrs;                /* rate-sensitivity exponent n */
  double gamd0;              /* reference shear rate, 1/s */
  double tau0f, tau0b;       /* initial CRSS, forward/backward, MPa */
  double tau1, thet0, thet1; /* Voce parameters, MPa */
  double hself, hlat;        /* self/latent hardening ratios */
} mth_phase;

/* Run parameters: the subset of the reference namelist (src/io.c:25-94) that
 * drives the EVPFFT solve, plus the phase-field/DRX block. */
typedef struct {
  int    cell_dim[3];        /* CellDim */
  int    n_phases;           /* N_phases */
  mth_phase phase[MTH_NPH_MAX];
  double time_step;          /* TimeStep [s] */
  int    n_steps;            /* N_steps */
  double err;                /* Err: Green-iteration tolerance */
  int    iter_max;           /* IterMax */
  int    velgrad_bc_flag[6]; /* VelGrad_BC_Flag (Voigt 11,22,33,23,13,12) */
  double velgrad_bc[6];      /* VelGrad_BC */
  int    stress_bc_flag[6];  /* Stress_BC_Flag */
  double stress_bc[6];       /* Stress_BC */
  int    elast_bc;           /* ElastBC: 0 -> Gamma(k=0) = -S0, 1 -> 0 */
  int    update_flag;        /* Update_Flag: texture update */
  int    hard_flag;          /* Hard_Flag: Voce hardening */
  int    precision;          /* mth_precision */
  double newton_tol;         /* local Newton tolerance; <=0 selects the default
                                (1e-10 FP64 as in src/evolution.c:104, 1e-6 mixed).  A solve
                                ends when its last step is within it; in the mixed modes also
                                when the next step is bounded within it (|gradient| over the
                                smallest eigenvalue of the elastic Hessian base) */
  int    newton_itmax;       /* <=0 selects 500 (src/evolution.c:105) */
  /* Phase-field / DRX block (src/io.c:71-90) */
  double pf_length_scale;    /* dx [m] */
  double pf_time_step;       /* dt of one PF substep [s] */
  double e_gb;               /* GB energy [J/m^2] */
  double m_gb;               /* GB mobility [m^4/(J s)] */
  double pf_width_cells;     /* L_gb / dx; the reference hard-codes 3 (src/pf_xrx.c:1493) */
  double stored_energy_scale;/* Scale_Fdeform (alpha in PF_XRX) */
  double shear_modulus;      /* mu in the stored energy alpha*mu*b^2 [GPa] */
  double burgers;            /* b [nm] */
  int    nucleus_radius;     /* bound on the squared distance [cells^2] a nucleus paints (key nucleus_radius) */
  double rho_nucleation;     /* nucleation threshold on rho_tot [1e12/m^2] */
  double rho0;               /* initial dislocation density [1e12/m^2] */
  double rho_k;              /* rho = rho0 + rho_k * accumulated slip [1e12/m^2] */
  int    pf_substeps;        /* PF substeps per mechanical step; 0 disables DRX */
  uint64_t seed;             /* counter-based RNG seed */
  double nucleation_prob;    /* per-step nucleation probability of a candidate voxel */
  int    device;             /* CUDA device ordinal the context runs on */
  int    pf_cell_dim[3];     /* CellDim_pf: grid of the phase field.  Zeros or equal to
                                cell_dim: the mechanical grid.  Otherwise grain ids and rho
                                are carried to the PF grid and the relaxed ids back as
                                InterpolateGrid and Update_microstructure do
                                (src/integrated.c:496-760,821-860); each entry >= 2. */
  /* Dislocation-density law of phase 1: the reference's shipped
   * DD_BASED_FLAG path (StrainRate_Orowan src/constitutive.c:507-721,
   * DislocationEvolution :1346-1520 with first-order GNDs, AvgDislocation
   * :1669-1760); namelist keys of src/io.c:47-68. */
  int    flow_law;           /* 0: power law + Voce harden; 1: dislocation density */
  double dd_a0;              /* a0: lattice parameter [nm]; b = a0/sqrt(2) */
  double dd_L0;              /* L0: GND length scale */
  double dd_T;               /* T__K [K] */
  double dd_q_slip;          /* Q_slip [1e-19 J] */
  double dd_q_bulk;          /* Q_bulk [1e-19 J] */
  double dd_c[8];            /* C_1 .. C_8 */
  double dd_chi[6];          /* Selfinter, Coplanar, CrossSlip, GlissileJunction, HirthLock,
                                LomerCottrellLock */
  double dd_rho_ssd0;        /* rho_SSD_initial [1e12/m^2] */
  double dd_d0;              /* D_0 */
  double dd_nu;              /* Poisson ratio (4th value of ElastConst_PhaseI) */
} mth_params;

/* Per-step record; the reference prints the scalars to vm.out
 * (src/evolution.c:1621-1625) and keeps the tensors in globals. */
typedef struct {
  int    step;
  int    iterations;         /* Green iterations taken */
  double time;               /* TimeTot */
  double sig_avg[3][3];      /* <sigma> (SigAvg) */
  double sig_avg_ph1[3][3];  /* <sigma> over phase 1 (SigAvg1) */
  double disgrad_avg[3][3];  /* <grad u> actual (DisGradAvg_actual) */
  double eps_avg[3][3];      /* <eps^p> (EpsAvg) */
  double edot_avg[3][3];     /* <edot^p> (EdotAvg) */
  double e_vm, evmp, d_vm, dvmp, s_vm, s_vm1;
  double err_s, err_e;       /* final normalised errors */
  long long newton_iters;    /* local Newton iterations summed over voxels and Green iterations */
  long long newton_failed;   /* voxel solves that hit the iteration cap */
  int    n_new_grains;       /* DRX nuclei seeded this step */
  /* dislocation-density law: the dd.out columns after TIME and EVM
   * (src/evolution.c:1566-1569): volume averages of the per-system sums of
   * rho_F, rho_P, rho_s, rho_m, |rho_GND|, rho_dipole, rho_forest */
  double dd_avg[7];
} mth_step_report;

typedef enum {
  MTH_FIELD_SIG = 0,      /* 9 doubles/voxel, Cauchy stress (3x3 row-major) */
  MTH_FIELD_EPS = 1,      /* 9: plastic strain */
  MTH_FIELD_EDOT = 2,     /* 9: plastic strain rate */
  MTH_FIELD_STRAIN = 3,   /* 9: sym(grad u) */
  MTH_FIELD_ROT = 4,      /* 9: crystal->sample transformation (TranMat_xt2sa) */
  MTH_FIELD_CRSS = 5,     /* 12: forward CRSS per slip system */
  MTH_FIELD_GAMACUM = 6,  /* 1: accumulated shear */
  MTH_FIELD_GRAIN = 7,    /* 1: grain id (as double) */
  MTH_FIELD_RHO = 8,      /* 1: total dislocation density */
  MTH_FIELD_RHO_SSD = 9,  /* 12: statistically stored density per system (dislocation-density law) */
  MTH_FIELD_RHO_GND = 10, /* 36: GND densities per system: screw (12), edge I (12), edge II (12) */
  MTH_FIELD_DISGRAD = 11  /* 9: displacement gradient grad u (DisGrad, 3x3 row-major); needs mth_track_disgrad */
} mth_field;

/* Library */
const char* mth_version(void);
const char* mth_last_error(void);   /* thread-local message of the last failure */

/* Context lifecycle: replaces SetupJob/Evolution/DestroyJob (src/evp.c:23-26).
 * mth_step runs the Green iterations with their bookkeeping on the GPU and
 * queues them in groups, reading a convergence flag once per group.
 * Environment read by mth_create, for tests and comparisons only:
 *   MTH_FFT_TILES="ks,kg"      tile widths of the strided / Green TMA passes
 *   MTH_PDL=0                  no programmatic dependent launches
 *   MTH_HOST_BOOK=1            per-iteration bookkeeping on the host
 *   MTH_TEST_FAIL_TILE_WAIT=1  tile waits report a time-out (failure-path test) */
typedef struct mth_ctx mth_ctx;
mth_status mth_create(const mth_params* params, mth_ctx** out);
/* Voxel microstructure in the reference's text order: z fastest, then y, then
 * x (pIDX, src/evp.h:53).  Euler angles are Bunge degrees as in the file
 * (src/init.c:255-273); phase is 1-based.  Replaces InitMicroStruct
 * (src/init.c:233-396) and InitFields (src/init.c:444-515). */
mth_status mth_upload_microstructure(mth_ctx* ctx, const int* grain, const int* phase,
                                     const double* euler_deg, size_t n_voxels);
/* One mechanical step: Green iteration + end-of-step updates, the body of
 * the loop in Evolution (src/evolution.c:1319-1693). */
mth_status mth_step(mth_ctx* ctx, mth_step_report* report);
/* Copy a field to host memory as doubles (count = voxels * components). */
mth_status mth_download_field(mth_ctx* ctx, int field, double* host, size_t count);
/* Keep the full displacement gradient DisGrad (src/evolution.c:1319-1405),
 * for MTH_FIELD_DISGRAD and MTH_IOUT_DISGRAD.  The strain field holds its
 * symmetric part; with tracking on, each step also accumulates the
 * antisymmetric part (3 planes per voxel: the step's uniform rotation
 * increment and the local one from the Green operator's antisymmetric
 * part), at the cost of one inverse transform of 3 components per step.
 * Switch it on after mth_upload_microstructure and before the first
 * mth_step (MTH_ERR_STATE otherwise); on = 0 switches it off and frees the
 * planes.  mth_adjoint refuses a context that tracks it. */
mth_status mth_track_disgrad(mth_ctx* ctx, int on);
mth_status mth_destroy(mth_ctx* ctx);

/* Batch local solve: the per-voxel Newton of UpdateStress
 * (src/evolution.c:44-310) over n independent voxels, all inputs on the host
 * in the 6-component Lebensohn-Tome basis (chg_basis, src/kinematics.c:14-93).
 *   sig [n*6]   in: initial guess = lambda; out: converged stress
 *   eps_p [n*6] plastic strain at t
 *   strain [n*6] total strain sym(grad u)
 *   rot [n*9]   crystal->sample rotation, row-major
 *   crss [n*12] forward CRSS per system (backward = forward + (tau0b-tau0f))
 *   edot [n*6]  out: plastic strain rate
 *   err [n*2]   out: |sig-lambda|, |eps_tot-strain| (src/evolution.c:291-299)
 * c066 is the 6x6 reference stiffness.  Phase 1 parameters come from params;
 * power law only (flow_law = 1 returns MTH_ERR_UNSUPPORTED). */
mth_status mth_local_solve(const mth_params* params, const double c066[36], size_t n,
                           double* sig, const double* eps_p, const double* strain,
                           const double* rot, const double* crss, double* edot,
                           double* err, long long* newton_iters);

/* Sparse phase-field relaxation on arrays: PF_XRX (src/pf_xrx.c:1469-1698,
 * whose argument list this follows) on one grid: `substeps` explicit
 * substeps from sharp interfaces (one order parameter per voxel), with the
 * result the reference's sequential sweep gives.  rho: stored-energy density
 * of each voxel [1e12/m^2]; init_gid: grain ids above it are recrystallised
 * (a voxel they pass 0.5 at loses its stored energy, src/pf_xrx.c:1217-1219);
 * rho_avg: the caller's table of per-grain window averages (grain id g at
 * g-1, rho_avg_len entries), read and updated as the reference does -- pass
 * the same table to consecutive calls.  Outputs the relaxed grain ids (first
 * maximum of each list) and, when the pointers are not NULL, every voxel's
 * list in stored order, up to MTH_PF_K entries (ids, values, count).  FP64
 * when params->precision is MTH_FP64, FP32 otherwise.  Coefficients from
 * params (pf_length_scale, pf_time_step, e_gb, m_gb, pf_width_cells,
 * stored_energy_scale, shear_modulus, burgers).  A list over MTH_PF_K
 * entries, over 32 ids in a 3x3x3 neighbourhood or a grain id outside the
 * table returns MTH_ERR_UNSUPPORTED.  A voxel left without a positive eta
 * gets grain id 0, as Update_gID gives it (the reference then stops on the
 * assert of GetStatistics that every voxel's etas sum above 0.5, src/pf_xrx.c:1383-1386). */
#define MTH_PF_K 16
mth_status mth_pf_relax(const mth_params* params, const int cell_dim[3], const int* grain, const double* rho,
                        int substeps, int init_gid, double* rho_avg, int rho_avg_len, int* grain_out,
                        int* ids_out, double* phi_out, int* cnt_out);

/* DRX nucleation on arrays: NucleationCheckDRX (src/integrated.c:161-494)
 * with a counter-based generator.  A voxel nucleates when it is a
 * grain-boundary voxel as the reference marks it (its +x, -x, +y, -y or +z
 * neighbour in another grain, src/evolution.c:816-829 with
 * src/constitutive.c:724-873), its phase (1-based) is a crystal phase of
 * params, rho > params->rho_nucleation and u(params->seed, step*N + voxel) <
 * params->nucleation_prob.  Nuclei are numbered first_id, first_id+1, ... in
 * voxel order and paint every voxel within squared distance
 * params->nucleus_radius (the reference's key, compared with |d|^2), without
 * periodic images, later nuclei over earlier ones (src/integrated.c:397-402).
 * sites receives up to cap nucleus voxels; *n_new the number of nuclei. */
mth_status mth_nucleate(const mth_params* params, const int cell_dim[3], int* grain, const int* phase,
                        const double* rho, long long step, int first_id, long long* sites, long long cap,
                        int* n_new);

/* Allocation-free batch local solve.  No counterpart in the reference.
 * Same computation and argument meaning as mth_local_solve, but every array
 * is a DEVICE pointer owned by the caller, and the call allocates nothing:
 * no cudaMalloc/cudaFree and no allocating library routine.  It is meant for
 * callers that cannot allocate device memory during a solve: a host
 * application that hands out all device memory from its own preallocated pool
 * (an allocation behind its back would bypass the pool's accounting and could
 * fail on a GPU that the pool has filled), and code that must not trigger the
 * implicit device synchronisation a cudaMalloc/cudaFree can cause.
 * Its only scratch (per-block partial sums) is a fixed array in the library's
 * device image, held by every GPU that loads the library until the process
 * exits; n may not exceed MTH_NOALLOC_MAX_VOXELS (MTH_ERR_ARG otherwise).
 * The first call on each device looks up that array's device address; a
 * cudaDeviceReset by the caller invalidates the address the library keeps.
 * All calls share the array: calls that overlap on the GPU (different
 * streams or threads) race, so serialise them.  stream: a cudaStream_t
 * passed as void* (NULL = the default stream); the call synchronises the
 * stream and returns after it has finished the solve (newton_iters is read
 * back from the device), so it cannot be made while the stream (or, for
 * NULL, any stream) is being captured into a graph.  The
 * solve runs on params->device; the caller's current device is the same
 * after the call as before it. */
#define MTH_NOALLOC_MAX_VOXELS (1LL << 20)
mth_status mth_local_solve_noalloc(const mth_params* params, const double c066[36], size_t n,
                                   double* d_sig, const double* d_eps_p, const double* d_strain,
                                   const double* d_rot, const double* d_crss, double* d_edot,
                                   double* d_err, long long* newton_iters, void* stream);

/* Field files in the format of the reference's writers (src/io.c:247-541):
 * raw native values, no header, voxels in pIDX order (z fastest).
 *   MTH_IOUT_SIG, _EPS (plastic strain), _EDOT, _ELS (elastic strain
 *   sym(grad u) - eps_p, WriteElsMPI): six files "<prefix>_<c>_S<step>.iout"
 *   of doubles, c = 1..6 for the components 11, 22, 33, 23, 13, 12;
 *   MTH_IOUT_DISGRAD: six files as above of the displacement gradient's
 *   entries 11, 22, 33, 23, 13, 12 (WriteDisgradMPI, src/io.c:283-320;
 *   needs mth_track_disgrad);
 *   MTH_IOUT_GRAIN: "<prefix>_S<step>.iout", int32 grain ids (WriteGrainMPI);
 *   MTH_IOUT_TEXTURE: "<prefix>_S<step>.iout", 48-byte records {double
 *   Bunge angles in degrees [3]; int 1-based coordinates [3]; int grain;
 *   int phase; int 0} (WriteTextureMPI).
 * <step> is printed with 6 digits (%06d).  The fields are copied on the
 * device when mth_write_iout is called (in order with the context's work);
 * the copy to the host, the conversion and the file writes run on a
 * background thread while the caller continues.  One write is in flight per
 * context: the next mth_write_iout waits for the previous one and returns
 * its error if it failed; mth_iout_wait waits and returns the status. */
typedef enum {
  MTH_IOUT_SIG = 0,
  MTH_IOUT_EPS = 1,
  MTH_IOUT_EDOT = 2,
  MTH_IOUT_ELS = 3,
  MTH_IOUT_GRAIN = 4,
  MTH_IOUT_TEXTURE = 5,
  MTH_IOUT_DISGRAD = 6
} mth_iout_kind;
mth_status mth_write_iout(mth_ctx* ctx, int kind, const char* prefix, int step);
mth_status mth_iout_wait(mth_ctx* ctx);

/* Batches of independent volumes (RVEs) on one GPU.  Each member has its own
 * parameters (material, loading, precision), microstructure and grid size;
 * mth_batch_step advances every member by one mechanical step, with the same
 * results as mth_step on each member alone.  The step is one CUDA-graph
 * launch: a device-side loop whose body is one Green iteration of all
 * members (their kernels as parallel branches, each with its bookkeeping);
 * converged members are switched off on the device and the loop ends when
 * none is left.
 * The reference runs one volume per job (src/evp.c:7-32) and has no
 * counterpart.  Recrystallisation (pf_substeps > 0) is not supported in a
 * batch (MTH_ERR_UNSUPPORTED); all members must name the same device. */
typedef struct mth_batch mth_batch;
mth_status mth_batch_create(const mth_params* params, int n, mth_batch** out);
mth_status mth_batch_upload(mth_batch* batch, int member, const int* grain, const int* phase,
                            const double* euler_deg, size_t n_voxels);
/* reports: n entries (may be NULL) */
mth_status mth_batch_step(mth_batch* batch, mth_step_report* reports);
mth_status mth_batch_download_field(mth_batch* batch, int member, int field, double* host, size_t n_values);
mth_status mth_batch_destroy(mth_batch* batch);
/* The FFT passes mth_batch_create chose for a member by timing Green
 * iterations of a scratch volume of its grid and precision (once per grid and
 * precision in the process): *tma 1 for the tensor-map (TMA) tile passes, 0
 * for the shared-memory passes; *kz_strided and *kz_green the kz columns per
 * tile block of the strided (y, x) and the Green passes (0 when *tma is 0).
 * No reference counterpart. */
mth_status mth_batch_passes(const mth_batch* batch, int member, int* tma, int* kz_strided, int* kz_green);

/* Per-kernel device timing.  When enabled, every kernel launch of the context
 * is bracketed by CUDA events on the context's stream; times are summed per
 * kernel class.  Launch counts are kept whether or not timing is enabled.
 * The reference has no timers (no MPI_Wtime in src/); this replaces ad hoc
 * printf timing for the benchmark. */
#define MTH_PROF_MAX 16
typedef struct {
  int       n_kernels;
  char      name[MTH_PROF_MAX][32];
  double    ms[MTH_PROF_MAX];           /* summed device time per class */
  long long launches[MTH_PROF_MAX];     /* launches per class */
  double    bytes[MTH_PROF_MAX];        /* algorithmic HBM bytes moved, summed */
  long long total_launches;
} mth_profile;
mth_status mth_profile_enable(mth_ctx* ctx, int on);
mth_status mth_profile_read(mth_ctx* ctx, mth_profile* out, int reset);

/* Calibration gradient by the adjoint of the converged fixed point.  The
 * reference computes no gradients; this entry point runs the forward
 * solve for n_steps mechanical steps from a freshly uploaded context and
 * returns the misfit of the volume-averaged stress-strain curve
 *   J = sum_n (<sigma_33>_n - target_n)^2
 * and its derivatives with respect to the phase-1 parameters
 * (tau0, tau1, thet0, thet1, nrs): tau0 shifts the forward and the
 * backward initial CRSS together; tau1, thet0, thet1 are the Voce
 * parameters of harden (src/constitutive.c:275-326) and nrs the exponent
 * of the power law (src/constitutive.c:5-67).  Per mechanical step, in
 * reverse order, one linear solve of the projected tangent problem (the
 * transposed linearised Green iteration at the converged state) and the
 * transposed local Jacobians of the flow rule, the Voce update and the
 * lattice rotation.  States are stored every checkpoint_every steps and
 * the steps between are recomputed.  Requires: every voxel of phase 1,
 * a crystal; no phase-field DRX; ElastBC = 1; stress-controlled components
 * only on the diagonal (11, 22, 33), with Stress_BC_Flag the complement of
 * VelGrad_BC_Flag.  After the call the context holds the state after
 * n_steps. */
typedef struct {
  int n_steps;              /* mechanical steps of the forward run (>= 1) */
  int checkpoint_every;     /* steps between stored states; <= 0 selects 10 */
  const double* target;     /* n_steps values of <sigma_33> to fit */
  double cg_tol;            /* relative residual of each linear solve; <= 0 selects
                               1e-7 (MTH_FP64) or 1e-5 (mixed modes) */
  int cg_itmax;             /* <= 0 selects 2000 */
} mth_adjoint_opts;
typedef struct {
  double misfit;            /* J */
  double grad[5];           /* dJ/d(tau0, tau1, thet0, thet1, nrs) */
  long long cg_iterations;  /* summed over the reverse steps */
  int cg_iterations_max;    /* largest count of one step */
  int recomputed_steps;     /* forward steps run again from checkpoints */
  double forward_ms;        /* wall time of the first forward sweep */
  double reverse_ms;        /* recomputation + reverse sweep */
} mth_adjoint_result;
/* s33 (may be NULL): n_steps values of <sigma_33> of the forward run. */
mth_status mth_adjoint(mth_ctx* ctx, const mth_adjoint_opts* opts, double* s33, mth_adjoint_result* result);

/* Host-side readers for the reference's input files. */
/* input.in namelist (src/io.c:96-164); fills params and copies the file
 * names of the .sx files and the microstructure. */
mth_status mth_read_namelist(const char* path, mth_params* params,
                             char* slip_path_1, char* slip_path_2, char* ms_path,
                             size_t path_cap);
/* single-crystal .sx file (src/init.c:52-231) into params->phase[iphase]. */
mth_status mth_read_sx(const char* path, mth_params* params, int iphase);
/* voxel microstructure text (src/init.c:255-270): cell_dim[0]*cell_dim[1]*
 * cell_dim[2] lines, z fastest; the i,j,k columns are checked against the
 * line order as the reference does (src/init.c:262-266). */
mth_status mth_read_microstructure(const char* path, const int cell_dim[3], int* grain, int* phase,
                                   double* euler_deg);

#ifdef __cplusplus
}
#endif
#endif /* MTH_H */

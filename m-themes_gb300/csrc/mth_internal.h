// mth_internal.h -- declarations shared by the CUDA translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "mth_common.cuh"

namespace mth {

// Radix plan of one axis: n = prod(radix[0..nst)).
struct FftPlan {
  int n;
  int nst;
  int radix[8];
};

struct FftGeom {
  int n0, n1, n2, kz;      // grid and half-spectrum length along z
  int kzs;                 // half-spectrum row stride: kz rounded up to even, so
                           // that FP32 spectrum rows start on 16-byte boundaries
  long long plane, kplane; // elements per real plane / per spectrum plane (n0*n1*kzs)
  FftPlan px, py, pz;
  size_t smem_budget;      // dynamic shared memory per block (bytes)
};

struct AddVec { double v[6]; };

// Per-iteration inputs of the Green-iteration kernels, read from device
// memory so that a captured graph replays unchanged: the uniform strain
// increment added by the inverse z pass (6 doubles, LT basis; null: none)
// and the live flag of the volume (null: live; 0: the kernels return at
// once, which switches a converged volume of a batch off).
struct IterIn {
  const double* add;
  const int* live;
  int pdl;   // host side: launch the pass as a programmatic dependent of the kernel before it
};
// The kernels of the Green iteration's chain start with is_live.  Launched
// as programmatic dependents (launch_chain) they may begin while the kernel
// before them drains, so they first wait there for that grid and its memory
// (griddepcontrol.wait; it returns at once after an ordinary launch), then
// read the live flag.
__device__ __forceinline__ void chain_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ bool is_live(const IterIn& in) {
  chain_wait();
  return !in.live || *in.live;
}
#ifdef __CUDACC__
// Launch of a chain kernel: with pdl, as a programmatic dependent of the
// previous kernel in the stream (its launch and prologue overlap that
// kernel's last blocks); the kernel must begin with chain_wait.
template <typename... KArgs, typename... Args>
inline cudaError_t launch_chain(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, int pdl,
                                Args... args) {
  if (!pdl) {
    k<<<grid, block, smem, st>>>(args...);
    return cudaGetLastError();
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k, args...);
}
#endif

// Green-operator constants, passed by value (kernel parameter space).
struct GreenConst {
  double c0[81];      // C0_ijkl (chg_basis of C066, src/init.c:376)
  double s066[36];    // S066 = C066^-1 (used at k=0 when ElastBC=0)
  float c0f[81];      // single-precision copies for the FP32 pass
  float s066f[36];
  int elast_bc;
};

// Flow-rule, hardening and reference-medium constants, passed by value.
struct NewtonConst {
  PhaseConst ph[2];
  double s0dev[25];     // 5x5 deviatoric block of S066
  double s0hh;          // hydrostatic entry of S066
  double dt;
  double tol;
  int itmax;
  int flow_off;         // 1: Schmid tensors zero (Update_Flag=0 at istep 0)
  int ph1_only;         // 1: no crystal phase but phase 1 (sigma is 0 elsewhere), so the
                        // phase-1 stress sums equal the total ones
  int bound_stop;       // 1: also end a local solve when the next Newton step is bounded
                        // below the tolerance (ET_STOT_MIN; the FP32 flow-rule modes)
  // float copies (fill_float_consts)
  float s0devf[25];
  float s0hhf, dtf, tolf;
};

// Fill the float copies of the double constants of nc and its phases.
void fill_float_consts(NewtonConst& nc);

bool make_plan(int n, FftPlan* p);

// TMA-staged passes (fft_tma.cu) for grids whose three line lengths have
// compile-time plans.  tma_create builds the tensor maps over the fields and
// spectra; tma_has(t, pass) says whether pass 0 (z), 1 (y / x strided) or
// 2 (x + Green) has them.  err: device flag raised by a timed-out wait.
struct TmaMaps;
template <typename T>
TmaMaps* tma_create(const FftGeom& g, T* sig, T* strain, T* wspin, c2<T>* spec, c2<T>* anti, int ks = 0,
                    int kg = 0);   // ks, kg: kz columns per tile of the strided / Green passes (0: default)
void tma_destroy(TmaMaps* t);
// failure-path test hook of the tile passes: 1 makes each block's first
// tile wait report a time-out (the copies are still drained); device-wide
cudaError_t tma_set_wait_probe(int on);
bool tma_has(const TmaMaps* t, int pass);
void tma_tiles(const TmaMaps* t, int* ks, int* kg);   // the tile widths in use
int tma_tile_choice(bool fp32, int pass, int i);      // compiled width i (0..2) of pass 1 (strided) / 2 (Green)
template <typename T>
cudaError_t tma_fft_z_r2c(const TmaMaps* t, const FftGeom& g, const c2<T>* tw, const IterIn& it, int* err,
                          cudaStream_t st);
template <typename T>
cudaError_t tma_fft_z_c2r(const TmaMaps* t, const FftGeom& g, int which, const c2<T>* tw, T scale, const IterIn& it,
                          int* err, cudaStream_t st);
template <typename T>
cudaError_t tma_fft_strided(const TmaMaps* t, const FftGeom& g, int which, int sign, const c2<T>* tw,
                            const IterIn& it, int* err, cudaStream_t st);
template <typename T>
cudaError_t tma_fft_x_green(const TmaMaps* t, const FftGeom& g, const GreenConst& gc, const c2<T>* twf,
                            const c2<T>* twi, const IterIn& it, int* err, cudaStream_t st);

template <typename T>
cudaError_t launch_fft_z_r2c(const FftGeom& g, const T* in, c2<T>* out, int ncomp, const c2<T>* tw, const IterIn& it,
                             cudaStream_t st);
template <typename T>
cudaError_t launch_fft_z_c2r(const FftGeom& g, const c2<T>* spec, T* field, int ncomp, const c2<T>* tw, T scale,
                             const IterIn& it, int mode, cudaStream_t st);
template <typename T>
cudaError_t launch_fft_strided(const FftGeom& g, c2<T>* spec, int ncomp, int axis, int sign, const c2<T>* tw,
                               const IterIn& it, cudaStream_t st);
template <typename T>
cudaError_t launch_fft_x_green(const FftGeom& g, const GreenConst& gc, c2<T>* spec, c2<T>* anti, const c2<T>* twf,
                               const c2<T>* twi, const IterIn& it, cudaStream_t st);

// Per-voxel field pointers of one RVE; TSt is the storage type.
template <typename TSt>
struct Fields {
  TSt* sig;      // 6 planes, LT basis, sample axes
  TSt* strain;   // 6 planes: sym(grad u)
  TSt* epsp;     // 6 planes: plastic strain
  TSt* edot;     // 6 planes: plastic strain rate
  TSt* rot;      // 9 planes: crystal->sample matrix, row-major
  TSt* crss;     // 12 planes: forward CRSS
  TSt* gamacum;  // 1 plane
  TSt* wspin;    // 3 planes: antisymmetric part of the accumulated grad-u increment
  TSt* ddc;      // dislocation-density law: 36 planes, per system passing stress (12),
                 // tau_0 + cutting stress (12), reference rate (12) of the step; else null
  const uint8_t* phase;  // 0-based phase index
  const int* eclass;     // elastic class of the voxel (row of etab)
  const double* etab;    // ETAB_W doubles per class
  const float* etabf;    // float copy of etab
  long long nv;
};

// Elastic-class table row.  The reference builds the stiffness C_gr of each
// voxel once, from its initial orientation (src/init.c:272-283), and never
// rotates it with the lattice; only the Schmid tensors follow the texture
// (update_schmid).  Voxels with equal phase and initial Euler angles share a
// row.  Packed symmetric 5x5 blocks in the LT basis, sample axes:
constexpr int ETAB_W = 48;
constexpr int ET_STOT = 0;    // S066_dev + S_gr (15): Hessian base of the local solve
constexpr int ET_SEL = 15;    // S_gr dev (15)
constexpr int ET_SEL_HH = 30; // S_gr hydrostatic
constexpr int ET_CGR = 31;    // C_gr dev (15)
constexpr int ET_CGR_HH = 46; // C_gr hydrostatic
constexpr int ET_STOT_MIN = 47; // smallest eigenvalue of the S066_dev + S_gr block (a lower bound)

// Partial sums written per block by the Newton kernel.
constexpr int NPART = 16;   // err_s, err_e, sig[6], sig_ph1[6], newton_iters, newton_failed
// Partial sums written per block by the end-of-step kernel.
constexpr int NPART_END = 12;  // epsp[6], edot[6]

// law: 0 power law + Voce, 1 dislocation density (per-system constants in
// Fields::ddc, harden off)
cudaError_t launch_newton(int mixed, const NewtonConst& nc, const void* fields, double* partials, int nblocks,
                          const IterIn& it, cudaStream_t st, int law = 0);
// kernel attributes the Newton launches need, set on the current device
cudaError_t prepare_newton_kernels();
cudaError_t launch_end_step(int mixed, const NewtonConst& nc, const void* fields, const double anti_uniform[3],
                            int do_orient, int do_harden, double* partials, int nblocks, cudaStream_t st, int law = 0);
cudaError_t launch_setup(int mixed, const NewtonConst& nc, const void* fields, const double* euler,
                         const double d6[6], int nblocks, cudaStream_t st);
cudaError_t launch_local_solve(const NewtonConst& nc, long long n, double* sig, const double* epsp,
                               const double* strain, const double* rot, const double* crss, const double* etab,
                               double* edot, double* err, long long* iters, cudaStream_t st);
// ------------------------------------------------------------ DRX / phase field
constexpr int PF_K = 16;   // (id, eta) entries a voxel's list holds
constexpr int PF_NM = 32;  // ids of a voxel's 3x3x3 neighbourhood N(v)
constexpr int PF_RW = 128; // ids one row (x, y) of voxels writes to the rho_avg table per substep
constexpr int PF_RB = 16;  // rows per block of the table-writer prefix

struct PfCoef { double mcoef, kappa, mwell, edisl; };

// Overflow bits of a phase-field run (launch_pf_relax's *bad): a capacity
// above was exceeded or a grain id fell outside the rho_avg table.
enum { PF_BAD_LIST = 1, PF_BAD_NEIGH = 2, PF_BAD_ROW = 4, PF_BAD_TABLE = 8 };

// Device state of the phase field (drx.cu).  Every per-voxel array is
// slot-major ([slot][voxel]) so a warp's loads of one slot coalesce.
template <typename T>
struct PfBuffers {
  int* ids[2];        // lists, in stored order: ids, etas, lengths
  T* phi[2];
  uint8_t* cnt[2];
  int* gid;           // first-maximum grain id after the last substep
  T* energy;          // stored energy of the call (DefEng_buf), reset to 100 where a recrystallised id passed 0.5
  int* nid;           // N(v) in scan order [PF_NM][nv], and its length
  uint8_t* ncnt;
  uint8_t* upd[2];    // update flags, fixed-point iterates
  int* tail;          // id the list's last entry carries when the sweep reaches the voxel
  uint8_t* tmode;     // 0 unchanged, 1 weak last entry relabelled, 2 (tail, 0) appended
  T* wavg;            // window averages of the held entries [PF_K + 1][nv]
  uint8_t* ow[2];     // stored-energy resets of this substep, fixed-point iterates
  int* rw_id;         // per row: the ids it writes to the table, the last value, and the
  T* rw_val;          // first and last z of a writer [PF_RW][rows]
  int* rw_zf;
  int* rw_zl;
  uint8_t* rw_n;
  int* blk_row;       // per block of PF_RB rows and table entry: the last row up to that block
  T* blk_val;         // writing the id, and the value it wrote ([nblk][table_cap]; row -1: none)
  T* table;           // rho_avg table: grain id g at g - 1
  int table_len;      // entries the kernels may use (<= table_cap)
  int table_cap;      // entries allocated
  int nblk;
  unsigned int* word; // [0] fixed-point change counter, [1] overflow bits
  int cur;            // list buffer holding the result
  int rows;
};

template <typename T>
cudaError_t pf_alloc(PfBuffers<T>& b, const int dims[3], int table_len);
template <typename T>
void pf_free(PfBuffers<T>& b);
// grow the table to at least len entries, keeping its contents (new entries 0)
template <typename T>
cudaError_t pf_table_reserve(PfBuffers<T>& b, int len, cudaStream_t st);

cudaError_t launch_nucleation_candidates(const int dims[3], const int* grain, const uint8_t* crystal, const double* rho,
                                         double rho_nuc, double prob, uint64_t seed, uint64_t counter0,
                                         long long* out, unsigned long long* count, long long cap, cudaStream_t st);
cudaError_t launch_paint_nuclei(const int dims[3], const long long* sites, int nn, int radius2, int first_id,
                                int* winner, int* grain, cudaStream_t st);
// PF_XRX on the device: substeps sweeps from (grain, 1) per voxel with the
// table in b; ids above init_gid are recrystallised.  Synchronises the
// stream once per fixed-point iteration; *launches counts the kernels,
// *bad the overflow bits.
template <typename T>
cudaError_t launch_pf_relax(const int dims[3], const int* grain, const T* rho, int substeps, int init_gid,
                            const PfCoef& co, PfBuffers<T>& b, cudaStream_t st, int* launches, unsigned* bad);
// DRX microstructure update on the fields: rho from accumulated slip,
// adoption of the relaxed grain ids and the reset of recrystallised voxels.
cudaError_t launch_drx_rho(int mixed, const void* fields, double rho0, double rho_k, double* rho_d, void* rho_t,
                           cudaStream_t st);
// cnt: scratch of 2 n_drx ints (per recrystallised grain: its voxels, those
// that joined it in this step)
cudaError_t launch_drx_update(int mixed, const void* fields, int* grain, const int* grain_prev, const int* gid_new,
                              int first_drx_id, int n_drx, const double* drx_rot, const int* drx_class,
                              double tau0f, int nsys, int* cnt, cudaStream_t st);
cudaError_t launch_class_histogram(long long nv, const uint8_t* crystal, const int* eclass, unsigned long long* hist,
                                   cudaStream_t st);
// grid transfer between the mechanical and the phase-field grid
cudaError_t launch_resample_nearest(const int ns[3], const int* src, const int nd[3], int* dst, cudaStream_t st);
cudaError_t launch_resample_trilinear(const int ns[3], const double* src, const int nd[3], void* dst, int to_float,
                                      cudaStream_t st);
cudaError_t launch_gather_rot(int mixed, const void* rot, long long nv, const long long* sites, int nn, double* out,
                              cudaStream_t st);

// ------------------------------------------------- dislocation-density law
// Constants of phase 1 (device-resident copy per context): Burgers vector,
// shear modulus, Poisson ratio, C_1..C_8, kT [eV], reduced activation
// energies, L0, D_0, T; junction strengths and the projection cosines/sines
// of the forest and parallel densities (src/init.c:1096-1126); crystal-axes
// Schmid vectors, screw sense vectors b x n and slip directions.
// Constants of the dislocation-density law in precision T: the material
// coefficients of StrainRate_Orowan and DislocationEvolution folded on the
// host in FP64, the slip-system geometry and the 12 x 12 projection tables.
// The density kernels take them by value, so they are read from the
// kernel-parameter constant bank.
template <typename T>
struct DdCoef {
  T rm;      // rho_m = rm sqrt(rho_P rho_F)
  T tp;      // tau_pass = tp sqrt(|rho_P + rho_m|)
  T tcut;    // tau_cut = tcut sqrt(rho_F)
  T g0;      // gdot_0 = g0 rho_m / sqrt(rho_F)
  T dip;     // d_dipole = dip / (|rss| + eps)
  T eps;
  T c4, c5, c6;
  T ann;     // thermal annihilation: ann rho_s^2
  T clb;     // climb: clb d_dipole rho_s^2 exp(clb_h |p| + clb_0), p the hydrostatic stress
  T clb_h, clb_0;
  T gnd;     // GND rate per shear-rate gradient: 1 / (b L0)
  T m[NSYS][5], bp[NSYS][3], bb[NSYS][3];
  T chi[NSYS][NSYS], cs[NSYS][NSYS], ss[NSYS][NSYS], cg1[NSYS][NSYS], sg1[NSYS][NSYS], cg3[NSYS][NSYS],
      sg3[NSYS][NSYS];
};
struct DdConst {
  int nsys;
  DdCoef<double> d;
  DdCoef<float> f;
};
// Per-voxel state, 12 planes each (voxel index fastest).
template <typename T>
struct DdFields {
  T* rho_s;    // statistically stored density
  T* g1;       // GND: screw
  T* g2;       // GND: edge I
  T* g3;       // GND: edge II (stays 0 with first-order GNDs)
  T* dipole;   // rho_dipole, rho_forest: accumulated for the dd.out averages
  T* forest;
  T* gamdot;   // shear rate at the converged stress of the step
  const uint8_t* gb;   // per voxel: bit 2a / 2a+1 = neighbour +/- along axis a in the same grain
};
cudaError_t launch_dd_init(int mixed, const void* dd, const uint8_t* phase, long long P, double rho0, cudaStream_t st);
cudaError_t launch_dd_prep(int mixed, const DdConst& dc, const void* dd, const void* fields, cudaStream_t st);
cudaError_t launch_dd_gamdot(int mixed, const DdConst& dc, const void* dd, const void* fields, int flow_off,
                             cudaStream_t st);
cudaError_t launch_dd_evolve(int mixed, const DdConst& dc, const void* dd, const void* fields, const int dims[3],
                             double dt, int do_grad, double* partials, cudaStream_t st);
constexpr int NPART_DD = 7;

long long noalloc_max_voxels();
cudaError_t launch_local_solve_noalloc(const NewtonConst& nc, long long n, double* sig, const double* epsp,
                                       const double* strain, const double* rot, const double* crss, double* edot,
                                       double* err, long long* iters_host, cudaStream_t st);
// field planes (6 LT planes when sym, else nc planes) -> voxel-major doubles
cudaError_t launch_to_host_layout(int mixed, const void* src, long long P, int nc, int sym, double* dst,
                                  cudaStream_t st);
// DisGrad = strain planes (6 LT) + antisymmetric planes (W21, W02, W10) -> voxel-major 3x3 doubles
cudaError_t launch_disgrad_to_host(int mixed, const void* strain, const void* skew, long long P, double* dst,
                                   cudaStream_t st);
// skew += u + wspin per voxel, (W21, W02, W10) planes
cudaError_t launch_disgrad_skew(int mixed, const void* wspin, void* skew, long long P, const double u[3],
                                cudaStream_t st);
cudaError_t launch_reduce_partials(const double* partials, int nblocks, int width, double* out, const IterIn& it,
                                   cudaStream_t st);

// the per-iteration bookkeeping on the device (book.cu, book.cuh)
struct IterBook;
cudaError_t launch_iter_book(IterBook* b, const double* red, double* add, int* live, int first, cudaStream_t st,
                             int pdl);

}  // namespace mth

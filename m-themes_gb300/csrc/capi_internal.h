// capi_internal.h -- the context structure and the host helpers shared by
// the translation units of the C-ABI (capi*.cu).  Not installed; the public
// interface is include/mth.h.
#pragma once
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <chrono>
#include <map>
#include <string>
#include <thread>
#include <tuple>
#include <vector>
#include "../../include/mth.h"
#include "mth_common.cuh"
#include "mth_internal.h"
#include "book.cuh"
#include "adjoint.h"

using namespace mth;

// Records the message returned by mth_last_error and returns s.
mth_status set_err(mth_status s, const char* fmt, ...);

#define CK(call)                                                                              \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess)                                                                    \
      return set_err(MTH_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                     __FILE__, __LINE__);                                                     \
  } while (0)
#define SETDEV(c) CK(cudaSetDevice((c)->p.device))

// Host-side tensor helpers (FP64) of capi.cu.
namespace capi_host {
typedef double t33[3][3];
void t2v(const t33 t, double* v, int nv);
void v2t(const double* v, t33 t, int nv);
void m2t4(const double c[6][6], double* t);
bool inv6(const double a[6][6], double out[6][6]);
double von_mises(const t33 t);
void voigt_to_full(const double* v, t33 m);
bool radix_ok(int n);
mth_status fill_phase(const mth_phase& in, PhaseConst& ph);
int pkh(int i, int j);
void euler_to_rot(const double* e, double R[9]);
void class_row(const PhaseConst& ph, const double R[9], double* row);
void class_row_add_s0(double* row, const double s066[6][6]);
}  // namespace capi_host
using namespace capi_host;

// ---------------------------------------------------------------- context
constexpr long long MAX_CANDIDATES = 1LL << 20;   // nucleation candidates collected per step
constexpr int MAX_NUCLEI = 65536;                 // nuclei kept per step (first in voxel order)

struct mth_ctx {
  mth_params p;
  int mixed;
  int n[3];
  long long nv;
  FftGeom geom;
  NewtonConst nc;
  GreenConst gc;
  cudaStream_t st;
  int nblocks;
  // device memory
  void* fieldmem;
  Fields<float> ff;
  Fields<double> fd;
  void* spec;
  void* anti;
  TmaMaps* tma;       // tensor maps of the TMA passes (null members: shared-memory passes)
  int* err_d;         // raised by a timed-out wait in a kernel
  int* err_h;         // pinned copy
  double* add_d;      // uniform strain increment of the current Green iteration (6, device)
  double* add_h;      // pinned staging of add_d
  int* live_d;        // live flag read by the iteration kernels (1 outside a batch)
  bool in_batch;      // red, err_d, add_d, live_d and the stream belong to a batch
  bool tma_off;       // shared-memory passes even where tensor maps exist (tuning)
  struct IoutWriter* iout;   // background writer of per-step field files
  double* dl_d;       // download staging in the host layout
  size_t dl_cap;      // doubles
  // state of the mechanical step in progress (mth_step and the batch driver)
  int it_nnew;
  uint8_t* phase_d;
  int* grain_d;
  int* eclass_d;
  double* etab_d;
  float* etabf_d;      // float copy of the class table for the FP32 paths
  int nclass;
  double* partials;
  double* red;
  double* red_h;  // pinned
  void* tw[3][2]; // per axis, forward/inverse
  // profiling
  int prof_on;
  double prof_ms[MTH_PROF_MAX];
  double prof_bytes[MTH_PROF_MAX];
  long long prof_launch[MTH_PROF_MAX];
  std::vector<cudaEvent_t>* ev_pool;
  std::vector<int>* ev_pending;   // class of each pending pair (events 2i, 2i+1)
  // macro state (FP64, host)
  t33 udot, udot_s, udot_a, scauchy;
  int vbc[6], sbc[6], creep;
  t33 disgrad_avg, disgrad_avg_t;
  double c066[6][6], s066[6][6], s0_4[81];
  double wgt, wgt_ph1, e_vm, d_vm, time_tot;
  IterBook bk;        // the step's per-iteration bookkeeping (host copy)
  IterBook* bk_d;     // its device copy (mth_step's device-side bookkeeping)
  int* book_h;        // pinned: live flag, iteration, non-finite flag read after a group of iterations
  bool host_book;     // bookkeeping on the host after every iteration instead (test hook)
  int pdl;            // programmatic dependent launches along the iteration's kernels
  int istep;
  int uploaded;
  // dynamic recrystallisation
  int drx;
  int first_drx_id, next_grain_id;
  std::vector<double>* etab_h;       // host copy of the elastic-class table
  std::vector<double>* drx_rot_h;    // 9 per recrystallised grain
  std::vector<int>* drx_class_h;
  double* drx_rot_d;
  int* drx_class_d;
  int* drx_cnt_d;     // per recrystallised grain: voxels, voxels that joined it this step
  size_t drx_cap;
  PfBuffers<float> pff;
  PfBuffers<double> pfd;
  PfCoef pfc;
  double* rho_d;
  void* rho_t;
  int* grain_prev_d;
  int* winner_d;
  long long* sites_d;
  unsigned long long* count_d;
  uint8_t* crystal_d;
  unsigned long long* hist_d;
  double* gather_d;
  // phase field on a grid of its own (CellDim_pf != CellDim)
  bool pf_resample;
  int npf[3];
  long long nvpf;
  int* grain_pf_d;      // grain ids carried to the PF grid
  double* rho_pf_d;     // rho on the PF grid (FP64)
  void* rho_pf_t;       // rho on the PF grid in the PF precision
  int* gid_coarse_d;    // relaxed ids carried back to the mechanical grid
  size_t hist_cap;
  double tau0f;
  int nsys;
  int adj_solid;        // every voxel is of phase 1 and crystalline (adjoint precondition)
  double last_au[3];    // uniform spin increment of the last end of step
  void* skew_d;         // DisGrad's antisymmetric part, planes (W21, W02, W10), while tracked (mth_track_disgrad)
  // dislocation-density law
  int dd;
  DdConst* ddc;         // phase-1 constants of the dislocation-density law (host; kernel parameters)
  void* dd_mem;         // 84 state planes + 36 per-step constant planes
  DdFields<float> ddf;
  DdFields<double> ddd;
  uint8_t* gb_d;        // same-grain neighbour flags per voxel
  double dd_avg[NPART_DD];
};

struct IoutWriter;
void iout_free(IoutWriter* w);
void ctx_free(mth_ctx* c);
void ctx_set_tiles(mth_ctx* c, int ks, int kg);   // tensor maps with these tile widths

// ------------------------------------------------------------- profiling
enum { K_FFT_Z_R2C = 0, K_FFT_Y, K_FFT_X_GREEN, K_FFT_Z_C2R, K_NEWTON, K_REDUCE, K_END_STEP, K_SPIN, K_SETUP, K_DRX,
       K_PF, K_ADJ_LOCAL, K_ADJ_CG, K_DD, K_BOOK, K_NCLASS };
void prof_begin(mth_ctx* c);
void prof_end(mth_ctx* c, int cls, int kernels, double bytes);
void prof_resolve(mth_ctx* c);   // after the stream has been synchronised
mth_status pf_bad_status(unsigned bad);   // MTH_ERR_UNSUPPORTED naming the exceeded capacities
const char* prof_class_name(int cls);

#define LAUNCHN(cls, kernels, bytes, call)         \
  do {                                             \
    prof_begin(c);                                 \
    cudaError_t e__ = (call);                      \
    prof_end(c, cls, (kernels), (double)(bytes));  \
    if (e__ != cudaSuccess)                        \
      return set_err(MTH_ERR_CUDA, "launch of the %s kernels failed: %s (%s:%d)", prof_class_name(cls), \
                     cudaGetErrorString(e__), __FILE__, __LINE__);                                   \
  } while (0)
#define LAUNCH(cls, bytes, call) LAUNCHN(cls, 1, bytes, call)

// Phases of a mechanical step (capi.cu), shared by mth_step, the batch
// driver and the adjoint.
IterIn iter_in(const mth_ctx* c);
mth_status launch_reduce(mth_ctx* c, int width, bool gated);
mth_status reduce_to_host(mth_ctx* c, int width, double* out);
template <typename T>
mth_status green_iteration(mth_ctx* c);
mth_status step_begin(mth_ctx* c);
bool iter_more(const mth_ctx* c);
void iter_add(mth_ctx* c);
mth_status iter_finish(mth_ctx* c, const double* red);
mth_status step_end(mth_ctx* c, mth_step_report* rep);

// adjoint.h -- device views and launchers of the calibration adjoint.
#pragma once
#include <cuda_runtime.h>
#include "mth_internal.h"

namespace mth {

// Per-step scalars of the reverse sweep.
struct AdjStepArgs {
  double au[3];     // uniform part of the spin increment of the step
  double seed;      // d misfit / d <sigma_33> of the step, divided by the voxel count
  int flow_off, do_orient, do_harden;
};

// Device arrays one reverse step reads and writes (planes of nv values).
template <typename T>
struct AdjViews {
  long long nv;
  // forward snapshot of the step: state before it (rotation, CRSS,
  // accumulated shear), converged stress and local spin after it
  const T* s_sig;
  const T* s_rot;
  const T* s_crss;
  const T* s_gam;
  const T* s_wspin;
  // adjoint of the per-voxel state (FP64): eps_p (6), CRSS (12), accumulated
  // shear (1), rotation vector (3); spin adjoint of the later step (3)
  double* ep;
  double* tau;
  double* gam;
  double* phi;
  double* wnext;
  double* sigbar;   // 6: stress adjoint of the step
  T* ct;            // 16: tangent stiffness (packed 5x5 + hydrostatic)
  T* rhs;           // 9: C_t sigbar (6) and the spin adjoint difference (3)
  const T* mu;      // 6: solution of the projected tangent problem
};

// k = 0 block of the projection: the stress-controlled macroscopic
// components, as a 6x6 matrix in the LT basis.
struct AdjProj {
  double ps[36];
};

template <typename T>
cudaError_t launch_adj_pre(const NewtonConst& nc, const AdjStepArgs& a, const AdjViews<T>& b, const int* eclass,
                           const double* etab, double* partials, cudaStream_t st);
template <typename T>
cudaError_t launch_adj_post(const NewtonConst& nc, const AdjStepArgs& a, const AdjViews<T>& b, double* partials,
                            cudaStream_t st);
cudaError_t launch_adj_sum_tau(const double* tau, int nsys, long long P, double* partials, cudaStream_t st);
template <typename T>
cudaError_t launch_adj_ct_apply(const T* ct, T* p, const T* r, double beta, int update_p, T* out, long long P,
                                cudaStream_t st);
template <typename T>
cudaError_t launch_adj_dot(const T* a, const T* b, long long P, double* partials, cudaStream_t st);
template <typename T>
cudaError_t launch_adj_cg_update(T* x, T* r, const T* p, const T* ap, double alpha, long long P, double* partials,
                                 cudaStream_t st);
// nin = 6: Q f; nin = 9: Q f + W^T w (planes 6..8 of the spectra)
template <typename T>
cudaError_t launch_adj_x_proj(const FftGeom& g, const AdjProj& pj, c2<T>* spec, int nin, const c2<T>* twf,
                              const c2<T>* twi, cudaStream_t st);

}  // namespace mth

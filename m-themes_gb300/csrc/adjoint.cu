// adjoint.cu -- kernels of the calibration adjoint: the per-voxel
// transposed Jacobians (adj_local.cuh), the conjugate-gradient solve of the
// projected tangent problem  Q C_t mu = Q g  and its Fourier-space operators.
//
// Q is the orthogonal projection (in the L2 inner product of LT 6-vectors)
// onto the strain fields the converged Green iteration can reach: at k != 0
// the compatible fields sym(a (x) n) -- at wave vectors with a Nyquist
// component the span of sym(a (x) n) and sym(b (x) m) with n, m the two
// directions the forward Green operator averages (green_op.cuh); at k = 0
// the stress-controlled macroscopic components.  W^T is the transpose of
// the map from the compatible strain increment of a step to the local
// lattice spin that the forward x pass accumulates: W(eps-hat) =
// n x (eps-hat n), so W^T(w-hat) = sym((w-hat x n) (x) n), itself
// compatible.  Both act in the x pass of the forward FFT pipeline
// (fft_green.cu); the z and y passes are the forward's own kernels.
#include <cstdio>
#include "mth_common.cuh"
#include "mth_internal.h"
#include "green_op.cuh"
#include "fft_core.cuh"
#include "fft_smem.cuh"
#include "adj_local.cuh"
#include "adjoint.h"

namespace mth {

// FP64 block sum of W values for 256-thread blocks, one partial per block.
template <int W>
__device__ __forceinline__ void adj_block_sum(double (&v)[W], double* out) {
  // 256-thread blocks, fixed order: the values are staged in shared memory,
  // 16 threads per component each sum 16 of them, one thread per component
  // sums the 16 partials (one DADD per value instead of a shuffle tree in
  // every thread: GB300's FP64 pipe runs at 1/64 of the FP32 rate)
  constexpr int NT = 256;
  static_assert(W <= 16, "at most 16 components");
  __shared__ double sv[W][NT];
  __shared__ double sp[W][16];
  const int t = threadIdx.x;
#pragma unroll
  for (int i = 0; i < W; i++) sv[i][t] = v[i];
  __syncthreads();
  {
    const int comp = t >> 4, chunk = t & 15;
    if (comp < W) {
      double a = 0.0;
#pragma unroll
      for (int k = 0; k < NT / 16; k++) a += sv[comp][k * 16 + chunk];
      sp[comp][chunk] = a;
    }
  }
  __syncthreads();
  if (t < W) {
    double a = 0.0;
#pragma unroll
    for (int k = 0; k < 16; k++) a += sp[t][k];
    out[(size_t)blockIdx.x * W + t] = a;
  }
}

// ----------------------------------------------------- per-voxel kernels
template <typename T>
__global__ void __launch_bounds__(256) adj_pre_kernel(const NewtonConst nc, AdjStepArgs a, AdjViews<T> b,
                                                      const int* __restrict__ eclass, const double* __restrict__ etab,
                                                      double* __restrict__ partials) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long P = b.nv;
  double th[4] = {0, 0, 0, 0};
  if (v < P) {
    const PhaseConst& ph = nc.ph[0];
    adj::StepFlags sf;
    sf.dt = nc.dt;
    for (int i = 0; i < 3; i++) sf.au[i] = a.au[i];
    sf.flow_off = a.flow_off;
    sf.do_orient = a.do_orient;
    sf.do_harden = a.do_harden;
    double sig[6], R[9], tau[NSYS], wsp[3];
    for (int i = 0; i < 6; i++) sig[i] = (double)b.s_sig[i * P + v];
    for (int i = 0; i < 9; i++) R[i] = (double)b.s_rot[i * P + v];
    for (int s = 0; s < NSYS; s++) tau[s] = s < ph.nsys ? (double)b.s_crss[s * P + v] : 1.0;
    const double gam = (double)b.s_gam[v];
    for (int i = 0; i < 3; i++) wsp[i] = a.do_orient ? (double)b.s_wspin[i * P + v] : 0.0;
    adj::AdjState in, out;
    for (int i = 0; i < 6; i++) in.ep[i] = b.ep[i * P + v];
    for (int s = 0; s < NSYS; s++) in.tau[s] = b.tau[s * P + v];
    in.gam = b.gam[v];
    for (int i = 0; i < 3; i++) in.phi[i] = b.phi[i * P + v];
    adj::FlowEval f;
    adj::flow_eval(ph, sig, R, tau, sf.flow_off, f);
    const double seed6[6] = {0.0, a.seed * 2.0 * RSQ6, 0.0, 0.0, 0.0, a.seed * RSQ3};
    double sigbar[6], wbar[3];
    adj::adj_pre(ph, sf, sig, R, gam, wsp, f, in, seed6, out, sigbar, wbar, th);
    const double* row = etab + (size_t)eclass[v] * ETAB_W;
    double ct[16];
    if (!adj::tangent_stiffness(ph, sf, f, row + ET_SEL, row[ET_SEL_HH], ct)) {
      for (int i = 0; i < 16; i++) ct[i] = 0.0;
      th[0] = th[0] + __longlong_as_double(0x7ff8000000000000ULL);   // NaN: reported by the host
    }
    double g6[6];
    adj::ct_apply<double, double>(ct, sigbar, g6);
    for (int i = 0; i < 6; i++) {
      b.ep[i * P + v] = out.ep[i];
      b.sigbar[i * P + v] = sigbar[i];
      b.rhs[i * P + v] = (T)g6[i];
    }
    for (int s = 0; s < NSYS; s++) b.tau[s * P + v] = out.tau[s];
    b.gam[v] = out.gam;
    for (int i = 0; i < 3; i++) {
      b.phi[i * P + v] = out.phi[i];
      b.rhs[(6 + i) * P + v] = (T)(wbar[i] - b.wnext[i * P + v]);
      b.wnext[i * P + v] = wbar[i];
    }
    for (int i = 0; i < 16; i++) b.ct[i * P + v] = (T)ct[i];
  }
  adj_block_sum<4>(th, partials);
}

template <typename T>
__global__ void __launch_bounds__(256) adj_post_kernel(const NewtonConst nc, AdjStepArgs a, AdjViews<T> b,
                                                       double* __restrict__ partials) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long P = b.nv;
  double th[4] = {0, 0, 0, 0};
  if (v < P) {
    const PhaseConst& ph = nc.ph[0];
    adj::StepFlags sf;
    sf.dt = nc.dt;
    for (int i = 0; i < 3; i++) sf.au[i] = a.au[i];
    sf.flow_off = a.flow_off;
    sf.do_orient = a.do_orient;
    sf.do_harden = a.do_harden;
    double sig[6], R[9], tau[NSYS];
    for (int i = 0; i < 6; i++) sig[i] = (double)b.s_sig[i * P + v];
    for (int i = 0; i < 9; i++) R[i] = (double)b.s_rot[i * P + v];
    for (int s = 0; s < NSYS; s++) tau[s] = s < ph.nsys ? (double)b.s_crss[s * P + v] : 1.0;
    adj::FlowEval f;
    adj::flow_eval(ph, sig, R, tau, sf.flow_off, f);
    double ct[16], d[6], qbar[6];
    for (int i = 0; i < 16; i++) ct[i] = (double)b.ct[i * P + v];
    for (int i = 0; i < 6; i++) d[i] = (double)b.mu[i * P + v] - b.sigbar[i * P + v];
    adj::ct_apply<double, double>(ct, d, qbar);
    adj::AdjState st;
    for (int i = 0; i < 6; i++) st.ep[i] = b.ep[i * P + v];
    for (int s = 0; s < NSYS; s++) st.tau[s] = b.tau[s * P + v];
    st.gam = b.gam[v];
    for (int i = 0; i < 3; i++) st.phi[i] = b.phi[i * P + v];
    adj::adj_post(ph, sf, sig, f, qbar, st, th);
    for (int i = 0; i < 6; i++) b.ep[i * P + v] = st.ep[i];
    for (int s = 0; s < NSYS; s++) b.tau[s * P + v] = st.tau[s];
    for (int i = 0; i < 3; i++) b.phi[i * P + v] = st.phi[i];
  }
  adj_block_sum<4>(th, partials);
}

// sum over voxels and active systems of the CRSS adjoint (d/d tau0)
__global__ void __launch_bounds__(256) adj_sum_tau_kernel(const double* __restrict__ tau, int nsys, long long P,
                                                          double* __restrict__ partials) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double s[1] = {0.0};
  if (v < P)
    for (int k = 0; k < nsys; k++) s[0] += tau[k * P + v];
  adj_block_sum<1>(s, partials);
}

// ------------------------------------------------------------ CG kernels
// update_p: p = r + beta p first; then out = C_t p.
template <typename T>
__global__ void __launch_bounds__(256) adj_ct_apply_kernel(const T* __restrict__ ct, T* __restrict__ p,
                                                           const T* __restrict__ r, T beta, int update_p,
                                                           T* __restrict__ out, long long P) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= P) return;
  T x[6], c[16], y[6];
#pragma unroll
  for (int i = 0; i < 6; i++) {
    T pv = p[i * P + v];
    if (update_p) {
      pv = r[i * P + v] + beta * pv;
      p[i * P + v] = pv;
    }
    x[i] = pv;
  }
#pragma unroll
  for (int i = 0; i < 16; i++) c[i] = ct[i * P + v];
  adj::ct_apply<T, T>(c, x, y);
#pragma unroll
  for (int i = 0; i < 6; i++) out[i * P + v] = y[i];
}

template <typename T>
__global__ void __launch_bounds__(256) adj_dot_kernel(const T* __restrict__ a, const T* __restrict__ b, long long P,
                                                      double* __restrict__ partials) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double s[1] = {0.0};
  if (v < P)
#pragma unroll
    for (int i = 0; i < 6; i++) s[0] += to_f64(a[i * P + v]) * to_f64(b[i * P + v]);   // exact products
  adj_block_sum<1>(s, partials);
}

// x += alpha p ; r -= alpha Ap ; partial |r|^2
template <typename T>
__global__ void __launch_bounds__(256) adj_cg_update_kernel(T* __restrict__ x, T* __restrict__ r, const T* __restrict__ p,
                                                            const T* __restrict__ ap, T alpha, long long P,
                                                            double* __restrict__ partials) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double s[1] = {0.0};
  if (v < P)
#pragma unroll
    for (int i = 0; i < 6; i++) {
      const long long o = i * P + v;
      x[o] += alpha * p[o];
      const T rv = r[o] - alpha * ap[o];
      r[o] = rv;
      s[0] += to_f64(rv) * to_f64(rv);
    }
  adj_block_sum<1>(s, partials);
}

// --------------------------------------------------- Fourier projection
// f (6 LT complex) -> Q f at wave vector (kx, ky, kz); with NIN == 9 the
// three further inputs w are the spin adjoint and W^T w is added.
template <typename T>
__device__ __forceinline__ void proj_point(const AdjProj& pj, int kx, int ky, int kz, int n0, int n1, int n2,
                                           const c2<T>* in, int nin, c2<T> out[6]) {
  if (kx == 0 && ky == 0 && kz == 0) {
    for (int i = 0; i < 6; i++) {
      T re = 0, im = 0;
      for (int j = 0; j < 6; j++) {
        re += (T)pj.ps[i * 6 + j] * in[j].x;
        im += (T)pj.ps[i * 6 + j] * in[j].y;
      }
      out[i] = mk<T>(re, im);
    }
    return;
  }
  T fr[3][3], fi[3][3];
  {
    T re[6], im[6];
#pragma unroll
    for (int i = 0; i < 6; i++) { re[i] = in[i].x; im[i] = in[i].y; }
    lt_to_cart<T>(re, fr);
    lt_to_cart<T>(im, fi);
  }
  T f[3] = {freq<T>(kx, n0), freq<T>(ky, n1), freq<T>(kz, n2)};
  const bool q0 = (2 * kx == n0), q1 = (2 * ky == n1), q2 = (2 * kz == n2);
  const T nrm = sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
  const T n[3] = {f[0] / nrm, f[1] / nrm, f[2] / nrm};
  const bool anyq = q0 || q1 || q2;
  const bool anyv = (!q0 && kx != 0) || (!q1 && ky != 0) || (!q2 && kz != 0);
  T orr[3][3], oi[3][3];
  if (anyq && anyv) {
    // complement of the reachable space: c (x) c, c = n x m / |n x m|
    const T m[3] = {q0 ? n[0] : -n[0], q1 ? n[1] : -n[1], q2 ? n[2] : -n[2]};
    T c[3] = {n[1] * m[2] - n[2] * m[1], n[2] * m[0] - n[0] * m[2], n[0] * m[1] - n[1] * m[0]};
    const T cn = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
#pragma unroll
    for (int i = 0; i < 3; i++) c[i] /= cn;
    T sr = 0, si = 0;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        sr += c[i] * fr[i][j] * c[j];
        si += c[i] * fi[i][j] * c[j];
      }
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        orr[i][j] = fr[i][j] - sr * c[i] * c[j];
        oi[i][j] = fi[i][j] - si * c[i] * c[j];
      }
  } else {
    // sym(a (x) n), a = 2 f n - (n f n) n
    T fnr[3], fni[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
      fnr[i] = fr[i][0] * n[0] + fr[i][1] * n[1] + fr[i][2] * n[2];
      fni[i] = fi[i][0] * n[0] + fi[i][1] * n[1] + fi[i][2] * n[2];
    }
    const T nnr = n[0] * fnr[0] + n[1] * fnr[1] + n[2] * fnr[2];
    const T nni = n[0] * fni[0] + n[1] * fni[1] + n[2] * fni[2];
    T ar[3], ai[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
      ar[i] = (T)2 * fnr[i] - nnr * n[i];
      ai[i] = (T)2 * fni[i] - nni * n[i];
    }
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        orr[i][j] = (T)0.5 * (ar[i] * n[j] + ar[j] * n[i]);
        oi[i][j] = (T)0.5 * (ai[i] * n[j] + ai[j] * n[i]);
      }
  }
  if (nin == 9) {
    // + sym((w x n) (x) n)
    const c2<T>* w = in + 6;
    const T ar[3] = {w[1].x * n[2] - w[2].x * n[1], w[2].x * n[0] - w[0].x * n[2], w[0].x * n[1] - w[1].x * n[0]};
    const T ai[3] = {w[1].y * n[2] - w[2].y * n[1], w[2].y * n[0] - w[0].y * n[2], w[0].y * n[1] - w[1].y * n[0]};
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        orr[i][j] += (T)0.5 * (ar[i] * n[j] + ar[j] * n[i]);
        oi[i][j] += (T)0.5 * (ai[i] * n[j] + ai[j] * n[i]);
      }
  }
  T vr[6], vi[6];
  cart_to_lt<T>(orr, vr);
  cart_to_lt<T>(oi, vi);
#pragma unroll
  for (int i = 0; i < 6; i++) out[i] = mk<T>(vr[i], vi[i]);
}

// Forward x transform of nin spectra, the projection per k, inverse x
// transform of the 6 results (written to planes 0..5).  One block: fixed y,
// kb consecutive kz, as fft_x_green_kernel.
template <typename T, int NC>
__global__ void __launch_bounds__(256) adj_x_proj_kernel(const AdjProj pj, c2<T>* __restrict__ spec, int nin,
                                                         long long kplane, int n0_, int n1, int n2, int kzn, int kzs,
                                                         int kb, FftPlan pl, const c2<T>* __restrict__ twf,
                                                         const c2<T>* __restrict__ twi) {
  const int n0 = NC > 0 ? NC : n0_;
  extern __shared__ unsigned char smraw[];
  c2<T>* tw_f = reinterpret_cast<c2<T>*>(smraw);
  c2<T>* tw_i = tw_f + n0;
  const int ls = n0 + 1;
  c2<T>* d0 = tw_i + n0;
  c2<T>* d1 = d0 + nin * kb * ls;
  const int k0 = blockIdx.x * kb;
  const int y = blockIdx.y;
  const long long S = (long long)n1 * kzs;
  const long long base = (long long)y * kzs + k0;
  load_twiddles<T>(tw_f, twf, n0);
  load_twiddles<T>(tw_i, twi, n0);
  for (int idx = threadIdx.x; idx < nin * n0 * kb; idx += blockDim.x) {
    const int kk = idx % kb;
    const int e = (idx / kb) % n0;
    const int c = idx / (kb * n0);
    c2<T> v = mk<T>(0, 0);
    if (k0 + kk < kzn) v = spec[c * kplane + base + e * S + kk];
    d0[(c * kb + kk) * ls + e] = v;
  }
  __syncthreads();
  c2<T>* r = do_fft<T, NC>(d0, d1, n0, ls, nin * kb, pl, tw_f, -1);
  c2<T>* other = (r == d0) ? d1 : d0;
  for (int idx = threadIdx.x; idx < n0 * kb; idx += blockDim.x) {
    const int kk = idx % kb;
    const int kx = idx / kb;
    if (k0 + kk >= kzn) continue;
    c2<T> s[9], o[6];
    for (int c = 0; c < nin; c++) s[c] = r[(c * kb + kk) * ls + kx];
    proj_point<T>(pj, kx, y, k0 + kk, n0, n1, n2, s, nin, o);
#pragma unroll
    for (int c = 0; c < 6; c++) r[(c * kb + kk) * ls + kx] = o[c];
  }
  __syncthreads();
  c2<T>* r2 = do_fft<T, NC>(r, other, n0, ls, 6 * kb, pl, tw_i, +1);
  for (int idx = threadIdx.x; idx < 6 * n0 * kb; idx += blockDim.x) {
    const int kk = idx % kb;
    const int e = (idx / kb) % n0;
    const int c = idx / (kb * n0);
    if (k0 + kk < kzn) spec[c * kplane + base + e * S + kk] = r2[(c * kb + kk) * ls + e];
  }
}

// ------------------------------------------------------------ launchers
static int blocks_of(long long P) { return (int)((P + 255) / 256); }

template <typename T>
cudaError_t launch_adj_pre(const NewtonConst& nc, const AdjStepArgs& a, const AdjViews<T>& b, const int* eclass,
                           const double* etab, double* partials, cudaStream_t st) {
  adj_pre_kernel<T><<<blocks_of(b.nv), 256, 0, st>>>(nc, a, b, eclass, etab, partials);
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch_adj_post(const NewtonConst& nc, const AdjStepArgs& a, const AdjViews<T>& b, double* partials,
                            cudaStream_t st) {
  adj_post_kernel<T><<<blocks_of(b.nv), 256, 0, st>>>(nc, a, b, partials);
  return cudaGetLastError();
}
cudaError_t launch_adj_sum_tau(const double* tau, int nsys, long long P, double* partials, cudaStream_t st) {
  adj_sum_tau_kernel<<<blocks_of(P), 256, 0, st>>>(tau, nsys, P, partials);
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch_adj_ct_apply(const T* ct, T* p, const T* r, double beta, int update_p, T* out, long long P,
                                cudaStream_t st) {
  adj_ct_apply_kernel<T><<<blocks_of(P), 256, 0, st>>>(ct, p, r, (T)beta, update_p, out, P);
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch_adj_dot(const T* a, const T* b, long long P, double* partials, cudaStream_t st) {
  adj_dot_kernel<T><<<blocks_of(P), 256, 0, st>>>(a, b, P, partials);
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch_adj_cg_update(T* x, T* r, const T* p, const T* ap, double alpha, long long P, double* partials,
                                 cudaStream_t st) {
  adj_cg_update_kernel<T><<<blocks_of(P), 256, 0, st>>>(x, r, p, ap, (T)alpha, P, partials);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_adj_x_proj(const FftGeom& g, const AdjProj& pj, c2<T>* spec, int nin, const c2<T>* twf,
                              const c2<T>* twi, cudaStream_t st) {
  int kb = 16;
  auto smem = [&](int kbv) { return sizeof(c2<T>) * ((size_t)2 * g.n0 + 2 * (size_t)nin * kbv * (g.n0 + 1)); };
  while (kb > 1 && smem(kb) > g.smem_budget) kb >>= 1;
  const size_t sm = smem(kb);
  auto k = adj_x_proj_kernel<T, 0>;
  switch (g.n0) {
#define MTH_CASE(N) case N: k = adj_x_proj_kernel<T, N>; break;
    MTH_CASE(16) MTH_CASE(32) MTH_CASE(48) MTH_CASE(64) MTH_CASE(96) MTH_CASE(128) MTH_CASE(256)
#undef MTH_CASE
    default: break;
  }
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  dim3 grid((g.kz + kb - 1) / kb, g.n1);
  k<<<grid, 256, sm, st>>>(pj, spec, nin, g.kplane, g.n0, g.n1, g.n2, g.kz, g.kzs, kb, g.px, twf, twi);
  return cudaGetLastError();
}

#define INST(T)                                                                                                   \
  template cudaError_t launch_adj_pre<T>(const NewtonConst&, const AdjStepArgs&, const AdjViews<T>&, const int*,  \
                                         const double*, double*, cudaStream_t);                                    \
  template cudaError_t launch_adj_post<T>(const NewtonConst&, const AdjStepArgs&, const AdjViews<T>&, double*,    \
                                          cudaStream_t);                                                           \
  template cudaError_t launch_adj_ct_apply<T>(const T*, T*, const T*, double, int, T*, long long, cudaStream_t); \
  template cudaError_t launch_adj_dot<T>(const T*, const T*, long long, double*, cudaStream_t);                   \
  template cudaError_t launch_adj_cg_update<T>(T*, T*, const T*, const T*, double, long long, double*,            \
                                               cudaStream_t);                                                      \
  template cudaError_t launch_adj_x_proj<T>(const FftGeom&, const AdjProj&, c2<T>*, int, const c2<T>*,          \
                                            const c2<T>*, cudaStream_t);
INST(float)
INST(double)
#undef INST

}  // namespace mth

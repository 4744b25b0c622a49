// fft_green.cu -- 3-D real FFT passes and the fused Green-operator pass.
//
// Replaces the 9+9 FFTW-MPI transforms and the GAMMA contraction of one
// Green iteration (src/evolution.c:1361-1405, GAMMA from src/init.c:541-591).
// Every pass is a batch of 1-D transforms done in shared memory with a
// mixed-radix (4/2/3) Stockham autosort, so each line is read from and
// written to HBM exactly once per pass:
//   fft_z_r2c   : 6 real stress planes -> 6 half spectra along z (two real
//                 lines packed per complex transform)
//   fft_strided : complex lines along y or x, in place (forward/inverse)
//   fft_x_green : forward x transform, Gamma0 applied at every k, antisymmetric
//                 part accumulated for the lattice spin, inverse x transform
//   fft_z_c2r   : half spectra -> real planes, fused with the strain update
//                 DisGrad += dDisGradAvg + Re(.)/Nxyz of src/evolution.c:1402
#include <cstdio>
#include "mth_common.cuh"
#include "mth_internal.h"
#include "green_op.cuh"
#include "fft_core.cuh"
#include "fft_smem.cuh"

namespace mth {

// ------------------------------------------------------------- z passes
// One block: lb consecutive (x,y) lines, npair = ceil(ncomp/2) packed
// transforms per line.
template <typename T, int NC>
__global__ void __launch_bounds__(256) fft_z_r2c_kernel(const T* __restrict__ in, c2<T>* __restrict__ out, int ncomp,
                                                        long long plane, long long kplane, int nlines, int n2_,
                                                        int kzs, int lb, FftPlan pl, const c2<T>* __restrict__ twg,
                                                        IterIn it) {
  if (!is_live(it)) return;
  const int n2 = NC > 0 ? NC : n2_;
  extern __shared__ unsigned char smraw[];
  c2<T>* tw = reinterpret_cast<c2<T>*>(smraw);
  const int npair = (ncomp + 1) / 2;
  const int ls = n2 + 1;
  c2<T>* d0 = tw + n2;
  c2<T>* d1 = d0 + npair * lb * ls;
  const int line0 = blockIdx.x * lb;
  const int nl_here = min(lb, nlines - line0);
  load_twiddles<T>(tw, twg, n2);
  for (int idx = threadIdx.x; idx < npair * lb * n2; idx += blockDim.x) {
    const int z = idx % n2;
    const int l = (idx / n2) % lb;
    const int p = idx / (n2 * lb);
    T a = 0, b = 0;
    if (l < nl_here) {
      const long long o = (long long)(line0 + l) * n2 + z;
      a = in[(2 * p) * plane + o];
      if (2 * p + 1 < ncomp) b = in[(2 * p + 1) * plane + o];
    }
    d0[(p * lb + l) * ls + z] = mk<T>(a, b);
  }
  __syncthreads();
  c2<T>* r = do_fft<T, NC>(d0, d1, n2, ls, npair * lb, pl, tw, -1);
  const int kz = n2 / 2 + 1;
  for (int idx = threadIdx.x; idx < npair * lb * kz; idx += blockDim.x) {
    const int k = idx % kz;
    const int l = (idx / kz) % lb;
    const int p = idx / (kz * lb);
    if (l >= nl_here) continue;
    const c2<T>* X = r + (p * lb + l) * ls;
    c2<T> xk = X[k], xm = X[(n2 - k) % n2];
    // A = (X[k] + conj(X[-k]))/2 ; B = -i (X[k] - conj(X[-k]))/2
    c2<T> A = mk<T>((T)0.5 * (xk.x + xm.x), (T)0.5 * (xk.y - xm.y));
    c2<T> B = mk<T>((T)0.5 * (xk.y + xm.y), (T)-0.5 * (xk.x - xm.x));
    const long long o = (long long)(line0 + l) * kzs + k;
    out[(2 * p) * kplane + o] = A;
    if (2 * p + 1 < ncomp) out[(2 * p + 1) * kplane + o] = B;
  }
}

// mode 0: field = val*scale + add ; mode 1: field += val*scale + add
template <typename T, int NC>
__global__ void __launch_bounds__(256) fft_z_c2r_kernel(const c2<T>* __restrict__ spec, T* __restrict__ field, int ncomp,
                                                        long long plane, long long kplane, int nlines, int n2_,
                                                        int kzs, int lb, FftPlan pl, const c2<T>* __restrict__ twg, T scale,
                                                        IterIn it, int mode) {
  if (!is_live(it)) return;
  const int n2 = NC > 0 ? NC : n2_;
  extern __shared__ unsigned char smraw[];
  c2<T>* tw = reinterpret_cast<c2<T>*>(smraw);
  const int npair = (ncomp + 1) / 2;
  const int ls = n2 + 1;
  c2<T>* d0 = tw + n2;
  c2<T>* d1 = d0 + npair * lb * ls;
  const int line0 = blockIdx.x * lb;
  const int nl_here = min(lb, nlines - line0);
  const int kz = n2 / 2 + 1;
  load_twiddles<T>(tw, twg, n2);
  for (int idx = threadIdx.x; idx < npair * lb * kz; idx += blockDim.x) {
    const int k = idx % kz;
    const int l = (idx / kz) % lb;
    const int p = idx / (kz * lb);
    c2<T> A = mk<T>(0, 0), B = mk<T>(0, 0);
    if (l < nl_here) {
      const long long o = (long long)(line0 + l) * kzs + k;
      A = spec[(2 * p) * kplane + o];
      if (2 * p + 1 < ncomp) B = spec[(2 * p + 1) * kplane + o];
    }
    if (k == 0 || 2 * k == n2) { A.y = 0; B.y = 0; }
    c2<T>* X = d0 + (p * lb + l) * ls;
    X[k] = mk<T>(A.x - B.y, A.y + B.x);                       // A + iB
    if (k > 0 && 2 * k < n2) X[n2 - k] = mk<T>(A.x + B.y, -A.y + B.x);  // conj(A) + i conj(B)
  }
  __syncthreads();
  c2<T>* r = do_fft<T, NC>(d0, d1, n2, ls, npair * lb, pl, tw, +1);
  __shared__ T addv[6];
  if (threadIdx.x < 6) addv[threadIdx.x] = it.add ? (T)it.add[threadIdx.x] : (T)0;
  __syncthreads();
  for (int idx = threadIdx.x; idx < ncomp * lb * n2; idx += blockDim.x) {
    const int z = idx % n2;
    const int l = (idx / n2) % lb;
    const int c = idx / (n2 * lb);
    if (l >= nl_here) continue;
    const c2<T> X = r[((c >> 1) * lb + l) * ls + z];
    const T val = (c & 1) ? X.y : X.x;
    const long long o = (long long)c * plane + (long long)(line0 + l) * n2 + z;
    const T v = val * scale + addv[c];
    if (mode == 0) field[o] = v;
    else field[o] += v;
  }
}

// ------------------------------------------------------- strided passes
// Lines along a dimension of length L with element stride S (in complex
// elements); the block covers kb consecutive kz and one outer index.
// base(outer) = outer * ostride.
template <typename T, int NC>
__global__ void __launch_bounds__(256) fft_strided_kernel(c2<T>* __restrict__ spec, int ncomp, long long kplane,
                                                          int L_, long long S, long long ostride, int kzn, int kb,
                                                          FftPlan pl, const c2<T>* __restrict__ twg, int sign, IterIn it) {
  if (!is_live(it)) return;
  const int L = NC > 0 ? NC : L_;
  extern __shared__ unsigned char smraw[];
  c2<T>* tw = reinterpret_cast<c2<T>*>(smraw);
  const int ls = L + 1;
  const int nl = ncomp * kb;
  c2<T>* d0 = tw + L;
  c2<T>* d1 = d0 + nl * ls;
  const int k0 = blockIdx.x * kb;
  const long long base = (long long)blockIdx.y * ostride + k0;
  load_twiddles<T>(tw, twg, L);
  for (int idx = threadIdx.x; idx < ncomp * L * kb; idx += blockDim.x) {
    const int kk = idx % kb;
    const int e = (idx / kb) % L;
    const int c = idx / (kb * L);
    c2<T> v = mk<T>(0, 0);
    if (k0 + kk < kzn) v = spec[c * kplane + base + e * S + kk];
    d0[(c * kb + kk) * ls + e] = v;
  }
  __syncthreads();
  c2<T>* r = do_fft<T, NC>(d0, d1, L, ls, nl, pl, tw, sign);
  for (int idx = threadIdx.x; idx < ncomp * L * kb; idx += blockDim.x) {
    const int kk = idx % kb;
    const int e = (idx / kb) % L;
    const int c = idx / (kb * L);
    if (k0 + kk < kzn) spec[c * kplane + base + e * S + kk] = r[(c * kb + kk) * ls + e];
  }
}

// x pass fused with Gamma0: forward transform along x of the 6 stress
// spectra, Delta = Gamma0 : sigma-hat per k, antisymmetric part added to
// the spin accumulator, inverse transform along x.  One block: fixed y,
// kb consecutive kz.
template <typename T, int NC>
__global__ void __launch_bounds__(256) fft_x_green_kernel(const GreenConst gc, c2<T>* __restrict__ spec, c2<T>* __restrict__ anti_acc,
                                                          long long kplane, int n0_, int n1, int n2, int kzn, int kzs, int kb,
                                                          FftPlan pl, const c2<T>* __restrict__ twf,
                                                          const c2<T>* __restrict__ twi, IterIn it) {
  if (!is_live(it)) return;
  const int n0 = NC > 0 ? NC : n0_;
  extern __shared__ unsigned char smraw[];
  c2<T>* tw_f = reinterpret_cast<c2<T>*>(smraw);
  c2<T>* tw_i = tw_f + n0;
  const int ls = n0 + 1;
  const int nl = 6 * kb;
  c2<T>* d0 = tw_i + n0;
  c2<T>* d1 = d0 + nl * ls;
  const int k0 = blockIdx.x * kb;
  const int y = blockIdx.y;
  const long long S = (long long)n1 * kzs;
  const long long base = (long long)y * kzs + k0;
  load_twiddles<T>(tw_f, twf, n0);
  load_twiddles<T>(tw_i, twi, n0);
  for (int idx = threadIdx.x; idx < 6 * n0 * kb; idx += blockDim.x) {
    const int kk = idx % kb;
    const int e = (idx / kb) % n0;
    const int c = idx / (kb * n0);
    c2<T> v = mk<T>(0, 0);
    if (k0 + kk < kzn) v = spec[c * kplane + base + e * S + kk];
    d0[(c * kb + kk) * ls + e] = v;
  }
  __syncthreads();
  c2<T>* r = do_fft<T, NC>(d0, d1, n0, ls, nl, pl, tw_f, -1);
  c2<T>* other = (r == d0) ? d1 : d0;
  for (int idx = threadIdx.x; idx < n0 * kb; idx += blockDim.x) {
    const int kk = idx % kb;
    const int kx = idx / kb;
    if (k0 + kk >= kzn) continue;
    c2<T> s[6], a[3];
#pragma unroll
    for (int c = 0; c < 6; c++) s[c] = r[(c * kb + kk) * ls + kx];
    green_point<T>(gc, kx, y, k0 + kk, n0, n1, n2, s, a);
#pragma unroll
    for (int c = 0; c < 6; c++) r[(c * kb + kk) * ls + kx] = s[c];
    const long long o = base + kx * S + kk;
#pragma unroll
    for (int c = 0; c < 3; c++) anti_acc[c * kplane + o] = cadd<T>(anti_acc[c * kplane + o], a[c]);
  }
  __syncthreads();
  c2<T>* r2 = do_fft<T, NC>(r, other, n0, ls, nl, pl, tw_i, +1);
  for (int idx = threadIdx.x; idx < 6 * n0 * kb; idx += blockDim.x) {
    const int kk = idx % kb;
    const int e = (idx / kb) % n0;
    const int c = idx / (kb * n0);
    if (k0 + kk < kzn) spec[c * kplane + base + e * S + kk] = r2[(c * kb + kk) * ls + e];
  }
}

// ------------------------------------------------------------ launchers
// line lengths with compile-time kernels; other even 2^a 3^b lengths use the
// runtime-plan kernels
#define MTH_CT_SIZES(X) X(16) X(32) X(48) X(64) X(96) X(128) X(256)

static size_t z_smem(int n2, int npair, int lb, size_t esz) { return (size_t)esz * (n2 + 2 * npair * lb * (n2 + 1)); }

template <typename T>
static int pick_lb(int n2, int npair, int nlines, size_t budget) {
  int lb = 16;
  while (lb > 1 && z_smem(n2, npair, lb, sizeof(c2<T>)) > budget) lb >>= 1;
  if (lb > nlines) lb = nlines;
  return lb;
}

template <typename T>
cudaError_t launch_fft_z_r2c(const FftGeom& g, const T* in, c2<T>* out, int ncomp, const c2<T>* tw, const IterIn& it,
                             cudaStream_t st) {
  const int npair = (ncomp + 1) / 2;
  const int nlines = g.n0 * g.n1;
  const int lb = pick_lb<T>(g.n2, npair, nlines, g.smem_budget);
  const size_t sm = z_smem(g.n2, npair, lb, sizeof(c2<T>));
  auto k = fft_z_r2c_kernel<T, 0>;
  switch (g.n2) {
#define MTH_CASE(N) case N: k = fft_z_r2c_kernel<T, N>; break;
    MTH_CT_SIZES(MTH_CASE)
#undef MTH_CASE
    default: break;
  }
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k<<<(nlines + lb - 1) / lb, 256, sm, st>>>(in, out, ncomp, g.plane, g.kplane, nlines, g.n2, g.kzs, lb, g.pz, tw, it);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_fft_z_c2r(const FftGeom& g, const c2<T>* spec, T* field, int ncomp, const c2<T>* tw, T scale,
                             const IterIn& it, int mode, cudaStream_t st) {
  const int npair = (ncomp + 1) / 2;
  const int nlines = g.n0 * g.n1;
  const int lb = pick_lb<T>(g.n2, npair, nlines, g.smem_budget);
  const size_t sm = z_smem(g.n2, npair, lb, sizeof(c2<T>));
  auto k = fft_z_c2r_kernel<T, 0>;
  switch (g.n2) {
#define MTH_CASE(N) case N: k = fft_z_c2r_kernel<T, N>; break;
    MTH_CT_SIZES(MTH_CASE)
#undef MTH_CASE
    default: break;
  }
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k<<<(nlines + lb - 1) / lb, 256, sm, st>>>(spec, field, ncomp, g.plane, g.kplane, nlines, g.n2, g.kzs, lb, g.pz,
                                             tw, scale, it, mode);
  return cudaGetLastError();
}

static size_t s_smem(int L, int nl, size_t esz, int ntw) { return esz * ((size_t)ntw * L + 2 * (size_t)nl * (L + 1)); }

template <typename T>
static int pick_kb(int L, int ncomp, size_t budget, int ntw) {
  int kb = 16;
  while (kb > 1 && s_smem(L, ncomp * kb, sizeof(c2<T>), ntw) > budget) kb >>= 1;
  return kb;
}

// axis 1 (y) or 0 (x)
template <typename T>
cudaError_t launch_fft_strided(const FftGeom& g, c2<T>* spec, int ncomp, int axis, int sign, const c2<T>* tw,
                               const IterIn& it, cudaStream_t st) {
  const int L = axis == 1 ? g.n1 : g.n0;
  const long long S = axis == 1 ? g.kzs : (long long)g.n1 * g.kzs;
  const long long ostride = axis == 1 ? (long long)g.n1 * g.kzs : g.kzs;
  const int nouter = axis == 1 ? g.n0 : g.n1;
  const FftPlan& pl = axis == 1 ? g.py : g.px;
  const int kb = pick_kb<T>(L, ncomp, g.smem_budget, 1);
  const size_t sm = s_smem(L, ncomp * kb, sizeof(c2<T>), 1);
  auto k = fft_strided_kernel<T, 0>;
  switch (L) {
#define MTH_CASE(N) case N: k = fft_strided_kernel<T, N>; break;
    MTH_CT_SIZES(MTH_CASE)
#undef MTH_CASE
    default: break;
  }
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  dim3 grid((g.kz + kb - 1) / kb, nouter);
  k<<<grid, 256, sm, st>>>(spec, ncomp, g.kplane, L, S, ostride, g.kz, kb, pl, tw, sign, it);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_fft_x_green(const FftGeom& g, const GreenConst& gc, c2<T>* spec, c2<T>* anti, const c2<T>* twf,
                               const c2<T>* twi, const IterIn& it, cudaStream_t st) {
  const int kb = pick_kb<T>(g.n0, 6, g.smem_budget, 2);
  const size_t sm = s_smem(g.n0, 6 * kb, sizeof(c2<T>), 2);
  auto k = fft_x_green_kernel<T, 0>;
  switch (g.n0) {
#define MTH_CASE(N) case N: k = fft_x_green_kernel<T, N>; break;
    MTH_CT_SIZES(MTH_CASE)
#undef MTH_CASE
    default: break;
  }
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  dim3 grid((g.kz + kb - 1) / kb, g.n1);
  k<<<grid, 256, sm, st>>>(gc, spec, anti, g.kplane, g.n0, g.n1, g.n2, g.kz, g.kzs, kb, g.px, twf, twi, it);
  return cudaGetLastError();
}

#define INST(T)                                                                                                      \
  template cudaError_t launch_fft_z_r2c<T>(const FftGeom&, const T*, c2<T>*, int, const c2<T>*, const IterIn&,     \
                                           cudaStream_t);                                                            \
  template cudaError_t launch_fft_z_c2r<T>(const FftGeom&, const c2<T>*, T*, int, const c2<T>*, T, const IterIn&, int, \
                                           cudaStream_t);                                                            \
  template cudaError_t launch_fft_strided<T>(const FftGeom&, c2<T>*, int, int, int, const c2<T>*, const IterIn&,      \
                                             cudaStream_t);                                                          \
  template cudaError_t launch_fft_x_green<T>(const FftGeom&, const GreenConst&, c2<T>*, c2<T>*, const c2<T>*, const c2<T>*, \
                                            const IterIn&, cudaStream_t);
INST(float)
INST(double)
#undef INST

}  // namespace mth

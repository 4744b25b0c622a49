// fft_smem.cuh -- batched 1-D FFTs in shared memory (mixed radix 4/2/3,
// Stockham autosort), shared by the Green-iteration passes and the adjoint's
// projection pass.
#pragma once
#include "mth_common.cuh"
#include "mth_internal.h"
#include "fft_core.cuh"

namespace mth {

// ---------------------------------------------------------------- smem FFT
// Stockham autosort over nl lines of length n stored at d0 + l*ls.  Stage s
// with radix R takes element j + r*n/R, multiplies by W^(k*r) (k = j mod Ns,
// W = exp(sign*2*pi*i/(Ns*R))), does an R-point DFT and writes element
// (j/Ns)*Ns*R + k + r*Ns.  The result is in d0 or d1 (returned).
template <typename T>
__device__ c2<T>* smem_fft(c2<T>* d0, c2<T>* d1, int n, int ls, int nl, const FftPlan& pl, const c2<T>* tw,
                           int sign) {
  int Ns = 1;
  for (int s = 0; s < pl.nst; s++) {
    const int R = pl.radix[s];
    const int nb = n / R;
    const int total = nl * nb;
    const int twstep = n / (Ns * R);
    for (int w = threadIdx.x; w < total; w += blockDim.x) {
      const int l = w / nb, j = w - l * nb;
      const c2<T>* in = d0 + l * ls;
      c2<T>* out = d1 + l * ls;
      const int k = j % Ns;
      c2<T> v[4];
#pragma unroll
      for (int r = 0; r < 4; r++) {
        if (r < R) {
          v[r] = in[j + r * nb];
          if (r) v[r] = cmul<T>(v[r], tw[k * r * twstep]);
        }
      }
      if (R == 2) {
        c2<T> a = v[0], b = v[1];
        v[0] = cadd<T>(a, b);
        v[1] = csub<T>(a, b);
      } else if (R == 4) {
        c2<T> s02 = cadd<T>(v[0], v[2]), d02 = csub<T>(v[0], v[2]);
        c2<T> s13 = cadd<T>(v[1], v[3]), d13 = csub<T>(v[1], v[3]);
        // W = sign*i ; W*d13
        c2<T> wd = mk<T>(-(T)sign * d13.y, (T)sign * d13.x);
        v[0] = cadd<T>(s02, s13);
        v[2] = csub<T>(s02, s13);
        v[1] = cadd<T>(d02, wd);
        v[3] = csub<T>(d02, wd);
      } else {  // R == 3
        const T h = (T)0.86602540378443864676 * (T)sign;
        c2<T> t = cadd<T>(v[1], v[2]), u = csub<T>(v[1], v[2]);
        c2<T> m = mk<T>(v[0].x - (T)0.5 * t.x, v[0].y - (T)0.5 * t.y);
        c2<T> iu = mk<T>(-h * u.y, h * u.x);
        v[0] = cadd<T>(v[0], t);
        v[1] = cadd<T>(m, iu);
        v[2] = csub<T>(m, iu);
      }
      const int idxD = (j / Ns) * Ns * R + k;
#pragma unroll
      for (int r = 0; r < 4; r++)
        if (r < R) out[idxD + r * Ns] = v[r];
    }
    __syncthreads();
    c2<T>* t = d0;
    d0 = d1;
    d1 = t;
    Ns *= R;
  }
  return d0;
}

template <typename T>
__device__ void load_twiddles(c2<T>* s, const c2<T>* g, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) s[i] = g[i];
}

template <typename T, int N, int S = 0, int NS = 1>
__device__ __forceinline__ c2<T>* smem_fft_ct(c2<T>* d0, c2<T>* d1, int ls, int nl, const c2<T>* tw, int sign) {
  if constexpr (S < ct_nst(N)) {
    constexpr int R = ct_radix(N, S);
    constexpr int NB = N / R;
    constexpr int TWS = N / (NS * R);
    const int total = nl * NB;
    for (int w = threadIdx.x; w < total; w += blockDim.x) {
      const int l = w / NB, j = w - l * NB;
      const int k = j % NS;
      const c2<T>* in = d0 + l * ls;
      c2<T>* out = d1 + l * ls;
      c2<T> v[4];
#pragma unroll
      for (int r = 0; r < R; r++) {
        v[r] = in[j + r * NB];
        if (r && NS > 1) v[r] = cmul<T>(v[r], tw[k * r * TWS]);
      }
      butterfly<T, R>(v, sign);
      const int idxD = (j / NS) * NS * R + k;
#pragma unroll
      for (int r = 0; r < R; r++) out[idxD + r * NS] = v[r];
    }
    __syncthreads();
    return smem_fft_ct<T, N, S + 1, NS * R>(d1, d0, ls, nl, tw, sign);
  } else {
    return d0;
  }
}

// NC > 0: compile-time line length; NC == 0: runtime plan.
template <typename T, int NC>
__device__ __forceinline__ c2<T>* do_fft(c2<T>* d0, c2<T>* d1, int n, int ls, int nl, const FftPlan& pl,
                                         const c2<T>* tw, int sign) {
  if constexpr (NC > 0) return smem_fft_ct<T, NC>(d0, d1, ls, nl, tw, sign);
  else return smem_fft<T>(d0, d1, n, ls, nl, pl, tw, sign);
}

}  // namespace mth

// green_op.cuh -- the Green operator at one wave vector, shared by the
// shared-memory and the TMA x passes.
#pragma once
#include "mth_common.cuh"
#include "mth_internal.h"

namespace mth {

// Frequency of index idx on an axis of n points: idx/n - round(idx/n) of
// src/init.c:778-786 (the Nyquist index maps to -1/2), from integers.
template <typename T> __device__ __forceinline__ T freq(int idx, int n) {
  const int k = (2 * idx >= n) ? idx - n : idx;
  return (T)k / (T)n;
}
template <typename T> __device__ __forceinline__ T c0_at(const GreenConst& gc, int i);
template <> __device__ __forceinline__ float c0_at<float>(const GreenConst& gc, int i) { return gc.c0f[i]; }
template <> __device__ __forceinline__ double c0_at<double>(const GreenConst& gc, int i) { return gc.c0[i]; }
template <typename T> __device__ __forceinline__ T s066_at(const GreenConst& gc, int i);
template <> __device__ __forceinline__ float s066_at<float>(const GreenConst& gc, int i) { return gc.s066f[i]; }
template <> __device__ __forceinline__ double s066_at<double>(const GreenConst& gc, int i) { return gc.s066[i]; }

// Delta = -Omega(n) (sig n) (x) n for one n; accumulates into dsym (LT, 6
// complex) and danti (3 complex: [2][1], [0][2], [1][0]) with weight wgt.
template <typename T>
__device__ __forceinline__ void green_apply_n(const GreenConst& gc, const T n[3], const c2<T> s[3][3], T wgt, c2<T> dsym[6],
                                              c2<T> danti[3]) {
  T A[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int k = i; k < 3; k++) {
      T a = 0;
#pragma unroll
      for (int j = 0; j < 3; j++)
#pragma unroll
        for (int l = 0; l < 3; l++) a += c0_at<T>(gc, ((i * 3 + j) * 3 + k) * 3 + l) * n[j] * n[l];
      A[i][k] = a;
      A[k][i] = a;
    }
  T det = A[0][0] * (A[1][1] * A[2][2] - A[1][2] * A[2][1]) - A[0][1] * (A[1][0] * A[2][2] - A[1][2] * A[2][0]) +
          A[0][2] * (A[1][0] * A[2][1] - A[2][0] * A[1][1]);
  T id = (T)1 / det;
  T O[3][3];
  O[0][0] = (A[1][1] * A[2][2] - A[1][2] * A[2][1]) * id;
  O[0][1] = (A[0][2] * A[2][1] - A[0][1] * A[2][2]) * id;
  O[0][2] = (A[0][1] * A[1][2] - A[0][2] * A[1][1]) * id;
  O[1][0] = O[0][1];
  O[1][1] = (A[0][0] * A[2][2] - A[0][2] * A[2][0]) * id;
  O[1][2] = (A[0][2] * A[1][0] - A[0][0] * A[1][2]) * id;
  O[2][0] = O[0][2];
  O[2][1] = O[1][2];
  O[2][2] = (A[0][0] * A[1][1] - A[0][1] * A[1][0]) * id;
  c2<T> t[3], v[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    t[k] = mk<T>(s[k][0].x * n[0] + s[k][1].x * n[1] + s[k][2].x * n[2],
                 s[k][0].y * n[0] + s[k][1].y * n[1] + s[k][2].y * n[2]);
  }
#pragma unroll
  for (int i = 0; i < 3; i++)
    v[i] = mk<T>(-(O[i][0] * t[0].x + O[i][1] * t[1].x + O[i][2] * t[2].x) * wgt,
                 -(O[i][0] * t[0].y + O[i][1] * t[1].y + O[i][2] * t[2].y) * wgt);
  // Delta_ij = v_i n_j
  T r2 = (T)RSQ2, r3 = (T)RSQ3, r6 = (T)RSQ6;
  c2<T> d00 = cscale<T>(v[0], n[0]), d11 = cscale<T>(v[1], n[1]), d22 = cscale<T>(v[2], n[2]);
  c2<T> d12 = cscale<T>(v[1], n[2]), d21 = cscale<T>(v[2], n[1]);
  c2<T> d02 = cscale<T>(v[0], n[2]), d20 = cscale<T>(v[2], n[0]);
  c2<T> d01 = cscale<T>(v[0], n[1]), d10 = cscale<T>(v[1], n[0]);
  dsym[0] = cadd<T>(dsym[0], cscale<T>(csub<T>(d11, d00), r2));
  dsym[1] = cadd<T>(dsym[1], cscale<T>(csub<T>(cscale<T>(d22, (T)2), cadd<T>(d00, d11)), r6));
  dsym[2] = cadd<T>(dsym[2], cscale<T>(cadd<T>(d12, d21), r2));
  dsym[3] = cadd<T>(dsym[3], cscale<T>(cadd<T>(d02, d20), r2));
  dsym[4] = cadd<T>(dsym[4], cscale<T>(cadd<T>(d01, d10), r2));
  dsym[5] = cadd<T>(dsym[5], cscale<T>(cadd<T>(cadd<T>(d00, d11), d22), r3));
  danti[0] = cadd<T>(danti[0], cscale<T>(csub<T>(d21, d12), (T)0.5));
  danti[1] = cadd<T>(danti[1], cscale<T>(csub<T>(d02, d20), (T)0.5));
  danti[2] = cadd<T>(danti[2], cscale<T>(csub<T>(d10, d01), (T)0.5));
}

// sig: LT components of sigma-hat at k (in), replaced by LT of sym(Delta);
// anti: antisymmetric part of Delta.  When k has Nyquist components the
// operator is the mean of Gamma at n(k) and n(-k): the reference keeps only
// the real part of its complex inverse transform (src/evolution.c:1402),
// which equals the transform of the Hermitian part of Delta-hat.
template <typename T>
__device__ __forceinline__ void green_point(const GreenConst& gc, int kx, int ky, int kz, int n0, int n1, int n2,
                                            c2<T> sig[6], c2<T> anti[3]) {
  c2<T> dsym[6], danti[3];
#pragma unroll
  for (int i = 0; i < 6; i++) dsym[i] = mk<T>(0, 0);
#pragma unroll
  for (int i = 0; i < 3; i++) danti[i] = mk<T>(0, 0);
  if (kx == 0 && ky == 0 && kz == 0) {
    if (gc.elast_bc == 0) {
      for (int i = 0; i < 6; i++) {
        T re = 0, im = 0;
        for (int j = 0; j < 6; j++) {
          re -= s066_at<T>(gc, i * 6 + j) * sig[j].x;
          im -= s066_at<T>(gc, i * 6 + j) * sig[j].y;
        }
        dsym[i] = mk<T>(re, im);
      }
    }
  } else {
    c2<T> s[3][3];
    {
      T re[6], im[6], tr[3][3], ti[3][3];
#pragma unroll
      for (int i = 0; i < 6; i++) { re[i] = sig[i].x; im[i] = sig[i].y; }
      lt_to_cart<T>(re, tr);
      lt_to_cart<T>(im, ti);
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) s[i][j] = mk<T>(tr[i][j], ti[i][j]);
    }
    T f[3] = {freq<T>(kx, n0), freq<T>(ky, n1), freq<T>(kz, n2)};
    const bool q0 = (2 * kx == n0), q1 = (2 * ky == n1), q2 = (2 * kz == n2);
    T nrm = sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    T n[3] = {f[0] / nrm, f[1] / nrm, f[2] / nrm};
    const bool anyq = q0 || q1 || q2;
    const bool anyv = (!q0 && kx != 0) || (!q1 && ky != 0) || (!q2 && kz != 0);
    if (anyq && anyv) {
      green_apply_n<T>(gc, n, s, (T)0.5, dsym, danti);
      T m[3] = {q0 ? n[0] : -n[0], q1 ? n[1] : -n[1], q2 ? n[2] : -n[2]};
      green_apply_n<T>(gc, m, s, (T)0.5, dsym, danti);
    } else {
      green_apply_n<T>(gc, n, s, (T)1, dsym, danti);
    }
  }
#pragma unroll
  for (int i = 0; i < 6; i++) sig[i] = dsym[i];
#pragma unroll
  for (int i = 0; i < 3; i++) anti[i] = danti[i];
}

}  // namespace mth

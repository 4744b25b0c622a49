// fft_core.cuh -- radix plans and butterflies of the shared-memory FFTs.
#pragma once
#include "mth_common.cuh"

namespace mth {

// Compile-time variant for the line lengths the workloads use: the radix
// plan (4s, then 2s, then 3s, as make_plan) and every index computation fold
// into constants.
__host__ __device__ constexpr int ct_nst(int n) {
  int s = 0;
  while (n % 4 == 0) { n /= 4; s++; }
  while (n % 2 == 0) { n /= 2; s++; }
  while (n % 3 == 0) { n /= 3; s++; }
  return s;
}
__host__ __device__ constexpr int ct_radix(int n, int idx) {
  int s = 0;
  while (n % 4 == 0) { if (s == idx) return 4; n /= 4; s++; }
  while (n % 2 == 0) { if (s == idx) return 2; n /= 2; s++; }
  while (n % 3 == 0) { if (s == idx) return 3; n /= 3; s++; }
  return 1;
}

// Plans of the in-register tile FFTs (fft_tma.cu): the largest radix up to
// RMAX first (16, 8, 4, then 2, then 3), so a line needs fewer stages, each
// one pair of block-wide synchronisations.
__host__ __device__ constexpr int tl_nst(int n, int rmax) {
  int s = 0;
  for (int r = rmax; r >= 4; r /= 2)
    while (n % r == 0) { n /= r; s++; }
  while (n % 2 == 0) { n /= 2; s++; }
  while (n % 3 == 0) { n /= 3; s++; }
  return s;
}
__host__ __device__ constexpr int tl_radix(int n, int idx, int rmax) {
  int s = 0;
  for (int r = rmax; r >= 4; r /= 2)
    while (n % r == 0) { if (s == idx) return r; n /= r; s++; }
  while (n % 2 == 0) { if (s == idx) return 2; n /= 2; s++; }
  while (n % 3 == 0) { if (s == idx) return 3; n /= 3; s++; }
  return 1;
}

// x * W^m for W = exp(sign 2 pi i / 16), m in 0..15, by the values of
// cos(k pi / 8) (exact constants, no table)
template <typename T, int M>
__device__ __forceinline__ c2<T> rot16(c2<T> x, int sign) {
  constexpr int m = M & 15;
  constexpr double C1 = 0.92387953251128675613, S1 = 0.38268343236508977173, H = 0.70710678118654752440;
  constexpr double cr[4] = {1.0, C1, H, S1};   // cos(k pi/8), k = 0..3
  constexpr int q = m / 4, k = m % 4;         // W^m = i^(sign q) * W^k
  const T c = (T)cr[k], sn = (T)sign * (T)cr[(4 - k) & 3] * (k ? (T)1 : (T)0);
  c2<T> y = k ? mk<T>(x.x * c - x.y * sn, x.x * sn + x.y * c) : x;
  // multiply by (sign i)^q
  if constexpr (q == 1) y = mk<T>(-(T)sign * y.y, (T)sign * y.x);
  if constexpr (q == 2) y = mk<T>(-y.x, -y.y);
  if constexpr (q == 3) y = mk<T>((T)sign * y.y, -(T)sign * y.x);
  return y;
}

template <typename T, int R>
__device__ __forceinline__ void butterfly(c2<T>* v, int sign);

// radix-4 DFT of a[0], a[S], a[2S], a[3S] into the same places
template <typename T, int S>
__device__ __forceinline__ void dft4_strided(c2<T>* a, int sign) {
  c2<T> s02 = cadd<T>(a[0], a[2 * S]), d02 = csub<T>(a[0], a[2 * S]);
  c2<T> s13 = cadd<T>(a[S], a[3 * S]), d13 = csub<T>(a[S], a[3 * S]);
  c2<T> wd = mk<T>(-(T)sign * d13.y, (T)sign * d13.x);
  a[0] = cadd<T>(s02, s13);
  a[2 * S] = csub<T>(s02, s13);
  a[S] = cadd<T>(d02, wd);
  a[3 * S] = csub<T>(d02, wd);
}

template <typename T, int R>
__device__ __forceinline__ void butterfly(c2<T>* v, int sign) {
  if constexpr (R == 16) {
    // n = n1 + 4 n2, k = k1 + 4 k2: DFT4 over n2, twiddle W16^(n1 k1), DFT4 over n1
    c2<T> a[16];
#pragma unroll
    for (int n1 = 0; n1 < 4; n1++) {
      c2<T> b[4] = {v[n1], v[n1 + 4], v[n1 + 8], v[n1 + 12]};
      dft4_strided<T, 1>(b, sign);
#pragma unroll
      for (int k1 = 0; k1 < 4; k1++) a[n1 * 4 + k1] = b[k1];
    }
    a[5] = rot16<T, 1>(a[5], sign);
    a[6] = rot16<T, 2>(a[6], sign);
    a[7] = rot16<T, 3>(a[7], sign);
    a[9] = rot16<T, 2>(a[9], sign);
    a[10] = rot16<T, 4>(a[10], sign);
    a[11] = rot16<T, 6>(a[11], sign);
    a[13] = rot16<T, 3>(a[13], sign);
    a[14] = rot16<T, 6>(a[14], sign);
    a[15] = rot16<T, 9>(a[15], sign);
#pragma unroll
    for (int k1 = 0; k1 < 4; k1++) {
      dft4_strided<T, 4>(a + k1, sign);
#pragma unroll
      for (int k2 = 0; k2 < 4; k2++) v[k1 + 4 * k2] = a[k1 + 4 * k2];
    }
  } else if constexpr (R == 8) {
    // n = n1 + 2 n2, k = k1 + 4 k2: DFT4 over n2, twiddle W8^(n1 k1), DFT2 over n1
    c2<T> e[4] = {v[0], v[2], v[4], v[6]}, o[4] = {v[1], v[3], v[5], v[7]};
    dft4_strided<T, 1>(e, sign);
    dft4_strided<T, 1>(o, sign);
    o[1] = rot16<T, 2>(o[1], sign);
    o[2] = rot16<T, 4>(o[2], sign);
    o[3] = rot16<T, 6>(o[3], sign);
#pragma unroll
    for (int k1 = 0; k1 < 4; k1++) {
      v[k1] = cadd<T>(e[k1], o[k1]);
      v[k1 + 4] = csub<T>(e[k1], o[k1]);
    }
  } else if constexpr (R == 2) {
    c2<T> a = v[0], b = v[1];
    v[0] = cadd<T>(a, b);
    v[1] = csub<T>(a, b);
  } else if constexpr (R == 4) {
    c2<T> s02 = cadd<T>(v[0], v[2]), d02 = csub<T>(v[0], v[2]);
    c2<T> s13 = cadd<T>(v[1], v[3]), d13 = csub<T>(v[1], v[3]);
    c2<T> wd = mk<T>(-(T)sign * d13.y, (T)sign * d13.x);
    v[0] = cadd<T>(s02, s13);
    v[2] = csub<T>(s02, s13);
    v[1] = cadd<T>(d02, wd);
    v[3] = csub<T>(d02, wd);
  } else {
    const T h = (T)0.86602540378443864676 * (T)sign;
    c2<T> t = cadd<T>(v[1], v[2]), u = csub<T>(v[1], v[2]);
    c2<T> m = mk<T>(v[0].x - (T)0.5 * t.x, v[0].y - (T)0.5 * t.y);
    c2<T> iu = mk<T>(-h * u.y, h * u.x);
    v[0] = cadd<T>(v[0], t);
    v[1] = cadd<T>(m, iu);
    v[2] = csub<T>(m, iu);
  }
}

}  // namespace mth

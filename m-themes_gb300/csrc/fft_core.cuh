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

template <typename T, int R>
__device__ __forceinline__ void butterfly(c2<T> v[4], int sign) {
  if constexpr (R == 2) {
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

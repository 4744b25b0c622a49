// mth_common.cuh -- shared types and helpers of the sm_103a EVPFFT kernels.
//
// Field layout in HBM: structure of arrays, one plane of N0*N1*N2 values per
// component, voxel index (x*N1+y)*N2+z with z fastest (the reference's pIDX,
// src/evp.h:53).  Symmetric tensors are stored as 6 components in the
// Lebensohn-Tome basis of chg_basis (src/kinematics.c:27-53): components 0..4
// deviatoric, 5 hydrostatic.  Spectra are half spectra along z
// (N2/2+1 points), one plane per component, index (x*N1+y)*Kz+kz.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace mth {

constexpr int NSYS = 12;
constexpr double RSQ2 = 0.70710678118654744;
constexpr double RSQ3 = 0.57735026918962584;
constexpr double RSQ6 = 0.40824829046386304;

template <typename T> struct cplx;
template <> struct cplx<float> { using type = float2; };
template <> struct cplx<double> { using type = double2; };
template <typename T> using c2 = typename cplx<T>::type;

template <typename T> __host__ __device__ __forceinline__ c2<T> mk(T a, T b) { c2<T> r; r.x = a; r.y = b; return r; }
template <typename T> __device__ __forceinline__ c2<T> cadd(c2<T> a, c2<T> b) { return mk<T>(a.x + b.x, a.y + b.y); }
template <typename T> __device__ __forceinline__ c2<T> csub(c2<T> a, c2<T> b) { return mk<T>(a.x - b.x, a.y - b.y); }
template <typename T> __device__ __forceinline__ c2<T> cmul(c2<T> a, c2<T> b) {
  return mk<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename T> __device__ __forceinline__ c2<T> cscale(c2<T> a, T s) { return mk<T>(a.x * s, a.y * s); }
template <typename T> __device__ __forceinline__ c2<T> conjg(c2<T> a) { return mk<T>(a.x, -a.y); }

// Symmetric 3x3 tensor (Cartesian) <-> 6-vector in the LT basis.
// v2t: t = sum_i v_i B_i ; t2v: v_i = t : B_i  (chg_basis opt 1 / opt 2).
template <typename T> __host__ __device__ __forceinline__ void lt_to_cart(const T* v, T t[3][3]) {
  const T r2 = (T)RSQ2, r3 = (T)RSQ3, r6 = (T)RSQ6;
  t[0][0] = -r2 * v[0] - r6 * v[1] + r3 * v[5];
  t[1][1] = r2 * v[0] - r6 * v[1] + r3 * v[5];
  t[2][2] = (T)2 * r6 * v[1] + r3 * v[5];
  t[1][2] = t[2][1] = r2 * v[2];
  t[0][2] = t[2][0] = r2 * v[3];
  t[0][1] = t[1][0] = r2 * v[4];
}
template <typename T> __host__ __device__ __forceinline__ void cart_to_lt(const T t[3][3], T* v) {
  const T r2 = (T)RSQ2, r3 = (T)RSQ3, r6 = (T)RSQ6;
  v[0] = r2 * (t[1][1] - t[0][0]);
  v[1] = r6 * ((T)2 * t[2][2] - t[0][0] - t[1][1]);
  v[2] = r2 * (t[1][2] + t[2][1]);
  v[3] = r2 * (t[0][2] + t[2][0]);
  v[4] = r2 * (t[0][1] + t[1][0]);
  v[5] = r3 * (t[0][0] + t[1][1] + t[2][2]);
}

// Q (5x5, row-major) maps deviatoric LT components from sample to crystal
// axes: a_c = Q a_s, with A_c = T^T A_s T and T the crystal->sample matrix
// (TranMat_xt2sa).  Q_ij = B_i : (T^T B_j T).
template <typename T> __host__ __device__ __forceinline__ void rot_to_q(const T R[9], T Q[25]) {
#pragma unroll
  for (int j = 0; j < 5; j++) {
    T bj[6] = {0, 0, 0, 0, 0, 0};
    bj[j] = (T)1;
    T b[3][3], m[3][3], c[3][3];
    lt_to_cart<T>(bj, b);
    // m = b T
#pragma unroll
    for (int p = 0; p < 3; p++)
#pragma unroll
      for (int q = 0; q < 3; q++) m[p][q] = b[p][0] * R[0 * 3 + q] + b[p][1] * R[1 * 3 + q] + b[p][2] * R[2 * 3 + q];
    // c = T^T m
#pragma unroll
    for (int p = 0; p < 3; p++)
#pragma unroll
      for (int q = 0; q < 3; q++) c[p][q] = R[0 * 3 + p] * m[0][q] + R[1 * 3 + p] * m[1][q] + R[2 * 3 + p] * m[2][q];
    T v[6];
    cart_to_lt<T>(c, v);
#pragma unroll
    for (int i = 0; i < 5; i++) Q[i * 5 + j] = v[i];
  }
}

// Per-phase constants of the flow rule in crystal axes.
struct PhaseConst {
  int type;          // 0 crystal, 1 gas
  int nsys;
  double nrs, gamd0;
  double tau_back_minus_fwd;   // tau0b - tau0f (harden shifts both alike)
  double s_xt[6];    // crystal-axes compliance, diagonal in the LT basis
  double c_xt[6];    // crystal-axes stiffness, diagonal in the LT basis
  double m_xt[NSYS][5];  // Schmid tensors in crystal axes (Schm_xt)
  double bn[NSYS][3], bb[NSYS][3];
  double hard[NSYS][NSYS];
  double tau0f, tau1, thet0, thet1;
  int nrs_int;       // >0 when nrs is an integer: exponent fast path
  // float copies for the FP32 flow rule (filled by fill_float_consts)
  float nrsf, gamd0f, tau_offf;
  float m_xtf[NSYS][5];
  float bnf[NSYS][3], bbf[NSYS][3];
  float hardf[NSYS][NSYS];
  float tau0ff, tau1f, thet0f, thet1f;
};

// Constant of precision T from its double and float copies: the FP32 paths
// read float constants instead of converting doubles on the FP64 pipe.
template <typename T>
__host__ __device__ __forceinline__ T cpick(double d, float f);
template <>
__host__ __device__ __forceinline__ float cpick<float>(double, float f) { return f; }
template <>
__host__ __device__ __forceinline__ double cpick<double>(double d, float) { return d; }

#ifdef __CUDACC__
// FP32 <-> FP64 conversions by integer operations on the two words of the
// double: GB300 executes F2F conversions on its FP64 pipe (1/64 of the FP32
// rate), these run on the integer pipes.  f32_to_f64 is exact for normal
// numbers, zeros, infinities and NaNs and flushes FP32 subnormals to signed
// zero.  f64_to_f32 rounds to nearest even, as the hardware conversion does,
// for results in the FP32 normal range, flushes smaller magnitudes to signed
// zero, and returns +-inf above the range and a quiet NaN for a NaN.
__device__ __forceinline__ double f32_to_f64(float x) {
  const unsigned u = __float_as_uint(x);
  const unsigned sgn = u & 0x80000000u, mag = u & 0x7fffffffu;
  // exponent bias 127 -> 1023: add (1023 - 127) << 20 to the high word
  unsigned hi = sgn | ((mag >> 3) + (896u << 20));
  unsigned lo = u << 29;
  if (mag < 0x00800000u) {          // zero or subnormal
    hi = sgn;
    lo = 0u;
  } else if (mag >= 0x7f800000u) {  // inf or NaN: all-ones exponent, same mantissa
    hi |= 0x7ff00000u;
  }
  return __hiloint2double((int)hi, (int)lo);
}
__device__ __forceinline__ float f64_to_f32(double x) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const unsigned sgn = hi & 0x80000000u, mhi = hi & 0x7fffffffu;
  const int e = (int)(mhi >> 20) - 896;   // FP32 biased exponent
  // exponent and the top 23 mantissa bits (meaningful for 0 < e < 255)
  unsigned b = ((mhi - (896u << 20)) << 3) | (lo >> 29);
  const unsigned r = lo & 0x1fffffffu;    // the 29 bits rounded off
  // round to nearest even; a carry out of the mantissa steps the exponent
  // (to inf from the largest binade)
  b += (r > 0x10000000u || (r == 0x10000000u && (b & 1u))) ? 1u : 0u;
  if (e <= 0) b = 0u;
  else if (e >= 255) b = (mhi > 0x7ff00000u || (mhi == 0x7ff00000u && lo != 0u)) ? 0x7fc00000u : 0x7f800000u;
  return __uint_as_float(sgn | b);
}
__device__ __forceinline__ double to_f64(float x) { return f32_to_f64(x); }
__device__ __forceinline__ double to_f64(double x) { return x; }
#endif

}  // namespace mth

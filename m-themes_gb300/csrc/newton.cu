// newton.cu -- per-voxel kernels: the local stress solve of UpdateStress
// (src/evolution.c:44-310) with the power-law flow rule of StrainRate_eval
// (src/constitutive.c:5-67), the end-of-step updates (plastic strain,
// update_orient src/constitutive.c:196-273, harden src/constitutive.c:275-326)
// and the set-up of InitMicroStruct/InitFields (src/init.c:233-515).
//
// One thread per voxel, structure-of-arrays fields, coalesced loads.
//
// Local problem.  The reference solves, per voxel and in the 6-component
// Lebensohn-Tome basis, R(s) = s - lambda + C066 (S s + e_p + edot_p(s) dt - e)
// = 0 by Newton with a line search on |R|^2 (src/evolution.c:129-253).  Here
// the same root is found from the equivalent system S0 R = 0 (S0 = C066^-1),
// which is the gradient of the strictly convex potential
//   Phi(s) = 1/2 (s-lambda).S0.(s-lambda) + 1/2 s.S.s + (e_p - e).s + dt psi(s),
//   psi(s) = sum_a gamd0 tau_a |r_a|^(n+1) / (n+1),  r_a = m_a.s / tau_a,
// so Newton's direction is always a descent direction and the Hessian
// S0 + S + dt sum_a w_a m_a m_a^T is symmetric positive definite (Cholesky).
// The solve runs in crystal axes: there the cubic compliance S is diagonal and
// the Schmid tensors m_a are the constants of the .sx file, so no per-voxel
// Schmid field is stored (update_schmid, src/kinematics.c:430-463, becomes a
// 5x5 rotation of the stress).  The hydrostatic component decouples exactly
// for cubic crystals (edot_p has no trace, src/constitutive.c:50) and is
// solved in closed form.  Convergence: |step| <= tol |lambda|, as the
// reference's erral (src/evolution.c:264-270).
#include <type_traits>
#include <cstdio>
#include <cmath>
#include <atomic>
#include "mth_common.cuh"
#include "mth_internal.h"

namespace mth {

// |r|^e for the flow rule; integer exponents by repeated squaring.
template <typename T>
__device__ __forceinline__ T pow_abs(T a, int ei, T ef) {
  if (ei > 0) {
    T r = (T)1, b = a;
    int e = ei;
    while (e) {
      if (e & 1) r *= b;
      b *= b;
      e >>= 1;
    }
    return r;
  }
  return a > (T)0 ? (T)pow(a, ef) : (T)0;
}

// class-table row pointer of precision T
template <typename T>
__device__ __forceinline__ const T* cpick_ptr(const double* d, const float* f);
template <>
__device__ __forceinline__ const float* cpick_ptr<float>(const double*, const float* f) { return f; }
template <>
__device__ __forceinline__ const double* cpick_ptr<double>(const double* d, const float*) { return d; }

// Flow rule in crystal axes at deviatoric stress x (5).  tauf: forward CRSS
// per system; the backward CRSS is forward + tau_off.  Returns edot (5),
// optional Hessian contribution D (15, packed upper triangle) and
// psi = sum gamd0 tau |r|^(n+1)/(n+1) = sum gamd0 |rss| |r|^n/(n+1).
// gam (optional) receives the shear rates.
template <typename TF, bool WANT_D>
__device__ __forceinline__ void flow_rule(const PhaseConst& ph, const TF x[5], const TF* tauf, TF tau_off, TF ed[5],
                                          TF D[15], TF& psi, TF* gam) {
#pragma unroll
  for (int i = 0; i < 5; i++) ed[i] = 0;
  if (WANT_D) {
#pragma unroll
    for (int i = 0; i < 15; i++) D[i] = 0;
  }
  psi = 0;
  const int ns = ph.nsys;
  const TF n = cpick<TF>(ph.nrs, ph.nrsf);
  const TF g0 = cpick<TF>(ph.gamd0, ph.gamd0f);
  const TF inv_np1 = (TF)1 / (n + (TF)1);
  const int nm1 = ph.nrs_int > 0 ? ph.nrs_int - 1 : 0;
  // fully unrolled over the NSYS slots so the per-voxel CRSS stay in registers
#pragma unroll
  for (int s = 0; s < NSYS; s++) {
    if (s < ns) {
      TF m[5];
#pragma unroll
      for (int i = 0; i < 5; i++) m[i] = cpick<TF>(ph.m_xt[s][i], ph.m_xtf[s][i]);
      const TF rss = m[0] * x[0] + m[1] * x[1] + m[2] * x[2] + m[3] * x[3] + m[4] * x[4];
      const TF tau = rss < (TF)0 ? tauf[s] + tau_off : tauf[s];
      const TF itau = (TF)1 / tau;
      const TF r = rss * itau;
      const TF ar = fabs(r);
      const TF pnm1 = pow_abs<TF>(ar, nm1, n - (TF)1);   // |r|^(n-1)
      const TF pn = pnm1 * ar;                             // |r|^n
      const TF g = g0 * (r > (TF)0 ? pn : -pn);
      if (gam) gam[s] = g;
#pragma unroll
      for (int i = 0; i < 5; i++) ed[i] += m[i] * g;
      if (WANT_D) {
        const TF w = g0 * n * pnm1 * itau;
        int q = 0;
#pragma unroll
        for (int i = 0; i < 5; i++)
#pragma unroll
          for (int j = i; j < 5; j++) D[q++] += w * m[i] * m[j];
      }
      psi += g0 * fabs(rss) * pn * inv_np1;
    } else if (gam) {
      gam[s] = 0;
    }
  }
}

// Dislocation-density flow rule of StrainRate_Orowan, forward plus backward
// jumps (src/constitutive.c:507-721), in crystal axes: per system
// gdot = g0 sinh((|rss| - tp)/td) sign(rss) where |rss| > tp, else 0, with
// tp the passing stress, td = tau_0 + cutting stress and g0 the reference
// rate of the step (from the dislocation densities, dd.cu).  It is the
// gradient of the convex potential psi = sum g0 td (cosh(t) - 1),
// t = max(|rss| - tp, 0)/td, written 2 g0 td sinh^2(t/2).
template <typename TF, bool WANT_D>
__device__ __forceinline__ void flow_rule_dd(const PhaseConst& ph, const TF x[5], const TF* tp, const TF* td,
                                             const TF* g0, TF ed[5], TF D[15], TF& psi, TF* gam) {
#pragma unroll
  for (int i = 0; i < 5; i++) ed[i] = 0;
  if (WANT_D) {
#pragma unroll
    for (int i = 0; i < 15; i++) D[i] = 0;
  }
  psi = 0;
  const int ns = ph.nsys;
#pragma unroll
  for (int s = 0; s < NSYS; s++) {
    if (s < ns) {
      TF m[5];
#pragma unroll
      for (int i = 0; i < 5; i++) m[i] = cpick<TF>(ph.m_xt[s][i], ph.m_xtf[s][i]);
      const TF rss = m[0] * x[0] + m[1] * x[1] + m[2] * x[2] + m[3] * x[3] + m[4] * x[4];
      const TF ar = fabs(rss);
      TF g = 0, w = 0;
      if (ar > tp[s]) {
        const TF t = (ar - tp[s]) / td[s];
        const TF sh = sinh(t);
        g = g0[s] * (rss > (TF)0 ? sh : -sh);
        if (WANT_D) w = g0[s] * cosh(t) / td[s];
        const TF h = sinh((TF)0.5 * t);
        psi += (TF)2 * g0[s] * td[s] * h * h;
      }
      if (gam) gam[s] = g;
#pragma unroll
      for (int i = 0; i < 5; i++) ed[i] += m[i] * g;
      if (WANT_D) {
        int q = 0;
#pragma unroll
        for (int i = 0; i < 5; i++)
#pragma unroll
          for (int j = i; j < 5; j++) D[q++] += w * m[i] * m[j];
      }
    } else if (gam) {
      gam[s] = 0;
    }
  }
}

// Slip laws of the local solve.  Power law: forward CRSS per system, the
// backward one offset by tau_off.  Dislocation density: passing stress,
// tau_0 + cutting stress and reference rate per system.
template <typename TF>
struct PlSlip {
  TF tauf[NSYS];
  TF tau_off;
  template <bool WANT_D>
  __device__ __forceinline__ void flow(const PhaseConst& ph, const TF x[5], TF ed[5], TF D[15], TF& psi,
                                       TF* gam) const {
    flow_rule<TF, WANT_D>(ph, x, tauf, tau_off, ed, D, psi, gam);
  }
};
template <typename TF>
struct DdSlip {
  TF tp[NSYS], td[NSYS], g0[NSYS];
  template <bool WANT_D>
  __device__ __forceinline__ void flow(const PhaseConst& ph, const TF x[5], TF ed[5], TF D[15], TF& psi,
                                       TF* gam) const {
    flow_rule_dd<TF, WANT_D>(ph, x, tp, td, g0, ed, D, psi, gam);
  }
};
// The power law's state with the CRSS in shared memory (the cooperative
// kernel, whose registers bound how many blocks share an SM): tauf points
// at this thread's NSYS values, rows of NSYS + 1 so that a warp's threads
// read distinct banks.
template <typename TF>
struct PlSlipSh {
  const TF* tauf;
  TF tau_off;
  template <bool WANT_D>
  __device__ __forceinline__ void flow(const PhaseConst& ph, const TF x[5], TF ed[5], TF D[15], TF& psi,
                                       TF* gam) const {
    flow_rule<TF, WANT_D>(ph, x, tauf, tau_off, ed, D, psi, gam);
  }
};
// slip-law state of voxel v from the fields (LAW 0: power law, 1: dislocation density)
template <int LAW, typename TF, typename TSt>
struct SlipOf;
template <typename TF, typename TSt>
struct SlipOf<0, TF, TSt> {
  using type = PlSlip<TF>;
  __device__ __forceinline__ static void load(const PhaseConst& ph, const Fields<TSt>& f, long long v, type& sl) {
    const long long P = f.nv;
#pragma unroll
    for (int s = 0; s < NSYS; s++) sl.tauf[s] = s < ph.nsys ? (TF)f.crss[s * P + v] : (TF)1;
    sl.tau_off = cpick<TF>(ph.tau_back_minus_fwd, ph.tau_offf);
  }
};
template <typename TF, typename TSt>
struct SlipOf<1, TF, TSt> {
  using type = DdSlip<TF>;
  __device__ __forceinline__ static void load(const PhaseConst& ph, const Fields<TSt>& f, long long v, type& sl) {
    const long long P = f.nv;
#pragma unroll
    for (int s = 0; s < NSYS; s++) {
      const bool a = s < ph.nsys;
      sl.tp[s] = a ? (TF)f.ddc[s * P + v] : (TF)0;
      sl.td[s] = a ? (TF)f.ddc[(NSYS + s) * P + v] : (TF)1;
      sl.g0[s] = a ? (TF)f.ddc[(2 * NSYS + s) * P + v] : (TF)0;
    }
  }
};

__device__ __forceinline__ int pk(int i, int j) {  // packed upper-triangle index of 5x5
  if (i > j) { int t = i; i = j; j = t; }
  return i * 5 - (i * (i - 1)) / 2 + (j - i);
}

template <typename T>
__device__ __forceinline__ void symv5(const T* K, const T* x, T* y) {
#pragma unroll
  for (int i = 0; i < 5; i++) {
    T s = 0;
#pragma unroll
    for (int j = 0; j < 5; j++) s += K[pk(i, j)] * x[j];
    y[i] = s;
  }
}

// 1/d for a positive normal FP64 pivot, without FP64-pipe work besides
// three DFMA: the FP32 hardware reciprocal (rcp.approx.ftz.f32, within 1 ulp)
// of d's mantissa m in [1, 2), truncated to 24 bits, gives 1/m to within
// 2^-22; its exponent is shifted by d's with integer operations; one
// cubically convergent Newton step x <- x (1 + e + e^2), e = 1 - d x,
// takes the relative error from 2^-22 to below 2^-64, so the result is
// within an ulp or two of 1/d without the special-case handling of a
// correctly rounded divide.
template <bool QUAD = false>
__device__ __forceinline__ double pivot_rcp_nr(double d) {
  const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
  const int E = (int)((hi >> 20) & 0x7ffu);   // biased exponent of d (1..2046)
  const float m = __uint_as_float(0x3f800000u | ((hi & 0xfffffu) << 3) | (lo >> 29));
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(m));
  const unsigned ru = __float_as_uint(r);     // 1/m in (0.5, 1]
  // 1/d = (1/m) 2^(1023 - (E - 1023)): biased FP64 exponent Er - 127 + 2046 - E
  const int eo = (int)((ru >> 23) & 0xffu) + 1919 - E;
  unsigned xhi = ((unsigned)eo << 20) | ((ru >> 3) & 0xfffffu);
  unsigned xlo = ru << 29;
  if (eo <= 0) xhi = xlo = 0u;                // 1/d below the normal range
  const double x = __hiloint2double((int)xhi, (int)xlo);
  const double e = fma(-d, x, 1.0);
  if constexpr (QUAD) return fma(x, e, x);   // quadratic step: within 2^-43 of 1/d
  return fma(x, fma(e, e, e), x);
}
// QUAD: the quadratic step, for solves whose result is rounded to FP32 (a
// pivot reciprocal off by 2^-43 is a backward error of that size in D,
// far below the FP32 rounding of the assembled Hessian and of the step)
template <typename T, bool NR, bool QUAD = false>
__device__ __forceinline__ T pivot_inv(T d) {
  if constexpr (NR && sizeof(T) == 8) return pivot_rcp_nr<QUAD>(d);
  else return (T)1 / d;
}

// dj > 0 for a pivot; for the FP64 solves of the mixed modes (NR) tested on
// the high word with integer operations instead of an FP64 compare: a
// positive finite double has a high word in [1, 0x7fefffff] (this also
// rejects +inf and the subnormals below 2^-1042, which the reciprocal
// estimate flushes).
template <typename T, bool NR>
__device__ __forceinline__ bool pivot_positive(T d) {
  if constexpr (NR && sizeof(T) == 8) return (unsigned)__double2hiint(d) - 1u < 0x7fefffffu;
  else return d > (T)0;
}

// LDL^T solve of the packed symmetric positive definite 5x5 matrix A:
// x = A^-1 b.  Returns false when a pivot is not positive.  NR: pivot
// reciprocals by pivot_rcp_nr (FP64 solves of the mixed modes).
template <typename T, bool NR = false, bool QUAD = false>
__device__ __forceinline__ bool ldl_solve5(const T* A, const T* b, T* x) {
  // U[i][k] = L[i][k] d[k], the column before its scaling by 1/d[k], kept so
  // the updates need no products L d
  T L[5][5], U[5][5], id[5];
#pragma unroll
  for (int j = 0; j < 5; j++) {
    T dj = A[pk(j, j)];
#pragma unroll
    for (int k = 0; k < 5; k++)
      if (k < j) dj -= U[j][k] * L[j][k];
    if (!pivot_positive<T, NR>(dj)) return false;
    id[j] = pivot_inv<T, NR, QUAD>(dj);
#pragma unroll
    for (int i = 0; i < 5; i++)
      if (i > j) {
        T a = A[pk(i, j)];
#pragma unroll
        for (int k = 0; k < 5; k++)
          if (k < j) a -= U[i][k] * L[j][k];
        U[i][j] = a;
        L[i][j] = a * id[j];
      }
  }
  T y[5];
#pragma unroll
  for (int i = 0; i < 5; i++) {
    T a = b[i];
#pragma unroll
    for (int k = 0; k < 5; k++)
      if (k < i) a -= L[i][k] * y[k];
    y[i] = a;
  }
#pragma unroll
  for (int i = 4; i >= 0; i--) {
    T a = y[i] * id[i];
#pragma unroll
    for (int k = 0; k < 5; k++)
      if (k > i) a -= L[k][i] * x[k];
    x[i] = a;
  }
  return true;
}

// LDL^T solve of a TF system in precision TL.  FP32 -> FP64 (and back):
// the conversions by integer operations (f32_to_f64, f64_to_f32), as GB300
// executes F2F conversions on its 1/64-rate FP64 pipe; the pivot
// reciprocals with the quadratic step (the FP64 solve of an FP32 system is
// rounded to FP32; 5 DFMA fewer per solve, the 400 Newton launches of the
// 128^3 benchmark 2.3 % faster).
template <typename TF, typename TL>
__device__ __forceinline__ bool ldl_solve5_wide(const TF* H, const TF* b, TF* x) {
  TL Hl[15], bl[5], pl[5];
  if constexpr (sizeof(TF) == 4 && sizeof(TL) == 8) {
#pragma unroll
    for (int i = 0; i < 15; i++) Hl[i] = f32_to_f64(H[i]);
#pragma unroll
    for (int i = 0; i < 5; i++) bl[i] = f32_to_f64(b[i]);
    const bool ok = ldl_solve5<TL, true, true>(Hl, bl, pl);
#pragma unroll
    for (int i = 0; i < 5; i++) x[i] = f64_to_f32(pl[i]);
    return ok;
  } else {
#pragma unroll
    for (int i = 0; i < 15; i++) Hl[i] = (TL)H[i];
#pragma unroll
    for (int i = 0; i < 5; i++) bl[i] = (TL)b[i];
    const bool ok = ldl_solve5<TL, true>(Hl, bl, pl);
#pragma unroll
    for (int i = 0; i < 5; i++) x[i] = (TF)pl[i];
    return ok;
  }
}

// Result of one voxel solve.
template <typename TF>
struct VoxelOut {
  TF conv_s, conv_e;   // the voxel's error contributions, in the flow-rule precision
  int iters;
  int failed;
};

// ------------------------------------------------- the local solve, in pieces
// nw_init (set-up), nw_pass_a (one flow-rule evaluation and what it decides;
// when the next Newton direction is needed it returns the system H p = -g),
// nw_pass_b (the move the direction gives) and nw_finish (back to sample
// axes, error contributions).  solve_voxel runs them with its own Jacobian
// solve in between; newton_coop_kernel runs the Jacobian solves of all the
// threads of a block between them, done by as few threads as there are
// systems.  The linear term c and the Hessian base K of Phi, constant during
// a solve, are in registers (NewtonRegs) or in shared memory (NewtonShared:
// component-major, one column per thread, so the registers hold only what
// changes).
template <typename TF>
struct NewtonShared {
  TF (*K)[256];   // [15][256]
  TF (*c)[256];   // [5][256]
  int t;
  __device__ __forceinline__ TF k(int i) const { return K[i][t]; }
  __device__ __forceinline__ TF cc(int i) const { return c[i][t]; }
  __device__ __forceinline__ void set_k(int i, TF v) const { K[i][t] = v; }
  __device__ __forceinline__ void set_c(int i, TF v) const { c[i][t] = v; }
};
// the same in registers (one solve per thread)
template <typename TF>
struct NewtonRegs {
  TF K[15], c[5];
  __device__ __forceinline__ TF k(int i) const { return K[i]; }
  __device__ __forceinline__ TF cc(int i) const { return c[i]; }
  __device__ __forceinline__ void set_k(int i, TF v) { K[i] = v; }
  __device__ __forceinline__ void set_c(int i, TF v) { c[i] = v; }
};
template <typename TF>
struct NewtonState {
  TF x[5];                     // iterate (crystal axes)
  TF h, ref2, dh, hstep2, tol2, ls_thr2;
  TF xt[5];                    // point evaluated next
  TF p[5], pn2, slope, phi0, alpha;
  TF edf[5], psif;             // rates and psi at the last evaluated point
  int it, ls, pass;
  bool done, near_root, trial, failed;
};

template <typename TF, typename Store, typename Load>
__device__ __forceinline__ void nw_init(NewtonState<TF>& s, Store& sh, const NewtonConst& nc,
                                        const TF* __restrict__ et, const Load& load) {
  const TF shh = et[ET_SEL_HH];
  TF lam6[6], eps6[6], ep6[6], Q[25];
  {
    TF R[9];
    load(lam6, eps6, ep6, R, false);
    rot_to_q<TF>(R, Q);
  }
  TF s0s[5];
#pragma unroll
  for (int i = 0; i < 5; i++) {
    TF a = 0;
#pragma unroll
    for (int j = 0; j < 5; j++) a += cpick<TF>(nc.s0dev[i * 5 + j], nc.s0devf[i * 5 + j]) * lam6[j];
    s0s[i] = a;
  }
#pragma unroll
  for (int i = 0; i < 5; i++) {
    TF a = 0, b = 0, e = 0, d = 0;
#pragma unroll
    for (int j = 0; j < 5; j++) {
      a += Q[i * 5 + j] * lam6[j];
      b += Q[i * 5 + j] * eps6[j];
      e += Q[i * 5 + j] * ep6[j];
      d += Q[i * 5 + j] * s0s[j];
    }
    s.x[i] = a;
    sh.set_c(i, -d + e - b);
  }
  {
    TF St[25], t[25];
#pragma unroll
    for (int i = 0; i < 5; i++)
#pragma unroll
      for (int j = 0; j < 5; j++) St[i * 5 + j] = et[ET_STOT + pk(i, j)];
#pragma unroll
    for (int i = 0; i < 5; i++)
#pragma unroll
      for (int j = 0; j < 5; j++) {
        TF a = 0;
#pragma unroll
        for (int k = 0; k < 5; k++) a += Q[i * 5 + k] * St[k * 5 + j];
        t[i * 5 + j] = a;
      }
#pragma unroll
    for (int i = 0; i < 5; i++)
#pragma unroll
      for (int j = i; j < 5; j++) {
        TF a = 0;
#pragma unroll
        for (int k = 0; k < 5; k++) a += t[i * 5 + k] * Q[j * 5 + k];
        sh.set_k(pk(i, j), a);
      }
  }
  const TF s0hh = cpick<TF>(nc.s0hh, nc.s0hhf);
  s.h = (s0hh * lam6[5] + eps6[5] - ep6[5]) / (s0hh + shh);
  TF ref2 = 0;
#pragma unroll
  for (int i = 0; i < 6; i++) ref2 += lam6[i] * lam6[i];
  s.ref2 = ref2;
  s.dh = s.h - lam6[5];
  const TF tol = cpick<TF>(nc.tol, nc.tolf);
  s.tol2 = tol * tol;
  s.ls_thr2 = (TF)1e-6 * ref2;
  s.hstep2 = s.dh * s.dh;
#pragma unroll
  for (int i = 0; i < 5; i++) {
    s.xt[i] = s.x[i];
    s.p[i] = 0;
  }
  s.pn2 = s.slope = s.phi0 = 0;
  s.alpha = 1;
  s.it = s.ls = s.pass = 0;
  s.done = s.near_root = s.trial = s.failed = false;
}

template <typename TF>
__device__ __forceinline__ void nw_accept(NewtonState<TF>& s) {
#pragma unroll
  for (int i = 0; i < 5; i++) s.x[i] += s.alpha * s.p[i];
  const TF step2 = s.alpha * s.alpha * s.pn2 + s.hstep2;
  s.hstep2 = 0;
  s.near_root = step2 <= s.ls_thr2;
  TF den2 = s.ref2;
  if (!(den2 > (TF)0))
    den2 = s.x[0] * s.x[0] + s.x[1] * s.x[1] + s.x[2] * s.x[2] + s.x[3] * s.x[3] + s.x[4] * s.x[4] + s.h * s.h;
  if (!(den2 > (TF)0) || step2 <= s.tol2 * den2) s.done = true;
  s.it++;
}

// Newton with a backtracking line search on Phi for large steps.  One
// flow-rule evaluation site: every evaluation (with its Hessian) is at the
// point the solve moves to next, so an accepted line-search trial supplies
// the next Newton step and the last accepted iterate supplies the final
// rates, without evaluating any point twice.  At most 41 (itmax + 1)
// passes: each Newton step takes at most 40 trials + 1.
// Returns 0: pass done, no solve; 1: the Newton direction is needed (H, mg
// filled); 2: the solve has ended.
template <typename TF, typename Store, typename Slip>
__device__ __forceinline__ int nw_pass_a(NewtonState<TF>& s, const Store& sh, const NewtonConst& nc,
                                         const PhaseConst& ph, const Slip& slip, const TF* __restrict__ et, TF H[15],
                                         TF mg[5]) {
  if (s.pass >= 41 * (nc.itmax + 1)) return 2;
  s.pass++;
  const TF dt = cpick<TF>(nc.dt, nc.dtf);
  TF Df[15];
  if (nc.flow_off) {
#pragma unroll
    for (int i = 0; i < 5; i++) s.edf[i] = 0;
#pragma unroll
    for (int i = 0; i < 15; i++) Df[i] = 0;
    s.psif = 0;
  } else {
    slip.template flow<true>(ph, s.xt, s.edf, Df, s.psif, nullptr);
  }
  TF Kx[5];
#pragma unroll
  for (int i = 0; i < 5; i++) {
    TF a = 0;
#pragma unroll
    for (int j = 0; j < 5; j++) a += sh.k(pk(i, j)) * s.xt[j];
    Kx[i] = a;
  }
  if (s.trial) {
    TF phi = 0;
#pragma unroll
    for (int i = 0; i < 5; i++) phi += s.xt[i] * ((TF)0.5 * Kx[i] + sh.cc(i));
    phi += dt * s.psif;
    if (!(phi <= s.phi0 + (TF)1e-4 * s.alpha * s.slope)) {
      TF den = (TF)2 * (phi - s.phi0 - s.slope * s.alpha);
      TF an = den > (TF)0 ? -s.slope * s.alpha * s.alpha / den : (TF)0.5 * s.alpha;
      an = fmin(an, (TF)0.5 * s.alpha);
      s.alpha = fmax(an, (TF)0.1 * s.alpha);
      s.ls++;
#pragma unroll
      for (int i = 0; i < 5; i++) s.xt[i] = s.x[i] + s.alpha * s.p[i];
      if (!(s.alpha * s.alpha * s.pn2 <= (TF)1e-28 * (s.ref2 + (TF)1)) && s.ls < 40) return 0;
      nw_accept(s);
      s.trial = false;
      return 0;
    }
    nw_accept(s);
    s.trial = false;
  }
  if (s.done || s.it >= nc.itmax) return 2;
  TF g[5];
#pragma unroll
  for (int i = 0; i < 5; i++) g[i] = Kx[i] + sh.cc(i) + dt * s.edf[i];
  if (sizeof(TF) == 4 && nc.bound_stop) {
    TF den2 = s.ref2;
    if (!(den2 > (TF)0))
      den2 = s.x[0] * s.x[0] + s.x[1] * s.x[1] + s.x[2] * s.x[2] + s.x[3] * s.x[3] + s.x[4] * s.x[4] + s.h * s.h;
    const TF mu = et[ET_STOT_MIN];
    const TF gn2 = g[0] * g[0] + g[1] * g[1] + g[2] * g[2] + g[3] * g[3] + g[4] * g[4];
    if (gn2 <= s.tol2 * den2 * mu * mu) {
      s.done = true;
      return 2;
    }
  }
#pragma unroll
  for (int i = 0; i < 15; i++) H[i] = sh.k(i) + dt * Df[i];
#pragma unroll
  for (int i = 0; i < 5; i++) mg[i] = -g[i];
  // Phi at x (= xt here), for a line search along the coming direction
  TF phi0 = 0;
#pragma unroll
  for (int i = 0; i < 5; i++) phi0 += s.x[i] * ((TF)0.5 * Kx[i] + sh.cc(i));
  s.phi0 = phi0 + dt * s.psif;
  return 1;
}

// the move along the solved direction p of -g (mg); false: the solve failed
template <typename TF>
__device__ __forceinline__ bool nw_pass_b(NewtonState<TF>& s, const NewtonConst& nc, const TF p[5], bool ok,
                                          const TF mg[5]) {
  if (!ok) {
    s.failed = true;
    return false;
  }
  s.pn2 = 0;
  s.slope = 0;
#pragma unroll
  for (int i = 0; i < 5; i++) {
    s.p[i] = p[i];
    s.pn2 += p[i] * p[i];
    s.slope -= mg[i] * p[i];
  }
  s.alpha = 1;
  if (s.pn2 > s.ls_thr2 && !nc.flow_off) {
    s.ls = 0;
    s.trial = true;
#pragma unroll
    for (int i = 0; i < 5; i++) s.xt[i] = s.x[i] + s.alpha * s.p[i];
    return true;
  }
  nw_accept(s);
#pragma unroll
  for (int i = 0; i < 5; i++) s.xt[i] = s.x[i];
  return true;
}

template <typename TF, typename Load>
__device__ __forceinline__ VoxelOut<TF> nw_finish(const NewtonState<TF>& s, const NewtonConst& nc,
                                                  const TF* __restrict__ et, const Load& load, TF* sig6, TF* ed6) {
  VoxelOut<TF> o;
  o.iters = s.it;
  o.failed = (s.failed || !s.done) ? 1 : 0;
  const TF dt = cpick<TF>(nc.dt, nc.dtf);
  const TF shh = et[ET_SEL_HH];
  TF lam6[6], eps6[6], ep6[6], Q[25];
  {
    TF R[9];
    load(lam6, eps6, ep6, R, true);
    rot_to_q<TF>(R, Q);
  }
  TF ss[5], es[5];
#pragma unroll
  for (int j = 0; j < 5; j++) {
    TF a = 0, b = 0;
#pragma unroll
    for (int i = 0; i < 5; i++) {
      a += Q[i * 5 + j] * s.x[i];
      b += Q[i * 5 + j] * s.edf[i];
    }
    ss[j] = a;
    es[j] = b;
  }
  TF cs = s.dh * s.dh, ce = 0;
#pragma unroll
  for (int i = 0; i < 5; i++) {
    const TF ds = ss[i] - lam6[i];
    cs += ds * ds;
    TF de = ep6[i] + dt * es[i] - eps6[i];
#pragma unroll
    for (int j = 0; j < 5; j++) de += et[ET_SEL + pk(i, j)] * ss[j];
    ce += de * de;
  }
  {
    const TF de = ep6[5] + shh * s.h - eps6[5];
    ce += de * de;
  }
  o.conv_s = sqrt(cs);
  o.conv_e = sqrt(ce);
#pragma unroll
  for (int j = 0; j < 5; j++) {
    sig6[j] = ss[j];
    ed6[j] = es[j];
  }
  sig6[5] = s.h;
  ed6[5] = 0;
  return o;
}

// Local solve of one crystal voxel.  lam6/eps6/ep6: LT sample-frame inputs
// (lambda = current stress, total strain, plastic strain); Q: sample->crystal
// 5x5 of the current lattice orientation; et: elastic-class row (initial
// orientation); tauf: forward CRSS.  Outputs sig6 (sample frame) and ed6
// (plastic strain rate, sample frame).
// TF: flow rule, residual, Hessian assembly, line search and frame
// transforms; TL: precision of the Jacobian (Hessian) solve.  FP64 mode:
// both double.  Mixed mode: TF = float, TL = double: the FP32-assembled 5x5
// system is factored and solved in FP64 at every Newton step.  Mixed
// root-FP64 mode (ROOT_ONLY): the FP64 solve only for the steps within
// 1e-3 |lambda| of the root, which set the converged answer, and the FP32
// factorisation for the large early steps, whose direction only has to be a
// descent direction (GB300 issues FP64 at 1/64 of the FP32 rate).  Fast
// mode: all float.
// load(lam6, eps6, ep6, R, again) fills the voxel's inputs; it is called
// at the start and again (again = true: loads the compiler may not merge
// with the first) for the back-transform and the error norms, so neither
// the inputs nor the 5x5 frame rotation stay live across the Newton loop.
template <typename TF, typename TL, bool ROOT_ONLY, typename Slip, typename Load>
__device__ VoxelOut<TF> solve_voxel(const NewtonConst& nc, const PhaseConst& ph, const TF* __restrict__ et, const Slip& slip,
                                    const Load& load, TF* sig6, TF* ed6) {
  NewtonState<TF> s;
  NewtonRegs<TF> r;
  nw_init(s, r, nc, et, load);
  for (;;) {
    TF H[15], mg[5];
    const int k = nw_pass_a(s, r, nc, ph, slip, et, H, mg);
    if (k == 2) break;
    if (k == 0) continue;
    TF p[5];
    bool ok;
    if (sizeof(TL) > sizeof(TF) && (!ROOT_ONLY || s.near_root)) {
      // Jacobian solve in TL (FP64) of the TF-assembled system: at every
      // step, or (ROOT_ONLY) for the steps within 1e-3 |lambda| of the
      // root, which set the converged answer
      ok = ldl_solve5_wide<TF, TL>(H, mg, p);
    } else {
      ok = ldl_solve5<TF>(H, mg, p);
    }
    if (!nw_pass_b(s, nc, p, ok, mg)) break;
  }
  return nw_finish(s, nc, et, load, sig6, ed6);
}

// ------------------------------------------------------------ reductions
template <int W>
__device__ __forceinline__ void block_reduce_store(double (&v)[W], double* out) {
  __shared__ double sm[W][8];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < W; i++) {
    double a = v[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
    if (lane == 0) sm[i][wid] = a;
  }
  __syncthreads();
  if (threadIdx.x < W) {
    double a = 0;
    const int nw = blockDim.x >> 5;
    for (int w = 0; w < nw; w++) a += sm[threadIdx.x][w];
    out[(size_t)blockIdx.x * W + threadIdx.x] = a;
  }
}

// Block sum of W per-thread values for 256-thread blocks, in FP64 in a fixed
// order: the values are staged in shared memory (in their own precision);
// 16 threads per component each sum 16 of them (stride 16), one thread per
// component sums the 16 partials.  The row stride 256 + 16 keeps the
// two components read by one warp on opposite bank halves.
template <typename TV, int W>
__device__ __forceinline__ void block_reduce_smem(const TV (&v)[W], double* out) {
  constexpr int NT = 256, LD = NT + 16;
  static_assert(W <= 16, "at most 16 components");
  __shared__ TV sv[W][LD];
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
      for (int k = 0; k < NT / 16; k++) a += (double)sv[comp][k * 16 + chunk];
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

// Block sums of the Newton kernel's NPART values, as block_reduce_smem, with
// two exact savings: when ph1_only the phase-1 stress sums (components
// 8..13) are the total ones (2..7), added once and written twice; the
// Newton-iteration and failure counts (14, 15: small integers) are summed in
// the staging precision, exact below 2^24.
constexpr int NRED_LD = 256 + 16;   // row stride of the staged values
template <typename TV>
__device__ __forceinline__ void newton_block_reduce_in(const TV (&v)[NPART], double* out, bool ph1_only,
                                                       TV (*sv)[NRED_LD], double (*sp)[16]);
template <typename TV>
__device__ __forceinline__ void newton_block_reduce(const TV (&v)[NPART], double* out, bool ph1_only) {
  __shared__ TV sv[NPART][NRED_LD];
  __shared__ double sp[NPART][16];
  newton_block_reduce_in<TV>(v, out, ph1_only, sv, sp);
}
// the same with the staging buffers given (the cooperative kernel lays them
// over its system buffers, free once its pass loop has ended)
template <typename TV>
__device__ __forceinline__ void newton_block_reduce_in(const TV (&v)[NPART], double* out, bool ph1_only,
                                                       TV (*sv)[NRED_LD], double (*sp)[16]) {
  constexpr int NT = 256;
  const int t = threadIdx.x;
#pragma unroll
  for (int i = 0; i < NPART; i++)
    if (!ph1_only || i < 8 || i >= 14) sv[i][t] = v[i];
  __syncthreads();
  {
    const int comp = t >> 4, chunk = t & 15;
    if (comp >= 14) {
      TV a = 0;
#pragma unroll
      for (int k = 0; k < NT / 16; k++) a += sv[comp][k * 16 + chunk];
      sp[comp][chunk] = (double)a;
    } else if (!ph1_only || comp < 8) {
      double a = 0.0;
#pragma unroll
      for (int k = 0; k < NT / 16; k++) a += to_f64(sv[comp][k * 16 + chunk]);
      sp[comp][chunk] = a;
    }
  }
  __syncthreads();
  if (t < NPART) {
    const int src = (ph1_only && t >= 8 && t < 14) ? t - 6 : t;
    double a = 0.0;
#pragma unroll
    for (int k = 0; k < 16; k++) a += sp[src][k];
    out[(size_t)blockIdx.x * NPART + t] = a;
  }
}

// Loads of a global value that the compiler keeps as separate loads (used to
// re-read a voxel's inputs after the Newton loop instead of holding them).
__device__ __forceinline__ float ld_again(const float* p) {
  float v;
  asm volatile("ld.global.cg.f32 %0, [%1];" : "=f"(v) : "l"(__cvta_generic_to_global(p)));
  return v;
}
__device__ __forceinline__ double ld_again(const double* p) {
  double v;
  asm volatile("ld.global.cg.f64 %0, [%1];" : "=d"(v) : "l"(__cvta_generic_to_global(p)));
  return v;
}
template <typename T>
__device__ __forceinline__ T ld_sel(const T* p, bool again) { return again ? ld_again(p) : *p; }

// ------------------------------------------------------------ Newton kernel
template <typename TSt, typename TF, typename TS, int MINB, bool ROOT_ONLY = false, int LAW = 0>
__global__ void __launch_bounds__(256, MINB) newton_kernel(const NewtonConst nc, Fields<TSt> f, double* __restrict__ partials,
                                                                IterIn it) {
  if (!is_live(it)) return;
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long P = f.nv;
  TF acc[NPART];
#pragma unroll
  for (int i = 0; i < NPART; i++) acc[i] = (TF)0;
  if (v < P) {
    const int jph = f.phase[v];
    const PhaseConst& ph = nc.ph[jph];
    if (ph.type == 0) {
      typename SlipOf<LAW, TF, TSt>::type slip;
      SlipOf<LAW, TF, TSt>::load(ph, f, v, slip);
      auto load = [&](TF* lam6, TF* eps6, TF* ep6, TF* R, bool again) {
#pragma unroll
        for (int i = 0; i < 6; i++) {
          lam6[i] = (TF)ld_sel(f.sig + i * P + v, again);
          eps6[i] = (TF)ld_sel(f.strain + i * P + v, again);
          ep6[i] = (TF)ld_sel(f.epsp + i * P + v, again);
        }
#pragma unroll
        for (int i = 0; i < 9; i++) R[i] = (TF)ld_sel(f.rot + i * P + v, again);
      };
      TF s6[6], e6[6];
      const TF* et = cpick_ptr<TF>(f.etab, f.etabf) + (size_t)f.eclass[v] * ETAB_W;
      VoxelOut<TF> o = solve_voxel<TF, TS, ROOT_ONLY>(nc, ph, et, slip, load, s6, e6);
#pragma unroll
      for (int i = 0; i < 6; i++) {
        f.sig[i * P + v] = (TSt)s6[i];
        f.edot[i * P + v] = (TSt)e6[i];
      }
      acc[0] = o.conv_s;
      acc[1] = o.conv_e;
#pragma unroll
      for (int i = 0; i < 6; i++) {
        acc[2 + i] = s6[i];
        acc[8 + i] = jph == 0 ? s6[i] : (TF)0;
      }
      acc[14] = (TF)o.iters;    // small integers: exact in float
      acc[15] = (TF)o.failed;
    } else {
#pragma unroll
      for (int i = 0; i < 6; i++) {
        f.sig[i * P + v] = (TSt)0;
        f.edot[i * P + v] = (TSt)0;
      }
    }
  }
  newton_block_reduce<TF>(acc, partials, nc.ph1_only != 0);
}

// Newton kernel of the mixed modes with the FP64 Jacobian solve at every
// step.  A warp runs its Newton passes until its slowest thread has ended,
// so with the solves done by each thread about a third of the lanes of every
// FP64 instruction idled.  Here the block's threads step their solves in
// lock-step passes (a block-wide vote ends the loop): in each pass the
// threads that need a Newton direction put their 5x5 systems in shared
// memory, in thread order, the first n threads of the block solve the n
// systems in FP64, and each thread reads its direction back.  Every voxel's
// iterates and result are those of solve_voxel.
#ifndef MTH_COOP_TAU_SMEM
#define MTH_COOP_TAU_SMEM 1   // power-law CRSS of the cooperative kernel in shared memory
#endif
template <typename TSt, typename TF, typename TL, int MINB, int LAW = 0>
__global__ void __launch_bounds__(256, MINB) newton_coop_kernel(const NewtonConst nc, Fields<TSt> f,
                                                                double* __restrict__ partials, IterIn it) {
  if (!is_live(it)) return;
  // the systems of a pass (H, -g in / direction out), and after the pass
  // loop the block sums' staging buffers, in one static buffer
  constexpr size_t SYS_B = sizeof(TF) * 20 * 256, RED_B = sizeof(TF) * NPART * NRED_LD + sizeof(double) * NPART * 16;
  __shared__ __align__(16) unsigned char sbuf[SYS_B > RED_B ? SYS_B : RED_B];
  TF(*sH)[256] = reinterpret_cast<TF(*)[256]>(sbuf);
  TF(*sB)[256] = reinterpret_cast<TF(*)[256]>(sbuf + sizeof(TF) * 15 * 256);
  extern __shared__ __align__(16) unsigned char coop_dyn[];   // K [15][256], c [5][256], CRSS [256][NSYS + 1]
  __shared__ int sOk[256];
  __shared__ int sWarp[8];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const long long v = (long long)blockIdx.x * blockDim.x + t;
  const long long P = f.nv;
  TF acc[NPART];
#pragma unroll
  for (int i = 0; i < NPART; i++) acc[i] = (TF)0;
  int jph = 0;
  bool active = false;
  const TF* et = nullptr;
  // power law: the CRSS in shared memory, after K and c
  using SlipT = std::conditional_t<LAW == 0 && MTH_COOP_TAU_SMEM, PlSlipSh<TF>, typename SlipOf<LAW, TF, TSt>::type>;
  SlipT slip;
  NewtonState<TF> s;
  const NewtonShared<TF> sh{reinterpret_cast<TF(*)[256]>(coop_dyn),
                            reinterpret_cast<TF(*)[256]>(coop_dyn + 15 * 256 * sizeof(TF)), t};
  auto load = [&](TF* lam6, TF* eps6, TF* ep6, TF* R, bool again) {
#pragma unroll
    for (int i = 0; i < 6; i++) {
      lam6[i] = (TF)ld_sel(f.sig + i * P + v, again);
      eps6[i] = (TF)ld_sel(f.strain + i * P + v, again);
      ep6[i] = (TF)ld_sel(f.epsp + i * P + v, again);
    }
#pragma unroll
    for (int i = 0; i < 9; i++) R[i] = (TF)ld_sel(f.rot + i * P + v, again);
  };
  if (v < P) {
    jph = f.phase[v];
    const PhaseConst& ph = nc.ph[jph];
    if (ph.type == 0) {
      if constexpr (LAW == 0 && MTH_COOP_TAU_SMEM) {
        TF* tau = reinterpret_cast<TF*>(coop_dyn + 20 * 256 * sizeof(TF)) + t * (NSYS + 1);
#pragma unroll
        for (int q = 0; q < NSYS; q++) tau[q] = q < ph.nsys ? (TF)f.crss[q * P + v] : (TF)1;
        slip.tauf = tau;
        slip.tau_off = cpick<TF>(ph.tau_back_minus_fwd, ph.tau_offf);
      } else {
        SlipOf<LAW, TF, TSt>::load(ph, f, v, slip);
      }
      et = cpick_ptr<TF>(f.etab, f.etabf) + (size_t)f.eclass[v] * ETAB_W;
      nw_init(s, sh, nc, et, load);
      active = true;
    } else {
#pragma unroll
      for (int i = 0; i < 6; i++) {
        f.sig[i * P + v] = (TSt)0;
        f.edot[i * P + v] = (TSt)0;
      }
    }
  }
  const bool crystal = active;
  // every thread of the block takes part in every barrier of this loop
  while (__syncthreads_or(active)) {
    TF H[15], mg[5];
    int need = 0;
    if (active) {
      const int r = nw_pass_a(s, sh, nc, nc.ph[jph], slip, et, H, mg);
      if (r == 2) active = false;
      need = r == 1;
    }
    // slots of the systems, in thread order
    const unsigned m = __ballot_sync(0xffffffffu, need);
    if (lane == 0) sWarp[w] = __popc(m);
    __syncthreads();
    int base = 0, n = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
      base += k < w ? sWarp[k] : 0;
      n += sWarp[k];
    }
    const int slot = base + __popc(m & ((1u << lane) - 1u));
    if (need) {
#pragma unroll
      for (int i = 0; i < 15; i++) sH[i][slot] = H[i];
#pragma unroll
      for (int i = 0; i < 5; i++) sB[i][slot] = mg[i];
    }
    __syncthreads();
    if (t < n) {
      TF Hs[15], bs[5], ps[5];
#pragma unroll
      for (int i = 0; i < 15; i++) Hs[i] = sH[i][t];
#pragma unroll
      for (int i = 0; i < 5; i++) bs[i] = sB[i][t];
      const bool ok = ldl_solve5_wide<TF, TL>(Hs, bs, ps);
#pragma unroll
      for (int i = 0; i < 5; i++) sB[i][t] = ps[i];
      sOk[t] = ok ? 1 : 0;
    }
    __syncthreads();
    if (need) {
      TF pd[5];
#pragma unroll
      for (int i = 0; i < 5; i++) pd[i] = sB[i][slot];
      if (!nw_pass_b(s, nc, pd, sOk[slot] != 0, mg)) active = false;
    }
  }
  if (crystal) {
    TF s6[6], e6[6];
    const VoxelOut<TF> o = nw_finish(s, nc, et, load, s6, e6);
#pragma unroll
    for (int i = 0; i < 6; i++) {
      f.sig[i * P + v] = (TSt)s6[i];
      f.edot[i * P + v] = (TSt)e6[i];
    }
    acc[0] = o.conv_s;
    acc[1] = o.conv_e;
#pragma unroll
    for (int i = 0; i < 6; i++) {
      acc[2 + i] = s6[i];
      acc[8 + i] = jph == 0 ? s6[i] : (TF)0;
    }
    acc[14] = (TF)o.iters;
    acc[15] = (TF)o.failed;
  }
  newton_block_reduce_in<TF>(acc, partials, nc.ph1_only != 0, reinterpret_cast<TF(*)[NRED_LD]>(sbuf),
                             reinterpret_cast<double(*)[16]>(sbuf + sizeof(TF) * NPART * NRED_LD));
}

// newton_coop_kernel for the FP32 fields with the FP64 solve, with its 33 KB
// of dynamic shared memory (K and c of each thread's solve, its CRSS)
constexpr size_t COOP_DYN = (20 + (MTH_COOP_TAU_SMEM ? NSYS + 1 : 0)) * 256 * sizeof(float);

// the opt-in above 48 KB of shared memory per block, once per device (also
// done by prepare_newton_kernels when a context is created, so that no
// attribute call falls inside a stream capture)
template <int MINB, int LAW>
static cudaError_t coop_attr() {
  static bool attr[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev >= 0 && dev < 64 && attr[dev]) return cudaSuccess;
  e = cudaFuncSetAttribute(newton_coop_kernel<float, float, double, MINB, LAW>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)COOP_DYN);
  if (e == cudaSuccess && dev >= 0 && dev < 64) attr[dev] = true;
  return e;
}

template <int MINB, int LAW>
static cudaError_t launch_coop(const NewtonConst& nc, const Fields<float>& f, double* partials, int nblocks,
                               const IterIn& it, cudaStream_t st) {
  cudaError_t e = coop_attr<MINB, LAW>();
  if (e != cudaSuccess) return e;
  return launch_chain(newton_coop_kernel<float, float, double, MINB, LAW>, dim3(nblocks), dim3(256), COOP_DYN, st,
                      it.pdl, nc, f, partials, it);
}

// blocks per SM the cooperative kernel is compiled for: 4 (64 registers,
// 54.5 KB of shared memory per block with the block sums' buffers laid over
// the system buffers and the CRSS in shared memory) against 3 (80
// registers): 301.2 against 319.7 ms for the 300 Newton launches of three
// 128^3 steps (307.2 ms with the CRSS in registers; 5 blocks at 48
// registers, 352.8 ms)
#ifndef MTH_COOP_MINB
#define MTH_COOP_MINB 4
#endif
cudaError_t prepare_newton_kernels() { return coop_attr<MTH_COOP_MINB, 0>(); }

void fill_float_consts(NewtonConst& nc) {
  for (int k = 0; k < 2; k++) {
    PhaseConst& ph = nc.ph[k];
    ph.nrsf = (float)ph.nrs;
    ph.gamd0f = (float)ph.gamd0;
    ph.tau_offf = (float)ph.tau_back_minus_fwd;
    for (int s = 0; s < NSYS; s++) {
      for (int i = 0; i < 5; i++) ph.m_xtf[s][i] = (float)ph.m_xt[s][i];
      for (int i = 0; i < 3; i++) {
        ph.bnf[s][i] = (float)ph.bn[s][i];
        ph.bbf[s][i] = (float)ph.bb[s][i];
      }
      for (int j = 0; j < NSYS; j++) ph.hardf[s][j] = (float)ph.hard[s][j];
    }
    ph.tau0ff = (float)ph.tau0f;
    ph.tau1f = (float)ph.tau1;
    ph.thet0f = (float)ph.thet0;
    ph.thet1f = (float)ph.thet1;
  }
  for (int i = 0; i < 25; i++) nc.s0devf[i] = (float)nc.s0dev[i];
  nc.s0hhf = (float)nc.s0hh;
  nc.dtf = (float)nc.dt;
  nc.tolf = (float)nc.tol;
}

// blocks per SM of the one-solve-per-thread kernels: the
// dislocation-density law in the mixed modes, and the FP32-solve and
// near-root FP64 modes of the power law.  Measured at 128^3: the
// dislocation-density law 2.31e9 voxel-iterations/s with 2 blocks against
// 2.09e9 (3) and 2.12e9 (4); FP32 solves 2.55e9 with 3 against 2.52e9 (4);
// near-root FP64 solves the same with 3 and 4
#ifndef MTH_DD_MINB
#define MTH_DD_MINB 2
#endif
#ifndef MTH_FAST_MINB
#define MTH_FAST_MINB 3
#endif
#ifndef MTH_FP64_MINB
#define MTH_FP64_MINB 1   // FP64 mode: 1.01e8 with 1 (255 registers) against 0.99e8 with 2 (128, 516 B of spills)
#endif
cudaError_t launch_newton(int mixed, const NewtonConst& nc_in, const void* fields, double* partials, int nblocks,
                          const IterIn& it, cudaStream_t st, int law) {
  NewtonConst nc = nc_in;
  fill_float_consts(nc);
  if (law == 1) {
    // dislocation-density law: the FP64 Jacobian solve at every step in the
    // mixed modes (no FP32-solve variants)
    if (mixed) {
      const Fields<float>& f = *static_cast<const Fields<float>*>(fields);
      return launch_chain(newton_kernel<float, float, double, MTH_DD_MINB, false, 1>, dim3(nblocks), dim3(256), 0, st,
                          it.pdl, nc, f, partials, it);
    } else {
      const Fields<double>& f = *static_cast<const Fields<double>*>(fields);
      return launch_chain(newton_kernel<double, double, double, 1, false, 1>, dim3(nblocks), dim3(256), 0, st, it.pdl,
                          nc, f, partials, it);
    }
    return cudaGetLastError();
  }
  if (mixed == 2) {
    const Fields<float>& f = *static_cast<const Fields<float>*>(fields);
    return launch_chain(newton_kernel<float, float, float, MTH_FAST_MINB>, dim3(nblocks), dim3(256), 0, st, it.pdl, nc,
                        f, partials, it);
  } else if (mixed == 3) {
    const Fields<float>& f = *static_cast<const Fields<float>*>(fields);
    return launch_chain(newton_kernel<float, float, double, MTH_FAST_MINB, true>, dim3(nblocks), dim3(256), 0, st,
                        it.pdl, nc, f, partials, it);
  } else if (mixed) {
    const Fields<float>& f = *static_cast<const Fields<float>*>(fields);
    return launch_coop<MTH_COOP_MINB, 0>(nc, f, partials, nblocks, it, st);
  } else {
    const Fields<double>& f = *static_cast<const Fields<double>*>(fields);
    return launch_chain(newton_kernel<double, double, double, MTH_FP64_MINB>, dim3(nblocks), dim3(256), 0, st, it.pdl,
                        nc, f, partials, it);
  }
  return cudaGetLastError();
}

// ------------------------------------------------------- end-of-step kernel
// Eps += Edot dt (src/evolution.c:1500-1504), update_orient + Orientation
// (src/constitutive.c:142-273) and harden (src/constitutive.c:275-326).
// anti_u: uniform part of the lattice spin increment, (2,1),(0,2),(1,0)
// components of 2 Udot_a dt + antisym(sum dDisGradAvg).
template <typename TSt, typename TF, int LAW = 0>
__global__ void __launch_bounds__(256) end_step_kernel(const NewtonConst nc, Fields<TSt> f, double au0, double au1,
                                                       double au2, int do_orient, int do_harden,
                                                       double* __restrict__ partials) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long P = f.nv;
  TF acc[NPART_END];
#pragma unroll
  for (int i = 0; i < NPART_END; i++) acc[i] = (TF)0;
  if (v < P) {
    const int jph = f.phase[v];
    const PhaseConst& ph = nc.ph[jph];
    const TF dt = cpick<TF>(nc.dt, nc.dtf);
#pragma unroll
    for (int i = 0; i < 6; i++) {
      const TF ed = (TF)f.edot[i * P + v];
      const TF ep = (TF)f.epsp[i * P + v] + ed * dt;
      f.epsp[i * P + v] = (TSt)ep;
      acc[i] = ep;
      acc[6 + i] = ed;
    }
    if (ph.type == 0 && (do_orient || do_harden)) {
      TF R[9], Q[25], s6[6], x[5], gam[NSYS], ed[5], psi;
#pragma unroll
      for (int i = 0; i < 9; i++) R[i] = (TF)f.rot[i * P + v];
#pragma unroll
      for (int i = 0; i < 6; i++) s6[i] = (TF)f.sig[i * P + v];
      typename SlipOf<LAW, TF, TSt>::type slip;
      SlipOf<LAW, TF, TSt>::load(ph, f, v, slip);
      rot_to_q<TF>(R, Q);
#pragma unroll
      for (int i = 0; i < 5; i++) {
        TF a = 0;
#pragma unroll
        for (int j = 0; j < 5; j++) a += Q[i * 5 + j] * s6[j];
        x[i] = a;
      }
#pragma unroll
      for (int s = 0; s < NSYS; s++) gam[s] = 0;
      if (!nc.flow_off) slip.template flow<false>(ph, x, ed, nullptr, psi, gam);
      if (do_orient) {
        // plastic spin: RotSlip = -1/2 T sum_a gam_a (b_a x n_a)
        TF cx = 0, cy = 0, cz = 0;
#pragma unroll
        for (int s = 0; s < NSYS; s++) {
          if (s >= ph.nsys) break;
          const TF b0 = cpick<TF>(ph.bb[s][0], ph.bbf[s][0]), b1 = cpick<TF>(ph.bb[s][1], ph.bbf[s][1]),
                   b2 = cpick<TF>(ph.bb[s][2], ph.bbf[s][2]);
          const TF n0 = cpick<TF>(ph.bn[s][0], ph.bnf[s][0]), n1 = cpick<TF>(ph.bn[s][1], ph.bnf[s][1]),
                   n2 = cpick<TF>(ph.bn[s][2], ph.bnf[s][2]);
          cx += gam[s] * (b1 * n2 - b2 * n1);
          cy += gam[s] * (b2 * n0 - b0 * n2);
          cz += gam[s] * (b0 * n1 - b1 * n0);
        }
        TF ws[3];
#pragma unroll
        for (int i = 0; i < 3; i++) ws[i] = (TF)-0.5 * (R[i * 3 + 0] * cx + R[i * 3 + 1] * cy + R[i * 3 + 2] * cz);
        // Rot = (Udot_a + RotLoc - RotSlip) dt, as the vector (Rot21, Rot02, Rot10)
        TF w[3];
        w[0] = (TF)au0 + (TF)f.wspin[0 * P + v] - ws[0] * dt;
        w[1] = (TF)au1 + (TF)f.wspin[1 * P + v] - ws[1] * dt;
        w[2] = (TF)au2 + (TF)f.wspin[2 * P + v] - ws[2] * dt;
        // Orientation (src/constitutive.c:142-194)
        TF wn = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
        TF wt = tan(wn / (TF)2);
        if (fabs(wn) < (TF)1e-6) wn = (TF)1;
#pragma unroll
        for (int i = 0; i < 3; i++) w[i] *= wt / wn;
        TF om[3][3] = {{0, -w[2], w[1]}, {w[2], 0, -w[0]}, {-w[1], w[0], 0}};
        TF rot[3][3];
        wt = wt * wt;
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
          for (int j = 0; j < 3; j++) {
            TF o2 = om[i][0] * om[0][j] + om[i][1] * om[1][j] + om[i][2] * om[2][j];
            rot[i][j] = (TF)(i == j) + (TF)2 * (om[i][j] + o2) / ((TF)1 + wt);
          }
        TF Rn[9];
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
          for (int j = 0; j < 3; j++) Rn[i * 3 + j] = rot[i][0] * R[0 * 3 + j] + rot[i][1] * R[1 * 3 + j] + rot[i][2] * R[2 * 3 + j];
#pragma unroll
        for (int i = 0; i < 9; i++) f.rot[i * P + v] = (TSt)Rn[i];
      }
      if (do_harden) {
        const TF gamtot = (TF)f.gamacum[v];
        TF deltgam = 0;
#pragma unroll
        for (int s = 0; s < NSYS; s++) deltgam += fabs(gam[s]) * dt;   // gam is 0 past nsys
        if (deltgam > (TF)0) {
          const TF tau0 = cpick<TF>(ph.tau0f, ph.tau0ff), tau1 = cpick<TF>(ph.tau1, ph.tau1f),
                   th0 = cpick<TF>(ph.thet0, ph.thet0f), th1 = cpick<TF>(ph.thet1, ph.thet1f);
          const TF tiny = (TF)1e-4 * tau0;
          TF voce = 0;
          if (fabs(th0) > tiny) {
            voce = th1 * deltgam;
            if (fabs(tau1) > tiny) {
              // the Voce increment of harden (src/constitutive.c:293-316) with
              // exp(-dgam fact) - 1 as expm1 and the second bracket regrouped
              // as (e - 1)(gam fact + 1) + e dgam fact: the same value without
              // the cancellation of nearly equal terms (FP32 in mixed mode)
              const TF fact = fabs(th0 / tau1);
              const TF exp_ini = exp((TF)-1 * gamtot * fact);
              const TF em1 = expm1((TF)-1 * deltgam * fact);
              const TF exp_del = em1 + (TF)1;
              voce += (TF)-1 * (fact * tau1 - th1) / fact * exp_ini * em1 -
                      th1 / fact * exp_ini * (em1 * (gamtot * fact + (TF)1) + exp_del * deltgam * fact);
            }
          }
#pragma unroll
          for (int s = 0; s < NSYS; s++) {
            if (s >= ph.nsys) break;
            TF dtau = 0;
#pragma unroll
            for (int j = 0; j < NSYS; j++) dtau += cpick<TF>(ph.hard[s][j], ph.hardf[s][j]) * fabs(gam[j]) * dt;
            f.crss[s * P + v] = (TSt)((TF)f.crss[s * P + v] + dtau * voce / deltgam);
          }
          f.gamacum[v] = (TSt)(gamtot + deltgam);
        }
      }
    }
  }
  block_reduce_smem<TF, NPART_END>(acc, partials);
}

cudaError_t launch_end_step(int mixed, const NewtonConst& nc_in, const void* fields, const double au[3], int do_orient,
                            int do_harden, double* partials, int nblocks, cudaStream_t st, int law) {
  NewtonConst nc = nc_in;
  fill_float_consts(nc);
  if (law == 1) {
    if (mixed) {
      const Fields<float>& f = *static_cast<const Fields<float>*>(fields);
      end_step_kernel<float, float, 1><<<nblocks, 256, 0, st>>>(nc, f, au[0], au[1], au[2], do_orient, 0, partials);
    } else {
      const Fields<double>& f = *static_cast<const Fields<double>*>(fields);
      end_step_kernel<double, double, 1><<<nblocks, 256, 0, st>>>(nc, f, au[0], au[1], au[2], do_orient, 0, partials);
    }
    return cudaGetLastError();
  }
  if (mixed) {
    const Fields<float>& f = *static_cast<const Fields<float>*>(fields);
    end_step_kernel<float, float><<<nblocks, 256, 0, st>>>(nc, f, au[0], au[1], au[2], do_orient, do_harden, partials);
  } else {
    const Fields<double>& f = *static_cast<const Fields<double>*>(fields);
    end_step_kernel<double, double><<<nblocks, 256, 0, st>>>(nc, f, au[0], au[1], au[2], do_orient, do_harden, partials);
  }
  return cudaGetLastError();
}

// ------------------------------------------------------------ set-up kernel
// Per voxel: crystal->sample matrix from Bunge angles (EulerToTransMatrix,
// src/kinematics.c:187-240, transposed as at src/init.c:276-278), the
// elastic initial stress C_gr : <grad u> (src/init.c:470-480) and the
// initial CRSS (src/init.c:1164-1170).  C066 is summed on the host from the
// elastic classes.
template <typename TSt>
__global__ void __launch_bounds__(256) setup_kernel(const NewtonConst nc, Fields<TSt> f, const double* __restrict__ euler,
                                                    AddVec d6) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long P = f.nv;
  if (v >= P) return;
  const int jph = f.phase[v];
  const PhaseConst& ph = nc.ph[jph];
#pragma unroll
  for (int i = 0; i < 6; i++) {
    f.strain[i * P + v] = (TSt)0;
    f.epsp[i * P + v] = (TSt)0;
    f.edot[i * P + v] = (TSt)0;
    f.sig[i * P + v] = (TSt)0;
  }
  for (int i = 0; i < 3; i++) f.wspin[i * P + v] = (TSt)0;
  f.gamacum[v] = (TSt)0;
  double R[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  if (ph.type == 0) {
    const double d2r = 3.14159265359 / 180.;
    const double t1 = euler[3 * v] * d2r, p = euler[3 * v + 1] * d2r, t2 = euler[3 * v + 2] * d2r;
    const double ct1 = cos(t1), st1 = sin(t1), cph = cos(p), sph = sin(p), ct2 = cos(t2), st2 = sin(t2);
    double a[3][3];
    a[0][0] = ct1 * ct2 - st1 * st2 * cph;
    a[0][1] = st1 * ct2 + ct1 * st2 * cph;
    a[0][2] = st2 * sph;
    a[1][0] = -1.0 * ct1 * st2 - st1 * ct2 * cph;
    a[1][1] = -1.0 * st1 * st2 + ct1 * ct2 * cph;
    a[1][2] = ct2 * sph;
    a[2][0] = st1 * sph;
    a[2][1] = -1.0 * ct1 * sph;
    a[2][2] = cph;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) R[i * 3 + j] = a[j][i];
    const double* et = f.etab + (size_t)f.eclass[v] * ETAB_W;
    double s6[6];
#pragma unroll
    for (int i = 0; i < 5; i++) {
      double s = 0;
#pragma unroll
      for (int j = 0; j < 5; j++) s += et[ET_CGR + pk(i, j)] * d6.v[j];
      s6[i] = s;
    }
    s6[5] = et[ET_CGR_HH] * d6.v[5];
#pragma unroll
    for (int i = 0; i < 6; i++) f.sig[i * P + v] = (TSt)s6[i];
    for (int s = 0; s < NSYS; s++) f.crss[s * P + v] = (TSt)(s < ph.nsys ? ph.tau0f : 0.0);
  } else {
    for (int s = 0; s < NSYS; s++) f.crss[s * P + v] = (TSt)0;
  }
#pragma unroll
  for (int i = 0; i < 9; i++) f.rot[i * P + v] = (TSt)R[i];
}

cudaError_t launch_setup(int mixed, const NewtonConst& nc, const void* fields, const double* euler, const double d6[6],
                         int nblocks, cudaStream_t st) {
  AddVec d;
  for (int i = 0; i < 6; i++) d.v[i] = d6[i];
  if (mixed) {
    const Fields<float>& f = *static_cast<const Fields<float>*>(fields);
    setup_kernel<float><<<nblocks, 256, 0, st>>>(nc, f, euler, d);
  } else {
    const Fields<double>& f = *static_cast<const Fields<double>*>(fields);
    setup_kernel<double><<<nblocks, 256, 0, st>>>(nc, f, euler, d);
  }
  return cudaGetLastError();
}

// ------------------------------------------------------------ downloads
// Field planes to voxel-major doubles for the host: a symmetric tensor of 6
// LT planes becomes the 3x3 row-major Cartesian tensor t = sum_i v_i B_i
// (the products and left-to-right sums of the host conversion, with
// rounded, uncontracted operations, so both give the same doubles); other
// fields are interleaved per voxel.
// the symmetric tensor of voxel v's 6 LT planes, row-major into o[9]
template <typename TSt>
__device__ __forceinline__ void sym_to_host(const TSt* __restrict__ src, long long P, long long v, double* o) {
  double a[6];
#pragma unroll
  for (int i = 0; i < 6; i++) a[i] = (double)src[i * P + v];
  const double r2 = RSQ2, r3 = RSQ3, r6 = RSQ6;
  const double t00 = __dadd_rn(__dadd_rn(__dmul_rn(a[0], -r2), __dmul_rn(a[1], -r6)), __dmul_rn(a[5], r3));
  const double t11 = __dadd_rn(__dadd_rn(__dmul_rn(a[0], r2), __dmul_rn(a[1], -r6)), __dmul_rn(a[5], r3));
  const double t22 = __dadd_rn(__dmul_rn(a[1], 2. * r6), __dmul_rn(a[5], r3));
  const double t12 = __dmul_rn(a[2], r2), t02 = __dmul_rn(a[3], r2), t01 = __dmul_rn(a[4], r2);
  o[0] = t00; o[1] = t01; o[2] = t02;
  o[3] = t01; o[4] = t11; o[5] = t12;
  o[6] = t02; o[7] = t12; o[8] = t22;
}

template <typename TSt>
__global__ void to_host_layout_kernel(const TSt* __restrict__ src, long long P, int nc, int sym,
                                      double* __restrict__ dst) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= P) return;
  if (sym) {
    sym_to_host(src, P, v, dst + 9 * v);
  } else {
    for (int i = 0; i < nc; i++) dst[nc * v + i] = (double)src[i * P + v];
  }
}

// DisGrad for the host: the symmetric part from the strain planes plus the
// antisymmetric part W, held as the planes (W21, W02, W10)
template <typename TSt>
__global__ void disgrad_to_host_kernel(const TSt* __restrict__ strain, const TSt* __restrict__ skew, long long P,
                                       double* __restrict__ dst) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= P) return;
  double* o = dst + 9 * v;
  sym_to_host(strain, P, v, o);
  const double w21 = (double)skew[v], w02 = (double)skew[P + v], w10 = (double)skew[2 * P + v];
  o[1] = __dsub_rn(o[1], w10);
  o[3] = __dadd_rn(o[3], w10);
  o[2] = __dadd_rn(o[2], w02);
  o[6] = __dsub_rn(o[6], w02);
  o[5] = __dsub_rn(o[5], w21);
  o[7] = __dadd_rn(o[7], w21);
}

cudaError_t launch_disgrad_to_host(int mixed, const void* strain, const void* skew, long long P, double* dst,
                                   cudaStream_t st) {
  const int nb = (int)((P + 255) / 256);
  if (mixed)
    disgrad_to_host_kernel<float><<<nb, 256, 0, st>>>(static_cast<const float*>(strain),
                                                       static_cast<const float*>(skew), P, dst);
  else
    disgrad_to_host_kernel<double><<<nb, 256, 0, st>>>(static_cast<const double*>(strain),
                                                        static_cast<const double*>(skew), P, dst);
  return cudaGetLastError();
}

// The antisymmetric part of DisGrad grows each step by that of its uniform
// increments (Udot dt at the step's start, the dDisGradAvg corrections
// before each iteration), u, and by that of the Gamma : sigma-hat terms added
// at src/evolution.c:1401, which the Green passes accumulate and the spin
// transform brings to wspin.  skew += u + wspin, all as (W21, W02, W10).
template <typename TSt>
__global__ void disgrad_skew_kernel(const TSt* __restrict__ wspin, TSt* __restrict__ skew, long long P, double u0,
                                    double u1, double u2) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= P) return;
  const double u[3] = {u0, u1, u2};
#pragma unroll
  for (int c = 0; c < 3; c++) skew[c * P + v] = (TSt)((double)skew[c * P + v] + (u[c] + (double)wspin[c * P + v]));
}

cudaError_t launch_disgrad_skew(int mixed, const void* wspin, void* skew, long long P, const double u[3],
                                cudaStream_t st) {
  const int nb = (int)((P + 255) / 256);
  if (mixed)
    disgrad_skew_kernel<float><<<nb, 256, 0, st>>>(static_cast<const float*>(wspin), static_cast<float*>(skew), P,
                                                    u[0], u[1], u[2]);
  else
    disgrad_skew_kernel<double><<<nb, 256, 0, st>>>(static_cast<const double*>(wspin), static_cast<double*>(skew),
                                                     P, u[0], u[1], u[2]);
  return cudaGetLastError();
}

cudaError_t launch_to_host_layout(int mixed, const void* src, long long P, int nc, int sym, double* dst,
                                  cudaStream_t st) {
  const int nb = (int)((P + 255) / 256);
  if (mixed)
    to_host_layout_kernel<float><<<nb, 256, 0, st>>>(static_cast<const float*>(src), P, nc, sym, dst);
  else
    to_host_layout_kernel<double><<<nb, 256, 0, st>>>(static_cast<const double*>(src), P, nc, sym, dst);
  return cudaGetLastError();
}

// --------------------------------------------------------- batch local solve
__global__ void __launch_bounds__(256) local_solve_kernel(const NewtonConst nc, long long n, double* __restrict__ sig,
                                                          const double* __restrict__ epsp,
                                                          const double* __restrict__ strain,
                                                          const double* __restrict__ rot,
                                                          const double* __restrict__ crss,
                                                          const double* __restrict__ etab, double* __restrict__ edot,
                                                          double* __restrict__ err, long long* __restrict__ iters) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  const PhaseConst& ph = nc.ph[0];
  double lam6[6], eps6[6], ep6[6], R[9], tauf[NSYS], s6[6], e6[6];
  for (int i = 0; i < 6; i++) {
    lam6[i] = sig[6 * v + i];
    eps6[i] = strain[6 * v + i];
    ep6[i] = epsp[6 * v + i];
  }
  for (int i = 0; i < 9; i++) R[i] = rot[9 * v + i];
  for (int s = 0; s < NSYS; s++) tauf[s] = s < ph.nsys ? crss[NSYS * v + s] : 1.0;
  auto load = [&](double* l, double* e, double* q, double* r, bool) {
    for (int i = 0; i < 6; i++) { l[i] = lam6[i]; e[i] = eps6[i]; q[i] = ep6[i]; }
    for (int i = 0; i < 9; i++) r[i] = R[i];
  };
  PlSlip<double> pl;
  for (int k = 0; k < NSYS; k++) pl.tauf[k] = tauf[k];
  pl.tau_off = ph.tau_back_minus_fwd;
  VoxelOut<double> o = solve_voxel<double, double, false>(nc, ph, etab + (size_t)v * ETAB_W, pl, load, s6, e6);
  for (int i = 0; i < 6; i++) {
    sig[6 * v + i] = s6[i];
    edot[6 * v + i] = e6[i];
  }
  err[2 * v] = o.conv_s;
  err[2 * v + 1] = o.conv_e;
  iters[v] = o.iters;
}

cudaError_t launch_local_solve(const NewtonConst& nc, long long n, double* sig, const double* epsp,
                               const double* strain, const double* rot, const double* crss, const double* etab,
                               double* edot, double* err, long long* iters, cudaStream_t st) {
  const int nb = (int)((n + 255) / 256);
  local_solve_kernel<<<nb, 256, 0, st>>>(nc, n, sig, epsp, strain, rot, crss, etab, edot, err, iters);
  return cudaGetLastError();
}

// --------------------------------------------------- deterministic reduction
// out[w] = sum over blocks (fixed order) of partials[b*width + w].  One
// 1024-thread block per component; each thread keeps four independent
// partial sums so four L2 loads are in flight instead of a chain of
// dependent ones.
constexpr int RED_NT = 1024;   // 32 warps: the second shuffle stage sums one value per warp
__global__ void __launch_bounds__(RED_NT) reduce_partials_kernel(const double* __restrict__ partials, int nblocks,
                                                                 int width, double* __restrict__ out, IterIn it) {
  if (!is_live(it)) return;
  __shared__ double sm[RED_NT / 32];
  for (int w = blockIdx.x; w < width; w += gridDim.x) {
    double a0 = 0, a1 = 0, a2 = 0, a3 = 0;
    int b = threadIdx.x;
    for (; b + 3 * RED_NT < nblocks; b += 4 * RED_NT) {
      a0 += partials[(size_t)b * width + w];
      a1 += partials[(size_t)(b + RED_NT) * width + w];
      a2 += partials[(size_t)(b + 2 * RED_NT) * width + w];
      a3 += partials[(size_t)(b + 3 * RED_NT) * width + w];
    }
    for (; b < nblocks; b += RED_NT) a0 += partials[(size_t)b * width + w];
    // warp sums by shuffles, then the 32 warp sums by warp 0
    double a = (a0 + a1) + (a2 + a3);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = a;
    __syncthreads();
    if (threadIdx.x < 32) {
      a = sm[threadIdx.x];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
      if (threadIdx.x == 0) out[w] = a;
    }
    __syncthreads();
  }
}

cudaError_t launch_reduce_partials(const double* partials, int nblocks, int width, double* out, const IterIn& it,
                                   cudaStream_t st) {
  return launch_chain(reduce_partials_kernel, dim3(width), dim3(RED_NT), 0, st, it.pdl, partials, nblocks, width, out,
                      it);
}


// ------------------------------------------------ allocation-free local solve
// Variant of local_solve_kernel for callers that cannot allocate device
// memory: the caller passes device pointers for every input and output, the
// elastic rows are built in the kernel from each voxel's rotation, and the
// only scratch (per-block Newton-iteration partial sums and their total)
// lives in the fixed array below, which every GPU that loads the library holds
// until the process exits.  Calls that overlap on the GPU share it and race.
namespace {
constexpr long long NOALLOC_MAX_VOXELS = 1LL << 20;
constexpr int NOALLOC_MAX_BLOCKS = (int)(NOALLOC_MAX_VOXELS / 256);
static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_MAX_BLOCKS + 1];

__global__ void __launch_bounds__(256) local_solve_noalloc_kernel(const NewtonConst nc, long long n, double* sig,
                                                                  const double* __restrict__ epsp,
                                                                  const double* __restrict__ strain,
                                                                  const double* __restrict__ rot,
                                                                  const double* __restrict__ crss,
                                                                  double* __restrict__ edot, double* __restrict__ err,
                                                                  double* __restrict__ scratch) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double acc[1] = {0.0};
  if (v < n) {
    const PhaseConst& ph = nc.ph[0];
    double lam6[6], eps6[6], ep6[6], R[9], Q[25], tauf[NSYS], s6[6], e6[6], et[ETAB_W];
    for (int i = 0; i < 6; i++) {
      lam6[i] = sig[6 * v + i];
      eps6[i] = strain[6 * v + i];
      ep6[i] = epsp[6 * v + i];
    }
    for (int i = 0; i < 9; i++) R[i] = rot[9 * v + i];
    for (int s = 0; s < NSYS; s++) tauf[s] = s < ph.nsys ? crss[NSYS * v + s] : 1.0;
    rot_to_q<double>(R, Q);
    // elastic row of this voxel: S_gr = Q^T diag(s_xt) Q, S_tot = S0 + S_gr
    for (int i = 0; i < 5; i++)
      for (int j = i; j < 5; j++) {
        double sg = 0;
        for (int k = 0; k < 5; k++) sg += Q[k * 5 + i] * ph.s_xt[k] * Q[k * 5 + j];
        et[ET_SEL + pk(i, j)] = sg;
        et[ET_STOT + pk(i, j)] = nc.s0dev[i * 5 + j] + sg;
      }
    et[ET_SEL_HH] = ph.s_xt[5];
    auto load = [&](double* l, double* e, double* q, double* r, bool) {
      for (int i = 0; i < 6; i++) { l[i] = lam6[i]; e[i] = eps6[i]; q[i] = ep6[i]; }
      for (int i = 0; i < 9; i++) r[i] = R[i];
    };
    PlSlip<double> pl;
    for (int k = 0; k < NSYS; k++) pl.tauf[k] = tauf[k];
    pl.tau_off = ph.tau_back_minus_fwd;
    VoxelOut<double> o = solve_voxel<double, double, false>(nc, ph, et, pl, load, s6, e6);
    for (int i = 0; i < 6; i++) {
      sig[6 * v + i] = s6[i];
      edot[6 * v + i] = e6[i];
    }
    err[2 * v] = o.conv_s;
    err[2 * v + 1] = o.conv_e;
    acc[0] = (double)o.iters;
  }
  block_reduce_store<1>(acc, scratch);
}

__global__ void noalloc_total_kernel(double* scratch, int nblocks) {
  __shared__ double sm[256];
  double a = 0;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) a += scratch[b];
  sm[threadIdx.x] = a;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sm[threadIdx.x] += sm[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) scratch[NOALLOC_MAX_BLOCKS] = sm[0];
}

// Device address of g_noalloc_scratch, looked up once per device with that
// device current (the host-side name is only a stand-in, not a device
// address).  Atomic slots: host threads that make their first calls on the
// same device at the same time both look the address up and store the same
// value.
constexpr int NOALLOC_MAX_DEVICES = 64;
std::atomic<double*> g_noalloc_ptr[NOALLOC_MAX_DEVICES];
}  // namespace

long long noalloc_max_voxels() { return NOALLOC_MAX_VOXELS; }

cudaError_t launch_local_solve_noalloc(const NewtonConst& nc, long long n, double* sig, const double* epsp,
                                       const double* strain, const double* rot, const double* crss, double* edot,
                                       double* err, long long* iters_host, cudaStream_t st) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return cudaErrorInvalidDevice;
  double* scratch = g_noalloc_ptr[dev].load(std::memory_order_acquire);
  if (!scratch) {
    e = cudaGetSymbolAddress((void**)&scratch, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_noalloc_ptr[dev].store(scratch, std::memory_order_release);
  }
  const int nb = (int)((n + 255) / 256);
  // the total slot is the only one read without being written first
  e = cudaMemsetAsync(scratch + NOALLOC_MAX_BLOCKS, 0, sizeof(double), st);
  if (e != cudaSuccess) return e;
  local_solve_noalloc_kernel<<<nb, 256, 0, st>>>(nc, n, sig, epsp, strain, rot, crss, edot, err, scratch);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  noalloc_total_kernel<<<1, 256, 0, st>>>(scratch, nb);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  double tot = 0;
  e = cudaMemcpyAsync(&tot, scratch + NOALLOC_MAX_BLOCKS, sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess) return e;
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return e;
  if (iters_host) *iters_host = (long long)tot;
  return cudaSuccess;
}

}  // namespace mth

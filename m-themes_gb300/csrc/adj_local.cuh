// adj_local.cuh -- per-voxel pieces of the calibration adjoint (host and
// device code: the same functions run in the adjoint kernels and in the CPU
// checks of their transposed Jacobians).
//
// The adjoint differentiates the converged fixed point of every mechanical
// step.  Per voxel, with the lattice rotation perturbed as dR = [dphi]x R
// (dphi a rotation vector in sample axes) and stresses/strains in the
// Lebensohn-Tome (LT) basis:
//   local law      eps    = S sig + eps_p + dt e(sig; R, tau, n)
//   end of step    eps_p' = eps_p + dt e(sig; R, tau, n)
//                  tau'   = tau + a(gdot) V(gam, dgam; tau1, thet0, thet1) / dgam
//                  gam'   = gam + dgam,  dgam = dt sum_s |gdot_s|
//                  R'     = C(w) R,  w = au + wspin + dt/2 R sum_s gdot_s (b_s x n_s)
// with e the power-law rate of StrainRate_eval (src/constitutive.c:5-67),
// V the Voce increment of harden (src/constitutive.c:275-326) and C the
// rotation of Orientation (src/constitutive.c:142-194), exactly as the
// forward end-of-step kernel evaluates them.
//
// adj_pre applies the transposed Jacobian of the end-of-step map to the
// adjoint of the state after the step, plus the seed of the macroscopic
// stress misfit; it returns the stress adjoint sigbar, the adjoint of the
// local spin field wbar and the adjoints of the state before the step (less
// the part that reaches them through the global solve).  adj_post adds that
// part: the transposed Jacobian of dt e at fixed stress applied to
// qbar = C_t (mu - sigbar), mu being the solution of the projected tangent
// problem.  tangent_stiffness gives C_t = (S + dt de/dsig)^-1.
#pragma once
#include <math.h>
#include "mth_common.cuh"

namespace mth {
namespace adj {

#define ADJ_HD __host__ __device__ __forceinline__

// ------------------------------------------------------------ dual numbers
// Forward-mode derivative carrier with K directions, for the closed-form
// Voce increment and the rotation update.
template <int K>
struct Dual {
  double v;
  double d[K];
};
template <int K> ADJ_HD Dual<K> dconst(double a) {
  Dual<K> r;
  r.v = a;
  for (int i = 0; i < K; i++) r.d[i] = 0.0;
  return r;
}
template <int K> ADJ_HD Dual<K> dvar(double a, int i) {
  Dual<K> r = dconst<K>(a);
  r.d[i] = 1.0;
  return r;
}
template <int K> ADJ_HD Dual<K> operator+(const Dual<K>& a, const Dual<K>& b) {
  Dual<K> r;
  r.v = a.v + b.v;
  for (int i = 0; i < K; i++) r.d[i] = a.d[i] + b.d[i];
  return r;
}
template <int K> ADJ_HD Dual<K> operator-(const Dual<K>& a, const Dual<K>& b) {
  Dual<K> r;
  r.v = a.v - b.v;
  for (int i = 0; i < K; i++) r.d[i] = a.d[i] - b.d[i];
  return r;
}
template <int K> ADJ_HD Dual<K> operator*(const Dual<K>& a, const Dual<K>& b) {
  Dual<K> r;
  r.v = a.v * b.v;
  for (int i = 0; i < K; i++) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
  return r;
}
template <int K> ADJ_HD Dual<K> operator/(const Dual<K>& a, const Dual<K>& b) {
  Dual<K> r;
  r.v = a.v / b.v;
  for (int i = 0; i < K; i++) r.d[i] = (a.d[i] - r.v * b.d[i]) / b.v;
  return r;
}
template <int K> ADJ_HD Dual<K> operator*(double s, const Dual<K>& a) {
  Dual<K> r;
  r.v = s * a.v;
  for (int i = 0; i < K; i++) r.d[i] = s * a.d[i];
  return r;
}
template <int K> ADJ_HD Dual<K> operator+(const Dual<K>& a, double s) {
  Dual<K> r = a;
  r.v += s;
  return r;
}
template <int K> ADJ_HD Dual<K> dexp(const Dual<K>& a) {
  Dual<K> r;
  r.v = exp(a.v);
  for (int i = 0; i < K; i++) r.d[i] = r.v * a.d[i];
  return r;
}
template <int K> ADJ_HD Dual<K> dexpm1(const Dual<K>& a) {
  Dual<K> r;
  r.v = expm1(a.v);
  const double e = exp(a.v);
  for (int i = 0; i < K; i++) r.d[i] = e * a.d[i];
  return r;
}
template <int K> ADJ_HD Dual<K> dfabs(const Dual<K>& a) { return a.v < 0.0 ? (-1.0) * a : a; }
template <int K> ADJ_HD Dual<K> dsqrt(const Dual<K>& a) {
  Dual<K> r;
  r.v = sqrt(a.v);
  for (int i = 0; i < K; i++) r.d[i] = r.v > 0.0 ? a.d[i] / (2.0 * r.v) : 0.0;
  return r;
}
template <int K> ADJ_HD Dual<K> dtan(const Dual<K>& a) {
  Dual<K> r;
  r.v = tan(a.v);
  for (int i = 0; i < K; i++) r.d[i] = (1.0 + r.v * r.v) * a.d[i];
  return r;
}
// plain doubles through the same templates
ADJ_HD double dexp(double a) { return exp(a); }
ADJ_HD double dexpm1(double a) { return expm1(a); }
ADJ_HD double dfabs(double a) { return fabs(a); }
ADJ_HD double dsqrt(double a) { return sqrt(a); }
ADJ_HD double dtan(double a) { return tan(a); }
ADJ_HD double val(double a) { return a; }
template <int K> ADJ_HD double val(const Dual<K>& a) { return a.v; }
template <typename N> ADJ_HD N num(double a);
template <> ADJ_HD double num<double>(double a) { return a; }
template <> ADJ_HD Dual<3> num<Dual<3>>(double a) { return dconst<3>(a); }
template <> ADJ_HD Dual<5> num<Dual<5>>(double a) { return dconst<5>(a); }

// --------------------------------------------------------- forward pieces
// Voce increment of harden at accumulated shear gam and increment dgam
// (dgam > 0), same branches and the same expm1 form as the forward kernel;
// tiny = 1e-4 tau0.
template <typename N>
ADJ_HD N voce_increment(N gam, N dgam, N tau1, N th0, N th1, double tiny) {
  N voce = num<N>(0.0);
  if (fabs(val(th0)) > tiny) {
    voce = th1 * dgam;
    if (fabs(val(tau1)) > tiny) {
      const N fact = dfabs(th0 / tau1);
      const N exp_ini = dexp((-1.0) * (gam * fact));
      const N em1 = dexpm1((-1.0) * (dgam * fact));
      const N exp_del = em1 + 1.0;
      voce = voce - ((fact * tau1 - th1) / fact) * exp_ini * em1 -
             (th1 / fact) * exp_ini * (em1 * (gam * fact + 1.0) + exp_del * dgam * fact);
    }
  }
  return voce;
}

// Rotation increment of Orientation for the spin vector w = (W21, W02, W10):
// C = I + 2 (O + O^2) / (1 + t^2), O = [w t/|w|]x, t = tan(|w|/2); |w| < 1e-6
// takes |w| := 1 in the scaling, as the forward kernel does.
template <typename N>
ADJ_HD void rot_increment(const N w[3], N C[3][3]) {
  N wn = dsqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
  N wt = dtan((0.5) * wn);
  if (fabs(val(wn)) < 1e-6) wn = num<N>(1.0);
  N ws[3];
  for (int i = 0; i < 3; i++) ws[i] = w[i] * (wt / wn);
  const N z = num<N>(0.0);
  N om[3][3] = {{z, (-1.0) * ws[2], ws[1]}, {ws[2], z, (-1.0) * ws[0]}, {(-1.0) * ws[1], ws[0], z}};
  const N den = wt * wt + 1.0;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      N o2 = om[i][0] * om[0][j] + om[i][1] * om[1][j] + om[i][2] * om[2][j];
      C[i][j] = (2.0) * ((om[i][j] + o2) / den) + (i == j ? 1.0 : 0.0);
    }
}

// Flow rule at the converged stress: the crystal-frame stress x = Q sig,
// per system the shear rate gdot, w = d gdot/d rss, d gdot/d tau and
// d gdot/d n, and the plastic rate in crystal (ex) and sample (es) axes.
struct FlowEval {
  double Q[25];
  double x[5];
  double gdot[NSYS], w[NSYS], dgdtau[NSYS], dgdn[NSYS];
  double ex[5], es[5];
};

ADJ_HD void flow_eval(const PhaseConst& ph, const double sig[6], const double R[9], const double* tau, int flow_off,
                      FlowEval& f) {
  rot_to_q<double>(R, f.Q);
  for (int i = 0; i < 5; i++) {
    double a = 0;
    for (int j = 0; j < 5; j++) a += f.Q[i * 5 + j] * sig[j];
    f.x[i] = a;
    f.ex[i] = 0;
  }
  const double n = ph.nrs, g0 = ph.gamd0;
  for (int s = 0; s < NSYS; s++) {
    f.gdot[s] = f.w[s] = f.dgdtau[s] = f.dgdn[s] = 0.0;
    if (s >= ph.nsys || flow_off) continue;
    double rss = 0;
    for (int i = 0; i < 5; i++) rss += ph.m_xt[s][i] * f.x[i];
    const double tp = rss < 0.0 ? tau[s] + ph.tau_back_minus_fwd : tau[s];
    const double r = rss / tp, ar = fabs(r);
    const double pnm1 = ar > 0.0 ? pow(ar, n - 1.0) : 0.0;
    const double pn = pnm1 * ar;
    const double g = g0 * (r > 0.0 ? pn : -pn);
    f.gdot[s] = g;
    f.w[s] = g0 * n * pnm1 / tp;
    f.dgdtau[s] = -n * g / tp;
    f.dgdn[s] = ar > 0.0 ? g * log(ar) : 0.0;
    for (int i = 0; i < 5; i++) f.ex[i] += ph.m_xt[s][i] * g;
  }
  for (int j = 0; j < 5; j++) {
    double a = 0;
    for (int i = 0; i < 5; i++) a += f.Q[i * 5 + j] * f.ex[i];
    f.es[j] = a;
  }
}

// L(Z) (5x3): column k = LT_dev(Z E_k - E_k Z), E_k = [e_k]x.  With
// dR = [dphi]x R:  d(Q s) = Q L(s) dphi  and  d(Q^T y) = -L(Q^T y) dphi.
ADJ_HD void lmat(const double z6[6], double L[5][3]) {
  double zc[3][3];
  double v[6] = {z6[0], z6[1], z6[2], z6[3], z6[4], 0.0};
  lt_to_cart<double>(v, zc);
  for (int k = 0; k < 3; k++) {
    double E[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    const int a = (k + 1) % 3, b = (k + 2) % 3;
    E[b][a] = 1.0;    // [e_k]x: E[(k+2)%3][(k+1)%3] = +1
    E[a][b] = -1.0;
    double M[3][3];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        double s = 0;
        for (int m = 0; m < 3; m++) s += zc[i][m] * E[m][j] - E[i][m] * zc[m][j];
        M[i][j] = s;
      }
    double o[6];
    cart_to_lt<double>(M, o);
    for (int i = 0; i < 5; i++) L[i][k] = o[i];
  }
}

// y += L^T u  (u: 5)
ADJ_HD void lmat_t_add(const double L[5][3], const double u[5], double y[3], double s) {
  for (int k = 0; k < 3; k++) {
    double a = 0;
    for (int i = 0; i < 5; i++) a += L[i][k] * u[i];
    y[k] += s * a;
  }
}

ADJ_HD int pk5(int i, int j) {
  if (i > j) { int t = i; i = j; j = t; }
  return i * 5 - (i * (i - 1)) / 2 + (j - i);
}

// Step data shared by all voxels.
struct StepFlags {
  double dt;
  double au[3];      // uniform part of the spin increment
  int flow_off, do_orient, do_harden;
};

// Adjoint of the per-voxel state (eps_p, tau, gam_acc, rotation).
struct AdjState {
  double ep[6];
  double tau[NSYS];
  double gam;
  double phi[3];
};

// ------------------------------------------------------------ adj_pre
// in: adjoint of the state after the step; seed: coefficient of sig (LT)
// in the objective's derivative (sigbar starts as seed6).  out: adjoint of
// the state before the step without the global-solve part; sigbar, wbar
// (adjoint of the spin field wspin), th += (tau1, thet0, thet1, n) adjoints.
ADJ_HD void adj_pre(const PhaseConst& ph, const StepFlags& sf, const double sig[6], const double R[9],
                    double gam_acc, const double wspin[3], const FlowEval& f, const AdjState& in,
                    const double seed6[6], AdjState& out, double sigbar[6], double wbar[3], double th[4]) {
  const double dt = sf.dt;
  double gbar[NSYS];
  for (int s = 0; s < NSYS; s++) gbar[s] = 0.0;
  for (int i = 0; i < 3; i++) { out.phi[i] = in.phi[i]; wbar[i] = 0.0; }
  // orientation update
  if (sf.do_orient) {
    double c[3] = {0, 0, 0};
    for (int s = 0; s < ph.nsys; s++) {
      const double* b = ph.bb[s];
      const double* n = ph.bn[s];
      c[0] += f.gdot[s] * (b[1] * n[2] - b[2] * n[1]);
      c[1] += f.gdot[s] * (b[2] * n[0] - b[0] * n[2]);
      c[2] += f.gdot[s] * (b[0] * n[1] - b[1] * n[0]);
    }
    double Rc[3];
    for (int i = 0; i < 3; i++) Rc[i] = R[i * 3 + 0] * c[0] + R[i * 3 + 1] * c[1] + R[i * 3 + 2] * c[2];
    Dual<3> w[3];
    for (int i = 0; i < 3; i++) w[i] = dvar<3>(sf.au[i] + wspin[i] + 0.5 * dt * Rc[i], i);
    Dual<3> C[3][3];
    rot_increment<Dual<3>>(w, C);
    // dphi' = C dphi + J dw,  [J e_k]x = (dC/dw_k) C^T
    for (int i = 0; i < 3; i++) {
      double a = 0;
      for (int j = 0; j < 3; j++) a += C[j][i].v * in.phi[j];
      out.phi[i] = a;   // C^T phibar'
    }
    if (fabs(val(dsqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]))) >= 1e-6) {
      for (int k = 0; k < 3; k++) {
        double A[3][3];
        for (int i = 0; i < 3; i++)
          for (int j = 0; j < 3; j++) {
            double s = 0;
            for (int m = 0; m < 3; m++) s += C[i][m].d[k] * C[j][m].v;
            A[i][j] = s;
          }
        const double jk[3] = {0.5 * (A[2][1] - A[1][2]), 0.5 * (A[0][2] - A[2][0]), 0.5 * (A[1][0] - A[0][1])};
        wbar[k] = jk[0] * in.phi[0] + jk[1] * in.phi[1] + jk[2] * in.phi[2];
      }
    }
    // w = au + wspin + dt/2 R c:  phibar += dt/2 (R c) x wbar ; gbar_s += dt/2 (b x n)_s . R^T wbar
    out.phi[0] += 0.5 * dt * (Rc[1] * wbar[2] - Rc[2] * wbar[1]);
    out.phi[1] += 0.5 * dt * (Rc[2] * wbar[0] - Rc[0] * wbar[2]);
    out.phi[2] += 0.5 * dt * (Rc[0] * wbar[1] - Rc[1] * wbar[0]);
    double u[3];
    for (int j = 0; j < 3; j++) u[j] = R[0 * 3 + j] * wbar[0] + R[1 * 3 + j] * wbar[1] + R[2 * 3 + j] * wbar[2];
    for (int s = 0; s < ph.nsys; s++) {
      const double* b = ph.bb[s];
      const double* n = ph.bn[s];
      const double bx = b[1] * n[2] - b[2] * n[1], by = b[2] * n[0] - b[0] * n[2], bz = b[0] * n[1] - b[1] * n[0];
      gbar[s] += 0.5 * dt * (bx * u[0] + by * u[1] + bz * u[2]);
    }
  }
  // hardening
  for (int s = 0; s < NSYS; s++) out.tau[s] = in.tau[s];
  out.gam = in.gam;
  if (sf.do_harden) {
    double dgam = 0;
    for (int s = 0; s < NSYS; s++) dgam += fabs(f.gdot[s]) * dt;
    if (dgam > 0.0) {
      Dual<5> V = voce_increment<Dual<5>>(dvar<5>(gam_acc, 0), dvar<5>(dgam, 1), dvar<5>(ph.tau1, 2),
                                          dvar<5>(ph.thet0, 3), dvar<5>(ph.thet1, 4), 1e-4 * ph.tau0f);
      const double F = V.v / dgam;
      double A = 0;   // sum_s taubar'_s a_s,  a_s = dt sum_j h_sj |gdot_j|
      double hb[NSYS];
      for (int j = 0; j < NSYS; j++) hb[j] = 0.0;
      for (int s = 0; s < ph.nsys; s++) {
        double a = 0;
        for (int j = 0; j < ph.nsys; j++) {
          a += ph.hard[s][j] * fabs(f.gdot[j]) * dt;
          hb[j] += in.tau[s] * ph.hard[s][j];
        }
        A += in.tau[s] * a;
      }
      const double dgbar = A * (V.d[1] - F) / dgam + in.gam;
      out.gam += A * V.d[0] / dgam;
      th[0] += A * V.d[2] / dgam;
      th[1] += A * V.d[3] / dgam;
      th[2] += A * V.d[4] / dgam;
      for (int j = 0; j < ph.nsys; j++) {
        const double sg = f.gdot[j] > 0.0 ? 1.0 : (f.gdot[j] < 0.0 ? -1.0 : 0.0);
        gbar[j] += dt * sg * (F * hb[j] + dgbar);
      }
    }
  }
  // plastic strain: eps_p' = eps_p + dt Q^T ex
  for (int i = 0; i < 6; i++) out.ep[i] = in.ep[i];
  double eb[5], ebx[5];
  for (int i = 0; i < 5; i++) eb[i] = dt * in.ep[i];
  for (int i = 0; i < 5; i++) {
    double a = 0;
    for (int j = 0; j < 5; j++) a += f.Q[i * 5 + j] * eb[j];
    ebx[i] = a;
  }
  for (int s = 0; s < ph.nsys; s++) {
    double a = 0;
    for (int i = 0; i < 5; i++) a += ph.m_xt[s][i] * ebx[i];
    gbar[s] += a;
  }
  {
    double L[5][3];
    double e6[6] = {f.es[0], f.es[1], f.es[2], f.es[3], f.es[4], 0.0};
    lmat(e6, L);
    lmat_t_add(L, eb, out.phi, -1.0);
  }
  // shear rates -> stress, CRSS, n, rotation
  for (int i = 0; i < 6; i++) sigbar[i] = seed6[i];
  double xb[5] = {0, 0, 0, 0, 0};
  for (int s = 0; s < ph.nsys; s++) {
    for (int i = 0; i < 5; i++) xb[i] += gbar[s] * f.w[s] * ph.m_xt[s][i];
    out.tau[s] += gbar[s] * f.dgdtau[s];
    th[3] += gbar[s] * f.dgdn[s];
  }
  double qx[5];
  for (int j = 0; j < 5; j++) {
    double a = 0;
    for (int i = 0; i < 5; i++) a += f.Q[i * 5 + j] * xb[i];
    qx[j] = a;
    sigbar[j] += a;
  }
  {
    double L[5][3];
    lmat(sig, L);
    lmat_t_add(L, qx, out.phi, 1.0);
  }
}

// ------------------------------------------------------------ adj_post
// st += transposed Jacobian of dt e(sig fixed; R, tau, n) applied to qbar,
// and eps_p's own adjoint += qbar.
ADJ_HD void adj_post(const PhaseConst& ph, const StepFlags& sf, const double sig[6], const FlowEval& f,
                     const double qbar[6], AdjState& st, double th[4]) {
  const double dt = sf.dt;
  for (int i = 0; i < 6; i++) st.ep[i] += qbar[i];
  if (sf.flow_off) return;
  double eb[5], ebx[5];
  for (int i = 0; i < 5; i++) eb[i] = dt * qbar[i];
  for (int i = 0; i < 5; i++) {
    double a = 0;
    for (int j = 0; j < 5; j++) a += f.Q[i * 5 + j] * eb[j];
    ebx[i] = a;
  }
  double xb[5] = {0, 0, 0, 0, 0};
  for (int s = 0; s < ph.nsys; s++) {
    double gb = 0;
    for (int i = 0; i < 5; i++) gb += ph.m_xt[s][i] * ebx[i];
    for (int i = 0; i < 5; i++) xb[i] += gb * f.w[s] * ph.m_xt[s][i];
    st.tau[s] += gb * f.dgdtau[s];
    th[3] += gb * f.dgdn[s];
  }
  double qx[5];
  for (int j = 0; j < 5; j++) {
    double a = 0;
    for (int i = 0; i < 5; i++) a += f.Q[i * 5 + j] * xb[i];
    qx[j] = a;
  }
  double L[5][3];
  lmat(sig, L);
  lmat_t_add(L, qx, st.phi, 1.0);
  double e6[6] = {f.es[0], f.es[1], f.es[2], f.es[3], f.es[4], 0.0};
  lmat(e6, L);
  lmat_t_add(L, eb, st.phi, -1.0);
}

// ------------------------------------------------------ tangent stiffness
// C_t = (S + dt de/dsig)^-1: deviatoric 5x5 (packed upper triangle, 15) and
// the hydrostatic entry 1/S_hh in ct[15].  sel: packed sample-axes
// deviatoric compliance of the voxel's elastic class.  Returns false when
// the 5x5 is not positive definite.
ADJ_HD bool tangent_stiffness(const PhaseConst& ph, const StepFlags& sf, const FlowEval& f, const double* sel,
                              double shh, double ct[16]) {
  double Dx[15];
  for (int i = 0; i < 15; i++) Dx[i] = 0.0;
  if (!sf.flow_off)
    for (int s = 0; s < ph.nsys; s++)
      for (int i = 0; i < 5; i++)
        for (int j = i; j < 5; j++) Dx[pk5(i, j)] += f.w[s] * ph.m_xt[s][i] * ph.m_xt[s][j];
  // M = S + dt Q^T Dx Q
  double M[5][5], T[5][5];
  for (int i = 0; i < 5; i++)
    for (int j = 0; j < 5; j++) {
      double a = 0;
      for (int k = 0; k < 5; k++) a += Dx[pk5(i, k)] * f.Q[k * 5 + j];
      T[i][j] = a;
    }
  for (int i = 0; i < 5; i++)
    for (int j = 0; j < 5; j++) {
      double a = 0;
      for (int k = 0; k < 5; k++) a += f.Q[k * 5 + i] * T[k][j];
      M[i][j] = sel[pk5(i, j)] + sf.dt * a;
    }
  // LDL^T of M, then the inverse column by column
  double L[5][5], d[5];
  for (int j = 0; j < 5; j++) {
    double dj = M[j][j];
    for (int k = 0; k < j; k++) dj -= L[j][k] * L[j][k] * d[k];
    if (!(dj > 0.0)) return false;
    d[j] = dj;
    L[j][j] = 1.0;
    for (int i = j + 1; i < 5; i++) {
      double a = M[i][j];
      for (int k = 0; k < j; k++) a -= L[i][k] * L[j][k] * d[k];
      L[i][j] = a / dj;
    }
  }
  double Ci[5][5];
  for (int c = 0; c < 5; c++) {
    double y[5];
    for (int i = 0; i < 5; i++) {
      double a = (i == c) ? 1.0 : 0.0;
      for (int k = 0; k < i; k++) a -= L[i][k] * y[k];
      y[i] = a;
    }
    for (int i = 4; i >= 0; i--) {
      double a = y[i] / d[i];
      for (int k = i + 1; k < 5; k++) a -= L[k][i] * Ci[k][c];
      Ci[i][c] = a;
    }
  }
  for (int i = 0; i < 5; i++)
    for (int j = i; j < 5; j++) ct[pk5(i, j)] = 0.5 * (Ci[i][j] + Ci[j][i]);
  ct[15] = 1.0 / shh;
  return true;
}

// y = C_t x for a 6-vector (packed deviatoric block + hydrostatic entry)
template <typename T, typename U>
ADJ_HD void ct_apply(const U* ct, const T x[6], T y[6]) {
  for (int i = 0; i < 5; i++) {
    T a = 0;
    for (int j = 0; j < 5; j++) a += (T)ct[pk5(i, j)] * x[j];
    y[i] = a;
  }
  y[5] = (T)ct[15] * x[5];
}

// ------------------------------------- forward end-of-step map (checks)
// The end-of-step update of one voxel as a function of everything the
// adjoint differentiates: returns the plastic rate es (sample, 5), the new
// CRSS, accumulated shear and rotation.  Used to check adj_pre / adj_post
// against finite differences.
ADJ_HD void end_step_map(const PhaseConst& ph, const StepFlags& sf, const double sig[6], const double R[9],
                         const double* tau, double gam_acc, const double wspin[3], double es[5], double* tau_n,
                         double& gam_n, double Rn[9]) {
  FlowEval f;
  flow_eval(ph, sig, R, tau, sf.flow_off, f);
  for (int i = 0; i < 5; i++) es[i] = f.es[i];
  for (int i = 0; i < 9; i++) Rn[i] = R[i];
  if (sf.do_orient) {
    double c[3] = {0, 0, 0};
    for (int s = 0; s < ph.nsys; s++) {
      const double* b = ph.bb[s];
      const double* n = ph.bn[s];
      c[0] += f.gdot[s] * (b[1] * n[2] - b[2] * n[1]);
      c[1] += f.gdot[s] * (b[2] * n[0] - b[0] * n[2]);
      c[2] += f.gdot[s] * (b[0] * n[1] - b[1] * n[0]);
    }
    double w[3];
    for (int i = 0; i < 3; i++)
      w[i] = sf.au[i] + wspin[i] + 0.5 * sf.dt * (R[i * 3 + 0] * c[0] + R[i * 3 + 1] * c[1] + R[i * 3 + 2] * c[2]);
    double C[3][3];
    rot_increment<double>(w, C);
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) Rn[i * 3 + j] = C[i][0] * R[0 * 3 + j] + C[i][1] * R[1 * 3 + j] + C[i][2] * R[2 * 3 + j];
  }
  for (int s = 0; s < NSYS; s++) tau_n[s] = tau[s];
  gam_n = gam_acc;
  if (sf.do_harden) {
    double dgam = 0;
    for (int s = 0; s < NSYS; s++) dgam += fabs(f.gdot[s]) * sf.dt;
    if (dgam > 0.0) {
      const double V = voce_increment<double>(gam_acc, dgam, ph.tau1, ph.thet0, ph.thet1, 1e-4 * ph.tau0f);
      for (int s = 0; s < ph.nsys; s++) {
        double a = 0;
        for (int j = 0; j < ph.nsys; j++) a += ph.hard[s][j] * fabs(f.gdot[j]) * sf.dt;
        tau_n[s] = tau[s] + a * V / dgam;
      }
      gam_n = gam_acc + dgam;
    }
  }
}

}  // namespace adj
}  // namespace mth

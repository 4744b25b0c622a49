// adj_local_check.cpp -- CPU check of the per-voxel transposed Jacobians of
// the calibration adjoint (m-themes_gb300/csrc/adj_local.cuh) against
// central finite differences of the end-of-step map they differentiate.
// Built and run by tests/test_adjoint_local.py with the host compiler.
// Prints one line per check: name, max relative error; exit status 1 when a
// check exceeds its tolerance.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <random>
#include "adj_local.cuh"

using namespace mth;
using namespace mth::adj;

static void fcc_phase(PhaseConst& ph, double nrs, std::mt19937_64& rng) {
  static const int sl[12][2][3] = {
      {{1, 1, -1}, {0, 1, 1}}, {{1, 1, -1}, {1, 0, 1}}, {{1, 1, -1}, {1, -1, 0}},
      {{1, -1, -1}, {0, 1, -1}}, {{1, -1, -1}, {1, 0, 1}}, {{1, -1, -1}, {1, 1, 0}},
      {{1, -1, 1}, {0, 1, 1}}, {{1, -1, 1}, {1, 0, -1}}, {{1, -1, 1}, {1, 1, 0}},
      {{1, 1, 1}, {0, 1, -1}}, {{1, 1, 1}, {1, 0, -1}}, {{1, 1, 1}, {1, -1, 0}}};
  memset(&ph, 0, sizeof(ph));
  ph.type = 0;
  ph.nsys = 12;
  ph.nrs = nrs;
  ph.gamd0 = 1.0;
  ph.tau0f = 16.0;
  ph.tau_back_minus_fwd = 0.0;
  ph.tau1 = 148.0;
  ph.thet0 = 250.0;
  ph.thet1 = 2.0;
  std::uniform_real_distribution<double> u(0.5, 1.5);
  for (int s = 0; s < 12; s++) {
    double nn = 0, nb = 0;
    for (int m = 0; m < 3; m++) { nn += sl[s][0][m] * sl[s][0][m]; nb += sl[s][1][m] * sl[s][1][m]; }
    for (int m = 0; m < 3; m++) { ph.bn[s][m] = sl[s][0][m] / sqrt(nn); ph.bb[s][m] = sl[s][1][m] / sqrt(nb); }
    double a[3][3];
    for (int m = 0; m < 3; m++)
      for (int n = 0; n < 3; n++) a[m][n] = 0.5 * (ph.bn[s][m] * ph.bb[s][n] + ph.bn[s][n] * ph.bb[s][m]);
    double v[6];
    cart_to_lt<double>(a, v);
    for (int i = 0; i < 5; i++) ph.m_xt[s][i] = v[i];
    for (int j = 0; j < 12; j++) ph.hard[s][j] = (s == j) ? 1.0 : 1.4 * u(rng) / 1.4;
  }
}

static void rodrigues(const double p[3], double E[9]) {
  const double t = sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
  double K[3][3] = {{0, -p[2], p[1]}, {p[2], 0, -p[0]}, {-p[1], p[0], 0}};
  const double a = t > 0 ? sin(t) / t : 1.0, b = t > 0 ? (1 - cos(t)) / (t * t) : 0.5;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      double k2 = 0;
      for (int m = 0; m < 3; m++) k2 += K[i][m] * K[m][j];
      E[i * 3 + j] = (i == j) + a * K[i][j] + b * k2;
    }
}
static void matmul3(const double A[9], const double B[9], double C[9]) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      double s = 0;
      for (int m = 0; m < 3; m++) s += A[i * 3 + m] * B[m * 3 + j];
      C[i * 3 + j] = s;
    }
}

// all differentiated inputs of one voxel
struct In {
  double sig[6];
  double phi[3];
  double tau[NSYS];
  double gam;
  double th[4];   // tau1, thet0, thet1, n
  double wsp[3];
};
constexpr int NIN = 6 + 3 + NSYS + 1 + 4 + 3;
static double* slot(In& z, int k) {
  if (k < 6) return &z.sig[k];
  k -= 6;
  if (k < 3) return &z.phi[k];
  k -= 3;
  if (k < NSYS) return &z.tau[k];
  k -= NSYS;
  if (k < 1) return &z.gam;
  k -= 1;
  if (k < 4) return &z.th[k];
  k -= 4;
  return &z.wsp[k];
}

struct Ctx {
  PhaseConst ph;
  StepFlags sf;
  double R0[9];
  double Rn0[9];   // R' at the base point
};

static void apply_th(const Ctx& c, const In& z, PhaseConst& ph) {
  ph = c.ph;
  ph.tau1 = z.th[0];
  ph.thet0 = z.th[1];
  ph.thet1 = z.th[2];
  ph.nrs = z.th[3];
}

// objective of the end-of-step map: a.(dt es) + b.tau' + c gam' + d.phi'
static double obj_pre(const Ctx& c, const In& z, const double a[5], const double b[NSYS], double cg, const double d[3]) {
  PhaseConst ph;
  apply_th(c, z, ph);
  double E[9], R[9];
  rodrigues(z.phi, E);
  matmul3(E, c.R0, R);
  double es[5], tn[NSYS], gn, Rn[9];
  end_step_map(ph, c.sf, z.sig, R, z.tau, z.gam, z.wsp, es, tn, gn, Rn);
  // phi' = axial(Rn Rn0^T)
  double A[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      double s = 0;
      for (int m = 0; m < 3; m++) s += Rn[i * 3 + m] * c.Rn0[j * 3 + m];
      A[i * 3 + j] = s;
    }
  const double ph3[3] = {0.5 * (A[7] - A[5]), 0.5 * (A[2] - A[6]), 0.5 * (A[3] - A[1])};
  double L = 0;
  for (int i = 0; i < 5; i++) L += a[i] * c.sf.dt * es[i];
  for (int s = 0; s < NSYS; s++) L += b[s] * tn[s];
  L += cg * gn;
  for (int i = 0; i < 3; i++) L += d[i] * ph3[i];
  return L;
}

// objective of the plastic rate at fixed stress: q.(dt es)
static double obj_post(const Ctx& c, const In& z, const double q[6]) {
  PhaseConst ph;
  apply_th(c, z, ph);
  double E[9], R[9];
  rodrigues(z.phi, E);
  matmul3(E, c.R0, R);
  FlowEval f;
  flow_eval(ph, z.sig, R, z.tau, c.sf.flow_off, f);
  double L = 0;
  for (int i = 0; i < 5; i++) L += q[i] * c.sf.dt * f.es[i];
  return L;
}

static double worst = 0;
static int failed = 0;
static void report(const char* name, const double* got, const double* want, int n, double tol) {
  double scale = 0, err = 0;
  for (int i = 0; i < n; i++) scale = fmax(scale, fabs(want[i]));
  for (int i = 0; i < n; i++) err = fmax(err, fabs(got[i] - want[i]));
  const double rel = scale > 0 ? err / scale : err;
  printf("%-28s max_rel_err %.3e (scale %.3e)\n", name, rel, scale);
  if (!(rel <= tol)) failed = 1;
  worst = fmax(worst, rel);
}

int main(int argc, char** argv) {
  const int cases = argc > 1 ? atoi(argv[1]) : 6;
  std::mt19937_64 rng(12345);
  std::normal_distribution<double> g(0.0, 1.0);
  std::uniform_real_distribution<double> u(0.0, 1.0);
  for (int cs = 0; cs < cases; cs++) {
    Ctx c;
    const double nrs = (cs % 3 == 0) ? 10.0 : (cs % 3 == 1 ? 12.5 : 20.0);
    fcc_phase(c.ph, nrs, rng);
    c.sf.dt = 1e-3;
    c.sf.flow_off = 0;
    c.sf.do_orient = (cs % 4 != 3);
    c.sf.do_harden = (cs % 5 != 4);
    for (int i = 0; i < 3; i++) c.sf.au[i] = 1e-3 * g(rng);
    {
      double p[3] = {3 * g(rng), 3 * g(rng), 3 * g(rng)};
      rodrigues(p, c.R0);
    }
    In z0;
    // a stress near the flow surface: |r| ~ 1 on the most stressed systems
    double sdir[6];
    double nrm = 0;
    for (int i = 0; i < 6; i++) { sdir[i] = g(rng); nrm += sdir[i] * sdir[i]; }
    for (int i = 0; i < 6; i++) z0.sig[i] = 45.0 * sdir[i] / sqrt(nrm);
    for (int i = 0; i < 3; i++) z0.phi[i] = 0.0;
    for (int s = 0; s < NSYS; s++) z0.tau[s] = 16.0 + 10.0 * u(rng);
    z0.gam = 0.02 * u(rng);
    z0.th[0] = c.ph.tau1;
    z0.th[1] = c.ph.thet0;
    z0.th[2] = c.ph.thet1;
    z0.th[3] = c.ph.nrs;
    for (int i = 0; i < 3; i++) z0.wsp[i] = 2e-4 * g(rng);
    {
      double es[5], tn[NSYS], gn;
      end_step_map(c.ph, c.sf, z0.sig, c.R0, z0.tau, z0.gam, z0.wsp, es, tn, gn, c.Rn0);
    }
    // ---- adj_pre against finite differences
    double a[5], b[NSYS], cg, d[3];
    for (int i = 0; i < 5; i++) a[i] = g(rng) * 1e3;
    for (int s = 0; s < NSYS; s++) b[s] = g(rng);
    cg = 10 * g(rng);
    for (int i = 0; i < 3; i++) d[i] = 100 * g(rng);
    AdjState in, out;
    memset(&in, 0, sizeof(in));
    for (int i = 0; i < 5; i++) in.ep[i] = a[i];
    for (int s = 0; s < NSYS; s++) in.tau[s] = b[s];
    in.gam = cg;
    for (int i = 0; i < 3; i++) in.phi[i] = d[i];
    FlowEval f;
    flow_eval(c.ph, z0.sig, c.R0, z0.tau, 0, f);
    double seed[6] = {0, 0, 0, 0, 0, 0}, sigbar[6], wbar[3], th[4] = {0, 0, 0, 0};
    adj_pre(c.ph, c.sf, z0.sig, c.R0, z0.gam, z0.wsp, f, in, seed, out, sigbar, wbar, th);
    double got[NIN], want[NIN];
    {
      int k = 0;
      for (int i = 0; i < 6; i++) got[k++] = sigbar[i];
      for (int i = 0; i < 3; i++) got[k++] = out.phi[i];
      for (int s = 0; s < NSYS; s++) got[k++] = out.tau[s];
      got[k++] = out.gam;
      for (int i = 0; i < 4; i++) got[k++] = th[i];
      for (int i = 0; i < 3; i++) got[k++] = wbar[i];
    }
    for (int k = 0; k < NIN; k++) {
      In zp = z0, zm = z0;
      const double base = *slot(z0, k);
      const double h = (k >= 6 && k < 9) ? 1e-6 : (k >= 6 + 3 + NSYS + 1 + 4 ? 1e-7 : 1e-6 * fmax(fabs(base), 1e-3));
      *slot(zp, k) += h;
      *slot(zm, k) -= h;
      want[k] = (obj_pre(c, zp, a, b, cg, d) - obj_pre(c, zm, a, b, cg, d)) / (2 * h);
    }
    char name[64];
    snprintf(name, sizeof name, "pre[%d] sigma", cs);
    report(name, got, want, 6, 2e-5);
    snprintf(name, sizeof name, "pre[%d] phi", cs);
    report(name, got + 6, want + 6, 3, 2e-5);
    snprintf(name, sizeof name, "pre[%d] tau", cs);
    report(name, got + 9, want + 9, NSYS, 2e-5);
    snprintf(name, sizeof name, "pre[%d] gam", cs);
    report(name, got + 21, want + 21, 1, 2e-5);
    snprintf(name, sizeof name, "pre[%d] theta", cs);
    report(name, got + 22, want + 22, 4, 2e-5);
    snprintf(name, sizeof name, "pre[%d] wspin", cs);
    report(name, got + 26, want + 26, 3, 2e-5);
    // ---- adj_post against finite differences
    double q[6];
    for (int i = 0; i < 6; i++) q[i] = 1e3 * g(rng);
    AdjState st;
    memset(&st, 0, sizeof(st));
    double th2[4] = {0, 0, 0, 0};
    adj_post(c.ph, c.sf, z0.sig, f, q, st, th2);
    {
      int k = 0;
      for (int i = 0; i < 3; i++) got[k++] = st.phi[i];
      for (int s = 0; s < NSYS; s++) got[k++] = st.tau[s];
      got[k++] = th2[3];
      const int idx[16] = {6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16, 17, 18, 19, 20, 25};
      for (int j = 0; j < 16; j++) {
        const int kk = idx[j];
        In zp = z0, zm = z0;
        const double base = *slot(z0, kk);
        const double h = (kk < 9) ? 1e-6 : 1e-6 * fmax(fabs(base), 1e-3);
        *slot(zp, kk) += h;
        *slot(zm, kk) -= h;
        want[j] = (obj_post(c, zp, q) - obj_post(c, zm, q)) / (2 * h);
      }
    }
    snprintf(name, sizeof name, "post[%d] phi", cs);
    report(name, got, want, 3, 2e-5);
    snprintf(name, sizeof name, "post[%d] tau", cs);
    report(name, got + 3, want + 3, NSYS, 2e-5);
    snprintf(name, sizeof name, "post[%d] n", cs);
    report(name, got + 15, want + 15, 1, 2e-5);
    // ---- tangent stiffness: C_t^-1 - S = dt d es / d sig
    {
      double Q[25], sel[15];
      rot_to_q<double>(c.R0, Q);
      const double sx[5] = {1 / 47000.0, 1 / 47000.0, 1 / 150800.0, 1 / 150800.0, 1 / 150800.0};
      for (int i = 0; i < 5; i++)
        for (int j = i; j < 5; j++) {
          double s = 0;
          for (int k = 0; k < 5; k++) s += Q[k * 5 + i] * sx[k] * Q[k * 5 + j];
          sel[pk5(i, j)] = s;
        }
      double ct[16];
      const bool ok = tangent_stiffness(c.ph, c.sf, f, sel, 1.0 / 411200.0, ct);
      if (!ok) { printf("tangent_stiffness failed\n"); failed = 1; continue; }
      // check C_t (S + dt J) = I on the deviatoric block
      double J[5][5];
      for (int j = 0; j < 5; j++) {
        In zp = z0, zm = z0;
        const double h = 1e-6 * 45.0;
        zp.sig[j] += h;
        zm.sig[j] -= h;
        FlowEval fp, fm;
        flow_eval(c.ph, zp.sig, c.R0, zp.tau, 0, fp);
        flow_eval(c.ph, zm.sig, c.R0, zm.tau, 0, fm);
        for (int i = 0; i < 5; i++) J[i][j] = (fp.es[i] - fm.es[i]) / (2 * h);
      }
      double P[25], I[25];
      for (int i = 0; i < 5; i++)
        for (int j = 0; j < 5; j++) {
          double s = 0;
          for (int k = 0; k < 5; k++) s += ct[pk5(i, k)] * (sel[pk5(k, j)] + c.sf.dt * J[k][j]);
          P[i * 5 + j] = s;
          I[i * 5 + j] = (i == j) ? 1.0 : 0.0;
        }
      snprintf(name, sizeof name, "tangent[%d]", cs);
      report(name, P, I, 25, 1e-5);
    }
  }
  printf("worst %.3e\n", worst);
  return failed;
}

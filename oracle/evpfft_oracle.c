/*
 * evpfft_oracle.c -- ORACLE (test infrastructure only; never linked into the
 * product).
 *
 * CPU restatement, in FP64, of the M-THEMES EVPFFT mechanical step with the
 * power-law flow rule (StrainRate_eval, src/constitutive.c:5-67) and Voce
 * hardening (harden, src/constitutive.c:275-326) in place of the
 * dislocation-density law of the shipped build.  Each function below names
 * the reference lines it follows.  Array layout follows the reference: one
 * 3x3 tensor per voxel, voxel index (x*Ny+y)*Nz+z with z fastest
 * (pIDX, src/evp.h:53).
 *
 * Deliberate, documented choices where the reference is undefined:
 *  - line search: the reference reads an uninitialised `f2` on the second
 *    backtrack (src/evolution.c:237); here f2 holds the previous trial value
 *    as in the Numerical Recipes routine it was taken from, and the number of
 *    line searches that reach that branch is counted (orc_second_backtracks).
 *  - s_vm: the out-of-bounds SigDevAvg[3][3] (src/evolution.c:531) reads the
 *    value selected by svm_oob_mode (see oracle.h).
 *  - Schmid tensors before the first update_schmid call (Update_Flag=0,
 *    istep=0) are zero, which is what freshly mapped heap pages hold in the
 *    reference (src/init.c:1178 allocates, src/evolution.c:1334 fills).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "oracle.h"

#define R_PI 3.14159265359      /* PI, src/evp.h:77 */
#define R_TWO_PI 6.28318530718  /* TWO_PI, src/evp.h:78 */
#define NS MTH_NSYS_MAX

typedef double t33[3][3];
typedef double t3333[3][3][3][3];
typedef double m66[6][6];

/* ------------------------------------------------------------------ */
/* Lebensohn-Tome basis, chg_basis/chg_basis5 (src/kinematics.c:14-174) */
/* ------------------------------------------------------------------ */
static double Bb[6][3][3];
static int basis_ready = 0;

static void basis_init(void) {
  const double r2 = 0.70710678118654744, r3 = 0.57735026918962584, r6 = 0.40824829046386304;
  if (basis_ready) return;
  memset(Bb, 0, sizeof(Bb));
  Bb[1][0][0] = -r6; Bb[1][1][1] = -r6; Bb[1][2][2] = 2. * r6;
  Bb[0][0][0] = -r2; Bb[0][1][1] = r2;
  Bb[2][1][2] = r2; Bb[2][2][1] = r2;
  Bb[3][0][2] = r2; Bb[3][2][0] = r2;
  Bb[4][0][1] = r2; Bb[4][1][0] = r2;
  Bb[5][0][0] = r3; Bb[5][1][1] = r3; Bb[5][2][2] = r3;
  basis_ready = 1;
}
/* opt=2 / chg_basis5 opt=2: tensor -> vector (first nv components) */
static void t2v(const t33 t, double* v, int nv) {
  for (int i = 0; i < nv; i++) {
    double s = 0.0;
    for (int m = 0; m < 3; m++) for (int n = 0; n < 3; n++) s += t[m][n] * Bb[i][m][n];
    v[i] = s;
  }
}
/* opt=1: vector -> tensor */
static void v2t(const double* v, t33 t, int nv) {
  for (int m = 0; m < 3; m++) for (int n = 0; n < 3; n++) {
    double s = 0.0;
    for (int i = 0; i < nv; i++) s += v[i] * Bb[i][m][n];
    t[m][n] = s;
  }
}
/* opt=3: 6x6 -> 4th order */
static void m2t4(const m66 c, t3333 t) {
  for (int m = 0; m < 3; m++) for (int n = 0; n < 3; n++)
    for (int k = 0; k < 3; k++) for (int l = 0; l < 3; l++) {
      double s = 0.0;
      for (int i = 0; i < 6; i++) for (int j = 0; j < 6; j++) s += c[i][j] * Bb[i][m][n] * Bb[j][k][l];
      t[m][n][k][l] = s;
    }
}
/* opt=4: 4th order -> 6x6 */
static void t42m(const t3333 t, m66 c) {
  for (int i = 0; i < 6; i++) for (int j = 0; j < 6; j++) {
    double s = 0.0;
    for (int m = 0; m < 3; m++) for (int n = 0; n < 3; n++)
      for (int k = 0; k < 3; k++) for (int l = 0; l < 3; l++)
        s += t[m][n][k][l] * Bb[i][m][n] * Bb[j][k][l];
    c[i][j] = s;
  }
}

/* ------------------------------------------------------------------ */
/* 6x6 inverse: Crout LU with implicit pivoting, LU_dcmp/LU_bksb/LU_inv_66 */
/* (src/kinematics.c:282-428), including its tiny-pivot substitution and  */
/* the forward-substitution skip of leading |b|<=1e-5 entries.            */
/* ------------------------------------------------------------------ */
static int lu_inv66(m66 c) {
  const int n = 6;
  int indx[6], imax = 0;
  double vv[6], big, dum, sum, temp;
  for (int i = 0; i < n; i++) {
    big = 0.0;
    for (int j = 0; j < n; j++) if ((temp = fabs(c[i][j])) > big) big = temp;
    if (fabs(big) < 1e-5) return MTH_ERR_SINGULAR;
    vv[i] = 1.0 / big;
  }
  for (int j = 0; j < n; j++) {
    for (int i = 0; i < j; i++) {
      sum = c[i][j];
      for (int k = 0; k < i; k++) sum -= c[i][k] * c[k][j];
      c[i][j] = sum;
    }
    big = 0.0;
    for (int i = j; i < n; i++) {
      sum = c[i][j];
      for (int k = 0; k < j; k++) sum -= c[i][k] * c[k][j];
      c[i][j] = sum;
      if ((dum = vv[i] * fabs(sum)) >= big) { big = dum; imax = i; }
    }
    if (j != imax) {
      for (int k = 0; k < n; k++) { dum = c[imax][k]; c[imax][k] = c[j][k]; c[j][k] = dum; }
      vv[imax] = vv[j];
    }
    indx[j] = imax;
    if (fabs(c[j][j]) < 1e-5) c[j][j] = 1.0e-20;
    if (j != n - 1) {
      dum = 1.0 / c[j][j];
      for (int i = j + 1; i < n; i++) c[i][j] *= dum;
    }
  }
  m66 y;
  for (int jc = 0; jc < n; jc++) {
    double b[6] = {0, 0, 0, 0, 0, 0};
    b[jc] = 1.0;
    int ii = -1;
    for (int i = 0; i < n; i++) {
      int ip = indx[i];
      sum = b[ip];
      b[ip] = b[i];
      if (ii >= 0) for (int j = ii; j <= i - 1; j++) sum -= c[i][j] * b[j];
      else if (fabs(sum) > 1e-5) ii = i;
      b[i] = sum;
    }
    for (int i = n - 1; i >= 0; i--) {
      sum = b[i];
      for (int j = i + 1; j < n; j++) sum -= c[i][j] * b[j];
      b[i] = sum / c[i][i];
    }
    for (int i = 0; i < n; i++) y[i][jc] = b[i];
  }
  memcpy(c, y, sizeof(m66));
  return MTH_OK;
}

/* EulerToTransMatrix opt=2 (src/kinematics.c:187-240): Bunge angles
 * (radians) -> sample->crystal matrix a. */
static void euler_to_matrix(double t1, double ph, double t2, t33 a) {
  double ct1 = cos(t1), st1 = sin(t1), cph = cos(ph), sph = sin(ph), ct2 = cos(t2), st2 = sin(t2);
  a[0][0] = ct1 * ct2 - st1 * st2 * cph;
  a[0][1] = st1 * ct2 + ct1 * st2 * cph;
  a[0][2] = st2 * sph;
  a[1][0] = -1.0 * ct1 * st2 - st1 * ct2 * cph;
  a[1][1] = -1.0 * st1 * st2 + ct1 * ct2 * cph;
  a[1][2] = ct2 * sph;
  a[2][0] = st1 * sph;
  a[2][1] = -1.0 * ct1 * sph;
  a[2][2] = cph;
}

/* Ten4thTransform opt=2 (src/kinematics.c:243-280): c1 = a^T a^T a^T a^T c2 */
static void ten4_inverse_transform(t3333 c1, const t33 a, const t3333 c2) {
  for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++)
    for (int k = 0; k < 3; k++) for (int l = 0; l < 3; l++) {
      double s = 0.0;
      for (int m = 0; m < 3; m++) for (int n = 0; n < 3; n++)
        for (int p = 0; p < 3; p++) for (int q = 0; q < 3; q++)
          s += a[m][i] * a[n][j] * a[p][k] * a[q][l] * c2[m][n][p][q];
      c1[i][j][k][l] = s;
    }
}

/* ElastStiffnessMatrix (src/init.c:10-50): cubic C_ijkl from c11,c12,c44 */
static void cubic_stiffness(double c11, double c12, double c44, t3333 c) {
  memset(c, 0, sizeof(t3333));
  for (int i = 0; i < 3; i++) c[i][i][i][i] = c11;
  for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) if (i != j) {
    c[i][i][j][j] = c12;
    c[i][j][i][j] = c44;
    c[i][j][j][i] = c44;
  }
}

/* VonMises (src/kinematics.c:465-483) */
static double von_mises(const t33 t) {
  double tr = t[0][0] + t[1][1] + t[2][2], vm = 0.0;
  for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) {
    double d = (t[i][j] + t[j][i]) / 2. - (double)(i == j) * tr / 3.0;
    vm += d * d;
  }
  return sqrt(2. / 3. * vm);
}

/* VoigtToFull (src/kinematics.c:5-12) */
static void voigt_to_full(const double* v, t33 m) {
  m[0][0] = v[0]; m[0][1] = v[5]; m[0][2] = v[4];
  m[1][0] = v[5]; m[1][1] = v[1]; m[1][2] = v[3];
  m[2][0] = v[4]; m[2][1] = v[3]; m[2][2] = v[2];
}

/* ------------------------------------------------------------------ */
/* Complex FFT (mixed radix, recursive decimation in time).            */
/* ------------------------------------------------------------------ */
/* tw: exp(sign*2*pi*i*k/N) for k<N of the full length N; a sub-transform of
   length n uses every (N/n)-th entry */
static void fft1d_rec(const double* in, double* out, int n, int stride, const double* tw, int N,
                      double* scratch) {
  if (n == 1) { out[0] = in[0]; out[1] = in[1]; return; }
  int p = 2;
  while (n % p) p++;
  int m = n / p, step = N / n;
  for (int r = 0; r < p; r++)
    fft1d_rec(in + 2 * r * stride, scratch + 2 * r * m, m, stride * p, tw, N, out + 2 * r * m);
  for (int k = 0; k < m; k++) {
    for (int q = 0; q < p; q++) {
      double sr = 0.0, si = 0.0;
      int kk = k + q * m;
      for (int r = 0; r < p; r++) {
        int e = (int)(((long long)r * kk) % n) * step;
        double wr = tw[2 * e], wi = tw[2 * e + 1];
        double xr = scratch[2 * (r * m + k)], xi = scratch[2 * (r * m + k) + 1];
        sr += xr * wr - xi * wi;
        si += xr * wi + xi * wr;
      }
      out[2 * kk] = sr;
      out[2 * kk + 1] = si;
    }
  }
}

/* line: n complex values, transformed in place; work: 6n doubles */
static void fft1d(double* line, int n, const double* tw, double* work) {
  double* in = work;
  double* scr = work + 2 * n;
  double* out = work + 4 * n;
  memcpy(in, line, sizeof(double) * 2 * n);
  fft1d_rec(in, out, n, 1, tw, n, scr);
  memcpy(line, out, sizeof(double) * 2 * n);
}

static double* twiddles(int n, int sign) {
  double* tw = (double*)malloc(sizeof(double) * 2 * n);
  for (int k = 0; k < n; k++) {
    double a = sign * 2.0 * M_PI * (double)k / (double)n;
    tw[2 * k] = cos(a);
    tw[2 * k + 1] = sin(a);
  }
  return tw;
}

void orc_fft3d(double* d, int n0, int n1, int n2, int sign) {
  double* tw0 = twiddles(n0, sign);
  double* tw1 = twiddles(n1, sign);
  double* tw2 = twiddles(n2, sign);
#pragma omp parallel
  {
    int nmax = n0 > n1 ? n0 : n1;
    if (n2 > nmax) nmax = n2;
    double* line = (double*)malloc(sizeof(double) * 2 * nmax);
    double* work = (double*)malloc(sizeof(double) * 6 * nmax);
#pragma omp for collapse(2) schedule(static)
    for (int x = 0; x < n0; x++)
      for (int y = 0; y < n1; y++) fft1d(d + 2 * ((size_t)(x * n1 + y) * n2), n2, tw2, work);
#pragma omp for collapse(2) schedule(static)
    for (int x = 0; x < n0; x++)
      for (int z = 0; z < n2; z++) {
        for (int y = 0; y < n1; y++) {
          size_t o = 2 * ((size_t)(x * n1 + y) * n2 + z);
          line[2 * y] = d[o]; line[2 * y + 1] = d[o + 1];
        }
        fft1d(line, n1, tw1, work);
        for (int y = 0; y < n1; y++) {
          size_t o = 2 * ((size_t)(x * n1 + y) * n2 + z);
          d[o] = line[2 * y]; d[o + 1] = line[2 * y + 1];
        }
      }
#pragma omp for collapse(2) schedule(static)
    for (int y = 0; y < n1; y++)
      for (int z = 0; z < n2; z++) {
        for (int x = 0; x < n0; x++) {
          size_t o = 2 * ((size_t)(x * n1 + y) * n2 + z);
          line[2 * x] = d[o]; line[2 * x + 1] = d[o + 1];
        }
        fft1d(line, n0, tw0, work);
        for (int x = 0; x < n0; x++) {
          size_t o = 2 * ((size_t)(x * n1 + y) * n2 + z);
          d[o] = line[2 * x]; d[o + 1] = line[2 * x + 1];
        }
      }
    free(line);
    free(work);
  }
  free(tw0); free(tw1); free(tw2);
}

/* ------------------------------------------------------------------ */
/* Phase data, PlasticInit (src/init.c:52-231)                         */
/* ------------------------------------------------------------------ */
typedef struct {
  int type, nsys;
  double nsr, gam0;
  double tau[3];          /* tau0f, tau0b, tau1 */
  double thet[2];         /* thet0, thet1 */
  double hard[NS][NS];
  double bn[NS][3], bb[NS][3];
  double schm_xt[NS][5];
  t3333 cijkl;
  /* dislocation-density law (src/init.c:179-205,816-830,1096-1126) */
  int dd;
  double dd_b, dd_G, dd_nu, dd_c[8], dd_kT, dd_qslip, dd_qbulk, dd_L0, dd_d0, dd_T;
  double chi[NS][NS], cs[NS][NS], ss[NS][NS], cg1[NS][NS], sg1[NS][NS], cg3[NS][NS], sg3[NS][NS];
  double bp[NS][3];
} phase_t;

static int phase_init(const mth_phase* in, phase_t* ph) {
  memset(ph, 0, sizeof(*ph));
  ph->type = in->type;
  cubic_stiffness(in->c11, in->c12, in->c44, ph->cijkl);
  if (in->type != 0) return MTH_OK;   /* gas: nSYS stays 0 */
  if (in->nsys <= 0 || in->nsys > NS) return MTH_ERR_ARG;
  double tau1 = in->tau1, thet0 = in->thet0, thet1 = in->thet1;
  if (thet0 < thet1) return MTH_ERR_ARG;                      /* src/init.c:127-129 */
  if (tau1 < 1.e-6) { tau1 = 1.e-6; thet0 = thet1; }          /* src/init.c:130-133 */
  ph->nsys = in->nsys;
  ph->nsr = in->nrs;
  ph->gam0 = in->gamd0;
  ph->tau[0] = in->tau0f; ph->tau[1] = in->tau0b; ph->tau[2] = tau1;
  ph->thet[0] = thet0; ph->thet[1] = thet1;
  for (int j = 0; j < ph->nsys; j++) {
    double nn = sqrt(pow(in->bn[j][0], 2.0) + pow(in->bn[j][1], 2.0) + pow(in->bn[j][2], 2.0));
    double nb = sqrt(pow(in->bb[j][0], 2.0) + pow(in->bb[j][1], 2.0) + pow(in->bb[j][2], 2.0));
    for (int m = 0; m < 3; m++) { ph->bn[j][m] = in->bn[j][m] / nn; ph->bb[j][m] = in->bb[j][m] / nb; }
    double dot = 0.0;
    for (int m = 0; m < 3; m++) dot += ph->bn[j][m] * ph->bb[j][m];
    if (dot > 1e-3) return MTH_ERR_ARG;                        /* src/init.c:195-197 */
    t33 a;
    for (int m = 0; m < 3; m++) for (int n = 0; n < 3; n++)
      a[m][n] = (ph->bn[j][m] * ph->bb[j][n] + ph->bn[j][n] * ph->bb[j][m]) / 2.0;
    t2v(a, ph->schm_xt[j], 5);
  }
  for (int i = 0; i < ph->nsys; i++) for (int j = 0; j < ph->nsys; j++)
    ph->hard[i][j] = (i == j) ? in->hself : in->hlat;
  return MTH_OK;
}

/* Constants of the dislocation-density law (src/evp.h:77-86). */
#define DD_TRIAL_FREQ 1.0E10
#define DD_EV_IN_J 1.60217733e-19
#define DD_MY_J_IN_EV 0.62415063631
#define DD_BOLZ 1.380658e-23
#define DD_TAU0 1000.0        /* tau_0 of StrainRate_Orowan (src/constitutive.c:535) */
#define DD_EPS 5.0E-3         /* EPSILON of src/PFgrid.h:50, seen by DislocationEvolution */

/* Junction strength of slip systems i, j of an FCC crystal from their
 * geometry: self, coplanar (same plane), cross slip (collinear b), Hirth
 * (orthogonal b), and for 60-degree pairs on different planes glissile when
 * the junction b_i -/+ b_j lies in one of the two planes, Lomer-Cottrell when
 * it lies in neither.  For the system order of the FCC .sx files this gives
 * the matrix of InteractionStrengthMatrix (src/init.c:593-702). */
static double dd_junction(const phase_t* ph, int i, int j, const double str[6]) {
  if (i == j) return str[0];
  const double* ni = ph->bn[i]; const double* nj = ph->bn[j];
  const double* bi = ph->bb[i]; const double* bj = ph->bb[j];
  double nn = ni[0] * nj[0] + ni[1] * nj[1] + ni[2] * nj[2];
  double bbd = bi[0] * bj[0] + bi[1] * bj[1] + bi[2] * bj[2];
  if (fabs(fabs(nn) - 1.0) < 1e-6) return str[1];
  if (fabs(fabs(bbd) - 1.0) < 1e-6) return str[2];
  if (fabs(bbd) < 1e-6) return str[4];
  double sg = bbd > 0 ? 1.0 : -1.0, p[3];
  for (int m = 0; m < 3; m++) p[m] = bi[m] - sg * bj[m];
  double pi = p[0] * ni[0] + p[1] * ni[1] + p[2] * ni[2];
  double pj = p[0] * nj[0] + p[1] * nj[1] + p[2] * nj[2];
  return (fabs(pi) < 1e-6 || fabs(pj) < 1e-6) ? str[3] : str[5];
}

/* DD constants of a crystal phase from the run parameters: Burgers vector
 * b = a0/sqrt(2) (src/init.c:182), shear modulus of src/init.c:826, kT,
 * reduced activation energies, junction matrix and the projection cosines
 * of src/init.c:1107-1126 (screw sense vector n_j x b_j). */
static void dd_phase_init(const mth_params* p, const mth_phase* in, phase_t* ph) {
  ph->dd = 1;
  ph->dd_b = p->dd_a0 / sqrt(2.0);
  const double c11 = in->c11, c12 = in->c12, c44 = in->c44;
  ph->dd_G = 0.1 * (c11 - c12 + 3 * c44) + (0.5) * (5 * (c11 - c12) * c44) / (4 * c44 + 3 * (c11 - c12));
  ph->dd_nu = p->dd_nu;
  for (int k = 0; k < 8; k++) ph->dd_c[k] = p->dd_c[k];
  ph->dd_T = p->dd_T;
  ph->dd_kT = p->dd_T * DD_BOLZ * (1.0 / DD_EV_IN_J);
  ph->dd_qslip = p->dd_q_slip * DD_MY_J_IN_EV / ph->dd_kT;
  ph->dd_qbulk = p->dd_q_bulk * DD_MY_J_IN_EV / ph->dd_kT;
  ph->dd_L0 = p->dd_L0;
  ph->dd_d0 = p->dd_d0;
  for (int i = 0; i < ph->nsys; i++) {
    ph->bp[i][0] = ph->bb[i][1] * ph->bn[i][2] - ph->bb[i][2] * ph->bn[i][1];
    ph->bp[i][1] = ph->bb[i][2] * ph->bn[i][0] - ph->bb[i][0] * ph->bn[i][2];
    ph->bp[i][2] = ph->bb[i][0] * ph->bn[i][1] - ph->bb[i][1] * ph->bn[i][0];
  }
  for (int i = 0; i < ph->nsys; i++)
    for (int j = 0; j < ph->nsys; j++) {
      ph->chi[i][j] = dd_junction(ph, i, j, p->dd_chi);
      double sv[3] = {ph->bn[j][1] * ph->bb[j][2] - ph->bn[j][2] * ph->bb[j][1],
                      ph->bn[j][2] * ph->bb[j][0] - ph->bn[j][0] * ph->bb[j][2],
                      ph->bn[j][0] * ph->bb[j][1] - ph->bn[j][1] * ph->bb[j][0]};
      ph->cs[i][j] = fabs(ph->bn[i][0] * sv[0] + ph->bn[i][1] * sv[1] + ph->bn[i][2] * sv[2]);
      ph->ss[i][j] = fabs(sqrt(fabs(1.0 - ph->cs[i][j] * ph->cs[i][j])));
      ph->cg1[i][j] = fabs(ph->bn[i][0] * ph->bb[j][0] + ph->bn[i][1] * ph->bb[j][1] + ph->bn[i][2] * ph->bb[j][2]);
      ph->sg1[i][j] = fabs(sqrt(fabs(1.0 - ph->cg1[i][j] * ph->cg1[i][j])));
      ph->cg3[i][j] = fabs(ph->bn[i][0] * ph->bn[j][0] + ph->bn[i][1] * ph->bn[j][1] + ph->bn[i][2] * ph->bn[j][2]);
      ph->sg3[i][j] = fabs(sqrt(fabs(1.0 - ph->cg3[i][j] * ph->cg3[i][j])));
    }
}

/* Per-voxel state of the dislocation-density law (rows of NS). */
typedef struct {
  double *rho_s, *g1, *g2, *g3, *rho_m, *rho_F, *rho_P, *gam_acum, *trial_gam_acum;
  double dt;
} ddv_t;

/* StrainRate_Orowan, FORWARD_PLUS_BACKWARD branch (src/constitutive.c:
 * 507-721): forest/parallel densities from the trial densities, passing
 * stress from the mobile density of the previous evaluation, then the
 * mobile density, cutting stress and sinh rate law; writes rho_F, rho_P,
 * rho_m and trial_gam_acum as the reference does. */
static void flow_rule_dd(const phase_t* ph, const double sc[NS][5], const ddv_t* d, const double* s, double* edot,
                         m66 dedot, double* gamdot) {
  const int ns = ph->nsys;
  const double G = ph->dd_G, c1 = ph->dd_c[0], c2 = ph->dd_c[1], c3 = ph->dd_c[2], kT = ph->dd_kT;
  double gam[NS], gam2[NS];
  for (int i = 0; i < ns; i++) {
    double f = 0.0, pp = 0.0;
    for (int j = 0; j < ns; j++) {
      f += ph->chi[i][j] * (d->rho_s[j] * ph->cs[i][j] + fabs(d->g1[j] * ph->cg1[i][j]) +
                            fabs(d->g2[j] * ph->cs[i][j]) + fabs(d->g3[j] * ph->cg3[i][j]));
      pp += ph->chi[i][j] * (d->rho_s[j] * ph->ss[i][j] + fabs(d->g1[j] * ph->sg1[i][j]) +
                             fabs(d->g2[j] * ph->ss[i][j]) + fabs(d->g3[j] * ph->sg3[i][j]));
    }
    d->rho_F[i] = f;
    d->rho_P[i] = pp;
  }
  for (int i = 0; i < ns; i++) {
    const double b = ph->dd_b;
    double tau_pass = c1 * G * b * sqrt(fabs(d->rho_P[i] + d->rho_m[i])) * 1.0E-3;
    double rss = sc[i][0] * s[0] + sc[i][1] * s[1] + sc[i][2] * s[2] + sc[i][3] * s[3] + sc[i][4] * s[4];
    double tau_eff = fabs(rss) - tau_pass;
    double tau_cut = (kT / DD_MY_J_IN_EV) * sqrt(d->rho_F[i]) / c2 / c3 / b / b * 0.1;
    d->rho_m[i] = 2.0 * kT / c1 / c2 / c3 / G / (pow(b, 3.0)) * sqrt(d->rho_P[i] * d->rho_F[i]) * 160.2177;
    double gam_o = 1E-3 * (d->rho_m[i]) * DD_TRIAL_FREQ * c2 * b * exp(-1.0 * ph->dd_qslip) / sqrt(d->rho_F[i]);
    double t = fabs(rss) > tau_pass ? gam_o * sinh(tau_eff / (DD_TAU0 + tau_cut)) : 0.0;
    gam[i] = t * ((double)(2 * (rss > 0) - 1));
    gam2[i] = fabs(rss) > tau_pass ? gam_o * cosh(tau_eff / (tau_cut + DD_TAU0)) / (tau_cut + DD_TAU0) : 0.0;
    if (gamdot) gamdot[i] = gam[i];
    d->trial_gam_acum[i] = d->gam_acum[i] + gam[i] * d->dt;
  }
  for (int i = 0; i < 5; i++) {
    double e = 0.;
    for (int j = 0; j < ns; j++) e += sc[j][i] * gam[j];
    edot[i] = e;
  }
  edot[5] = 0.0;
  if (dedot) {
    for (int i = 0; i < 5; i++) for (int j = 0; j < 5; j++) {
      double a = 0.0;
      for (int k = 0; k < ns; k++) a += sc[k][i] * sc[k][j] * gam2[k];
      dedot[i][j] = a;
    }
    for (int i = 0; i < 6; i++) { dedot[i][5] = 0.0; dedot[5][i] = 0.0; }
  }
}

/* ------------------------------------------------------------------ */
/* Flow rule StrainRate_eval (src/constitutive.c:5-67); xkin is zero    */
/* throughout the reference (initialised at src/init.c:1165, never set). */
/* ------------------------------------------------------------------ */
static void flow_rule_pl(const phase_t* ph, const double sc[NS][5], const double tau_t[NS][2],
                         const double* s, double* edot, m66 dedot, double* gamdot) {
  double rss1[NS], rss2[NS];
  const int ns = ph->nsys;
  const double nsr = ph->nsr;
  for (int i = 0; i < ns; i++) {
    double rss = sc[i][0] * s[0] + sc[i][1] * s[1] + sc[i][2] * s[2] + sc[i][3] * s[3] + sc[i][4] * s[4];
    int isign = (rss - 0.0) < 0 ? 1 : 0;
    double r = (rss - 0.0) / tau_t[i][isign];
    rss1[i] = ph->gam0 * nsr * fabs(pow(r, nsr - 1.)) / tau_t[i][isign];
    rss2[i] = ph->gam0 * fabs(pow(r, nsr)) * ((double)(2 * (r > 0) - 1));
    if (gamdot) gamdot[i] = rss2[i];
  }
  for (int i = 0; i < 5; i++) {
    double e = 0.;
    for (int j = 0; j < ns; j++) e += sc[j][i] * rss2[j];
    edot[i] = e;
  }
  edot[5] = 0.0;
  if (dedot) {
    for (int i = 0; i < 5; i++) for (int j = 0; j < 5; j++) {
      double d = 0.0;
      for (int k = 0; k < ns; k++) d += sc[k][i] * sc[k][j] * rss1[k];
      dedot[i][j] = d;
    }
    for (int i = 0; i < 6; i++) { dedot[i][5] = 0.0; dedot[5][i] = 0.0; }
  }
}

/* the flow rule of the run: StrainRate_Orowan with per-voxel densities,
 * else StrainRate_eval */
static void flow_rule(const phase_t* ph, const double sc[NS][5], const double tau_t[NS][2], const ddv_t* d,
                      const double* s, double* edot, m66 dedot, double* gamdot) {
  if (d) flow_rule_dd(ph, sc, d, s, edot, dedot, gamdot);
  else flow_rule_pl(ph, sc, tau_t, s, edot, dedot, gamdot);
}

/* NR_quality (src/evolution.c:2-41): f = |R|^2/2 at sig */
static double nr_quality(const phase_t* ph, const double sc[NS][5], const double tau_t[NS][2], const ddv_t* d,
                         const m66 c066, double dt, const double* sig, const double* xlam,
                         const double* eps, const double* strain, const m66 sg, double* gamdot) {
  double edotp[6], tot[6], res[6], f = 0.0;
  flow_rule(ph, sc, tau_t, d, sig, edotp, NULL, gamdot);
  for (int i = 0; i < 6; i++) {
    tot[i] = eps[i] + edotp[i] * dt;
    for (int j = 0; j < 6; j++) tot[i] += sg[i][j] * sig[j];
  }
  for (int i = 0; i < 6; i++) {
    res[i] = sig[i] - xlam[i];
    for (int j = 0; j < 6; j++) res[i] += c066[i][j] * (tot[j] - strain[j]);
  }
  for (int i = 0; i < 6; i++) f += res[i] * res[i];
  return f / 2.0;
}

/* Newton with line search of UpdateStress for one crystal voxel
 * (src/evolution.c:68-299, NR_MODIFIED branch).  sig6 holds the start
 * value (= lambda) on entry and the solution on exit. */
typedef struct { double conv_s, conv_e; int iters; int cubic; int status; } newton_out;

static newton_out newton_voxel(const phase_t* ph, const double sc[NS][5], const double tau_t[NS][2],
                               const ddv_t* dd, const m66 c066, double dt, const m66 sg66, double* sig6,
                               const double* xlam6, const double* eps6, const double* strain6,
                               double* edotp6, double* gamdot, double tol, int itmax) {
  newton_out o = {0.0, 0.0, 0, 0, MTH_OK};
  double signorm = 0.0;
  /* |lambda| in the basis equals the Frobenius norm of the tensor */
  {
    t33 xl;
    v2t(xlam6, xl, 6);
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) signorm += xl[i][j] * xl[i][j];
    signorm = sqrt(signorm);
  }
  double erral = 10 * tol, conv_e = 0.0, conv_s = 0.0;
  int iterl = 0;
  while ((iterl < itmax) && (fabs(erral) > fabs(tol))) {
    iterl++;
    double sig_old[6], tot[6], res[6];
    m66 dedot, jinv, jac;
    for (int i = 0; i < 6; i++) sig_old[i] = sig6[i];
    flow_rule(ph, sc, tau_t, dd, sig6, edotp6, dedot, gamdot);
    for (int i = 0; i < 6; i++) {
      tot[i] = eps6[i] + edotp6[i] * dt;
      for (int j = 0; j < 6; j++) tot[i] += sg66[i][j] * sig6[j];
    }
    for (int i = 0; i < 6; i++) {
      res[i] = sig6[i] - xlam6[i];
      for (int j = 0; j < 6; j++) res[i] += c066[i][j] * (tot[j] - strain6[j]);
    }
    for (int i = 0; i < 6; i++) for (int j = 0; j < 6; j++) {
      double a = (double)(i == j);
      for (int k = 0; k < 6; k++) a += c066[i][k] * (sg66[k][j] + dedot[k][j] * dt);
      jinv[i][j] = a;
      jac[i][j] = a;
    }
    if (lu_inv66(jinv) != MTH_OK) { o.status = MTH_ERR_SINGULAR; break; }
    double f_old = 0.0, gradf[6], step[6];
    for (int i = 0; i < 6; i++) f_old += res[i] * res[i];
    f_old *= 0.5;
    for (int i = 0; i < 6; i++) {
      gradf[i] = 0.0;
      for (int j = 0; j < 6; j++) gradf[i] += res[j] * jac[j][i];
    }
    for (int i = 0; i < 6; i++) {
      step[i] = 0.0;
      for (int j = 0; j < 6; j++) step[i] -= jinv[i][j] * res[j];
    }
    const double stpmax = 10.0, ALF = 1.e-4, TOLX = 1.e-7;
    double sum = 0.0, slope = 0.0, test = 0.0;
    for (int i = 0; i < 6; i++) sum += step[i] * step[i];
    sum = sqrt(sum);
    if (sum > stpmax) for (int i = 0; i < 6; i++) step[i] *= stpmax / sum;
    for (int i = 0; i < 6; i++) slope += gradf[i] * step[i];
    if (slope >= 0) { o.status = MTH_ERR_NOT_CONVERGED; break; }   /* src/evolution.c:210-214 */
    for (int i = 0; i < 6; i++) {
      double t = fabs(step[i]) / fmax(fabs(sig_old[i]), 1.0);
      if (t > test) test = t;
    }
    double alamin = TOLX / test, alam = 1.0, alam2 = 0.0, f2 = 0.0, tmplam = 0.0;
    while (1) {
      for (int i = 0; i < 6; i++) sig6[i] = sig_old[i] + alam * step[i];
      double f_new = nr_quality(ph, sc, tau_t, dd, c066, dt, sig6, xlam6, eps6, strain6, sg66, gamdot);
      if (alam < alamin) {
        for (int i = 0; i < 6; i++) sig6[i] = sig_old[i];
        break;
      } else if (f_new <= f_old + ALF * alam * slope) {
        break;
      } else {
        if (fabs(alam - 1.0) < 1.e-4) {
          tmplam = -slope / (2.0 * (f_new - f_old - slope));
        } else {
          o.cubic++;
          double rhs1 = f_new - f_old - alam * slope;
          double rhs2 = f2 - f_old - alam2 * slope;
          double a = (rhs1 / (alam * alam) - rhs2 / (alam2 * alam2)) / (alam - alam2);
          double b = (-alam2 * rhs1 / (alam * alam) + alam * rhs2 / (alam2 * alam2)) / (alam - alam2);
          if (fabs(a) < 1e-4) tmplam = -slope / (2.0 * b);
          else {
            double disc = b * b - 3.0 * a * slope;
            if (disc < 0.0) tmplam = 0.5 * alam;
            else if (b <= 0.0) tmplam = (-b + sqrt(disc)) / (3.0 * a);
            else tmplam = -slope / (b + sqrt(disc));
          }
          if (tmplam > 0.5 * alam) tmplam = 0.5 * alam;
        }
      }
      alam2 = alam;
      f2 = f_new;
      alam = fmax(tmplam, 0.1 * alam);
    }
    double cnr = 0.0;
    conv_e = 0.0; conv_s = 0.0;
    for (int i = 0; i < 6; i++) {
      cnr += (sig6[i] - sig_old[i]) * (sig6[i] - sig_old[i]);
      conv_e += (tot[i] - strain6[i]) * (tot[i] - strain6[i]);
      conv_s += (sig6[i] - xlam6[i]) * (sig6[i] - xlam6[i]);
    }
    erral = sqrt(cnr) / signorm;
    conv_s = sqrt(conv_s);
    conv_e = sqrt(conv_e);
  }
  o.iters = iterl;
  o.conv_s = conv_s;
  o.conv_e = conv_e;
  if (o.status == MTH_OK && iterl >= itmax && fabs(erral) > fabs(tol)) o.status = MTH_ERR_NOT_CONVERGED;
  return o;
}

/* Schmid tensor of one voxel in sample axes, update_schmid
 * (src/kinematics.c:430-463); tm = TranMat_xt2sa */
static void schmid_sample(const phase_t* ph, const t33 tm, double sc[NS][5]) {
  for (int i = 0; i < ph->nsys; i++) {
    t33 a, ar;
    v2t(ph->schm_xt[i], a, 5);
    for (int m = 0; m < 3; m++) for (int n = 0; n < 3; n++) {
      double s = 0.0;
      for (int p = 0; p < 3; p++) for (int q = 0; q < 3; q++) s += tm[m][p] * tm[n][q] * a[p][q];
      ar[m][n] = s;
    }
    t2v(ar, sc[i], 5);
  }
}

/* ------------------------------------------------------------------ */
/* Context                                                            */
/* ------------------------------------------------------------------ */
struct orc_ctx {
  int n[3];
  size_t nv;
  int nthreads, svm_oob_mode;
  double wgt, wgt_ph1;
  int nphases;
  phase_t ph[MTH_NPH_MAX];
  int *grain, *phase;
  /* fields */
  t33 *sig, *eps, *edot, *disgrad, *velgrad, *tranmat;
  m66* sg66;                 /* inverse of C_gr */
  m66* cgr;                  /* C_gr (changes only by DRX) */
  double (*schm)[NS][5];
  double (*crss)[NS][2];
  double (*gamdot)[NS];
  double* gamacum;
  double* kbuf;              /* 9 complex fields */
  double (*nvec)[3];         /* unit wave vectors g (src/init.c:775-796) */
  double *conv_s, *conv_e;
  int* newton_it;
  unsigned char* newton_bad;
  /* macro state */
  m66 c066, s066;
  t3333 c0, s0;
  t3333 gc0, gs0;            /* C0 and S0 of the Green operator, frozen at set-up (src/init.c:1195) */
  mth_params par;
  int first_drx_id, next_grain_id, n_drx;
  double* drx_rot;           /* 9 per recrystallised grain */
  double* rho_avg_tab;       /* PF_XRX's rho_avg table, kept across steps */
  int rho_avg_len;
  t33 udot, udot_s, udot_a, scauchy;
  int vbc[6], sbc[6], creep, elast_bc, update_flag, hard_flag;
  double dt, err_tol, time_tot, e_vm, d_vm, s_vm, s_vm1, err_e, err_s;
  int iter_max, istep;
  double newton_tol;
  int newton_itmax;
  t33 disgrad_avg, ddisgrad_avg, ddisgrad_acum, disgrad_avg_t;
  t33 sig_avg, sig_avg1, sig_dev_avg, eps_avg, edot_avg;
  long long cubic_total;
  /* dislocation-density law (src/init.c:1055-1095) */
  int dd;
  double (*rho_s)[NS], (*rho_g1)[NS], (*rho_g2)[NS], (*rho_g3)[NS], (*rho_m)[NS], (*rho_F)[NS], (*rho_P)[NS];
  double (*rho_dipole)[NS], (*rho_forest)[NS], (*gam_acum)[NS], (*trial_gam_acum)[NS];
  double (*gadot_grad)[NS][3];
  unsigned char (*gbchk)[6];   /* GB_checkX/Y/Z of Gradient_ExchangeGrainID: [+x,-x,+y,-y,+z,(-y)] */
  double dd_avg[7];
};

static void* xcalloc(size_t n, size_t s) { return calloc(n ? n : 1, s); }

orc_ctx* orc_create(const mth_params* p, const int* grain, const int* phase, const double* euler_deg,
                    int nthreads, int svm_oob_mode, int* status) {
  basis_init();
  int st = MTH_OK;
  orc_ctx* c = (orc_ctx*)xcalloc(1, sizeof(orc_ctx));
  for (int i = 0; i < 3; i++) c->n[i] = p->cell_dim[i];
  c->nv = (size_t)c->n[0] * c->n[1] * c->n[2];
  c->nthreads = nthreads > 0 ? nthreads : 1;
#ifdef _OPENMP
  omp_set_num_threads(c->nthreads);
#endif
  c->svm_oob_mode = svm_oob_mode;
  c->wgt = 1. / (double)c->nv;
  c->nphases = p->n_phases;
  if (c->nphases < 1 || c->nphases > MTH_NPH_MAX) { st = MTH_ERR_ARG; goto fail; }
  for (int k = 0; k < c->nphases; k++) {
    st = phase_init(&p->phase[k], &c->ph[k]);
    if (st) goto fail;
  }
  size_t nv = c->nv;
  c->grain = (int*)xcalloc(nv, sizeof(int));
  c->phase = (int*)xcalloc(nv, sizeof(int));
  c->sig = (t33*)xcalloc(nv, sizeof(t33));
  c->eps = (t33*)xcalloc(nv, sizeof(t33));
  c->edot = (t33*)xcalloc(nv, sizeof(t33));
  c->disgrad = (t33*)xcalloc(nv, sizeof(t33));
  c->velgrad = (t33*)xcalloc(nv, sizeof(t33));
  c->tranmat = (t33*)xcalloc(nv, sizeof(t33));
  c->sg66 = (m66*)xcalloc(nv, sizeof(m66));
  c->cgr = (m66*)xcalloc(nv, sizeof(m66));
  c->schm = (double(*)[NS][5])xcalloc(nv, sizeof(double[NS][5]));
  c->crss = (double(*)[NS][2])xcalloc(nv, sizeof(double[NS][2]));
  c->gamdot = (double(*)[NS])xcalloc(nv, sizeof(double[NS]));
  c->gamacum = (double*)xcalloc(nv, sizeof(double));
  c->kbuf = (double*)xcalloc(nv * 9 * 2, sizeof(double));
  c->nvec = (double(*)[3])xcalloc(nv, sizeof(double[3]));
  c->conv_s = (double*)xcalloc(nv, sizeof(double));
  c->conv_e = (double*)xcalloc(nv, sizeof(double));
  c->newton_it = (int*)xcalloc(nv, sizeof(int));
  c->newton_bad = (unsigned char*)xcalloc(nv, 1);
  if (!c->kbuf || !c->schm || !c->sg66) { st = MTH_ERR_NOMEM; goto fail; }

  /* k-space unit vectors (src/init.c:775-796) */
  for (int x = 0; x < c->n[0]; x++) for (int y = 0; y < c->n[1]; y++) for (int z = 0; z < c->n[2]; z++) {
    size_t id = ((size_t)x * c->n[1] + y) * c->n[2] + z;
    double t[3];
    t[0] = (double)x * (double)(1.0 / c->n[0]);
    t[1] = (double)y * (double)(1.0 / c->n[1]);
    t[2] = (double)z * (double)(1.0 / c->n[2]);
    for (int m = 0; m < 3; m++) { t[m] -= round(t[m]); t[m] *= R_TWO_PI; }
    double g2 = sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
    if (x + y + z == 0) { g2 = 1.0; t[0] = t[1] = t[2] = 0.0; }
    for (int m = 0; m < 3; m++) c->nvec[id][m] = t[m] * (1. / g2);
  }

  /* boundary conditions (src/init.c:861-900) */
  {
    double vbc[6], sbc[6];
    for (int i = 0; i < 6; i++) {
      c->vbc[i] = p->velgrad_bc_flag[i];
      c->sbc[i] = p->stress_bc_flag[i];
      vbc[i] = p->velgrad_bc[i] * c->vbc[i];
      sbc[i] = p->stress_bc[i];
    }
    if (c->vbc[0] + c->vbc[1] + c->vbc[2] == 2) { st = MTH_ERR_ARG; goto fail; }
    for (int i = 0; i < 6; i++)
      if ((c->sbc[i] * c->vbc[i] != 0) || (c->sbc[i] + c->vbc[i] != 1)) { st = MTH_ERR_ARG; goto fail; }
    voigt_to_full(vbc, c->udot);
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) {
      c->udot_s[i][j] = (c->udot[i][j] + c->udot[j][i]) / 2.;
      c->udot_a[i][j] = (c->udot[i][j] - c->udot[j][i]) / 2.;
    }
    double d6[6];
    t33 dev;
    t2v((const double(*)[3])c->udot_s, d6, 6);
    v2t(d6, dev, 5);
    c->d_vm = 0.0;
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) c->d_vm += pow(dev[i][j], 2.0);
    c->d_vm = sqrt(2. / 3. * c->d_vm);
    c->creep = 0;
    for (int i = 0; i < 6; i++) c->creep += c->sbc[i];
    c->creep /= 6;
    voigt_to_full(sbc, c->scauchy);
  }
  c->elast_bc = p->elast_bc;
  c->update_flag = p->update_flag;
  c->hard_flag = p->hard_flag;
  c->dt = p->time_step;
  c->err_tol = p->err;
  c->iter_max = p->iter_max;
  c->newton_tol = p->newton_tol > 0 ? p->newton_tol : 1e-10;
  c->newton_itmax = p->newton_itmax > 0 ? p->newton_itmax : 500;

  /* InitFields macro part (src/init.c:453-457) */
  for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) {
    c->disgrad_avg[i][j] = c->udot[i][j] * c->dt;
    c->ddisgrad_avg[i][j] = 0.0;
    c->ddisgrad_acum[i][j] = 0.0;
  }
  /* microstructure (src/init.c:255-378) and the elastic initial stress of
     InitFields (src/init.c:459-487); C_gr is cached per grain id */
  {
    int nph1 = 0;
    m66 csum;
    memset(csum, 0, sizeof(csum));
    int cache_gid = -1, cache_ph = -1;
    double cache_e[3] = {0, 0, 0};
    m66 cache_c, cache_s;
    t33 cache_tm, cache_sig;
    for (size_t v = 0; v < nv; v++) {
      int jph = phase[v];
      if (jph < 1 || jph > c->nphases) { st = MTH_ERR_ARG; goto fail; }
      if (jph == 1) nph1++;
      c->grain[v] = grain[v];
      c->phase[v] = jph;
      const phase_t* ph = &c->ph[jph - 1];
      if (ph->type == 0) {
        double e0 = euler_deg[3 * v], e1 = euler_deg[3 * v + 1], e2 = euler_deg[3 * v + 2];
        if (!(grain[v] == cache_gid && jph == cache_ph && e0 == cache_e[0] && e1 == cache_e[1] && e2 == cache_e[2])) {
          double a1 = e0 * (R_PI / 180.), a2 = e1 * (R_PI / 180.), a3 = e2 * (R_PI / 180.);
          t33 sa2xt;
          t3333 caux, cg;
          euler_to_matrix(a1, a2, a3, sa2xt);
          for (int m = 0; m < 3; m++) for (int q = 0; q < 3; q++) cache_tm[m][q] = sa2xt[q][m];
          ten4_inverse_transform(caux, (const double(*)[3])sa2xt, (const double(*)[3][3][3])ph->cijkl);
          t42m((const double(*)[3][3][3])caux, cache_c);
          memcpy(cache_s, cache_c, sizeof(m66));
          if (lu_inv66(cache_s)) { st = MTH_ERR_SINGULAR; goto fail; }
          m2t4((const double(*)[6])cache_c, cg);
          for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) {
            double s = 0.0;
            for (int k = 0; k < 3; k++) for (int l = 0; l < 3; l++) s += cg[i][j][k][l] * c->disgrad_avg[k][l];
            if (c->creep == 1) s += c->scauchy[i][j];
            cache_sig[i][j] = s;
          }
          cache_gid = grain[v]; cache_ph = jph;
          cache_e[0] = e0; cache_e[1] = e1; cache_e[2] = e2;
        }
        memcpy(c->tranmat[v], cache_tm, sizeof(t33));
        memcpy(c->sg66[v], cache_s, sizeof(m66));
        memcpy(c->cgr[v], cache_c, sizeof(m66));
        memcpy(c->sig[v], cache_sig, sizeof(t33));
        for (int i = 0; i < 6; i++) for (int j = 0; j < 6; j++) csum[i][j] += cache_c[i][j];
        for (int i = 0; i < ph->nsys; i++) {
          c->crss[v][i][0] = ph->tau[0];
          c->crss[v][i][1] = ph->tau[1];
        }
      }
    }
    c->wgt_ph1 = (1.0 * (double)nph1) / (double)nv;
    for (int i = 0; i < 6; i++) for (int j = 0; j < 6; j++) c->c066[i][j] = csum[i][j] * c->wgt;
    memcpy(c->s066, c->c066, sizeof(m66));
    if (lu_inv66(c->s066)) { st = MTH_ERR_SINGULAR; goto fail; }
    m2t4((const double(*)[6])c->c066, c->c0);
    m2t4((const double(*)[6])c->s066, c->s0);
    memcpy(c->gc0, c->c0, sizeof(t3333));
    memcpy(c->gs0, c->s0, sizeof(t3333));
    c->par = *p;
    int gmax = 0;
    for (size_t v = 0; v < nv; v++) if (grain[v] > gmax) gmax = grain[v];
    c->first_drx_id = c->next_grain_id = gmax + 1;
  }
  c->e_vm = c->d_vm * c->dt;
  c->istep = 0;
  if (p->flow_law == 1) {
    if (c->ph[0].type != 0 || (c->nphases == 2 && c->ph[1].type == 0)) { st = MTH_ERR_UNSUPPORTED; goto fail; }
    dd_phase_init(p, &p->phase[0], &c->ph[0]);
    c->dd = 1;
    c->rho_s = (double(*)[NS])xcalloc(nv, sizeof(double[NS]));
    c->rho_g1 = (double(*)[NS])xcalloc(nv, sizeof(double[NS]));
    c->rho_g2 = (double(*)[NS])xcalloc(nv, sizeof(double[NS]));
    c->rho_g3 = (double(*)[NS])xcalloc(nv, sizeof(double[NS]));
    c->rho_m = (double(*)[NS])xcalloc(nv, sizeof(double[NS]));
    c->rho_F = (double(*)[NS])xcalloc(nv, sizeof(double[NS]));
    c->rho_P = (double(*)[NS])xcalloc(nv, sizeof(double[NS]));
    c->rho_dipole = (double(*)[NS])xcalloc(nv, sizeof(double[NS]));
    c->rho_forest = (double(*)[NS])xcalloc(nv, sizeof(double[NS]));
    c->gam_acum = (double(*)[NS])xcalloc(nv, sizeof(double[NS]));
    c->trial_gam_acum = (double(*)[NS])xcalloc(nv, sizeof(double[NS]));
    c->gadot_grad = (double(*)[NS][3])xcalloc(nv, sizeof(double[NS][3]));
    c->gbchk = (unsigned char(*)[6])xcalloc(nv, 6);
    for (size_t v = 0; v < nv; v++)
      for (int i = 0; i < NS; i++) c->rho_s[v][i] = p->dd_rho_ssd0;
    const int n0 = c->n[0], n1 = c->n[1], n2 = c->n[2];
    for (int x = 0; x < n0; x++) for (int y = 0; y < n1; y++) for (int z = 0; z < n2; z++) {
      size_t v = ((size_t)x * n1 + y) * n2 + z;
      int xp = (x + 1) % n0, xm = (x + n0 - 1) % n0, yp = (y + 1) % n1, ym = (y + n1 - 1) % n1;
      int zp = (z + 1) % n2;
      int g = c->grain[v];
      c->gbchk[v][0] = g == c->grain[((size_t)xp * n1 + y) * n2 + z];
      c->gbchk[v][1] = g == c->grain[((size_t)xm * n1 + y) * n2 + z];
      c->gbchk[v][2] = g == c->grain[((size_t)x * n1 + yp) * n2 + z];
      c->gbchk[v][3] = g == c->grain[((size_t)x * n1 + ym) * n2 + z];
      c->gbchk[v][4] = g == c->grain[((size_t)x * n1 + y) * n2 + zp];
      c->gbchk[v][5] = g == c->grain[((size_t)x * n1 + ym) * n2 + z];   /* -z flag compares with -y */
    }
  }
  if (status) *status = MTH_OK;
  return c;
fail:
  if (status) *status = st;
  orc_destroy(c);
  return NULL;
}

void orc_destroy(orc_ctx* c) {
  if (!c) return;
  free(c->grain); free(c->phase); free(c->sig); free(c->eps); free(c->edot); free(c->disgrad);
  free(c->velgrad); free(c->tranmat); free(c->sg66); free(c->schm); free(c->crss); free(c->gamdot);
  free(c->gamacum); free(c->kbuf); free(c->nvec); free(c->conv_s); free(c->conv_e);
  free(c->newton_it); free(c->newton_bad);
  free(c->cgr); free(c->drx_rot); free(c->rho_avg_tab);
  free(c->rho_s); free(c->rho_g1); free(c->rho_g2); free(c->rho_g3); free(c->rho_m); free(c->rho_F);
  free(c->rho_P); free(c->rho_dipole); free(c->rho_forest); free(c->gam_acum); free(c->trial_gam_acum);
  free(c->gadot_grad); free(c->gbchk);
  free(c);
}

/* update_schmid over the grid (src/kinematics.c:430-463) */
static void update_schmid_all(orc_ctx* c) {
#pragma omp parallel for schedule(static)
  for (long long v = 0; v < (long long)c->nv; v++) {
    const phase_t* ph = &c->ph[c->phase[v] - 1];
    if (ph->type == 0) schmid_sample(ph, (const double(*)[3])c->tranmat[v], c->schm[v]);
  }
}

/* Green operator application, src/evolution.c:1373-1387 with GAMMA from
 * CalcGAMMA (src/init.c:541-591) evaluated at each k instead of stored. */
static void gamma_apply(const orc_ctx* c, size_t v, const double* nv, double* ks /* 9 complex */) {
  double G[3][3][3][3];
  if (v == 0) {
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++)
      for (int k = 0; k < 3; k++) for (int l = 0; l < 3; l++)
        G[i][j][k][l] = (c->elast_bc == 0) ? -1.0 * c->gs0[i][j][k][l] : 0.0;
  } else {
    double io[3][3], om[3][3];
    for (int i = 0; i < 3; i++) for (int k = 0; k < 3; k++) {
      double s = 0.0;
      for (int j = 0; j < 3; j++) for (int l = 0; l < 3; l++) s += c->gc0[i][j][k][l] * nv[j] * nv[l];
      io[i][k] = s;
    }
    /* M3Inverse (src/init.c:517-539) */
    double det = io[0][0] * (io[1][1] * io[2][2] - io[1][2] * io[2][1])
               - io[0][1] * (io[1][0] * io[2][2] - io[1][2] * io[2][0])
               + io[0][2] * (io[1][0] * io[2][1] - io[2][0] * io[1][1]);
    om[0][0] = io[1][1] * io[2][2] - io[1][2] * io[2][1];
    om[0][1] = io[0][2] * io[2][1] - io[0][1] * io[2][2];
    om[0][2] = io[0][1] * io[1][2] - io[0][2] * io[1][1];
    om[1][0] = io[1][2] * io[2][0] - io[1][0] * io[2][2];
    om[1][1] = io[0][0] * io[2][2] - io[0][2] * io[2][0];
    om[1][2] = io[0][2] * io[1][0] - io[0][0] * io[1][2];
    om[2][0] = io[1][0] * io[2][1] - io[1][1] * io[2][0];
    om[2][1] = io[0][1] * io[2][0] - io[0][0] * io[2][1];
    om[2][2] = io[0][0] * io[1][1] - io[0][1] * io[1][0];
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) om[i][j] /= det;
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++)
      for (int k = 0; k < 3; k++) for (int l = 0; l < 3; l++)
        G[i][j][k][l] = -1.0 * om[i][k] * nv[j] * nv[l];
  }
  double outr[9], outi[9];
  for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) {
    double sr = 0.0, si = 0.0;
    for (int k = 0; k < 3; k++) for (int l = 0; l < 3; l++) {
      sr += G[i][j][k][l] * ks[2 * (k * 3 + l)];
      si += G[i][j][k][l] * ks[2 * (k * 3 + l) + 1];
    }
    outr[i * 3 + j] = sr;
    outi[i * 3 + j] = si;
  }
  for (int q = 0; q < 9; q++) { ks[2 * q] = outr[q]; ks[2 * q + 1] = outi[q]; }
}

/* get_smacro (src/evolution.c:473-547) */
static void get_smacro(orc_ctx* c) {
  static const int IJV[2][6] = {{0, 1, 2, 1, 0, 0}, {0, 1, 2, 2, 2, 1}};
  for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) {
    double s = 0.0, s1 = 0.0;
    for (size_t v = 0; v < c->nv; v++) {
      s += c->sig[v][i][j];
      if (c->phase[v] == 1) s1 += c->sig[v][i][j];
    }
    c->sig_avg[i][j] = s * c->wgt;
    c->sig_avg1[i][j] = s1 * (c->wgt / c->wgt_ph1);
  }
  for (int a = 0; a < 6; a++) {
    int ii = IJV[0][a], jj = IJV[1][a];
    c->ddisgrad_avg[ii][jj] = 0.0;
    if (c->vbc[a] == 0) {
      for (int b = 0; b < 6; b++) {
        int kk = IJV[0][b], ll = IJV[1][b];
        c->ddisgrad_avg[ii][jj] += c->s0[ii][jj][kk][ll] * c->sbc[b] * (c->scauchy[kk][ll] - c->sig_avg[kk][ll]);
      }
    }
  }
  for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) c->ddisgrad_acum[i][j] += c->ddisgrad_avg[i][j];
  double v6[6];
  t2v((const double(*)[3])c->sig_avg, v6, 6);
  v2t(v6, c->sig_dev_avg, 5);
  double oob = (c->svm_oob_mode == ORC_SVM_OOB_EPSAVG10) ? c->eps_avg[1][0]
             : (c->svm_oob_mode == ORC_SVM_OOB_SIGAVG1_00) ? c->sig_avg1[0][0] : 0.0;
  double svm = 0.0;
  for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) {
    if (i != j) svm += c->sig_dev_avg[i][j] * c->sig_dev_avg[i][j];
    else {
      double d = c->sig_dev_avg[i][j] - (c->sig_dev_avg[1][1] + c->sig_dev_avg[2][2] + oob) / 3.0;
      svm += d * d;
    }
  }
  c->s_vm = sqrt(3. / 2. * svm);
  t2v((const double(*)[3])c->sig_avg1, v6, 6);
  v2t(v6, c->sig_dev_avg, 5);
  double svm1 = 0.0;
  for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) svm1 += c->sig_dev_avg[i][j] * c->sig_dev_avg[i][j];
  c->s_vm1 = sqrt(3. / 2. * svm1);
}

/* Orientation (src/constitutive.c:142-194) */
static void orientation(t33 tran, t33 rot) {
  double w[3] = {rot[2][1], rot[0][2], rot[1][0]};
  double wn = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
  double wt = tan(wn / 2.0);
  if (fabs(wn) < 1e-6) wn = 1.0;
  for (int i = 0; i < 3; i++) w[i] *= wt / wn;
  t33 om = {{0., -1. * w[2], w[1]}, {w[2], 0., -1. * w[0]}, {-1. * w[1], w[0], 0.}}, om2, tn;
  for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) {
    double s = 0.0;
    for (int k = 0; k < 3; k++) s += om[i][k] * om[k][j];
    om2[i][j] = s;
  }
  wt = wt * wt;
  for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++)
    rot[i][j] = (double)(i == j) + 2. * (om[i][j] + om2[i][j]) / (1. + wt);
  for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) {
    double s = 0.0;
    for (int k = 0; k < 3; k++) s += rot[i][k] * tran[k][j];
    tn[i][j] = s;
  }
  memcpy(tran, tn, sizeof(t33));
}

/* update_orient (src/constitutive.c:196-273) */
static void update_orient(orc_ctx* c) {
#pragma omp parallel for schedule(static)
  for (long long v = 0; v < (long long)c->nv; v++) {
    const phase_t* ph = &c->ph[c->phase[v] - 1];
    if (ph->type != 0) continue;
    t33 rl, lp, tm, rs, rot;
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) {
      rl[i][j] = (c->velgrad[v][i][j] - c->velgrad[v][j][i]) / 2.;
      lp[i][j] = 0.0;
      tm[i][j] = c->tranmat[v][i][j];
    }
    for (int is = 0; is < ph->nsys; is++) {
      double bs[3], ns[3];
      for (int i = 0; i < 3; i++) {
        bs[i] = 0.0; ns[i] = 0.0;
        for (int j = 0; j < 3; j++) { bs[i] += tm[i][j] * ph->bb[is][j]; ns[i] += tm[i][j] * ph->bn[is][j]; }
      }
      for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) lp[i][j] += bs[i] * ns[j] * c->gamdot[v][is];
    }
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) rs[i][j] = (lp[i][j] - lp[j][i]) / 2.;
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++)
      rot[i][j] = (c->udot_a[i][j] + rl[i][j] - rs[i][j]) * c->dt;
    orientation(tm, rot);
    memcpy(c->tranmat[v], tm, sizeof(t33));
  }
}

/* harden (src/constitutive.c:275-326) */
static void harden(orc_ctx* c) {
#pragma omp parallel for schedule(static)
  for (long long v = 0; v < (long long)c->nv; v++) {
    const phase_t* ph = &c->ph[c->phase[v] - 1];
    if (ph->type != 0) continue;
    double gamtot = c->gamacum[v], deltgam = 0.0;
    for (int i = 0; i < ph->nsys; i++) deltgam += fabs(c->gamdot[v][i]) * c->dt;
    for (int i = 0; i < ph->nsys; i++) {
      double dtau = 0.;
      for (int j = 0; j < ph->nsys; j++) dtau += ph->hard[i][j] * fabs(c->gamdot[v][j]) * c->dt;
      double tau0 = ph->tau[0], tau1 = ph->tau[2], thet0 = ph->thet[0], thet1 = ph->thet[1];
      double tiny = 1.e-4 * tau0, voce = 0.0;
      if (fabs(thet0) > tiny) {
        voce = thet1 * deltgam;
        if (fabs(tau1) > tiny) {
          double fact = fabs(thet0 / tau1);
          double exp_ini = exp(-1.0 * gamtot * fact);
          double exp_del = exp(-1.0 * deltgam * fact);
          voce += -1. * (fact * tau1 - thet1) / fact * exp_ini * (exp_del - 1.0) -
                  thet1 / fact * exp_ini * (exp_del * ((gamtot + deltgam) * fact + 1.0) - (gamtot * fact + 1.0));
        }
      }
      c->crss[v][i][0] += dtau * voce / deltgam;
      c->crss[v][i][1] += dtau * voce / deltgam;
    }
    c->gamacum[v] = gamtot + deltgam;
  }
}

/* Gradient_ShearRate (src/constitutive.c:875-1108): per system, one-sided
 * or central differences of the shear rate across the x, y, z neighbours
 * that lie in the same grain (GB_check flags), 0 where neither does;
 * periodic. */
static void dd_gradient_rate(orc_ctx* c) {
  const int n0 = c->n[0], n1 = c->n[1], n2 = c->n[2];
#pragma omp parallel for schedule(static)
  for (int x = 0; x < n0; x++)
    for (int y = 0; y < n1; y++)
      for (int z = 0; z < n2; z++) {
        const size_t v = ((size_t)x * n1 + y) * n2 + z;
        const size_t nb[6] = {((size_t)((x + 1) % n0) * n1 + y) * n2 + z, ((size_t)((x + n0 - 1) % n0) * n1 + y) * n2 + z,
                              ((size_t)x * n1 + (y + 1) % n1) * n2 + z, ((size_t)x * n1 + (y + n1 - 1) % n1) * n2 + z,
                              ((size_t)x * n1 + y) * n2 + (z + 1) % n2, ((size_t)x * n1 + y) * n2 + (z + n2 - 1) % n2};
        for (int i = 0; i < NS; i++)
          for (int a = 0; a < 3; a++) {
            const int up = c->gbchk[v][2 * a], dn = c->gbchk[v][2 * a + 1];
            double g;
            if (!up && dn) g = c->gamdot[v][i] - c->gamdot[nb[2 * a + 1]][i];
            else if (up && !dn) g = c->gamdot[nb[2 * a]][i] - c->gamdot[v][i];
            else if (up && dn) g = (c->gamdot[nb[2 * a]][i] - c->gamdot[nb[2 * a + 1]][i]) / 2.0;
            else g = 0.0;
            c->gadot_grad[v][i][a] = g;
          }
      }
}

/* DislocationEvolution with first-order GNDs (src/constitutive.c:1346-1520)
 * and AvgDislocation (src/constitutive.c:1669-1760). */
static void dd_evolution(orc_ctx* c) {
  const size_t nv = c->nv;
#pragma omp parallel for schedule(static)
  for (long long v = 0; v < (long long)nv; v++) {
    const phase_t* ph = &c->ph[c->phase[v] - 1];
    if (ph->type != 0) continue;
    const double b = ph->dd_b, G = ph->dd_G;
    double sig6[6];
    t2v((const double(*)[3])c->sig[v], sig6, 6);
    for (int i = 0; i < ph->nsys; i++) {
      const double* sc = c->schm[v][i];
      double rss = sc[0] * sig6[0] + sc[1] * sig6[1] + sc[2] * sig6[2] + sc[3] * sig6[3] + sc[4] * sig6[4];
      double hydro = (sig6[0] + sig6[1] + sig6[2]) / 3.0;
      double d_dipole = sqrt(3.0) * G * b / 16.0 / R_PI / (1 - ph->dd_nu) / (fabs(rss) + DD_EPS);
      double ag = fabs(c->gamdot[v][i]);
      const double c4 = ph->dd_c[3], c5 = ph->dd_c[4], c6 = ph->dd_c[5], c7 = ph->dd_c[6];
      c->rho_dipole[v][i] += ag * (c6 * (d_dipole)*c->rho_m[v][i]) * c->dt;
      c->rho_forest[v][i] += ag * (c4 * sqrt(c->rho_F[v][i])) * c->dt;
      double rs = c->rho_s[v][i];
      double dot_ssd = ag * (c4 * sqrt(c->rho_F[v][i]) + c6 * (d_dipole)*c->rho_m[v][i] - c5 * rs) -
                       c7 * 1.6 * 1E12 * 1E-9 * rs * rs -
                       4 * 1E12 * (d_dipole) * (ph->dd_d0 / b) * pow(rs, 2.0) *
                           exp((fabs(hydro) * b * b * b * 100 / (1.38 * ph->dd_T)) - 1.0) * exp(-1.0 * ph->dd_qbulk);
      c->rho_s[v][i] += dot_ssd * c->dt;
      c->gam_acum[v][i] = c->trial_gam_acum[v][i];
      const double* gg = c->gadot_grad[v][i];
      double g_screw = gg[0] * ph->bp[i][0] + gg[1] * ph->bp[i][1] + gg[2] * ph->bp[i][2];
      c->rho_g1[v][i] += g_screw / b / ph->dd_L0 * c->dt;
      double g_edge = gg[0] * ph->bb[i][0] + gg[1] * ph->bb[i][1] + gg[2] * ph->bb[i][2];
      c->rho_g2[v][i] += -1.0 * g_edge / b / ph->dd_L0 * c->dt;
      c->rho_g3[v][i] += 0.0 * c->dt;
    }
  }
  double s[7] = {0, 0, 0, 0, 0, 0, 0};
  for (size_t v = 0; v < nv; v++) {
    const phase_t* ph = &c->ph[c->phase[v] - 1];
    if (ph->type != 0) continue;
    for (int i = 0; i < ph->nsys; i++) {
      s[0] += c->rho_F[v][i];
      s[1] += c->rho_P[v][i];
      s[2] += c->rho_s[v][i];
      s[3] += c->rho_m[v][i];
      s[4] += sqrt(c->rho_g1[v][i] * c->rho_g1[v][i] + c->rho_g2[v][i] * c->rho_g2[v][i] +
                   c->rho_g3[v][i] * c->rho_g3[v][i]);
      s[5] += c->rho_dipole[v][i];
      s[6] += c->rho_forest[v][i];
    }
  }
  for (int k = 0; k < 7; k++) c->dd_avg[k] = s[k] * (1.0 / (double)nv);
}

/* Dynamic recrystallisation at the start of a mechanical step, in the order
 * of Evolution (src/evolution.c:850-1253), restated as in drx_oracle.c:
 * rho from accumulated slip, nucleation, phase-field relaxation, adoption
 * of the relaxed grain ids, reset of voxels that joined a recrystallised
 * grain (src/evolution.c:1120-1200) and the new reference medium C066/S0
 * (src/evolution.c:1200-1216; the Green operator keeps the initial C0). */
static int orc_drx_step(orc_ctx* c, int* n_new) {
  const size_t nv = c->nv;
  const mth_params* p = &c->par;
  const phase_t* ph0 = &c->ph[0];
  double* rho = (double*)malloc(sizeof(double) * nv);
  int* cry = (int*)malloc(sizeof(int) * nv);
  int* prev = (int*)malloc(sizeof(int) * nv);
  int* gnew = (int*)malloc(sizeof(int) * nv);
  long long* sites = (long long*)malloc(sizeof(long long) * 65536);
  for (size_t v = 0; v < nv; v++) {
    const int crystal = c->ph[c->phase[v] - 1].type == 0;
    cry[v] = crystal;
    rho[v] = crystal ? p->rho0 + p->rho_k * c->gamacum[v] : 0.0;
    prev[v] = c->grain[v];
  }
  long long ns = orc_nucleation_sites(c->n, c->grain, cry, rho, p->rho_nucleation, p->nucleation_prob, p->seed,
                                      c->istep, sites, 65536);
  int nn = (int)(ns < 65536 ? ns : 65536);
  if (nn > 0) {
    c->drx_rot = (double*)realloc(c->drx_rot, sizeof(double) * 9 * (size_t)(c->n_drx + nn));
    for (int k = 0; k < nn; k++) memcpy(c->drx_rot + 9 * (size_t)(c->n_drx + k), c->tranmat[sites[k]], sizeof(t33));
    orc_paint_nuclei(c->n, c->grain, sites, nn, c->next_grain_id, p->nucleus_radius);
    c->next_grain_id += nn;
    c->n_drx += nn;
  }
  *n_new = nn;
  int st = MTH_OK;
  if (c->next_grain_id > c->rho_avg_len) {   /* the table covers every grain id */
    const int len = c->next_grain_id + 1024;
    c->rho_avg_tab = (double*)realloc(c->rho_avg_tab, sizeof(double) * (size_t)len);
    for (int i = c->rho_avg_len; i < len; i++) c->rho_avg_tab[i] = 0.0;
    c->rho_avg_len = len;
  }
  if (c->n_drx > 0) {
    /* phase field on its own grid when CellDim_pf differs (InterpolateGrid,
     * src/integrated.c:674-760; coarse-graining src/integrated.c:821-860) */
    const int pf_zero = p->pf_cell_dim[0] == 0 && p->pf_cell_dim[1] == 0 && p->pf_cell_dim[2] == 0;
    int npf[3];
    for (int i = 0; i < 3; i++) npf[i] = pf_zero ? c->n[i] : p->pf_cell_dim[i];
    if (npf[0] != c->n[0] || npf[1] != c->n[1] || npf[2] != c->n[2]) {
      const size_t q = (size_t)npf[0] * npf[1] * npf[2];
      int* gpf = (int*)malloc(sizeof(int) * q);
      int* gnpf = (int*)malloc(sizeof(int) * q);
      double* rpf = (double*)malloc(sizeof(double) * q);
      orc_resample_nearest(c->n, c->grain, npf, gpf);
      orc_resample_trilinear(c->n, rho, npf, rpf);
      st = orc_pf_relax(p, npf, gpf, rpf, p->pf_substeps, c->first_drx_id - 1, c->rho_avg_tab, c->rho_avg_len,
                        gnpf, NULL, NULL, NULL, 0);
      orc_resample_nearest(npf, gnpf, c->n, gnew);
      free(gpf); free(gnpf); free(rpf);
    } else {
      st = orc_pf_relax(p, c->n, c->grain, rho, p->pf_substeps, c->first_drx_id - 1, c->rho_avg_tab,
                        c->rho_avg_len, gnew, NULL, NULL, NULL, 0);
    }
    /* per recrystallised grain: its voxels after the relaxation and those
       that joined it in this step; a grain whose joining voxels are under
       1 % of it (integer percent 0) resets none of them, they take its id
       only (the "growth" rollback, src/integrated.c:1537-1582) */
    long long* gtot = (long long*)calloc((size_t)c->n_drx, sizeof(long long));
    long long* gjoin = (long long*)calloc((size_t)c->n_drx, sizeof(long long));
    for (size_t v = 0; v < nv; v++) {
      const int g = gnew[v] != 0 ? gnew[v] : c->grain[v];
      const int k = g - c->first_drx_id;
      if (k < 0 || k >= c->n_drx) continue;
      gtot[k]++;
      if (g != prev[v] && cry[v]) gjoin[k]++;
    }
    for (size_t v = 0; v < nv && st == MTH_OK; v++) {
      /* a voxel left without a positive eta (grain id 0: the reference stops
         there on GetStatistics' assert, src/pf_xrx.c:1383-1386) keeps its grain */
      const int g = gnew[v] != 0 ? gnew[v] : c->grain[v];
      c->grain[v] = g;
      const int k = g - c->first_drx_id;
      if (g == prev[v] || !cry[v] || k < 0 || k >= c->n_drx) continue;
      if (gjoin[k] * 100 / gtot[k] == 0) continue;
      memset(c->sig[v], 0, sizeof(t33));
      c->gamacum[v] = 0.0;
      for (int i = 0; i < ph0->nsys; i++) { c->crss[v][i][0] = ph0->tau[0]; c->crss[v][i][1] = ph0->tau[1]; }
      memcpy(c->tranmat[v], c->drx_rot + 9 * (size_t)k, sizeof(t33));
      t33 sa2xt;
      t3333 caux;
      for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) sa2xt[i][j] = c->tranmat[v][j][i];
      ten4_inverse_transform(caux, (const double(*)[3])sa2xt, (const double(*)[3][3][3])ph0->cijkl);
      t42m((const double(*)[3][3][3])caux, c->cgr[v]);
      memcpy(c->sg66[v], c->cgr[v], sizeof(m66));
      if (lu_inv66(c->sg66[v])) st = MTH_ERR_SINGULAR;
    }
    free(gtot);
    free(gjoin);
    if (st == MTH_OK) {
      m66 csum;
      memset(csum, 0, sizeof(csum));
      for (size_t v = 0; v < nv; v++)
        if (cry[v]) for (int i = 0; i < 6; i++) for (int j = 0; j < 6; j++) csum[i][j] += c->cgr[v][i][j];
      for (int i = 0; i < 6; i++) for (int j = 0; j < 6; j++) c->c066[i][j] = csum[i][j] * c->wgt;
      memcpy(c->s066, c->c066, sizeof(m66));
      if (lu_inv66(c->s066)) st = MTH_ERR_SINGULAR;
      m2t4((const double(*)[6])c->c066, c->c0);
      m2t4((const double(*)[6])c->s066, c->s0);
    }
  }
  free(rho); free(cry); free(prev); free(gnew); free(sites);
  return st;
}

/* One mechanical step: body of the istep loop in Evolution
 * (src/evolution.c:1319-1693) on the power-law path. */
int orc_step(orc_ctx* c, mth_step_report* rep) {
  const size_t nv = c->nv;
  const int istep = c->istep;
  int st = MTH_OK;
  if (c->creep == 1 && c->e_vm > 0.3) return MTH_ERR_STATE;   /* src/evolution.c:606 */
  int n_new = 0;
  if (c->par.pf_substeps > 0 && istep > 0) {
    st = orc_drx_step(c, &n_new);
    if (st) return st;
  }
  /* src/evolution.c:1319-1332 */
#pragma omp parallel for schedule(static)
  for (long long v = 0; v < (long long)nv; v++)
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) {
      c->velgrad[v][i][j] = c->disgrad[v][i][j];
      if (c->creep == 1) c->disgrad[v][i][j] = c->disgrad_avg_t[i][j];
      else c->disgrad[v][i][j] += c->udot[i][j] * c->dt;
    }
  if (istep == 1 || c->update_flag == 1) update_schmid_all(c);   /* src/evolution.c:1334-1336 */
  memset(c->ddisgrad_avg, 0, sizeof(t33));
  memset(c->ddisgrad_acum, 0, sizeof(t33));
  int iter = 0;
  c->err_e = 2. * c->err_tol;
  c->err_s = 2. * c->err_tol;
  long long nit_total = 0, nbad_total = 0;
  const int n0 = c->n[0], n1 = c->n[1], n2 = c->n[2];
  while ((iter < c->iter_max) && (fmax(fabs(c->err_s), fabs(c->err_e)) > c->err_tol)) {
    iter++;
    /* forward FFT of the 6 independent stress components
       (src/evolution.c:1361-1372; sigma is symmetric so the (j,i) transforms
       equal the (i,j) ones) */
    double* buf = (double*)malloc(sizeof(double) * 2 * nv);
    static const int sym_i[6] = {0, 1, 2, 1, 0, 0}, sym_j[6] = {0, 1, 2, 2, 2, 1};
    for (int q = 0; q < 6; q++) {
      int i = sym_i[q], j = sym_j[q];
      for (size_t v = 0; v < nv; v++) { buf[2 * v] = c->sig[v][i][j]; buf[2 * v + 1] = 0.0; }
      orc_fft3d(buf, n0, n1, n2, -1);
      for (size_t v = 0; v < nv; v++) {
        c->kbuf[18 * v + 2 * (i * 3 + j)] = buf[2 * v];
        c->kbuf[18 * v + 2 * (i * 3 + j) + 1] = buf[2 * v + 1];
        c->kbuf[18 * v + 2 * (j * 3 + i)] = buf[2 * v];
        c->kbuf[18 * v + 2 * (j * 3 + i) + 1] = buf[2 * v + 1];
      }
    }
#pragma omp parallel for schedule(static)
    for (long long v = 0; v < (long long)nv; v++) gamma_apply(c, (size_t)v, c->nvec[v], c->kbuf + 18 * v);
    /* inverse FFT and strain update (src/evolution.c:1393-1405) */
    for (int q = 0; q < 9; q++) {
      int i = q / 3, j = q % 3;
      for (size_t v = 0; v < nv; v++) { buf[2 * v] = c->kbuf[18 * v + 2 * q]; buf[2 * v + 1] = c->kbuf[18 * v + 2 * q + 1]; }
      orc_fft3d(buf, n0, n1, n2, +1);
      for (size_t v = 0; v < nv; v++) c->disgrad[v][i][j] += c->ddisgrad_avg[i][j] + buf[2 * v] / (double)nv;
    }
    free(buf);
    /* UpdateStress (src/evolution.c:44-310) */
    int bad_status = MTH_OK;
#pragma omp parallel for schedule(dynamic, 64)
    for (long long v = 0; v < (long long)nv; v++) {
      const phase_t* ph = &c->ph[c->phase[v] - 1];
      c->newton_it[v] = 0;
      c->newton_bad[v] = 0;
      if (ph->type == 0) {
        double xl6[6], s6[6], e6[6], st6[6], ed6[6];
        t33 strain;
        for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++)
          strain[i][j] = (c->disgrad[v][i][j] + c->disgrad[v][j][i]) / 2.0;
        t2v((const double(*)[3])c->sig[v], xl6, 6);
        t2v((const double(*)[3])c->sig[v], s6, 6);
        t2v((const double(*)[3])c->eps[v], e6, 6);
        t2v((const double(*)[3])strain, st6, 6);
        ddv_t ddv, *dp = NULL;
        if (c->dd) {
          ddv.rho_s = c->rho_s[v]; ddv.g1 = c->rho_g1[v]; ddv.g2 = c->rho_g2[v]; ddv.g3 = c->rho_g3[v];
          ddv.rho_m = c->rho_m[v]; ddv.rho_F = c->rho_F[v]; ddv.rho_P = c->rho_P[v];
          ddv.gam_acum = c->gam_acum[v]; ddv.trial_gam_acum = c->trial_gam_acum[v]; ddv.dt = c->dt;
          dp = &ddv;
        }
        newton_out o = newton_voxel(ph, (const double(*)[5])c->schm[v], (const double(*)[2])c->crss[v], dp,
                                    (const double(*)[6])c->c066, c->dt, (const double(*)[6])c->sg66[v],
                                    s6, xl6, e6, st6, ed6, c->gamdot[v], c->newton_tol, c->newton_itmax);
        if (o.status == MTH_ERR_SINGULAR) bad_status = MTH_ERR_SINGULAR;
        c->newton_it[v] = o.iters;
        c->newton_bad[v] = (o.status != MTH_OK);
        if (o.cubic) {
#pragma omp atomic
          c->cubic_total += o.cubic;
        }
        v2t(s6, c->sig[v], 6);
        v2t(ed6, c->edot[v], 6);
        c->conv_s[v] = o.conv_s;
        c->conv_e[v] = o.conv_e;
      } else {
        memset(c->sig[v], 0, sizeof(t33));
        memset(c->edot[v], 0, sizeof(t33));
        c->conv_s[v] = 0.0;
        c->conv_e[v] = 0.0;
      }
    }
    if (bad_status) st = bad_status;
    double es = 0.0, ee = 0.0;
    for (size_t v = 0; v < nv; v++) {
      es += c->conv_s[v];
      ee += c->conv_e[v];
      nit_total += c->newton_it[v];
      nbad_total += c->newton_bad[v];
    }
    c->err_e = ee * c->wgt;
    c->err_s = es * c->wgt;
    get_smacro(c);
    if (fabs(c->e_vm) < 1E-5) c->err_e = 0.0;
    else c->err_e /= c->e_vm;
    c->err_s /= c->s_vm;
  }
  /* src/evolution.c:1471-1535 */
#pragma omp parallel for schedule(static)
  for (long long v = 0; v < (long long)nv; v++)
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++)
      c->velgrad[v][i][j] = (c->disgrad[v][i][j] - c->velgrad[v][i][j]) / c->dt;
  t33 actual, vgavg;
  for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) {
    actual[i][j] = c->disgrad_avg[i][j] + c->ddisgrad_acum[i][j];
    vgavg[i][j] = (actual[i][j] - c->disgrad_avg_t[i][j]) / c->dt;
  }
  c->e_vm = von_mises((const double(*)[3])actual);
  c->d_vm = von_mises((const double(*)[3])vgavg);
  c->time_tot += c->dt;
  memcpy(c->disgrad_avg_t, actual, sizeof(t33));
#pragma omp parallel for schedule(static)
  for (long long v = 0; v < (long long)nv; v++)
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) c->eps[v][i][j] += c->edot[v][i][j] * c->dt;
  t33 ea, da;
  memset(ea, 0, sizeof(ea));
  memset(da, 0, sizeof(da));
  for (size_t v = 0; v < nv; v++)
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) {
      ea[i][j] += c->eps[v][i][j] * c->wgt;
      da[i][j] += c->edot[v][i][j] * c->wgt;
    }
  memcpy(c->eps_avg, ea, sizeof(t33));
  memcpy(c->edot_avg, da, sizeof(t33));
  double evmp = 0.0, dvmp = 0.0;
  for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) {
    evmp += ea[i][j] * ea[i][j];
    dvmp += da[i][j] * da[i][j];
  }
  evmp = sqrt(2. / 3. * evmp);
  dvmp = sqrt(2. / 3. * dvmp);
  if (c->update_flag == 1 && istep > 1) update_orient(c);      /* src/evolution.c:1543-1546 */
  if (c->dd) {
    if (c->hard_flag == 1 && istep > 1) dd_gradient_rate(c);    /* src/evolution.c:1551-1559 */
    dd_evolution(c);                                            /* src/evolution.c:1564-1565 */
  } else if (c->hard_flag == 1) {
    harden(c);                                                  /* oracle patch point, src/evolution.c:1574 */
  }
  if (rep) {
    memset(rep, 0, sizeof(*rep));
    rep->step = istep;
    rep->iterations = iter;
    rep->time = c->time_tot;
    memcpy(rep->sig_avg, c->sig_avg, sizeof(t33));
    memcpy(rep->sig_avg_ph1, c->sig_avg1, sizeof(t33));
    memcpy(rep->disgrad_avg, actual, sizeof(t33));
    memcpy(rep->eps_avg, ea, sizeof(t33));
    memcpy(rep->edot_avg, da, sizeof(t33));
    rep->e_vm = c->e_vm; rep->evmp = evmp; rep->d_vm = c->d_vm; rep->dvmp = dvmp;
    rep->s_vm = c->s_vm; rep->s_vm1 = c->s_vm1;
    rep->err_s = c->err_s; rep->err_e = c->err_e;
    rep->newton_iters = nit_total;
    rep->newton_failed = nbad_total;
    rep->n_new_grains = n_new;
    if (c->dd) memcpy(rep->dd_avg, c->dd_avg, sizeof(c->dd_avg));
  }
  /* next macro guess (src/evolution.c:1691-1693) */
  for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++)
    c->disgrad_avg[i][j] = c->disgrad_avg_t[i][j] + c->udot[i][j] * c->dt;
  c->istep++;
  return st;
}

int orc_get_field(orc_ctx* c, int field, double* out) {
  const size_t nv = c->nv;
  for (size_t v = 0; v < nv; v++) {
    switch (field) {
      case MTH_FIELD_SIG: memcpy(out + 9 * v, c->sig[v], sizeof(t33)); break;
      case MTH_FIELD_EPS: memcpy(out + 9 * v, c->eps[v], sizeof(t33)); break;
      case MTH_FIELD_EDOT: memcpy(out + 9 * v, c->edot[v], sizeof(t33)); break;
      case MTH_FIELD_STRAIN:
        for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++)
          out[9 * v + 3 * i + j] = (c->disgrad[v][i][j] + c->disgrad[v][j][i]) / 2.0;
        break;
      case MTH_FIELD_ROT: memcpy(out + 9 * v, c->tranmat[v], sizeof(t33)); break;
      case MTH_FIELD_DISGRAD: memcpy(out + 9 * v, c->disgrad[v], sizeof(t33)); break;   /* DisGrad as kept */
      case MTH_FIELD_CRSS:
        for (int i = 0; i < NS; i++) out[NS * v + i] = c->crss[v][i][0];
        break;
      case MTH_FIELD_GAMACUM: out[v] = c->gamacum[v]; break;
      case MTH_FIELD_RHO_SSD:
        if (!c->dd) return MTH_ERR_ARG;
        for (int i = 0; i < NS; i++) out[NS * v + i] = c->rho_s[v][i];
        break;
      case MTH_FIELD_RHO_GND:
        if (!c->dd) return MTH_ERR_ARG;
        for (int i = 0; i < NS; i++) {
          out[3 * NS * v + i] = c->rho_g1[v][i];
          out[3 * NS * v + NS + i] = c->rho_g2[v][i];
          out[3 * NS * v + 2 * NS + i] = c->rho_g3[v][i];
        }
        break;
      case MTH_FIELD_GRAIN: out[v] = (double)c->grain[v]; break;
      case MTH_FIELD_RHO:
        out[v] = c->ph[c->phase[v] - 1].type == 0 ? c->par.rho0 + c->par.rho_k * c->gamacum[v] : 0.0;
        break;
      default: return MTH_ERR_ARG;
    }
  }
  return MTH_OK;
}

int orc_get_c066(orc_ctx* c, double* c066) {
  memcpy(c066, c->c066, sizeof(m66));
  return MTH_OK;
}

long long orc_second_backtracks(orc_ctx* c) { return c->cubic_total; }

int orc_local_solve(const mth_params* p, const double c066[36], size_t n, double* sig, const double* eps_p,
                    const double* strain, const double* rot, const double* crss, double* edot, double* err,
                    long long* newton_iters) {
  basis_init();
  phase_t ph;
  int st = phase_init(&p->phase[0], &ph);
  if (st) return st;
  if (ph.type != 0) return MTH_ERR_ARG;
  m66 c6;
  memcpy(c6, c066, sizeof(m66));
  double tol = p->newton_tol > 0 ? p->newton_tol : 1e-10;
  int itmax = p->newton_itmax > 0 ? p->newton_itmax : 500;
  long long tot = 0;
  int bad = MTH_OK;
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : tot)
  for (long long v = 0; v < (long long)n; v++) {
    t33 tm, sa2xt;
    t3333 caux;
    m66 cgr;
    double sc[NS][5], tau[NS][2], xl[6], gd[NS];
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) { tm[i][j] = rot[9 * v + 3 * i + j]; sa2xt[j][i] = tm[i][j]; }
    ten4_inverse_transform(caux, (const double(*)[3])sa2xt, (const double(*)[3][3][3])ph.cijkl);
    t42m((const double(*)[3][3][3])caux, cgr);
    if (lu_inv66(cgr)) { bad = MTH_ERR_SINGULAR; continue; }
    schmid_sample(&ph, (const double(*)[3])tm, sc);
    for (int i = 0; i < ph.nsys; i++) { tau[i][0] = crss[NS * v + i]; tau[i][1] = crss[NS * v + i] + (ph.tau[1] - ph.tau[0]); }
    for (int i = 0; i < 6; i++) xl[i] = sig[6 * v + i];
    newton_out o = newton_voxel(&ph, (const double(*)[5])sc, (const double(*)[2])tau, NULL, (const double(*)[6])c6,
                                p->time_step, (const double(*)[6])cgr, sig + 6 * v, xl, eps_p + 6 * v,
                                strain + 6 * v, edot + 6 * v, gd, tol, itmax);
    err[2 * v] = o.conv_s;
    err[2 * v + 1] = o.conv_e;
    tot += o.iters;
  }
  if (newton_iters) *newton_iters = tot;
  return bad;
}

// book.cuh -- the macroscopic bookkeeping of one Green iteration, written
// once for the host and the device: the uniform strain increment of the
// iteration (src/evolution.c:1319-1332), and from the reduced partial sums
// the error norms (src/evolution.c:1430-1455) and get_smacro
// (src/evolution.c:473-547: volume-averaged stress, the mixed-boundary
// strain correction, von Mises measures).  The host runs it in the batch
// and the adjoint; mth_step runs it in a one-warp kernel after each
// iteration, so iterations follow one another on the device without a host
// round trip.  Both builds compile it without FMA contraction; the basic
// operations and sqrt are correctly rounded on both, so the two give the
// same doubles.
#pragma once
#include <cmath>
#include "mth_common.cuh"

#ifdef __CUDACC__
#define MTH_HD __host__ __device__
#else
#define MTH_HD
#endif

namespace mth {

struct IterBook {
  // constants of the step
  double udot[3][3], scauchy[3][3], s0_4[81];
  int vbc[6], sbc[6];
  double wgt, wgt_ph1, dt, err, e_vm;
  int iter_max;
  // state
  double ddg[3][3], ddg_acum[3][3], ddg_applied[3][3], sig_avg[3][3], sig_avg1[3][3];
  double err_s, err_e, s_vm, s_vm1;
  int it_iter, nan;
  long long it_nit, it_nbad;
};

// component (m, n) of the Lebensohn-Tome basis tensor B_i (chg_basis,
// src/kinematics.c:27-53)
MTH_HD inline double book_basis(int i, int m, int n) {
  switch (i) {
    case 0: return m != n ? 0.0 : m == 0 ? -RSQ2 : m == 1 ? RSQ2 : 0.0;
    case 1: return m != n ? 0.0 : m == 2 ? 2. * RSQ6 : -RSQ6;
    case 2: return (m == 1 && n == 2) || (m == 2 && n == 1) ? RSQ2 : 0.0;
    case 3: return (m == 0 && n == 2) || (m == 2 && n == 0) ? RSQ2 : 0.0;
    case 4: return (m == 0 && n == 1) || (m == 1 && n == 0) ? RSQ2 : 0.0;
    default: return m == n ? RSQ3 : 0.0;
  }
}
MTH_HD inline void book_t2v(const double t[3][3], double* v, int nv) {
  for (int i = 0; i < nv; i++) {
    double s = 0;
    for (int m = 0; m < 3; m++)
      for (int n = 0; n < 3; n++) s += t[m][n] * book_basis(i, m, n);
    v[i] = s;
  }
}
MTH_HD inline void book_v2t(const double* v, double t[3][3], int nv) {
  for (int m = 0; m < 3; m++)
    for (int n = 0; n < 3; n++) {
      double s = 0;
      for (int i = 0; i < nv; i++) s += v[i] * book_basis(i, m, n);
      t[m][n] = s;
    }
}

MTH_HD inline bool book_finite(double x) {
#ifdef __CUDA_ARCH__
  return isfinite(x);
#else
  return std::isfinite(x);
#endif
}

// another iteration: IterMax not reached and Err not met
MTH_HD inline bool book_more(const IterBook& b) {
  return b.it_iter < b.iter_max && fmax(fabs(b.err_s), fabs(b.err_e)) > b.err;
}

// the uniform strain increment of the next iteration (add6, LT basis):
// the correction of the previous get_smacro, plus Udot dt on the first one
MTH_HD inline void book_add(IterBook& b, double* add6) {
  b.it_iter++;
  double u[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      u[i][j] = b.ddg[i][j] + (b.it_iter == 1 ? b.udot[i][j] * b.dt : 0.0);
      b.ddg_applied[i][j] += b.ddg[i][j];
    }
  book_t2v(u, add6, 6);
}

// get_smacro from the reduced sums red (NPART: err_s, err_e, sig[6],
// sig_ph1[6], Newton steps, failed solves).  The von Mises stress keeps the
// reference's formula, whose out-of-bounds word SigDevAvg[3][3]
// (src/evolution.c:531) holds SigAvg1[0][0] in the reference as built with
// g++ (SigAvg1 is laid out right after SigDevAvg's padding).
MTH_HD inline void book_smacro(IterBook& b, const double* red) {
  const int IJV[2][6] = {{0, 1, 2, 1, 0, 0}, {0, 1, 2, 2, 2, 1}};
  double s6[6], s16[6];
  for (int i = 0; i < 6; i++) {
    s6[i] = red[2 + i] * b.wgt;
    s16[i] = red[8 + i] * (b.wgt / b.wgt_ph1);
  }
  book_v2t(s6, b.sig_avg, 6);
  book_v2t(s16, b.sig_avg1, 6);
  for (int a = 0; a < 6; a++) {
    const int ii = IJV[0][a], jj = IJV[1][a];
    b.ddg[ii][jj] = 0.0;
    if (b.vbc[a] == 0)
      for (int q = 0; q < 6; q++) {
        const int kk = IJV[0][q], ll = IJV[1][q];
        b.ddg[ii][jj] += b.s0_4[((ii * 3 + jj) * 3 + kk) * 3 + ll] * b.sbc[q] * (b.scauchy[kk][ll] - b.sig_avg[kk][ll]);
      }
  }
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) b.ddg_acum[i][j] += b.ddg[i][j];
  double dev[3][3], v6[6];
  book_t2v(b.sig_avg, v6, 6);
  book_v2t(v6, dev, 5);
  const double oob = b.sig_avg1[0][0];
  double svm = 0;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      if (i != j) svm += dev[i][j] * dev[i][j];
      else {
        const double d = dev[i][j] - (dev[1][1] + dev[2][2] + oob) / 3.0;
        svm += d * d;
      }
    }
  b.s_vm = sqrt(3. / 2. * svm);
  book_t2v(b.sig_avg1, v6, 6);
  book_v2t(v6, dev, 5);
  double svm1 = 0;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) svm1 += dev[i][j] * dev[i][j];
  b.s_vm1 = sqrt(3. / 2. * svm1);
}

// the end of an iteration; false (and nan set) on a non-finite sum
MTH_HD inline bool book_finish(IterBook& b, const double* red, int npart) {
  for (int i = 0; i < npart; i++)
    if (!book_finite(red[i])) {
      b.nan = 1;
      return false;
    }
  b.it_nit += (long long)red[14];
  b.it_nbad += (long long)red[15];
  b.err_s = red[0] * b.wgt;
  b.err_e = red[1] * b.wgt;
  book_smacro(b, red);
  if (fabs(b.e_vm) < 1E-5) b.err_e = 0.0;
  else b.err_e /= b.e_vm;
  b.err_s /= b.s_vm;
  return true;
}

}  // namespace mth

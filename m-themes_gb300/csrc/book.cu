// book.cu -- the per-iteration bookkeeping of book.cuh as a one-warp
// kernel, so that mth_step can queue Green iterations without a host round
// trip.  GB300 issues FP64 at one warp instruction per sub-partition every
// few dozen cycles whatever the active lanes, so a one-thread version of
// the ~800 FP64 operations took 25 us per iteration; here the lanes compute
// the independent entries (the 9 entries of a tensor, the 6 of a vector)
// side by side, each with exactly the operations, in the order, of
// book.cuh's loops.  Compiled without FMA contraction like the host code;
// tests require the two to give the same doubles.
#include "book.cuh"
#include "mth_internal.h"

namespace mth {

// first: the step's start (live set, the first iteration's increment);
// otherwise the end of an iteration that ran (its reduced sums in red) and
// the increment of the next one.  live drops to 0 when the step's
// iterations are done (Err met or IterMax) or a sum is not finite, and the
// iteration kernels queued after that return at once.  One warp.
__global__ void __launch_bounds__(32) iter_book_kernel(IterBook* __restrict__ b, const double* __restrict__ red,
                                                       double* __restrict__ add, int* __restrict__ live, int first) {
  chain_wait();
  const int lane = threadIdx.x;
  __shared__ double s6[6], s16[6], sg[9], sg1[9], v6[6], v61[6], dv[9], dv1[9], u[9];
  __shared__ int more;
  if (first) {
    if (lane == 0) *live = 1;
  } else {
    if (!*live) return;
    // book_finish: a non-finite sum ends the step
    const bool ok = lane >= NPART || isfinite(red[lane]);
    if (!__all_sync(0xffffffffu, ok)) {
      if (lane == 0) {
        b->nan = 1;
        *live = 0;
      }
      return;
    }
    if (lane == 0) {
      b->it_nit += (long long)red[14];
      b->it_nbad += (long long)red[15];
      b->err_s = red[0] * b->wgt;
      b->err_e = red[1] * b->wgt;
    }
    // book_smacro
    if (lane < 6) s6[lane] = red[2 + lane] * b->wgt;
    else if (lane < 12) s16[lane - 6] = red[8 + lane - 6] * (b->wgt / b->wgt_ph1);
    __syncwarp();
    if (lane < 18) {   // v2t: sig_avg (lanes 0-8), sig_avg1 (lanes 9-17)
      const int e = lane % 9, m = e / 3, n = e % 3;
      const double* v = lane < 9 ? s6 : s16;
      double s = 0;
      for (int i = 0; i < 6; i++) s += v[i] * book_basis(i, m, n);
      if (lane < 9) {
        b->sig_avg[m][n] = s;
        sg[e] = s;
      } else {
        b->sig_avg1[m][n] = s;
        sg1[e] = s;
      }
    }
    __syncwarp();
    if (lane < 6) {   // the mixed-boundary correction, component a = lane
      const int IJV[2][6] = {{0, 1, 2, 1, 0, 0}, {0, 1, 2, 2, 2, 1}};
      const int ii = IJV[0][lane], jj = IJV[1][lane];
      double d = 0.0;
      if (b->vbc[lane] == 0)
        for (int q = 0; q < 6; q++) {
          const int kk = IJV[0][q], ll = IJV[1][q];
          d += b->s0_4[((ii * 3 + jj) * 3 + kk) * 3 + ll] * b->sbc[q] * (b->scauchy[kk][ll] - sg[kk * 3 + ll]);
        }
      b->ddg[ii][jj] = d;
    } else if (lane >= 6 && lane < 18) {   // t2v: of sig_avg (lanes 6-11), of sig_avg1 (lanes 12-17)
      const int i = (lane - 6) % 6;
      const double* t = lane < 12 ? sg : sg1;
      double s = 0;
      for (int m = 0; m < 3; m++)
        for (int n = 0; n < 3; n++) s += t[m * 3 + n] * book_basis(i, m, n);
      if (lane < 12) v6[i] = s;
      else v61[i] = s;
    }
    __syncwarp();
    if (lane < 9) {
      b->ddg_acum[lane / 3][lane % 3] += b->ddg[lane / 3][lane % 3];
    }
    if (lane < 18) {   // v2t of the deviatoric parts (5 components)
      const int e = lane % 9, m = e / 3, n = e % 3;
      const double* v = lane < 9 ? v6 : v61;
      double s = 0;
      for (int i = 0; i < 5; i++) s += v[i] * book_basis(i, m, n);
      if (lane < 9) dv[e] = s;
      else dv1[e] = s;
    }
    __syncwarp();
    if (lane == 0) {
      const double oob = sg1[0];
      double svm = 0;
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
          if (i != j) svm += dv[i * 3 + j] * dv[i * 3 + j];
          else {
            const double d = dv[i * 3 + j] - (dv[4] + dv[8] + oob) / 3.0;
            svm += d * d;
          }
        }
      b->s_vm = sqrt(3. / 2. * svm);
    } else if (lane == 1) {
      double svm1 = 0;
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) svm1 += dv1[i * 3 + j] * dv1[i * 3 + j];
      b->s_vm1 = sqrt(3. / 2. * svm1);
    }
    __syncwarp();
    if (lane == 0) {
      if (fabs(b->e_vm) < 1E-5) b->err_e = 0.0;
      else b->err_e /= b->e_vm;
      b->err_s /= b->s_vm;
    }
    __syncwarp();
  }
  // book_more, book_add
  if (lane == 0) {
    more = book_more(*b) ? 1 : 0;
    if (more) b->it_iter++;
    else *live = 0;
  }
  __syncwarp();
  if (!more) return;
  if (lane < 9) {
    const int i = lane / 3, j = lane % 3;
    u[lane] = b->ddg[i][j] + (b->it_iter == 1 ? b->udot[i][j] * b->dt : 0.0);
    b->ddg_applied[i][j] += b->ddg[i][j];
  }
  __syncwarp();
  if (lane < 6) {
    double s = 0;
    for (int m = 0; m < 3; m++)
      for (int n = 0; n < 3; n++) s += u[m * 3 + n] * book_basis(lane, m, n);
    add[lane] = s;
  }
}

cudaError_t launch_iter_book(IterBook* b, const double* red, double* add, int* live, int first, cudaStream_t st,
                             int pdl) {
  return launch_chain(iter_book_kernel, dim3(1), dim3(32), 0, st, pdl, b, red, add, live, first);
}

}  // namespace mth

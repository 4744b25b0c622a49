// dd.cu -- dislocation-density law: the per-step state of StrainRate_Orowan
// (src/constitutive.c:507-721), DislocationEvolution with first-order GNDs
// (src/constitutive.c:1346-1520), Gradient_ShearRate (src/constitutive.c:
// 875-1108) and AvgDislocation (src/constitutive.c:1669-1760).
//
// The reference recomputes the forest and parallel densities, the mobile
// density, the passing and cutting stresses and the reference rate inside
// every flow-rule evaluation, from densities that change only at the end of
// a mechanical step.  Here they are computed once per step (dd_prep) and the
// local Newton reads three numbers per slip system.  (The reference's
// passing stress uses the mobile density of the previous evaluation, which
// differs from the current one only at the first evaluation of a step; the
// converged stress is the same.)
//
// Arithmetic in FP64 except the forest/parallel sums, which run in the field
// precision (FP32 in the mixed modes); the densities are stored in it too.
#include <cstdio>
#include "mth_common.cuh"
#include "mth_internal.h"

namespace mth {

namespace {

constexpr double DD_TAU0 = 1000.0;       // tau_0 of StrainRate_Orowan
constexpr double DD_TRIAL_FREQ = 1.0e10; // TRIAL_FREQ_DRX
constexpr double DD_MY_J_IN_EV = 0.62415063631;
constexpr double DD_PI = 3.14159265359;
constexpr double DD_EPS = 5.0e-3;        // EPSILON seen by DislocationEvolution

template <int W>
__device__ __forceinline__ void dd_block_sum(double (&v)[W], double* out) {
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
    for (int w = 0; w < 8; w++) a += sm[threadIdx.x][w];
    out[(size_t)blockIdx.x * W + threadIdx.x] = a;
  }
}

// forest and parallel densities of every system of voxel v (from the
// densities at the start of the step), summed in the field precision T
// (the 12 x 12 sums are the bulk of the density kernels' arithmetic)
template <typename T>
__device__ __forceinline__ void forest_parallel(const DdConst& dc, const DdFields<T>& d, long long P, long long v,
                                                double* rf, double* rp) {
  T s[NSYS], a1[NSYS], a2[NSYS], a3[NSYS];
  for (int j = 0; j < NSYS; j++) {
    s[j] = d.rho_s[j * P + v];
    a1[j] = fabs(d.g1[j * P + v]);
    a2[j] = fabs(d.g2[j * P + v]);
    a3[j] = fabs(d.g3[j * P + v]);
  }
  for (int i = 0; i < dc.nsys; i++) {
    T f = 0, p = 0;
    for (int j = 0; j < dc.nsys; j++) {
      const T chi = cpick<T>(dc.chi[i][j], dc.chif[i][j]), cs = cpick<T>(dc.cs[i][j], dc.csf[i][j]);
      const T ss = cpick<T>(dc.ss[i][j], dc.ssf[i][j]);
      f += chi * (s[j] * cs + a1[j] * cpick<T>(dc.cg1[i][j], dc.cg1f[i][j]) + a2[j] * cs +
                  a3[j] * cpick<T>(dc.cg3[i][j], dc.cg3f[i][j]));
      p += chi * (s[j] * ss + a1[j] * cpick<T>(dc.sg1[i][j], dc.sg1f[i][j]) + a2[j] * ss +
                  a3[j] * cpick<T>(dc.sg3[i][j], dc.sg3f[i][j]));
    }
    rf[i] = (double)f;
    rp[i] = (double)p;
  }
}

__device__ __forceinline__ double mobile_density(const DdConst& dc, double rf, double rp) {
  const double b = dc.b;
  return 2.0 * dc.kT / dc.c[0] / dc.c[1] / dc.c[2] / dc.G / (b * b * b) * sqrt(rp * rf) * 160.2177;
}

// passing stress, tau_0 + cutting stress and reference rate per system
template <typename T>
__global__ void __launch_bounds__(256) dd_prep_kernel(const DdConst* __restrict__ dcp, DdFields<T> d, Fields<T> f) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long P = f.nv;
  if (v >= P) return;
  const DdConst& dc = *dcp;
  const bool crystal = f.phase[v] == 0;
  double rf[NSYS], rp[NSYS];
  if (crystal) forest_parallel(dc, d, P, v, rf, rp);
  const double b = dc.b, c1 = dc.c[0], c2 = dc.c[1], c3 = dc.c[2];
  for (int i = 0; i < NSYS; i++) {
    double tp = 0.0, td = 1.0, g0 = 0.0;
    if (crystal && i < dc.nsys) {
      const double rm = mobile_density(dc, rf[i], rp[i]);
      tp = c1 * dc.G * b * sqrt(fabs(rp[i] + rm)) * 1.0e-3;
      const double tcut = (dc.kT / DD_MY_J_IN_EV) * sqrt(rf[i]) / c2 / c3 / b / b * 0.1;
      td = DD_TAU0 + tcut;
      g0 = 1.0e-3 * rm * DD_TRIAL_FREQ * c2 * b * exp(-1.0 * dc.qslip) / sqrt(rf[i]);
    }
    f.ddc[i * P + v] = (T)tp;
    f.ddc[(NSYS + i) * P + v] = (T)td;
    f.ddc[(2 * NSYS + i) * P + v] = (T)g0;
  }
}

// shear rates at the converged stress (the last flow-rule evaluation of the
// step); 0 in gas voxels
template <typename T>
__global__ void __launch_bounds__(256) dd_gamdot_kernel(const DdConst* __restrict__ dcp, DdFields<T> d, Fields<T> f,
                                                        int flow_off) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long P = f.nv;
  if (v >= P) return;
  const DdConst& dc = *dcp;
  double x[5] = {0, 0, 0, 0, 0};
  const bool active = f.phase[v] == 0 && !flow_off;
  if (active) {
    double R[9], Q[25], s6[5];
    for (int i = 0; i < 9; i++) R[i] = (double)f.rot[i * P + v];
    for (int i = 0; i < 5; i++) s6[i] = (double)f.sig[i * P + v];
    rot_to_q<double>(R, Q);
    for (int i = 0; i < 5; i++) {
      double a = 0;
      for (int j = 0; j < 5; j++) a += Q[i * 5 + j] * s6[j];
      x[i] = a;
    }
  }
  for (int s = 0; s < NSYS; s++) {
    double g = 0.0;
    if (active && s < dc.nsys) {
      double rss = 0;
      for (int i = 0; i < 5; i++) rss += dc.m_xt[s][i] * x[i];
      const double tp = (double)f.ddc[s * P + v], td = (double)f.ddc[(NSYS + s) * P + v];
      const double g0 = (double)f.ddc[(2 * NSYS + s) * P + v];
      if (fabs(rss) > tp) g = g0 * sinh((fabs(rss) - tp) / td) * (rss > 0.0 ? 1.0 : -1.0);
    }
    d.gamdot[s * P + v] = (T)g;
  }
}

// DislocationEvolution + the per-block sums of AvgDislocation: rho_F,
// rho_P, rho_m (densities before the update, as the last flow evaluation
// saw them), rho_s, |rho_GND|, rho_dipole, rho_forest (after it).
template <typename T>
__global__ void __launch_bounds__(256) dd_evolve_kernel(const DdConst* __restrict__ dcp, DdFields<T> d, Fields<T> f,
                                                        int n0, int n1, int n2, double dt, int do_grad,
                                                        double* __restrict__ partials) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long P = f.nv;
  double acc[7] = {0, 0, 0, 0, 0, 0, 0};
  if (v < P && f.phase[v] == 0) {
    const DdConst& dc = *dcp;
    const int z = (int)(v % n2), y = (int)((v / n2) % n1), x = (int)(v / ((long long)n1 * n2));
    // neighbours +x, -x, +y, -y, +z, -z (periodic)
    long long nb[6];
    nb[0] = ((long long)((x + 1) % n0) * n1 + y) * n2 + z;
    nb[1] = ((long long)((x + n0 - 1) % n0) * n1 + y) * n2 + z;
    nb[2] = ((long long)x * n1 + (y + 1) % n1) * n2 + z;
    nb[3] = ((long long)x * n1 + (y + n1 - 1) % n1) * n2 + z;
    nb[4] = ((long long)x * n1 + y) * n2 + (z + 1) % n2;
    nb[5] = ((long long)x * n1 + y) * n2 + (z + n2 - 1) % n2;
    const unsigned gb = d.gb[v];
    double rf[NSYS], rp[NSYS];
    forest_parallel(dc, d, P, v, rf, rp);
    double R[9], Q[25], s6[6], xs[5];
    for (int i = 0; i < 9; i++) R[i] = (double)f.rot[i * P + v];
    for (int i = 0; i < 6; i++) s6[i] = (double)f.sig[i * P + v];
    rot_to_q<double>(R, Q);
    for (int i = 0; i < 5; i++) {
      double a = 0;
      for (int j = 0; j < 5; j++) a += Q[i * 5 + j] * s6[j];
      xs[i] = a;
    }
    const double hydro = (s6[0] + s6[1] + s6[2]) / 3.0;   // LT components 0..2, as DislocationEvolution
    const double b = dc.b, c4 = dc.c[3], c5 = dc.c[4], c6 = dc.c[5], c7 = dc.c[6];
    const double climb = exp((fabs(hydro) * b * b * b * 100 / (1.38 * dc.T)) - 1.0) * exp(-1.0 * dc.qbulk);
    for (int i = 0; i < dc.nsys; i++) {
      const double gd = (double)d.gamdot[i * P + v];
      double grad[3] = {0.0, 0.0, 0.0};
      if (do_grad) {
        for (int a = 0; a < 3; a++) {
          const int up = (gb >> (2 * a)) & 1, dn = (gb >> (2 * a + 1)) & 1;
          const double gp = (double)d.gamdot[i * P + nb[2 * a]], gm = (double)d.gamdot[i * P + nb[2 * a + 1]];
          if (!up && dn) grad[a] = gd - gm;
          else if (up && !dn) grad[a] = gp - gd;
          else if (up && dn) grad[a] = (gp - gm) / 2.0;
        }
      }
      double rss = 0;
      for (int k = 0; k < 5; k++) rss += dc.m_xt[i][k] * xs[k];
      const double rm = mobile_density(dc, rf[i], rp[i]);
      const double d_dipole = sqrt(3.0) * dc.G * b / 16.0 / DD_PI / (1 - dc.nu) / (fabs(rss) + DD_EPS);
      const double ag = fabs(gd);
      const double dip = (double)d.dipole[i * P + v] + ag * (c6 * d_dipole * rm) * dt;
      const double fst = (double)d.forest[i * P + v] + ag * (c4 * sqrt(rf[i])) * dt;
      const double rs = (double)d.rho_s[i * P + v];
      const double dot_ssd = ag * (c4 * sqrt(rf[i]) + c6 * d_dipole * rm - c5 * rs) - c7 * 1.6 * 1E12 * 1E-9 * rs * rs -
                             4 * 1E12 * d_dipole * (dc.d0 / b) * rs * rs * climb;
      const double rs_n = rs + dot_ssd * dt;
      const double g_screw = grad[0] * dc.bp[i][0] + grad[1] * dc.bp[i][1] + grad[2] * dc.bp[i][2];
      const double g_edge = grad[0] * dc.bb[i][0] + grad[1] * dc.bb[i][1] + grad[2] * dc.bb[i][2];
      const double g1 = (double)d.g1[i * P + v] + g_screw / b / dc.L0 * dt;
      const double g2 = (double)d.g2[i * P + v] + (-1.0 * g_edge) / b / dc.L0 * dt;
      const double g3 = (double)d.g3[i * P + v];
      d.dipole[i * P + v] = (T)dip;
      d.forest[i * P + v] = (T)fst;
      d.rho_s[i * P + v] = (T)rs_n;
      d.g1[i * P + v] = (T)g1;
      d.g2[i * P + v] = (T)g2;
      acc[0] += rf[i];
      acc[1] += rp[i];
      acc[2] += rs_n;
      acc[3] += rm;
      acc[4] += sqrt(g1 * g1 + g2 * g2 + g3 * g3);
      acc[5] += dip;
      acc[6] += fst;
    }
  }
  dd_block_sum<7>(acc, partials);
}

template <typename T>
__global__ void __launch_bounds__(256) dd_init_kernel(DdFields<T> d, const uint8_t* __restrict__ phase, long long P,
                                                      double rho0) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= P) return;
  for (int i = 0; i < NSYS; i++) {
    d.rho_s[i * P + v] = (T)rho0;   // every voxel, gas included, as src/init.c:1058-1060
    d.g1[i * P + v] = (T)0;
    d.g2[i * P + v] = (T)0;
    d.g3[i * P + v] = (T)0;
    d.dipole[i * P + v] = (T)0;
    d.forest[i * P + v] = (T)0;
    d.gamdot[i * P + v] = (T)0;
  }
}

int blocks_of(long long P) { return (int)((P + 255) / 256); }

}  // namespace

cudaError_t launch_dd_init(int mixed, const void* dd, const uint8_t* phase, long long P, double rho0, cudaStream_t st) {
  if (mixed) dd_init_kernel<float><<<blocks_of(P), 256, 0, st>>>(*static_cast<const DdFields<float>*>(dd), phase, P, rho0);
  else dd_init_kernel<double><<<blocks_of(P), 256, 0, st>>>(*static_cast<const DdFields<double>*>(dd), phase, P, rho0);
  return cudaGetLastError();
}

cudaError_t launch_dd_prep(int mixed, const DdConst* dc, const void* dd, const void* fields, cudaStream_t st) {
  if (mixed) {
    const Fields<float>& f = *static_cast<const Fields<float>*>(fields);
    dd_prep_kernel<float><<<blocks_of(f.nv), 256, 0, st>>>(dc, *static_cast<const DdFields<float>*>(dd), f);
  } else {
    const Fields<double>& f = *static_cast<const Fields<double>*>(fields);
    dd_prep_kernel<double><<<blocks_of(f.nv), 256, 0, st>>>(dc, *static_cast<const DdFields<double>*>(dd), f);
  }
  return cudaGetLastError();
}

cudaError_t launch_dd_gamdot(int mixed, const DdConst* dc, const void* dd, const void* fields, int flow_off,
                             cudaStream_t st) {
  if (mixed) {
    const Fields<float>& f = *static_cast<const Fields<float>*>(fields);
    dd_gamdot_kernel<float><<<blocks_of(f.nv), 256, 0, st>>>(dc, *static_cast<const DdFields<float>*>(dd), f, flow_off);
  } else {
    const Fields<double>& f = *static_cast<const Fields<double>*>(fields);
    dd_gamdot_kernel<double><<<blocks_of(f.nv), 256, 0, st>>>(dc, *static_cast<const DdFields<double>*>(dd), f,
                                                              flow_off);
  }
  return cudaGetLastError();
}

cudaError_t launch_dd_evolve(int mixed, const DdConst* dc, const void* dd, const void* fields, const int dims[3],
                             double dt, int do_grad, double* partials, cudaStream_t st) {
  if (mixed) {
    const Fields<float>& f = *static_cast<const Fields<float>*>(fields);
    dd_evolve_kernel<float><<<blocks_of(f.nv), 256, 0, st>>>(dc, *static_cast<const DdFields<float>*>(dd), f, dims[0],
                                                             dims[1], dims[2], dt, do_grad, partials);
  } else {
    const Fields<double>& f = *static_cast<const Fields<double>*>(fields);
    dd_evolve_kernel<double><<<blocks_of(f.nv), 256, 0, st>>>(dc, *static_cast<const DdFields<double>*>(dd), f,
                                                              dims[0], dims[1], dims[2], dt, do_grad, partials);
  }
  return cudaGetLastError();
}

}  // namespace mth

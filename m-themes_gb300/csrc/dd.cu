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
// Arithmetic in the field precision T (FP32 in the mixed modes, where the
// densities are stored in it too), with the material coefficients folded on
// the host in FP64 (DdCoef) and passed as kernel parameters; the per-block
// sums of the dd.out averages are FP64.  Loops over the slip systems are
// unrolled over the NSYS slots so the per-system values stay in registers.
#include <cstdio>
#include "mth_common.cuh"
#include "mth_internal.h"

namespace mth {

namespace {

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

// the densities of voxel v at the start of the step that the forest and
// parallel sums read: rho_s and |rho_GND| (3 kinds) of every system
template <typename T>
struct DdLocal {
  T s[NSYS], a1[NSYS], a2[NSYS], a3[NSYS];
};
template <typename T>
__device__ __forceinline__ void load_local(int nsys, const DdFields<T>& d, long long P, long long v, DdLocal<T>& l) {
#pragma unroll
  for (int j = 0; j < NSYS; j++) {
    if (j < nsys) {
      l.s[j] = d.rho_s[j * P + v];
      l.a1[j] = fabs(d.g1[j * P + v]);
      l.a2[j] = fabs(d.g2[j * P + v]);
      l.a3[j] = fabs(d.g3[j * P + v]);
    } else {
      l.s[j] = l.a1[j] = l.a2[j] = l.a3[j] = (T)0;
    }
  }
}
// forest (rf) and parallel (rp) density of system i
template <typename T>
__device__ __forceinline__ void forest_parallel(const DdCoef<T>& k, int i, const DdLocal<T>& l, T& rf, T& rp) {
  T f = 0, p = 0;
#pragma unroll
  for (int j = 0; j < NSYS; j++) {
    f += k.chi[i][j] * (l.s[j] * k.cs[i][j] + l.a1[j] * k.cg1[i][j] + l.a2[j] * k.cs[i][j] + l.a3[j] * k.cg3[i][j]);
    p += k.chi[i][j] * (l.s[j] * k.ss[i][j] + l.a1[j] * k.sg1[i][j] + l.a2[j] * k.ss[i][j] + l.a3[j] * k.sg3[i][j]);
  }
  rf = f;
  rp = p;
}

// deviatoric stress of voxel v in crystal axes
template <typename T>
__device__ __forceinline__ void crystal_stress(const Fields<T>& f, long long P, long long v, T (&x)[5]) {
  T R[9], Q[25], s6[5];
#pragma unroll
  for (int i = 0; i < 9; i++) R[i] = f.rot[i * P + v];
#pragma unroll
  for (int i = 0; i < 5; i++) s6[i] = f.sig[i * P + v];
  rot_to_q<T>(R, Q);
#pragma unroll
  for (int i = 0; i < 5; i++) {
    T a = 0;
#pragma unroll
    for (int j = 0; j < 5; j++) a += Q[i * 5 + j] * s6[j];
    x[i] = a;
  }
}

template <typename T>
__device__ __forceinline__ T resolved(const DdCoef<T>& k, int s, const T (&x)[5]) {
  return k.m[s][0] * x[0] + k.m[s][1] * x[1] + k.m[s][2] * x[2] + k.m[s][3] * x[3] + k.m[s][4] * x[4];
}

// passing stress, tau_0 + cutting stress and reference rate per system
template <typename T>
__global__ void __launch_bounds__(256) dd_prep_kernel(const DdCoef<T> k, int nsys, DdFields<T> d, Fields<T> f) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long P = f.nv;
  if (v >= P) return;
  const bool crystal = f.phase[v] == 0;
  DdLocal<T> l;
  if (crystal) load_local(nsys, d, P, v, l);
#pragma unroll
  for (int i = 0; i < NSYS; i++) {
    T tp = 0, td = 1, g0 = 0;
    if (crystal && i < nsys) {
      T rf, rp;
      forest_parallel(k, i, l, rf, rp);
      const T sf = sqrt(rf);
      const T rm = k.rm * sqrt(rp * rf);
      tp = k.tp * sqrt(fabs(rp + rm));
      td = (T)1000 + k.tcut * sf;   // tau_0 + cutting stress
      g0 = k.g0 * rm / sf;
    }
    f.ddc[i * P + v] = tp;
    f.ddc[(NSYS + i) * P + v] = td;
    f.ddc[(2 * NSYS + i) * P + v] = g0;
  }
}

// shear rates at the converged stress (the last flow-rule evaluation of the
// step); 0 in gas voxels
template <typename T>
__global__ void __launch_bounds__(256) dd_gamdot_kernel(const DdCoef<T> k, int nsys, DdFields<T> d, Fields<T> f,
                                                        int flow_off) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long P = f.nv;
  if (v >= P) return;
  T x[5] = {0, 0, 0, 0, 0};
  const bool active = f.phase[v] == 0 && !flow_off;
  if (active) crystal_stress(f, P, v, x);
#pragma unroll
  for (int s = 0; s < NSYS; s++) {
    T g = 0;
    if (active && s < nsys) {
      const T rss = resolved(k, s, x);
      const T tp = f.ddc[s * P + v], td = f.ddc[(NSYS + s) * P + v];
      const T g0 = f.ddc[(2 * NSYS + s) * P + v];
      if (fabs(rss) > tp) g = g0 * sinh((fabs(rss) - tp) / td) * (rss > (T)0 ? (T)1 : (T)-1);
    }
    d.gamdot[s * P + v] = g;
  }
}

// DislocationEvolution + the per-block sums of AvgDislocation: rho_F,
// rho_P, rho_m (densities before the update, as the last flow evaluation
// saw them), rho_s, |rho_GND|, rho_dipole, rho_forest (after it).  The
// per-voxel sums over the systems are in T, the block sums in FP64.
template <typename T>
__global__ void __launch_bounds__(256) dd_evolve_kernel(const DdCoef<T> k, int nsys, DdFields<T> d, Fields<T> f,
                                                        int n0, int n1, int n2, T dt, int do_grad,
                                                        double* __restrict__ partials) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long P = f.nv;
  double acc[7] = {0, 0, 0, 0, 0, 0, 0};
  if (v < P && f.phase[v] == 0) {
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
    DdLocal<T> l;
    load_local(nsys, d, P, v, l);
    T xs[5];
    crystal_stress(f, P, v, xs);
    // LT components 0..2, as DislocationEvolution
    const T hydro = (f.sig[v] + f.sig[P + v] + f.sig[2 * P + v]) / (T)3;
    const T climb = exp(fabs(hydro) * k.clb_h + k.clb_0);
    const T gdt = k.gnd * dt;
    T sum[7] = {0, 0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int i = 0; i < NSYS; i++) {
      if (i < nsys) {
        const T gd = d.gamdot[i * P + v];
        T grad[3] = {0, 0, 0};
        if (do_grad) {
#pragma unroll
          for (int a = 0; a < 3; a++) {
            const int up = (gb >> (2 * a)) & 1, dn = (gb >> (2 * a + 1)) & 1;
            const T gp = d.gamdot[i * P + nb[2 * a]], gm = d.gamdot[i * P + nb[2 * a + 1]];
            if (!up && dn) grad[a] = gd - gm;
            else if (up && !dn) grad[a] = gp - gd;
            else if (up && dn) grad[a] = (gp - gm) / (T)2;
          }
        }
        T rf, rp;
        forest_parallel(k, i, l, rf, rp);
        const T rss = resolved(k, i, xs);
        const T sf = sqrt(rf);
        const T rm = k.rm * sqrt(rp * rf);
        const T d_dipole = k.dip / (fabs(rss) + k.eps);
        const T ag = fabs(gd);
        const T dip = d.dipole[i * P + v] + ag * (k.c6 * d_dipole * rm) * dt;
        const T fst = d.forest[i * P + v] + ag * (k.c4 * sf) * dt;
        const T rs = l.s[i];
        const T dot_ssd = ag * (k.c4 * sf + k.c6 * d_dipole * rm - k.c5 * rs) - k.ann * rs * rs -
                          k.clb * d_dipole * rs * rs * climb;
        const T rs_n = rs + dot_ssd * dt;
        const T g_screw = grad[0] * k.bp[i][0] + grad[1] * k.bp[i][1] + grad[2] * k.bp[i][2];
        const T g_edge = grad[0] * k.bb[i][0] + grad[1] * k.bb[i][1] + grad[2] * k.bb[i][2];
        const T g1 = d.g1[i * P + v] + g_screw * gdt;
        const T g2 = d.g2[i * P + v] - g_edge * gdt;
        const T g3 = d.g3[i * P + v];
        d.dipole[i * P + v] = dip;
        d.forest[i * P + v] = fst;
        d.rho_s[i * P + v] = rs_n;
        d.g1[i * P + v] = g1;
        d.g2[i * P + v] = g2;
        sum[0] += rf;
        sum[1] += rp;
        sum[2] += rs_n;
        sum[3] += rm;
        sum[4] += sqrt(g1 * g1 + g2 * g2 + g3 * g3);
        sum[5] += dip;
        sum[6] += fst;
      }
    }
#pragma unroll
    for (int j = 0; j < 7; j++) acc[j] = (double)sum[j];
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

cudaError_t launch_dd_prep(int mixed, const DdConst& dc, const void* dd, const void* fields, cudaStream_t st) {
  if (mixed) {
    const Fields<float>& f = *static_cast<const Fields<float>*>(fields);
    dd_prep_kernel<float><<<blocks_of(f.nv), 256, 0, st>>>(dc.f, dc.nsys, *static_cast<const DdFields<float>*>(dd), f);
  } else {
    const Fields<double>& f = *static_cast<const Fields<double>*>(fields);
    dd_prep_kernel<double><<<blocks_of(f.nv), 256, 0, st>>>(dc.d, dc.nsys, *static_cast<const DdFields<double>*>(dd), f);
  }
  return cudaGetLastError();
}

cudaError_t launch_dd_gamdot(int mixed, const DdConst& dc, const void* dd, const void* fields, int flow_off,
                             cudaStream_t st) {
  if (mixed) {
    const Fields<float>& f = *static_cast<const Fields<float>*>(fields);
    dd_gamdot_kernel<float><<<blocks_of(f.nv), 256, 0, st>>>(dc.f, dc.nsys, *static_cast<const DdFields<float>*>(dd),
                                                             f, flow_off);
  } else {
    const Fields<double>& f = *static_cast<const Fields<double>*>(fields);
    dd_gamdot_kernel<double><<<blocks_of(f.nv), 256, 0, st>>>(dc.d, dc.nsys, *static_cast<const DdFields<double>*>(dd),
                                                              f, flow_off);
  }
  return cudaGetLastError();
}

cudaError_t launch_dd_evolve(int mixed, const DdConst& dc, const void* dd, const void* fields, const int dims[3],
                             double dt, int do_grad, double* partials, cudaStream_t st) {
  if (mixed) {
    const Fields<float>& f = *static_cast<const Fields<float>*>(fields);
    dd_evolve_kernel<float><<<blocks_of(f.nv), 256, 0, st>>>(dc.f, dc.nsys, *static_cast<const DdFields<float>*>(dd),
                                                             f, dims[0], dims[1], dims[2], (float)dt, do_grad,
                                                             partials);
  } else {
    const Fields<double>& f = *static_cast<const Fields<double>*>(fields);
    dd_evolve_kernel<double><<<blocks_of(f.nv), 256, 0, st>>>(dc.d, dc.nsys, *static_cast<const DdFields<double>*>(dd),
                                                              f, dims[0], dims[1], dims[2], dt, do_grad, partials);
  }
  return cudaGetLastError();
}

}  // namespace mth

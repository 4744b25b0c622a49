// drx.cu -- dynamic recrystallisation on the GPU: grain-boundary nucleation
// with a counter-based generator (NucleationCheckDRX, src/integrated.c:161-494)
// and the sparse order-parameter Allen-Cahn relaxation (PF_XRX / Update_grid /
// Update_gID, src/pf_xrx.c:6-66,895-1311,1469-1698) in the deterministic form
// documented in oracle/drx_oracle.c's restatement: at most PF_K order
// parameters per voxel, sorted by grain id; neighbourhood id set over the
// 3x3x3 block; stored-energy averages over the 7x7x7 window per grain id;
// explicit update with the 18-point Laplacian; argmax with ties to the
// smaller id.  One thread per voxel.  This translation unit is compiled
// without FMA contraction so that FP64 results are the separately rounded
// operations of the restatement, bit for bit.
#include <cstdint>
#include "mth_common.cuh"
#include "mth_internal.h"

namespace mth {

#define PF_EPS 5.0e-3
#define PF_KEEP 1.0e-4
constexpr int MAXIDS = 64;

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ULL;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
  return x ^ (x >> 31);
}
// uniform in (0, 1] from a (seed, counter) pair
__device__ __forceinline__ double uniform01(uint64_t seed, uint64_t counter) {
  uint64_t h = mix64(seed * 0xD1342543DE82EF95ULL + mix64(counter));
  return (double)((h >> 11) + 1) * (1.0 / 9007199254740992.0);
}

struct Dims {
  int n0, n1, n2;
  __device__ __forceinline__ long long idx(int x, int y, int z) const {
    x = (x % n0 + n0) % n0;
    y = (y % n1 + n1) % n1;
    z = (z % n2 + n2) % n2;
    return ((long long)x * n1 + y) * n2 + z;
  }
};

// -------------------------------------------------------------- nucleation
// Candidate: face neighbour in another grain (GB indicator,
// src/evolution.c:816-829), crystal phase, rho > rho_nuc, u(seed, counter) <
// prob.  Candidates are appended in arbitrary order; the host sorts them.
__global__ void nucleation_candidates_kernel(Dims d, const int* __restrict__ grain, const uint8_t* __restrict__ crystal,
                                             const double* __restrict__ rho, double rho_nuc, double prob,
                                             uint64_t seed, uint64_t counter0, long long* __restrict__ out,
                                             unsigned long long* __restrict__ count, long long cap) {
  const long long nv = (long long)d.n0 * d.n1 * d.n2;
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  if (!crystal[v]) return;
  const int x = (int)(v / ((long long)d.n1 * d.n2)), y = (int)((v / d.n2) % d.n1), z = (int)(v % d.n2);
  const int g = grain[v];
  const bool gb = (grain[d.idx(x + 1, y, z)] != g) | (grain[d.idx(x - 1, y, z)] != g) |
                  (grain[d.idx(x, y + 1, z)] != g) | (grain[d.idx(x, y - 1, z)] != g) |
                  (grain[d.idx(x, y, z + 1)] != g) | (grain[d.idx(x, y, z - 1)] != g);
  if (!gb || !(rho[v] > rho_nuc)) return;
  const double u = uniform01(seed, counter0 + (uint64_t)v);
  if (u < prob) {
    unsigned long long k = atomicAdd(count, 1ULL);
    if ((long long)k < cap) out[k] = v;
  }
}

// Disc painting: winner[v] = max nucleus index whose disc |d|^2 <= r^2
// (periodic) covers v; later nuclei win, as the sequential overwrite.
__global__ void paint_mark_kernel(Dims d, const long long* __restrict__ sites, int nn, int radius,
                                  int* __restrict__ winner) {
  const int side = 2 * radius + 1;
  const int per = side * side * side;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)nn * per) return;
  const int k = (int)(t / per);
  const int o = (int)(t % per);
  const int dx = o / (side * side) - radius, dy = (o / side) % side - radius, dz = o % side - radius;
  if (dx * dx + dy * dy + dz * dz > radius * radius) return;
  const long long v = sites[k];
  const int x = (int)(v / ((long long)d.n1 * d.n2)), y = (int)((v / d.n2) % d.n1), z = (int)(v % d.n2);
  atomicMax(&winner[d.idx(x + dx, y + dy, z + dz)], k);
}

__global__ void paint_apply_kernel(long long nv, int first_id, int* __restrict__ winner, int* __restrict__ grain) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  const int w = winner[v];
  if (w >= 0) {
    grain[v] = first_id + w;
    winner[v] = -1;
  }
}

// ------------------------------------------------------------ phase field
template <typename T>
__global__ void pf_init_kernel(long long nv, const int* __restrict__ grain, int* __restrict__ ids, T* __restrict__ phi,
                               uint8_t* __restrict__ cnt, int* __restrict__ gid) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  ids[v * PF_K] = grain[v];
  phi[v * PF_K] = (T)1;
  for (int s = 1; s < PF_K; s++) {
    ids[v * PF_K + s] = 0;
    phi[v * PF_K + s] = (T)0;
  }
  cnt[v] = 1;
  gid[v] = grain[v];
}

template <typename T>
__device__ __forceinline__ T eta_of(const int* ids, const T* phi, const uint8_t* cnt, long long w, int id) {
  const int c = cnt[w];
  for (int s = 0; s < c; s++)
    if (ids[w * PF_K + s] == id) return phi[w * PF_K + s];
  return (T)0;
}

__device__ __forceinline__ void sorted_insert(int* list, int& nl, int id) {
  int i = 0;
  while (i < nl && list[i] < id) i++;
  if (i < nl && list[i] == id) return;
  if (nl >= MAXIDS) return;
  for (int j = nl; j > i; j--) list[j] = list[j - 1];
  list[i] = id;
  nl++;
}

// Per voxel (x,y,z): for each grain id in the 7x7 patch of the x plane
// (y-3..y+3, z-3..z+3) the sum of rho in (y,z) order and the voxel count;
// up to PF_PATCH ids, else the patch is marked (n = 255) and the substep
// scans it directly.
template <typename T>
__global__ void __launch_bounds__(256) pf_patch_kernel(Dims d, const int* __restrict__ gid, const T* __restrict__ rho,
                                                       int* __restrict__ pl_id, T* __restrict__ pl_sum,
                                                       uint8_t* __restrict__ pl_cnt, uint8_t* __restrict__ pl_n) {
  const long long nv = (long long)d.n0 * d.n1 * d.n2;
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  const int x = (int)(v / ((long long)d.n1 * d.n2)), y = (int)((v / d.n2) % d.n1), z = (int)(v % d.n2);
  int id[PF_PATCH];
  T sm[PF_PATCH];
  int ct[PF_PATCH];
  int n = 0;
  bool over = false;
  for (int dy = -3; dy <= 3 && !over; dy++)
    for (int dz = -3; dz <= 3; dz++) {
      const long long w = d.idx(x, y + dy, z + dz);
      const int g = gid[w];
      int i = 0;
      while (i < n && id[i] != g) i++;
      if (i == n) {
        if (n == PF_PATCH) { over = true; break; }
        id[n] = g;
        sm[n] = (T)0;
        ct[n] = 0;
        n++;
      }
      sm[i] = sm[i] + rho[w];
      ct[i]++;
    }
  pl_n[v] = over ? (uint8_t)255 : (uint8_t)n;
  if (over) return;
  for (int i = 0; i < n; i++) {
    pl_id[(long long)i * nv + v] = id[i];
    pl_sum[(long long)i * nv + v] = sm[i];
    pl_cnt[(long long)i * nv + v] = (uint8_t)ct[i];
  }
}

template <typename T>
__global__ void __launch_bounds__(128) pf_substep_kernel(Dims d, const int* __restrict__ ids, const T* __restrict__ phi,
                                                         const uint8_t* __restrict__ cnt, int* __restrict__ ids2,
                                                         T* __restrict__ phi2, uint8_t* __restrict__ cnt2,
                                                         const int* __restrict__ gid, const T* __restrict__ rho,
                                                         T mcoef, T kappa, T mwell, T edisl,
                                                         const int* __restrict__ pl_id, const T* __restrict__ pl_sum,
                                                         const uint8_t* __restrict__ pl_cnt,
                                                         const uint8_t* __restrict__ pl_n) {
  const long long nv = (long long)d.n0 * d.n1 * d.n2;
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  const int x = (int)(v / ((long long)d.n1 * d.n2)), y = (int)((v / d.n2) % d.n1), z = (int)(v % d.n2);
  int nid[MAXIDS];
  int nn = 0;
  for (int dx = -1; dx <= 1; dx++)
    for (int dy = -1; dy <= 1; dy++)
      for (int dz = -1; dz <= 1; dz++) {
        const long long w = d.idx(x + dx, y + dy, z + dz);
        const int c = cnt[w];
        for (int s = 0; s < c; s++)
          if (phi[w * PF_K + s] > (T)PF_EPS) sorted_insert(nid, nn, ids[w * PF_K + s]);
      }
  const int cv = cnt[v];
  if (nn <= 1) {
    cnt2[v] = (uint8_t)cv;
    for (int s = 0; s < PF_K; s++) {
      ids2[v * PF_K + s] = s < cv ? ids[v * PF_K + s] : 0;
      phi2[v * PF_K + s] = s < cv ? phi[v * PF_K + s] : (T)0;
    }
    return;
  }
  int uid[MAXIDS];
  int nu = 0;
  for (int i = 0; i < nn; i++) sorted_insert(uid, nu, nid[i]);
  for (int s = 0; s < cv; s++) sorted_insert(uid, nu, ids[v * PF_K + s]);
  T wsum[MAXIDS];
  int wcnt[MAXIDS];
  for (int i = 0; i < nu; i++) {
    wsum[i] = (T)0;
    wcnt[i] = 0;
  }
  // window sums: the seven x planes' patch sums added in x order
  for (int dx = -3; dx <= 3; dx++) {
    const long long u = d.idx(x + dx, y, z);
    const int pn = pl_n[u];
    if (pn != 255) {
      for (int i = 0; i < nu; i++) {
        T ps = (T)0;
        int pc = 0;
        for (int j = 0; j < pn; j++)
          if (pl_id[(long long)j * nv + u] == uid[i]) {
            ps = pl_sum[(long long)j * nv + u];
            pc = pl_cnt[(long long)j * nv + u];
            break;
          }
        wsum[i] = wsum[i] + ps;
        wcnt[i] += pc;
      }
    } else {   // more ids in that patch than the list holds: scan it here
      for (int i = 0; i < nu; i++) {
        T ps = (T)0;
        int pc = 0;
        for (int dy = -3; dy <= 3; dy++)
          for (int dz = -3; dz <= 3; dz++) {
            const long long w = d.idx(x + dx, y + dy, z + dz);
            if (gid[w] == uid[i]) {
              ps = ps + rho[w];
              pc++;
            }
          }
        wsum[i] = wsum[i] + ps;
        wcnt[i] += pc;
      }
    }
  }
  T rbar[MAXIDS];
  for (int i = 0; i < nu; i++) rbar[i] = wcnt[i] > 0 ? wsum[i] / (T)wcnt[i] : (T)0;
  T sum_rex = 0, sum1 = 0, hdef = 0;
  for (int s = 0; s < cv; s++) {
    const int id = ids[v * PF_K + s];
    int i = 0;
    while (i < nu && uid[i] != id) i++;
    if (i < nu && wcnt[i] > 0 && rbar[i] > (T)0) {
      const T e = phi[v * PF_K + s];
      const T h = e * e * e * ((T)10.0 - (T)15.0 * e + (T)6.0 * e * e);
      sum_rex = sum_rex + e * e;
      sum1 = sum1 + h;
      hdef = hdef + h * rbar[i];
    }
  }
  int kid[PF_K + 1];
  T kval[PF_K + 1];
  int nk = 0;
  for (int a = 0; a < nn; a++) {
    const int id = nid[a];
    int i = 0;
    while (i < nu && uid[i] != id) i++;
    if (i == nu || !(rbar[i] > (T)0)) continue;
    const T c = eta_of<T>(ids, phi, cnt, v, id);
    const T f_r = eta_of<T>(ids, phi, cnt, d.idx(x + 1, y, z), id);
    const T f_l = eta_of<T>(ids, phi, cnt, d.idx(x - 1, y, z), id);
    const T f_f = eta_of<T>(ids, phi, cnt, d.idx(x, y + 1, z), id);
    const T f_b = eta_of<T>(ids, phi, cnt, d.idx(x, y - 1, z), id);
    const T f_u = eta_of<T>(ids, phi, cnt, d.idx(x, y, z + 1), id);
    const T f_d = eta_of<T>(ids, phi, cnt, d.idx(x, y, z - 1), id);
    const T e_lu = eta_of<T>(ids, phi, cnt, d.idx(x - 1, y, z + 1), id);
    const T e_lf = eta_of<T>(ids, phi, cnt, d.idx(x - 1, y - 1, z), id);
    const T e_ld = eta_of<T>(ids, phi, cnt, d.idx(x - 1, y, z - 1), id);
    const T e_lb = eta_of<T>(ids, phi, cnt, d.idx(x - 1, y + 1, z), id);
    const T e_rd = eta_of<T>(ids, phi, cnt, d.idx(x + 1, y, z - 1), id);
    const T e_ru = eta_of<T>(ids, phi, cnt, d.idx(x + 1, y, z + 1), id);
    const T e_rf = eta_of<T>(ids, phi, cnt, d.idx(x + 1, y - 1, z), id);
    const T e_rb = eta_of<T>(ids, phi, cnt, d.idx(x + 1, y + 1, z), id);
    const T e_cuf = eta_of<T>(ids, phi, cnt, d.idx(x, y - 1, z + 1), id);
    const T e_cdb = eta_of<T>(ids, phi, cnt, d.idx(x, y + 1, z - 1), id);
    const T e_cub = eta_of<T>(ids, phi, cnt, d.idx(x, y + 1, z + 1), id);
    const T e_cdf = eta_of<T>(ids, phi, cnt, d.idx(x, y - 1, z - 1), id);
    const T lap = (T)0.5 * (f_r + f_l + f_f + f_b + f_u + f_d) +
                  (T)0.125 * (e_lu + e_lf + e_ld + e_lb + e_rd + e_ru + e_rf + e_rb + e_cuf + e_cdb + e_cub + e_cdf) -
                  (T)4.5 * c;
    const T h = c * c * c * ((T)10.0 - (T)15.0 * c + (T)6.0 * c * c);
    const T dh = c * c * ((T)30.0 - (T)60.0 * c + (T)30.0 * c * c);
    const T drive = sum1 > (T)0 ? edisl * dh * ((sum1 - h) * rbar[i] - (hdef - h * rbar[i])) / (sum1 * sum1) : (T)0;
    const T val = c - mcoef * (mwell * (c * c * c - c + (T)3.0 * c * (sum_rex - c * c)) - kappa * lap + drive);
    if (val > (T)PF_KEEP) {
      kid[nk] = id;
      kval[nk] = val;
      nk++;
      if (nk > PF_K) {   // drop the smallest (ties: the larger id), keep id order
        int m = 0;
        for (int b = 1; b < nk; b++)
          if (kval[b] < kval[m] || (kval[b] == kval[m] && kid[b] > kid[m])) m = b;
        for (int b = m; b < nk - 1; b++) {
          kid[b] = kid[b + 1];
          kval[b] = kval[b + 1];
        }
        nk--;
      }
    }
  }
  cnt2[v] = (uint8_t)nk;
  for (int s = 0; s < PF_K; s++) {
    ids2[v * PF_K + s] = s < nk ? kid[s] : 0;
    phi2[v * PF_K + s] = s < nk ? kval[s] : (T)0;
  }
}

template <typename T>
__global__ void pf_argmax_kernel(long long nv, const int* __restrict__ ids, const T* __restrict__ phi,
                                 const uint8_t* __restrict__ cnt, int* __restrict__ gid) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  T best = (T)0;
  int g = gid[v];
  const int c = cnt[v];
  for (int s = 0; s < c; s++)
    if (phi[v * PF_K + s] > best) {
      best = phi[v * PF_K + s];
      g = ids[v * PF_K + s];
    }
  gid[v] = g;
}

// ------------------------------------------------------------- launchers
static inline int nb(long long n, int t) { return (int)((n + t - 1) / t); }

cudaError_t launch_nucleation_candidates(const int dims[3], const int* grain, const uint8_t* crystal, const double* rho,
                                         double rho_nuc, double prob, uint64_t seed, uint64_t counter0,
                                         long long* out, unsigned long long* count, long long cap, cudaStream_t st) {
  Dims d{dims[0], dims[1], dims[2]};
  const long long nv = (long long)dims[0] * dims[1] * dims[2];
  nucleation_candidates_kernel<<<nb(nv, 256), 256, 0, st>>>(d, grain, crystal, rho, rho_nuc, prob, seed, counter0,
                                                            out, count, cap);
  return cudaGetLastError();
}

cudaError_t launch_paint_nuclei(const int dims[3], const long long* sites, int nn, int radius, int first_id,
                                int* winner, int* grain, cudaStream_t st) {
  Dims d{dims[0], dims[1], dims[2]};
  const long long nv = (long long)dims[0] * dims[1] * dims[2];
  const int side = 2 * radius + 1;
  const long long work = (long long)nn * side * side * side;
  if (work > 0) paint_mark_kernel<<<nb(work, 256), 256, 0, st>>>(d, sites, nn, radius, winner);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  paint_apply_kernel<<<nb(nv, 256), 256, 0, st>>>(nv, first_id, winner, grain);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_pf_relax(const int dims[3], const int* grain, const T* rho, int substeps, const PfCoef& co,
                            PfBuffers<T>& b, cudaStream_t st) {
  Dims d{dims[0], dims[1], dims[2]};
  const long long nv = (long long)dims[0] * dims[1] * dims[2];
  pf_init_kernel<T><<<nb(nv, 256), 256, 0, st>>>(nv, grain, b.ids[0], b.phi[0], b.cnt[0], b.gid);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  int cur = 0;
  for (int s = 0; s < substeps; s++) {
    pf_patch_kernel<T><<<nb(nv, 256), 256, 0, st>>>(d, b.gid, rho, b.pl_id, b.pl_sum, b.pl_cnt, b.pl_n);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    pf_substep_kernel<T><<<nb(nv, 128), 128, 0, st>>>(d, b.ids[cur], b.phi[cur], b.cnt[cur], b.ids[1 - cur],
                                                      b.phi[1 - cur], b.cnt[1 - cur], b.gid, rho, (T)co.mcoef,
                                                      (T)co.kappa, (T)co.mwell, (T)co.edisl, b.pl_id, b.pl_sum,
                                                      b.pl_cnt, b.pl_n);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    cur = 1 - cur;
    pf_argmax_kernel<T><<<nb(nv, 256), 256, 0, st>>>(nv, b.ids[cur], b.phi[cur], b.cnt[cur], b.gid);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  b.cur = cur;
  return cudaSuccess;
}

template cudaError_t launch_pf_relax<float>(const int*, const int*, const float*, int, const PfCoef&, PfBuffers<float>&,
                                            cudaStream_t);
template cudaError_t launch_pf_relax<double>(const int*, const int*, const double*, int, const PfCoef&,
                                             PfBuffers<double>&, cudaStream_t);

}  // namespace mth

namespace mth {

// ------------------------------------------- microstructure update kernels
// rho = rho0 + rho_k * accumulated slip (crystal voxels; 0 in gas, which has
// no slip systems, as rho_tot in src/evolution.c:976-994)
template <typename TSt>
__global__ void drx_rho_kernel(Fields<TSt> f, double rho0, double rho_k, double* __restrict__ rho_d,
                               TSt* __restrict__ rho_t) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= f.nv) return;
  const double r = f.phase[v] == 0 ? rho0 + rho_k * (double)f.gamacum[v] : 0.0;
  rho_d[v] = r;
  rho_t[v] = (TSt)r;
}

// Voxels whose relaxed grain id differs from the id before this step's
// nucleation and belongs to a recrystallised grain become part of it: the
// treatment of growth==1 voxels after PF_XRX (src/evolution.c:1120-1200):
// stress zeroed, dislocation content reset (accumulated slip and CRSS back
// to the initial state), orientation and stiffness of the new grain.  Other
// id changes only relabel the voxel (src/integrated.c:1613-1615).
template <typename TSt>
__global__ void drx_update_kernel(Fields<TSt> f, int* __restrict__ grain, const int* __restrict__ grain_prev,
                                  const int* __restrict__ gid_new, int first_drx_id, int n_drx,
                                  const double* __restrict__ drx_rot, const int* __restrict__ drx_class, double tau0f,
                                  int nsys) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long P = f.nv;
  if (v >= P) return;
  const int gn = gid_new[v];
  grain[v] = gn;
  if (gn == grain_prev[v] || f.phase[v] != 0) return;
  const int k = gn - first_drx_id;
  if (k < 0 || k >= n_drx) return;
  for (int i = 0; i < 6; i++) f.sig[i * P + v] = (TSt)0;
  f.gamacum[v] = (TSt)0;
  for (int s = 0; s < NSYS; s++) f.crss[s * P + v] = (TSt)(s < nsys ? tau0f : 0.0);
  for (int i = 0; i < 9; i++) f.rot[i * P + v] = (TSt)drx_rot[9 * k + i];
  const_cast<int*>(f.eclass)[v] = drx_class[k];
}

__global__ void class_histogram_kernel(long long nv, const uint8_t* __restrict__ crystal, const int* __restrict__ eclass,
                                       unsigned long long* __restrict__ hist) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv || !crystal[v]) return;
  atomicAdd(&hist[eclass[v]], 1ULL);
}

cudaError_t launch_drx_rho(int mixed, const void* fields, double rho0, double rho_k, double* rho_d, void* rho_t,
                           cudaStream_t st) {
  if (mixed) {
    const Fields<float>& f = *static_cast<const Fields<float>*>(fields);
    drx_rho_kernel<float><<<nb(f.nv, 256), 256, 0, st>>>(f, rho0, rho_k, rho_d, static_cast<float*>(rho_t));
  } else {
    const Fields<double>& f = *static_cast<const Fields<double>*>(fields);
    drx_rho_kernel<double><<<nb(f.nv, 256), 256, 0, st>>>(f, rho0, rho_k, rho_d, static_cast<double*>(rho_t));
  }
  return cudaGetLastError();
}

cudaError_t launch_drx_update(int mixed, const void* fields, int* grain, const int* grain_prev, const int* gid_new,
                              int first_drx_id, int n_drx, const double* drx_rot, const int* drx_class, double tau0f,
                              int nsys, cudaStream_t st) {
  if (mixed) {
    const Fields<float>& f = *static_cast<const Fields<float>*>(fields);
    drx_update_kernel<float><<<nb(f.nv, 256), 256, 0, st>>>(f, grain, grain_prev, gid_new, first_drx_id, n_drx, drx_rot,
                                                            drx_class, tau0f, nsys);
  } else {
    const Fields<double>& f = *static_cast<const Fields<double>*>(fields);
    drx_update_kernel<double><<<nb(f.nv, 256), 256, 0, st>>>(f, grain, grain_prev, gid_new, first_drx_id, n_drx,
                                                             drx_rot, drx_class, tau0f, nsys);
  }
  return cudaGetLastError();
}

cudaError_t launch_class_histogram(long long nv, const uint8_t* crystal, const int* eclass, unsigned long long* hist,
                                   cudaStream_t st) {
  class_histogram_kernel<<<nb(nv, 256), 256, 0, st>>>(nv, crystal, eclass, hist);
  return cudaGetLastError();
}

// ------------------------------------------ PF <-> mechanical grid transfer
// InterpolateGrid / InterpolateGID (src/integrated.c:496-760) and the
// coarse-graining of gID_new (src/integrated.c:821-860): node coordinates
// x = i/(N-1) on [0,1], source cell floor(x/dx), dx = 1/(Ns-1), upper corner
// clamped to the last node (the reference aborts when rounding puts a node
// past the last source node; here the last cell is used).  Same operations
// in the same order as the oracle (this file is compiled without FMA
// contraction), so FP64 results are bit-identical.
__device__ __forceinline__ void axis_pos(int i, int nd, int ns, int& i0, int& i1, double& s) {
  if (nd < 2 || ns < 2) { i0 = 0; i1 = 0; s = 0.0; return; }
  const double dxd = 1.0 / (nd - 1), dxs = 1.0 / (ns - 1);
  const double x = 0.0 + (double)i * dxd;
  int ix = (int)floor(x / dxs);
  if (ix > ns - 1) ix = ns - 1;
  if (ix < 0) ix = 0;
  s = x / dxs - (double)ix;
  i0 = ix;
  i1 = ix + 1 < ns ? ix + 1 : ns - 1;
}

// integer field: value at the nearest of the eight corners, first minimum in
// the order 000,100,110,010,001,101,111,011 (TrilinearInterpolationINT)
__global__ void resample_nearest_kernel(Dims ds, const int* __restrict__ src, Dims dd, int* __restrict__ dst) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nv = (long long)dd.n0 * dd.n1 * dd.n2;
  if (v >= nv) return;
  const int k = (int)(v % dd.n2), j = (int)((v / dd.n2) % dd.n1), i = (int)(v / ((long long)dd.n1 * dd.n2));
  int x0, x1, y0, y1, z0, z1;
  double sx, sy, sz;
  axis_pos(i, dd.n0, ds.n0, x0, x1, sx);
  axis_pos(j, dd.n1, ds.n1, y0, y1, sy);
  axis_pos(k, dd.n2, ds.n2, z0, z1, sz);
  double dist[8];
  dist[0] = sx * sx + sy * sy + sz * sz;
  dist[1] = (1 - sx) * (1 - sx) + sy * sy + sz * sz;
  dist[2] = (1 - sx) * (1 - sx) + (1 - sy) * (1 - sy) + sz * sz;
  dist[3] = sx * sx + (1 - sy) * (1 - sy) + sz * sz;
  dist[4] = sx * sx + sy * sy + (1 - sz) * (1 - sz);
  dist[5] = (1 - sx) * (1 - sx) + sy * sy + (1 - sz) * (1 - sz);
  dist[6] = (1 - sx) * (1 - sx) + (1 - sy) * (1 - sy) + (1 - sz) * (1 - sz);
  dist[7] = sx * sx + (1 - sy) * (1 - sy) + (1 - sz) * (1 - sz);
  const int cx[8] = {x0, x1, x1, x0, x0, x1, x1, x0};
  const int cy[8] = {y0, y0, y1, y1, y0, y0, y1, y1};
  const int cz[8] = {z0, z0, z0, z0, z1, z1, z1, z1};
  int m = 0;
#pragma unroll
  for (int c = 1; c < 8; c++)
    if (dist[m] > dist[c]) m = c;
  dst[v] = src[((long long)cx[m] * ds.n1 + cy[m]) * ds.n2 + cz[m]];
}

// double field: trilinear interpolation, terms in the reference's order
// (TrilinearInterpolation); stored as TO
template <typename TO>
__global__ void resample_trilinear_kernel(Dims ds, const double* __restrict__ src, Dims dd, TO* __restrict__ dst) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nv = (long long)dd.n0 * dd.n1 * dd.n2;
  if (v >= nv) return;
  const int k = (int)(v % dd.n2), j = (int)((v / dd.n2) % dd.n1), i = (int)(v / ((long long)dd.n1 * dd.n2));
  int x0, x1, y0, y1, z0, z1;
  double sx, sy, sz;
  axis_pos(i, dd.n0, ds.n0, x0, x1, sx);
  axis_pos(j, dd.n1, ds.n1, y0, y1, sy);
  axis_pos(k, dd.n2, ds.n2, z0, z1, sz);
  auto V = [&](int a, int b, int c) { return src[((long long)a * ds.n1 + b) * ds.n2 + c]; };
  const double r = V(x0, y0, z0) * (1.0 - sx) * (1.0 - sy) * (1.0 - sz) + V(x1, y0, z0) * sx * (1.0 - sy) * (1.0 - sz) +
                   V(x0, y1, z0) * sy * (1.0 - sx) * (1.0 - sz) + V(x0, y0, z1) * sz * (1.0 - sy) * (1.0 - sx) +
                   V(x1, y0, z1) * sx * (1.0 - sy) * sz + V(x0, y1, z1) * sy * (1.0 - sx) * sz +
                   V(x1, y1, z0) * sx * (1.0 - sz) * sy + V(x1, y1, z1) * sx * sy * sz;
  dst[v] = (TO)r;
}

cudaError_t launch_resample_nearest(const int ns[3], const int* src, const int nd[3], int* dst, cudaStream_t st) {
  const long long nv = (long long)nd[0] * nd[1] * nd[2];
  resample_nearest_kernel<<<nb(nv, 256), 256, 0, st>>>(Dims{ns[0], ns[1], ns[2]}, src, Dims{nd[0], nd[1], nd[2]}, dst);
  return cudaGetLastError();
}

cudaError_t launch_resample_trilinear(const int ns[3], const double* src, const int nd[3], void* dst, int to_float,
                                      cudaStream_t st) {
  const long long nv = (long long)nd[0] * nd[1] * nd[2];
  if (to_float)
    resample_trilinear_kernel<float><<<nb(nv, 256), 256, 0, st>>>(Dims{ns[0], ns[1], ns[2]}, src,
                                                                  Dims{nd[0], nd[1], nd[2]}, static_cast<float*>(dst));
  else
    resample_trilinear_kernel<double><<<nb(nv, 256), 256, 0, st>>>(Dims{ns[0], ns[1], ns[2]}, src,
                                                                   Dims{nd[0], nd[1], nd[2]}, static_cast<double*>(dst));
  return cudaGetLastError();
}

// rotation matrices (9 components, component-major fields) of the parent
// voxels of the nn nuclei, as double, nucleus-major: out[k*9 + i]
template <typename TSt>
__global__ void gather_rot_kernel(const TSt* __restrict__ rot, long long nv, const long long* __restrict__ sites, int nn,
                                  double* __restrict__ out) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 9LL * nn) return;
  const long long k = t / 9;
  const int i = (int)(t - 9 * k);
  out[t] = (double)rot[(size_t)i * nv + sites[k]];
}

cudaError_t launch_gather_rot(int mixed, const void* rot, long long nv, const long long* sites, int nn, double* out,
                              cudaStream_t st) {
  if (nn <= 0) return cudaSuccess;
  if (mixed)
    gather_rot_kernel<float><<<nb(9LL * nn, 256), 256, 0, st>>>(static_cast<const float*>(rot), nv, sites, nn, out);
  else
    gather_rot_kernel<double><<<nb(9LL * nn, 256), 256, 0, st>>>(static_cast<const double*>(rot), nv, sites, nn, out);
  return cudaGetLastError();
}

}  // namespace mth

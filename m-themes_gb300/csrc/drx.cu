// drx.cu -- dynamic recrystallisation on the GPU: grain-boundary nucleation
// with a counter-based generator (NucleationCheckDRX, src/integrated.c:161-494)
// and the sparse order-parameter Allen-Cahn relaxation (PF_XRX / Update_grid /
// Update_gID, src/pf_xrx.c:6-66,895-1311,1469-1698), the reference's
// sequential sweep computed in parallel passes (section "phase field").
// This translation unit is compiled without FMA contraction so that FP64
// results are the separately rounded operations of the reference, bit for
// bit.
#include <cstdint>
#include "mth_common.cuh"
#include "mth_internal.h"

namespace mth {

#define PF_EPS 5.0e-3
#define PF_KEEP 1.0e-4

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

// The periodic 3x3x3 neighbourhood of voxel (x, y, z) without divisions:
// the wrapped coordinates of the three planes, rows and columns once, a
// neighbour's index by multiply-adds.
struct Nbhd {
  long long px[3];   // plane offsets of x-1, x, x+1 (times n1 n2)
  int py[3], pz[3];  // row offsets of y-1, y, y+1 (times n2); columns z-1, z, z+1
  __device__ __forceinline__ Nbhd(const Dims& d, int x, int y, int z) {
    const int xm = x == 0 ? d.n0 - 1 : x - 1, xp = x == d.n0 - 1 ? 0 : x + 1;
    const int ym = y == 0 ? d.n1 - 1 : y - 1, yp = y == d.n1 - 1 ? 0 : y + 1;
    const long long pl = (long long)d.n1 * d.n2;
    px[0] = xm * pl; px[1] = x * pl; px[2] = xp * pl;
    py[0] = ym * d.n2; py[1] = y * d.n2; py[2] = yp * d.n2;
    pz[0] = z == 0 ? d.n2 - 1 : z - 1; pz[1] = z; pz[2] = z == d.n2 - 1 ? 0 : z + 1;
  }
  // neighbour at offset (a, b, c), each in -1..1
  __device__ __forceinline__ long long at(int a, int b, int c) const { return px[a + 1] + py[b + 1] + pz[c + 1]; }
};

// -------------------------------------------------------------- nucleation
// Candidate: grain-boundary voxel as the reference marks it
// (src/evolution.c:816-829 from Gradient_ExchangeGrainID,
// src/constitutive.c:724-873: the +x, -x, +y, -y or +z neighbour in another
// grain -- its "-z" check compares with the -y neighbour), crystal phase,
// rho > rho_nuc, u(seed, counter) < prob.  Candidates are appended in
// arbitrary order; the host sorts them.
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
                  (grain[d.idx(x, y, z + 1)] != g);
  if (!gb || !(rho[v] > rho_nuc)) return;
  const double u = uniform01(seed, counter0 + (uint64_t)v);
  if (u < prob) {
    unsigned long long k = atomicAdd(count, 1ULL);
    if ((long long)k < cap) out[k] = v;
  }
}

// Disc painting (src/integrated.c:397-402): winner[v] = max nucleus index
// whose squared distance to v is <= radius2 (the reference's nucleus_radius,
// compared with |d|^2), without periodic images; later nuclei win, as the
// sequential overwrite.
__global__ void paint_mark_kernel(Dims d, const long long* __restrict__ sites, int nn, int r, int radius2,
                                  int* __restrict__ winner) {
  const int side = 2 * r + 1;
  const int per = side * side * side;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)nn * per) return;
  const int k = (int)(t / per);
  const int o = (int)(t % per);
  const int dx = o / (side * side) - r, dy = (o / side) % side - r, dz = o % side - r;
  if (dx * dx + dy * dy + dz * dz > radius2) return;
  const long long v = sites[k];
  const int x = (int)(v / ((long long)d.n1 * d.n2)) + dx, y = (int)((v / d.n2) % d.n1) + dy, z = (int)(v % d.n2) + dz;
  if (x < 0 || x >= d.n0 || y < 0 || y >= d.n1 || z < 0 || z >= d.n2) return;
  atomicMax(&winner[((long long)x * d.n1 + y) * d.n2 + z], k);
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
// PF_XRX / Update_grid / Update_gID (src/pf_xrx.c:6-66,895-1311,1469-1698)
// as the reference's sequential sweep computes it, in parallel passes.
//
// The reference sweeps x, y, z over the voxels and, while it does, changes
// the grid it reads: looking up an id a voxel does not hold takes over that
// voxel's last entry when the entry is below EPSILON (relabelling it) or
// appends (id, 0) (PFdata::operator[], src/PFgrid.h:70-90); it writes a
// global rho_avg table that later voxels read for ids they do not hold; and
// it resets the stored energy of a voxel a recrystallised id crosses
// (src/pf_xrx.c:1217-1219), which later voxels' window averages see.  Every
// one of these effects reaches a voxel only from voxels earlier in the sweep,
// and reads return the same value whatever the relabelling (a missing id
// reads the weak last entry's value, or 0), so each voxel's outcome is a
// function of the previous substep and of decisions of earlier voxels.  The
// passes compute those decisions to their fixed point (iterating until no
// voxel's decision changes, which happens after at most the length of the
// longest chain of dependent voxels, in practice two to four iterations):
//   nlist   N(v): ids with eta > EPSILON over the 3x3x3 block, scan order;
//   upd     whether the voxel holds more than one entry when the sweep
//           reaches it: it does if it held several, or if it held one strong
//           entry and one of its nine preceding stencil neighbours that
//           updates has an id it lacks in N (that neighbour's Laplacian
//           lookup appends it) -- fixed point;
//   tail    the id its last entry carries by then: the last such lookup, from
//           the latest preceding updating neighbour;
//   window  per held entry, the mean stored energy over the 7x7x7 window of
//           voxels whose initial grain id matches, with the resets of
//           earlier voxels in this substep;
//   rows    per row of voxels, the last value each id wrote to the table;
//   update  the new lists, with rho_avg of ids not held read from the latest
//           earlier writer (same row, then earlier rows, then the table) and
//           the energy resets this substep causes -- window/rows/update are
//           iterated to the fixed point of the resets;
//   table   each id's last writer's value into the table; finish: resets
//           applied, grain id = first maximum.
// Summation orders and the Laplacian's term order are the reference's, and
// this file is compiled without FMA contraction, so FP64 results equal the
// reference's sweep bit for bit (the oracle restates that sweep literally).

struct PfView {
  Dims d;
  long long nv;
  int rows;
};

// PFdata lookup by value: the entry's eta, else the weak last entry's, else 0
template <typename T>
__device__ __forceinline__ T pf_read_local(const int* id, const T* ph, int n, int j) {
  for (int k = 0; k < n; k++)
    if (id[k] == j) return ph[k];
  if (n > 0 && ph[n - 1] < (T)PF_EPS) return ph[n - 1];
  return (T)0;
}
template <typename T>
__device__ __forceinline__ T pf_read_g(const int* __restrict__ ids, const T* __restrict__ phi,
                                       const uint8_t* __restrict__ cnt, long long nv, long long w, int j) {
  const int n = cnt[w];
  for (int k = 0; k < n; k++)
    if (ids[(long long)k * nv + w] == j) return phi[(long long)k * nv + w];
  if (n > 0) {
    const T t = phi[(long long)(n - 1) * nv + w];
    if (t < (T)PF_EPS) return t;
  }
  return (T)0;
}
// PFdata lookup for assignment into a list under construction
template <typename T>
__device__ __forceinline__ void pf_write_local(int* id, T* ph, int& n, int j, T val, unsigned* bad) {
  for (int k = 0; k < n; k++)
    if (id[k] == j) { ph[k] = val; return; }
  if (n > 0 && ph[n - 1] < (T)PF_EPS) { id[n - 1] = j; ph[n - 1] = val; return; }
  if (n == PF_K) { *bad |= PF_BAD_LIST; return; }
  id[n] = j;
  ph[n] = val;
  n++;
}
// the list a voxel holds when the sweep reaches it: its stored list with the
// last entry relabelled or (tail, 0) appended
template <typename T>
__device__ __forceinline__ int pf_held(const PfView& g, const int* __restrict__ ids, const T* __restrict__ phi,
                                       const uint8_t* __restrict__ cnt, const int* __restrict__ tail,
                                       const uint8_t* __restrict__ tmode, long long v, int* hid, T* hph) {
  int n = cnt[v];
  for (int k = 0; k < n; k++) {
    hid[k] = ids[(long long)k * g.nv + v];
    hph[k] = phi[(long long)k * g.nv + v];
  }
  const int m = tmode[v];
  if (m == 1) hid[n - 1] = tail[v];
  else if (m == 2) { hid[n] = tail[v]; hph[n] = (T)0; n++; }
  return n;
}
// the nine stencil neighbours that precede v in the sweep, latest first
__constant__ int8_t c_pred[9][3] = {{0, 0, -1}, {0, -1, 1}, {0, -1, 0}, {0, -1, -1}, {-1, 1, 0},
                                    {-1, 0, 1}, {-1, 0, 0}, {-1, 0, -1}, {-1, -1, 0}};

template <typename T>
__global__ void pf_init_kernel(PfView g, const int* __restrict__ grain, const T* __restrict__ rho, int* __restrict__ ids,
                               T* __restrict__ phi, uint8_t* __restrict__ cnt, T* __restrict__ energy,
                               int* __restrict__ gid) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= g.nv) return;
  ids[v] = grain[v];
  phi[v] = (T)1;
  cnt[v] = 1;
  energy[v] = rho[v];
  gid[v] = grain[v];
}

template <typename T>
__global__ void __launch_bounds__(256) pf_nlist_kernel(PfView g, const int* __restrict__ ids, const T* __restrict__ phi,
                                                       const uint8_t* __restrict__ cnt, int* __restrict__ nid,
                                                       uint8_t* __restrict__ ncnt, unsigned* __restrict__ word) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= g.nv) return;
  const int x = (int)(v / ((long long)g.d.n1 * g.d.n2)), y = (int)((v / g.d.n2) % g.d.n1), z = (int)(v % g.d.n2);
  int L[PF_NM];
  int n = 0;
  unsigned bad = 0;
  const Nbhd nb(g.d, x, y, z);
  for (int dx = -1; dx <= 1; dx++)
    for (int dy = -1; dy <= 1; dy++)
      for (int dz = -1; dz <= 1; dz++) {
        const long long w = nb.at(dx, dy, dz);
        const int c = cnt[w];
        for (int k = 0; k < c; k++) {
          if (!(phi[(long long)k * g.nv + w] > (T)PF_EPS)) continue;
          const int j = ids[(long long)k * g.nv + w];
          bool seen = false;
          for (int a = 0; a < n; a++) seen |= (L[a] == j);
          if (seen) continue;
          if (n == PF_NM) { bad |= PF_BAD_NEIGH; continue; }
          L[n++] = j;
        }
      }
  ncnt[v] = (uint8_t)n;
  for (int a = 0; a < n; a++) nid[(long long)a * g.nv + v] = L[a];
  if (bad) atomicOr(&word[1], bad);
}

// One pass of the update flags' fixed point, in place.  The flags only turn
// on as the passes proceed (a flag is an OR over earlier voxels' flags), so
// reading some neighbours' flags of this pass and some of the last one still
// ends at the same fixed point, and a pass that changes nothing is at it.
// Within a warp (consecutive z of one row) the chain through the (0,0,-1)
// neighbour is resolved in the pass itself: u(z) = G(z) | (P(z) & u(z-1)),
// G the voxel's own and its other eight neighbours' part, P whether the
// z-1 neighbour's flag would carry over, solved for the warp's 32 lanes by
// a prefix over ballot masks.
template <typename T>
__global__ void __launch_bounds__(256) pf_upd_kernel(PfView g, const int* __restrict__ ids, const T* __restrict__ phi,
                                                     const uint8_t* __restrict__ cnt, const int* __restrict__ nid,
                                                     const uint8_t* __restrict__ ncnt, uint8_t* __restrict__ upd,
                                                     unsigned* __restrict__ word) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool in = v < g.nv;
  const int lane = threadIdx.x & 31;
  bool gen = false, prop = false, zin = false;
  uint8_t old = 0;
  if (in) {
    old = upd[v];
    const int c = cnt[v];
    gen = c > 1;
    if (c == 1 && phi[v] >= (T)PF_EPS) {
      const int X = ids[v];
      const int x = (int)(v / ((long long)g.d.n1 * g.d.n2)), y = (int)((v / g.d.n2) % g.d.n1), z = (int)(v % g.d.n2);
      for (int o = 0; o < 9; o++) {
        const int qx = x + c_pred[o][0], qy = y + c_pred[o][1], qz = z + c_pred[o][2];
        if (qx < 0 || qy < 0 || qy >= g.d.n1 || qz < 0 || qz >= g.d.n2) continue;
        const long long q = ((long long)qx * g.d.n1 + qy) * g.d.n2 + qz;
        const int nq = ncnt[q];
        const bool carries = nq >= 2 || (nq == 1 && nid[q] != X);
        if (o == 0) {   // (0,0,-1): the previous voxel of the row
          prop = carries;
          zin = upd[q] != 0;
        } else if (carries && upd[q]) {
          gen = true;
        }
      }
    }
  }
  // u = G | (P & u(z-1)) over the warp; lane 0 takes u(z-1) from the buffer
  const unsigned am = __activemask();
  unsigned gm = __ballot_sync(am, gen || (lane == 0 && prop && zin)), pm = __ballot_sync(am, prop);
#pragma unroll
  for (int s = 1; s < 32; s <<= 1) {
    gm |= pm & (gm << s);
    pm &= pm << s;
  }
  if (in) {
    const uint8_t u = (uint8_t)((gm >> lane) & 1u);
    if (u != old) {
      upd[v] = u;
      atomicAdd(&word[0], 1u);
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(256) pf_tail_kernel(PfView g, const int* __restrict__ ids, const T* __restrict__ phi,
                                                      const uint8_t* __restrict__ cnt, const int* __restrict__ nid,
                                                      const uint8_t* __restrict__ ncnt, const uint8_t* __restrict__ upd,
                                                      int* __restrict__ tail, uint8_t* __restrict__ tmode,
                                                      unsigned* __restrict__ word) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= g.nv) return;
  const int c = cnt[v];
  const bool weak = c > 0 && phi[(long long)(c - 1) * g.nv + v] < (T)PF_EPS;
  const int ns = weak ? c - 1 : c;
  int sid[PF_K];
  for (int k = 0; k < ns; k++) sid[k] = ids[(long long)k * g.nv + v];
  const int x = (int)(v / ((long long)g.d.n1 * g.d.n2)), y = (int)((v / g.d.n2) % g.d.n1), z = (int)(v % g.d.n2);
  int t = -1;
  for (int o = 0; o < 9 && t < 0; o++) {
    const int qx = x + c_pred[o][0], qy = y + c_pred[o][1], qz = z + c_pred[o][2];
    if (qx < 0 || qy < 0 || qy >= g.d.n1 || qz < 0 || qz >= g.d.n2) continue;
    const long long q = ((long long)qx * g.d.n1 + qy) * g.d.n2 + qz;
    if (!upd[q]) continue;
    for (int a = ncnt[q] - 1; a >= 0; a--) {
      const int j = nid[(long long)a * g.nv + q];
      bool strong = false;
      for (int k = 0; k < ns; k++) strong |= (sid[k] == j);
      if (!strong) { t = j; break; }
    }
  }
  uint8_t m = 0;
  if (t >= 0) {
    if (weak) m = 1;
    else if (c < PF_K) m = 2;
    else atomicOr(&word[1], (unsigned)PF_BAD_LIST);
  }
  tail[v] = t;
  tmode[v] = m;
}

// Window averages, one 8x8x8 tile of voxels per block: the tile and its
// 3-voxel halo (periodic) of initial grain ids, energies and this substep's
// resets are staged in shared memory once, and every voxel of the tile that
// updates sums its 7x7x7 window from there, in window order, one pass per
// held entry.  The window positions before the centre in that order are
// exactly the voxels earlier in the sweep (the first 171), so a reset applies
// there when the position lies inside the volume (a periodic image is a halo
// copy, refreshed only after the sweep).
constexpr int PF_WT = 8;
constexpr int PF_WH = PF_WT + 6;
template <typename T>
__global__ void __launch_bounds__(256) pf_window_kernel(PfView g, const int* __restrict__ ids,
                                                        const uint8_t* __restrict__ cnt, const int* __restrict__ tail,
                                                        const uint8_t* __restrict__ tmode, const int* __restrict__ gid0,
                                                        const T* __restrict__ energy, const uint8_t* __restrict__ ow,
                                                        T* __restrict__ wavg, int tiles_y, int tiles_z) {
  __shared__ int s_gid[PF_WH * PF_WH * PF_WH];
  __shared__ T s_e[PF_WH * PF_WH * PF_WH];
  __shared__ uint8_t s_reset[PF_WH * PF_WH * PF_WH];
  const int tz = blockIdx.x % tiles_z, ty = (blockIdx.x / tiles_z) % tiles_y, tx = blockIdx.x / (tiles_z * tiles_y);
  const int x0 = tx * PF_WT, y0 = ty * PF_WT, z0 = tz * PF_WT;
  for (int i = threadIdx.x; i < PF_WH * PF_WH * PF_WH; i += blockDim.x) {
    const int hz = i % PF_WH, hy = (i / PF_WH) % PF_WH, hx = i / (PF_WH * PF_WH);
    const int gx = x0 - 3 + hx, gy = y0 - 3 + hy, gz = z0 - 3 + hz;
    const bool in = gx >= 0 && gx < g.d.n0 && gy >= 0 && gy < g.d.n1 && gz >= 0 && gz < g.d.n2;
    const long long p = g.d.idx(gx, gy, gz);
    s_gid[i] = gid0[p];
    s_e[i] = energy[p];
    s_reset[i] = (uint8_t)(in && ow[p]);
  }
  __syncthreads();
  const int lz = threadIdx.x % PF_WT, ly = (threadIdx.x / PF_WT) % PF_WT;
  for (int half = 0; half < 2; half++) {
    const int lx = threadIdx.x / (PF_WT * PF_WT) + 4 * half;
    const int x = x0 + lx, y = y0 + ly, z = z0 + lz;
    if (x >= g.d.n0 || y >= g.d.n1 || z >= g.d.n2) continue;
    const long long v = ((long long)x * g.d.n1 + y) * g.d.n2 + z;
    const int c = cnt[v], mode = tmode[v];
    const int n = c + (mode == 2 ? 1 : 0);
    if (n <= 1) continue;
    for (int k = 0; k < n; k++) {
      const int id = (k == c || (mode == 1 && k == c - 1)) ? tail[v] : ids[(long long)k * g.nv + v];
      T A = (T)0;
      int C = 0;
      int q = 0;
      for (int i = 0; i < 7; i++)
        for (int j = 0; j < 7; j++) {
          const int base = ((lx + i) * PF_WH + (ly + j)) * PF_WH + lz;
          for (int m = 0; m < 7; m++, q++) {
            const int w = base + m;
            if (s_gid[w] == id) {
              A = A + ((q < 171 && s_reset[w]) ? (T)100 : s_e[w]);
              C++;
            }
          }
        }
      wavg[(long long)k * g.nv + v] = C > 0 ? A / (T)C : (T)0;
    }
  }
}

// Row summaries, one block per row of voxels (x, y): every id the row's
// updating voxels hold, with the first and last z holding it and the value
// the last one writes.  Ids go through a shared-memory hash (open addressing,
// 2 PF_RW slots); the order of the entries is immaterial (lookups are by id).
constexpr int PF_RHASH = 2 * PF_RW;
template <typename T>
__global__ void __launch_bounds__(128) pf_rows_kernel(PfView g, const int* __restrict__ ids,
                                                      const uint8_t* __restrict__ cnt, const int* __restrict__ tail,
                                                      const uint8_t* __restrict__ tmode, const T* __restrict__ wavg,
                                                      int* __restrict__ rw_id, T* __restrict__ rw_val,
                                                      int* __restrict__ rw_zf, int* __restrict__ rw_zl,
                                                      uint8_t* __restrict__ rw_n, unsigned* __restrict__ word) {
  __shared__ int h_id[PF_RHASH], h_zf[PF_RHASH], h_zl[PF_RHASH];
  __shared__ int h_n;
  const int r = blockIdx.x;
  for (int i = threadIdx.x; i < PF_RHASH; i += blockDim.x) {
    h_id[i] = 0;   // grain ids are >= 1 in a table-writing list; 0 marks a free slot
    h_zf[i] = INT_MAX;
    h_zl[i] = -1;
  }
  if (threadIdx.x == 0) h_n = 0;
  __syncthreads();
  unsigned bad = 0;
  // pass 1: slots, first and last z per id
  for (int z = threadIdx.x; z < g.d.n2; z += blockDim.x) {
    const long long v = (long long)r * g.d.n2 + z;
    const int c = cnt[v], mode = tmode[v];
    const int n = c + (mode == 2 ? 1 : 0);
    if (n <= 1) continue;
    for (int k = 0; k < n; k++) {
      const int id = (k == c || (mode == 1 && k == c - 1)) ? tail[v] : ids[(long long)k * g.nv + v];
      if (id < 1) { bad |= PF_BAD_TABLE; continue; }
      int slot = (int)(((unsigned)id * 2654435761u) % PF_RHASH), tries = 0;
      for (; tries < PF_RHASH; tries++, slot = (slot + 1) % PF_RHASH) {
        const int prev = atomicCAS(&h_id[slot], 0, id);
        if (prev == 0) { atomicAdd(&h_n, 1); break; }
        if (prev == id) break;
      }
      if (tries == PF_RHASH) { bad |= PF_BAD_ROW; continue; }
      atomicMin(&h_zf[slot], z);
      atomicMax(&h_zl[slot], z);
    }
  }
  __syncthreads();
  if (h_n > PF_RW) bad |= PF_BAD_ROW;
  // pass 2: the last writer's value, compacted into the summary
  __shared__ int h_pos[PF_RHASH];
  if (threadIdx.x == 0) {
    int e = 0;
    for (int i = 0; i < PF_RHASH; i++) h_pos[i] = (h_id[i] != 0 && e < PF_RW) ? e++ : -1;
    rw_n[r] = (uint8_t)e;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < PF_RHASH; i += blockDim.x) {
    const int e = h_pos[i];
    if (e < 0) continue;
    rw_id[(long long)e * g.rows + r] = h_id[i];
    rw_zf[(long long)e * g.rows + r] = h_zf[i];
    rw_zl[(long long)e * g.rows + r] = h_zl[i];
  }
  for (int z = threadIdx.x; z < g.d.n2; z += blockDim.x) {
    const long long v = (long long)r * g.d.n2 + z;
    const int c = cnt[v], mode = tmode[v];
    const int n = c + (mode == 2 ? 1 : 0);
    if (n <= 1) continue;
    for (int k = 0; k < n; k++) {
      const int id = (k == c || (mode == 1 && k == c - 1)) ? tail[v] : ids[(long long)k * g.nv + v];
      if (id < 1) continue;
      int slot = (int)(((unsigned)id * 2654435761u) % PF_RHASH);
      for (int tries = 0; tries < PF_RHASH && h_id[slot] != id; tries++) slot = (slot + 1) % PF_RHASH;
      if (h_id[slot] != id || h_pos[slot] < 0 || h_zl[slot] != z) continue;
      rw_val[(long long)h_pos[slot] * g.rows + r] = wavg[(long long)k * g.nv + v];
    }
  }
  if (bad) atomicOr(&word[1], bad);
}

// rho_avg of id j as the sweep leaves it just before voxel v: the latest
// earlier writer in v's row, else in the earlier rows of v's block of PF_RB
// rows, else the last writer up to the previous block (prefix table), else
// the table as the previous substep left it
template <typename T>
__device__ T pf_stale(const PfView& g, long long v, int j, const int* __restrict__ ids, const uint8_t* __restrict__ cnt,
                      const int* __restrict__ tail, const uint8_t* __restrict__ tmode, const T* __restrict__ wavg,
                      const int* __restrict__ rw_id, const T* __restrict__ rw_val, const int* __restrict__ rw_zf,
                      const int* __restrict__ rw_zl, const uint8_t* __restrict__ rw_n,
                      const int* __restrict__ blk_row, const T* __restrict__ blk_val, int table_cap,
                      const T* __restrict__ table, int table_len, unsigned* bad) {
  const int r = (int)(v / g.d.n2), z = (int)(v % g.d.n2);
  // v's row: the summary gives the first and last z holding j
  const int rn = rw_n[r];
  for (int e = 0; e < rn; e++) {
    if (rw_id[(long long)e * g.rows + r] != j) continue;
    const int zf = rw_zf[(long long)e * g.rows + r], zl = rw_zl[(long long)e * g.rows + r];
    if (zl < z) return rw_val[(long long)e * g.rows + r];
    if (zf < z) {   // the latest writer before v lies in [zf, z)
      for (long long w = v - 1; w >= (long long)r * g.d.n2 + zf; w--) {
        const int c = cnt[w], m = tmode[w];
        const int n = c + (m == 2 ? 1 : 0);
        if (n <= 1) continue;
        for (int k = 0; k < n; k++) {
          const int id = (k == c || (m == 1 && k == c - 1)) ? tail[w] : ids[(long long)k * g.nv + w];
          if (id == j) return wavg[(long long)k * g.nv + w];
        }
      }
    }
    break;
  }
  if (j < 1 || j > table_len) { *bad |= PF_BAD_TABLE; return (T)0; }
  const int blk = r / PF_RB;
  for (int q = r - 1; q >= blk * PF_RB; q--) {
    const int rn = rw_n[q];
    for (int e = 0; e < rn; e++)
      if (rw_id[(long long)e * g.rows + q] == j) return rw_val[(long long)e * g.rows + q];
  }
  if (blk > 0) {
    const long long at = (long long)(blk - 1) * table_cap + (j - 1);
    if (blk_row[at] >= 0) return blk_val[at];
  }
  return table[j - 1];
}

template <typename T>
__global__ void __launch_bounds__(128) pf_update_kernel(PfView g, const int* __restrict__ ids, const T* __restrict__ phi,
                                                        const uint8_t* __restrict__ cnt, const int* __restrict__ nid,
                                                        const uint8_t* __restrict__ ncnt, const int* __restrict__ tail,
                                                        const uint8_t* __restrict__ tmode, const T* __restrict__ wavg,
                                                        const int* __restrict__ rw_id, const T* __restrict__ rw_val,
                                                        const int* __restrict__ rw_zf, const int* __restrict__ rw_zl,
                                                        const uint8_t* __restrict__ rw_n, const int* __restrict__ blk_row,
                                                        const T* __restrict__ blk_val, int table_cap,
                                                        const T* __restrict__ table, int table_len, int init_gid, T mcoef,
                                                        T kappa, T mwell, T edisl,
                                                        const uint8_t* __restrict__ ow_in, uint8_t* __restrict__ ow_out,
                                                        int* __restrict__ ids2, T* __restrict__ phi2,
                                                        uint8_t* __restrict__ cnt2, unsigned* __restrict__ word) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= g.nv) return;
  const long long nv = g.nv;
  int hid[PF_K + 1];
  T hph[PF_K + 1];
  const int n = pf_held<T>(g, ids, phi, cnt, tail, tmode, v, hid, hph);
  int oid[PF_K];
  T oph[PF_K];
  int on = 0;
  unsigned bad = 0;
  bool reset = false;
  const int nn = ncnt[v];
  if (n > 1) {
    const int x = (int)(v / ((long long)g.d.n1 * g.d.n2)), y = (int)((v / g.d.n2) % g.d.n1), z = (int)(v % g.d.n2);
    const Nbhd nbh(g.d, x, y, z);
    T sum_rex = 0, sum1 = 0, hdef = 0;
    for (int k = 0; k < n; k++) {
      const T a = wavg[(long long)k * nv + v];
      if (a > (T)0) {
        const T e = hph[k];
        sum_rex = sum_rex + e * e;
        sum1 = sum1 + e * e * e * ((T)10.0 - (T)15.0 * e + (T)6.0 * e * e);
        hdef = hdef + (e * e * e * ((T)10.0 - (T)15.0 * e + (T)6.0 * e * e)) * a;
      }
    }
    for (int a = 0; a < nn; a++) {
      const int j = nid[(long long)a * nv + v];
      const T c = pf_read_local<T>(hid, hph, n, j);
      const T h = c * c * c * ((T)10.0 - (T)15.0 * c + (T)6.0 * c * c);
      const T dh = c * c * ((T)30.0 - (T)60.0 * c + (T)30.0 * c * c);
#define NB(a_, b_, c_) pf_read_g<T>(ids, phi, cnt, nv, nbh.at(a_, b_, c_), j)
      const T right = NB(1, 0, 0), left = NB(-1, 0, 0), front = NB(0, 1, 0), back = NB(0, -1, 0);
      const T up = NB(0, 0, 1), down = NB(0, 0, -1);
      const T lu = NB(-1, 0, 1), ld = NB(-1, 0, -1), lf = NB(-1, -1, 0), lb = NB(-1, 1, 0);
      const T cuf = NB(0, -1, 1), cub = NB(0, 1, 1), cdf = NB(0, -1, -1), cdb = NB(0, 1, -1);
      const T ru = NB(1, 0, 1), rdn = NB(1, 0, -1), rf = NB(1, -1, 0), rb = NB(1, 1, 0);
#undef NB
      // laplacian() receives left_up.. as its right_up.. parameters
      // (src/pf_xrx.c:6-9 against the call at :1193-1198)
      const T lap = (T)0.5 * (right + left + front + back + up + down) +
                    (T)0.125 * (cuf + cdf + cub + cdb + ld + lu + lf + lb + ru + rb + rdn + rf) - (T)4.5 * c;
      T ra;
      int k = 0;
      while (k < n && hid[k] != j) k++;
      if (k < n) ra = wavg[(long long)k * nv + v];
      else
        ra = pf_stale<T>(g, v, j, ids, cnt, tail, tmode, wavg, rw_id, rw_val, rw_zf, rw_zl, rw_n, blk_row, blk_val,
                         table_cap, table, table_len, &bad);
      if (ra > (T)0) {
        const T val = c - mcoef * (mwell * (c * c * c - c + (T)3.0 * c * (sum_rex - c * c)) - kappa * lap +
                                   edisl * dh * ((sum1 - h) * ra - (hdef - h * ra)) / (sum1 * sum1));
        if (j > init_gid && c < (T)0.5 && val > (T)0.5) reset = true;
        if (val > (T)PF_KEEP) pf_write_local<T>(oid, oph, on, j, val, &bad);
      }
    }
  } else if (n == 1) {
    for (int a = 0; a < nn; a++) {
      const int j = nid[(long long)a * nv + v];
      pf_write_local<T>(oid, oph, on, j, pf_read_local<T>(hid, hph, n, j), &bad);
    }
  }
  cnt2[v] = (uint8_t)on;
  for (int k = 0; k < on; k++) {
    ids2[(long long)k * nv + v] = oid[k];
    phi2[(long long)k * nv + v] = oph[k];
  }
  ow_out[v] = (uint8_t)reset;
  if ((uint8_t)reset != ow_in[v]) atomicAdd(&word[0], 1u);
  if (bad) atomicOr(&word[1], bad);
}

// Prefix of the table writers: per block of PF_RB rows and id, the last row
// writing the id in that block and its value (mark, write), then carried
// forward over the blocks (prefix), so that entry [b][j] is the last writer
// of j up to block b.  After the sweep, the last block's entries update the
// table (final).
__global__ void pf_blk_mark_kernel(PfView g, const int* __restrict__ rw_id, const uint8_t* __restrict__ rw_n,
                                   int* __restrict__ blk_row, int table_cap, int table_len,
                                   unsigned* __restrict__ word) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= g.rows) return;
  const long long base = (long long)(r / PF_RB) * table_cap;
  for (int e = 0; e < rw_n[r]; e++) {
    const int j = rw_id[(long long)e * g.rows + r];
    if (j < 1 || j > table_len) { atomicOr(&word[1], (unsigned)PF_BAD_TABLE); continue; }
    atomicMax(&blk_row[base + j - 1], r);
  }
}
template <typename T>
__global__ void pf_blk_write_kernel(PfView g, const int* __restrict__ rw_id, const T* __restrict__ rw_val,
                                    const uint8_t* __restrict__ rw_n, const int* __restrict__ blk_row,
                                    T* __restrict__ blk_val, int table_cap, int table_len) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= g.rows) return;
  const long long base = (long long)(r / PF_RB) * table_cap;
  for (int e = 0; e < rw_n[r]; e++) {
    const int j = rw_id[(long long)e * g.rows + r];
    if (j >= 1 && j <= table_len && blk_row[base + j - 1] == r) blk_val[base + j - 1] = rw_val[(long long)e * g.rows + r];
  }
}
template <typename T>
__global__ void pf_blk_prefix_kernel(int nblk, int* __restrict__ blk_row, T* __restrict__ blk_val, int table_cap,
                                     int table_len) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= table_len) return;
  int cr = blk_row[j];
  T cv = cr >= 0 ? blk_val[j] : (T)0;
  // eight blocks' rows loaded before any is written (each address is read
  // before it is written), then carried forward in order
  for (int b0 = 1; b0 < nblk; b0 += 8) {
    int rr[8];
#pragma unroll
    for (int u = 0; u < 8; u++) rr[u] = b0 + u < nblk ? blk_row[(long long)(b0 + u) * table_cap + j] : 0;
#pragma unroll
    for (int u = 0; u < 8; u++) {
      if (b0 + u >= nblk) break;
      const long long at = (long long)(b0 + u) * table_cap + j;
      if (rr[u] >= 0) {
        cr = rr[u];
        cv = blk_val[at];
      } else if (cr >= 0) {
        blk_row[at] = cr;
        blk_val[at] = cv;
      }
    }
  }
}
template <typename T>
__global__ void pf_table_final_kernel(int nblk, const int* __restrict__ blk_row, const T* __restrict__ blk_val,
                                      int table_cap, int table_len, T* __restrict__ table) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= table_len) return;
  const long long at = (long long)(nblk - 1) * table_cap + j;
  if (blk_row[at] >= 0) table[j] = blk_val[at];
}

// resets applied to the energy; grain id = first maximum, 0 when no eta > 0
// (Update_gID, src/pf_xrx.c:11-66)
template <typename T>
__global__ void pf_finish_kernel(PfView g, const int* __restrict__ ids, const T* __restrict__ phi,
                                 const uint8_t* __restrict__ cnt, const uint8_t* __restrict__ ow, T* __restrict__ energy,
                                 int* __restrict__ gid) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= g.nv) return;
  if (ow[v]) energy[v] = (T)100;
  T best = (T)0;
  int id = 0;
  const int c = cnt[v];
  for (int k = 0; k < c; k++) {
    const T e = phi[(long long)k * g.nv + v];
    if (best < e) { best = e; id = ids[(long long)k * g.nv + v]; }
  }
  gid[v] = id;
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

cudaError_t launch_paint_nuclei(const int dims[3], const long long* sites, int nn, int radius2, int first_id,
                                int* winner, int* grain, cudaStream_t st) {
  Dims d{dims[0], dims[1], dims[2]};
  const long long nv = (long long)dims[0] * dims[1] * dims[2];
  int r = 0;
  while ((r + 1) * (r + 1) <= radius2) r++;
  const int side = 2 * r + 1;
  const long long work = (long long)nn * side * side * side;
  if (work > 0 && radius2 >= 0) paint_mark_kernel<<<nb(work, 256), 256, 0, st>>>(d, sites, nn, r, radius2, winner);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  paint_apply_kernel<<<nb(nv, 256), 256, 0, st>>>(nv, first_id, winner, grain);
  return cudaGetLastError();
}

template <typename T>
cudaError_t pf_alloc(PfBuffers<T>& b, const int dims[3], int table_len) {
  memset(&b, 0, sizeof(b));
  const long long nv = (long long)dims[0] * dims[1] * dims[2];
  b.rows = dims[0] * dims[1];
  b.nblk = (b.rows + PF_RB - 1) / PF_RB;
  cudaError_t e = cudaSuccess;
  auto get = [&](void** p, size_t bytes) {
    if (e == cudaSuccess) e = cudaMalloc(p, bytes);
  };
  for (int i = 0; i < 2; i++) {
    get((void**)&b.ids[i], sizeof(int) * PF_K * nv);
    get((void**)&b.phi[i], sizeof(T) * PF_K * nv);
    get((void**)&b.cnt[i], (size_t)nv);
    get((void**)&b.upd[i], (size_t)nv);
    get((void**)&b.ow[i], (size_t)nv);
  }
  get((void**)&b.gid, sizeof(int) * nv);
  get((void**)&b.energy, sizeof(T) * nv);
  get((void**)&b.nid, sizeof(int) * PF_NM * nv);
  get((void**)&b.ncnt, (size_t)nv);
  get((void**)&b.tail, sizeof(int) * nv);
  get((void**)&b.tmode, (size_t)nv);
  get((void**)&b.wavg, sizeof(T) * (PF_K + 1) * nv);
  get((void**)&b.rw_id, sizeof(int) * PF_RW * (size_t)b.rows);
  get((void**)&b.rw_val, sizeof(T) * PF_RW * (size_t)b.rows);
  get((void**)&b.rw_zf, sizeof(int) * PF_RW * (size_t)b.rows);
  get((void**)&b.rw_zl, sizeof(int) * PF_RW * (size_t)b.rows);
  get((void**)&b.rw_n, (size_t)b.rows);
  get((void**)&b.word, sizeof(unsigned) * 2);
  if (e == cudaSuccess) e = pf_table_reserve(b, table_len, nullptr);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  return e;
}

template <typename T>
void pf_free(PfBuffers<T>& b) {
  for (int i = 0; i < 2; i++) {
    cudaFree(b.ids[i]); cudaFree(b.phi[i]); cudaFree(b.cnt[i]); cudaFree(b.upd[i]); cudaFree(b.ow[i]);
  }
  cudaFree(b.gid); cudaFree(b.energy); cudaFree(b.nid); cudaFree(b.ncnt); cudaFree(b.tail); cudaFree(b.tmode);
  cudaFree(b.wavg); cudaFree(b.rw_id); cudaFree(b.rw_val); cudaFree(b.rw_zf); cudaFree(b.rw_zl); cudaFree(b.rw_n); cudaFree(b.blk_row);
  cudaFree(b.blk_val);
  cudaFree(b.table); cudaFree(b.word);
  memset(&b, 0, sizeof(b));
}

template <typename T>
cudaError_t pf_table_reserve(PfBuffers<T>& b, int len, cudaStream_t st) {
  if (len <= b.table_cap) {
    b.table_len = b.table_cap;
    return cudaSuccess;
  }
  const int cap = len + 1024;
  T* t = nullptr;
  int* br = nullptr;
  T* bv = nullptr;
  const size_t nb_entries = (size_t)b.nblk * cap;
  cudaError_t e = cudaMalloc(&t, sizeof(T) * cap);
  if (e == cudaSuccess) e = cudaMalloc(&br, sizeof(int) * nb_entries);
  if (e == cudaSuccess) e = cudaMalloc(&bv, sizeof(T) * nb_entries);
  if (e == cudaSuccess) e = cudaMemsetAsync(t, 0, sizeof(T) * cap, st);
  if (e == cudaSuccess && b.table_cap > 0)
    e = cudaMemcpyAsync(t, b.table, sizeof(T) * b.table_cap, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    cudaFree(t);
    cudaFree(br);
    cudaFree(bv);
    return e;
  }
  cudaFree(b.table);
  cudaFree(b.blk_row);
  cudaFree(b.blk_val);
  b.table = t;
  b.blk_row = br;
  b.blk_val = bv;
  b.table_cap = b.table_len = cap;
  return cudaSuccess;
}

// fixed-point driver: the host reads the change counter after each iterate
static cudaError_t pf_read_counter(unsigned* word_d, unsigned* out, cudaStream_t st) {
  cudaError_t e = cudaMemcpyAsync(out, word_d, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e;
}

template <typename T>
cudaError_t launch_pf_relax(const int dims[3], const int* grain, const T* rho, int substeps, int init_gid,
                            const PfCoef& co, PfBuffers<T>& b, cudaStream_t st, int* launches, unsigned* bad) {
  PfView g{Dims{dims[0], dims[1], dims[2]}, (long long)dims[0] * dims[1] * dims[2], dims[0] * dims[1]};
  const long long nv = g.nv;
  int nl = 0;
  *bad = 0;
#define PF_CK(call)                        \
  do {                                     \
    cudaError_t e__ = (call);              \
    if (e__ != cudaSuccess) {              \
      *launches = nl;                      \
      return e__;                          \
    }                                      \
  } while (0)
#define PF_K_LAUNCH(...)          \
  do {                            \
    __VA_ARGS__;                  \
    nl++;                         \
    PF_CK(cudaGetLastError());    \
  } while (0)
  PF_CK(cudaMemsetAsync(b.word, 0, sizeof(unsigned) * 2, st));
  PF_K_LAUNCH(pf_init_kernel<T><<<nb(nv, 256), 256, 0, st>>>(g, grain, rho, b.ids[0], b.phi[0], b.cnt[0], b.energy, b.gid));
  int cur = 0;
  unsigned changed = 0;
  const int wtx = (dims[0] + PF_WT - 1) / PF_WT, wty = (dims[1] + PF_WT - 1) / PF_WT, wtz = (dims[2] + PF_WT - 1) / PF_WT;
  const int wtiles = wtx * wty * wtz;
  for (int s = 0; s < substeps; s++) {
    const int* ids = b.ids[cur];
    const T* phi = b.phi[cur];
    const uint8_t* cnt = b.cnt[cur];
    PF_K_LAUNCH(pf_nlist_kernel<T><<<nb(nv, 256), 256, 0, st>>>(g, ids, phi, cnt, b.nid, b.ncnt, b.word));
    // update flags to their fixed point (in place), two passes between
    // reads of the change counter (a pass at the fixed point changes
    // nothing, so a second one costs only its launch); the counter read is
    // the second pass's
    PF_CK(cudaMemsetAsync(b.upd[0], 0, (size_t)nv, st));
    const int a = 0;
    for (long long it = 0; it <= nv; it += 2) {
      PF_K_LAUNCH(pf_upd_kernel<T><<<nb(nv, 256), 256, 0, st>>>(g, ids, phi, cnt, b.nid, b.ncnt, b.upd[a], b.word));
      PF_CK(cudaMemsetAsync(b.word, 0, sizeof(unsigned), st));
      PF_K_LAUNCH(pf_upd_kernel<T><<<nb(nv, 256), 256, 0, st>>>(g, ids, phi, cnt, b.nid, b.ncnt, b.upd[a], b.word));
      PF_CK(pf_read_counter(b.word, &changed, st));
      if (changed == 0) break;
    }
    PF_K_LAUNCH(pf_tail_kernel<T><<<nb(nv, 256), 256, 0, st>>>(g, ids, phi, cnt, b.nid, b.ncnt, b.upd[a], b.tail,
                                                                b.tmode, b.word));
    // values, with the stored-energy resets to their fixed point
    PF_CK(cudaMemsetAsync(b.ow[0], 0, (size_t)nv, st));
    int o = 0;
    for (long long it = 0; it <= nv; it++) {
      PF_CK(cudaMemsetAsync(b.word, 0, sizeof(unsigned), st));
      PF_K_LAUNCH(pf_window_kernel<T><<<wtiles, 256, 0, st>>>(g, ids, cnt, b.tail, b.tmode, grain, b.energy, b.ow[o],
                                                               b.wavg, wty, wtz));
      PF_K_LAUNCH(pf_rows_kernel<T><<<g.rows, 128, 0, st>>>(g, ids, cnt, b.tail, b.tmode, b.wavg, b.rw_id, b.rw_val,
                                                              b.rw_zf, b.rw_zl, b.rw_n, b.word));
      // prefix of the table writers (their values change over the iterates)
      PF_CK(cudaMemsetAsync(b.blk_row, 0xff, sizeof(int) * (size_t)b.nblk * b.table_cap, st));
      if (b.table_len > 0) {
        PF_K_LAUNCH(pf_blk_mark_kernel<<<nb(g.rows, 256), 256, 0, st>>>(g, b.rw_id, b.rw_n, b.blk_row, b.table_cap,
                                                                         b.table_len, b.word));
        PF_K_LAUNCH(pf_blk_write_kernel<T><<<nb(g.rows, 256), 256, 0, st>>>(g, b.rw_id, b.rw_val, b.rw_n, b.blk_row,
                                                                             b.blk_val, b.table_cap, b.table_len));
        PF_K_LAUNCH(pf_blk_prefix_kernel<T><<<nb(b.table_len, 128), 128, 0, st>>>(b.nblk, b.blk_row, b.blk_val,
                                                                                   b.table_cap, b.table_len));
      }
      PF_K_LAUNCH(pf_update_kernel<T><<<nb(nv, 128), 128, 0, st>>>(
          g, ids, phi, cnt, b.nid, b.ncnt, b.tail, b.tmode, b.wavg, b.rw_id, b.rw_val, b.rw_zf, b.rw_zl, b.rw_n,
          b.blk_row, b.blk_val,
          b.table_cap, b.table, b.table_len,
          init_gid, (T)co.mcoef, (T)co.kappa, (T)co.mwell, (T)co.edisl, b.ow[o], b.ow[1 - o], b.ids[1 - cur],
          b.phi[1 - cur], b.cnt[1 - cur], b.word));
      o = 1 - o;
      PF_CK(pf_read_counter(b.word, &changed, st));
      if (changed == 0) break;
    }
    if (b.table_len > 0)
      PF_K_LAUNCH(pf_table_final_kernel<T><<<nb(b.table_len, 256), 256, 0, st>>>(b.nblk, b.blk_row, b.blk_val,
                                                                                   b.table_cap, b.table_len, b.table));
    cur = 1 - cur;
    PF_K_LAUNCH(pf_finish_kernel<T><<<nb(nv, 256), 256, 0, st>>>(g, b.ids[cur], b.phi[cur], b.cnt[cur], b.ow[o],
                                                                  b.energy, b.gid));
  }
  b.cur = cur;
  unsigned w[2] = {0, 0};
  PF_CK(cudaMemcpyAsync(w, b.word, sizeof(w), cudaMemcpyDeviceToHost, st));
  PF_CK(cudaStreamSynchronize(st));
  *bad = w[1];
  *launches = nl;
#undef PF_K_LAUNCH
#undef PF_CK
  return cudaSuccess;
}

template cudaError_t pf_alloc<float>(PfBuffers<float>&, const int*, int);
template cudaError_t pf_alloc<double>(PfBuffers<double>&, const int*, int);
template void pf_free<float>(PfBuffers<float>&);
template void pf_free<double>(PfBuffers<double>&);
template cudaError_t pf_table_reserve<float>(PfBuffers<float>&, int, cudaStream_t);
template cudaError_t pf_table_reserve<double>(PfBuffers<double>&, int, cudaStream_t);
template cudaError_t launch_pf_relax<float>(const int*, const int*, const float*, int, int, const PfCoef&,
                                            PfBuffers<float>&, cudaStream_t, int*, unsigned*);
template cudaError_t launch_pf_relax<double>(const int*, const int*, const double*, int, int, const PfCoef&,
                                             PfBuffers<double>&, cudaStream_t, int*, unsigned*);

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

// Per recrystallised grain k: its voxels after the relaxation (cnt[k]) and
// those of them that joined it in this step (cnt[n_drx + k]), for the
// "< 1 % grew" rule of src/integrated.c:1537-1582.
template <typename TSt>
__global__ void drx_count_kernel(Fields<TSt> f, const int* __restrict__ grain, const int* __restrict__ grain_prev,
                                 const int* __restrict__ gid_new, int first_drx_id, int n_drx,
                                 int* __restrict__ cnt) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= f.nv) return;
  const int gn = gid_new[v] != 0 ? gid_new[v] : grain[v];
  const int k = gn - first_drx_id;
  if (k < 0 || k >= n_drx) return;
  atomicAdd(&cnt[k], 1);
  if (gn != grain_prev[v] && f.phase[v] == 0) atomicAdd(&cnt[n_drx + k], 1);
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
                                  int nsys, const int* __restrict__ cnt) {
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long P = f.nv;
  if (v >= P) return;
  // a voxel the phase field left without a positive eta (grain id 0, where
  // the reference stops on GetStatistics' assert, src/pf_xrx.c:1383-1386)
  // keeps the grain it had
  const int gn = gid_new[v] != 0 ? gid_new[v] : grain[v];
  grain[v] = gn;
  if (gn == grain_prev[v] || f.phase[v] != 0) return;
  const int k = gn - first_drx_id;
  if (k < 0 || k >= n_drx) return;
  // a grain whose joining voxels are under 1 % of it (integer percent 0,
  // src/integrated.c:1562-1577) resets none of them: they take its id only
  if ((long long)cnt[n_drx + k] * 100 / cnt[k] == 0) return;
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
                              int nsys, int* cnt, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(cnt, 0, sizeof(int) * 2 * (size_t)n_drx, st);
  if (e != cudaSuccess) return e;
  if (mixed) {
    const Fields<float>& f = *static_cast<const Fields<float>*>(fields);
    drx_count_kernel<float><<<nb(f.nv, 256), 256, 0, st>>>(f, grain, grain_prev, gid_new, first_drx_id, n_drx, cnt);
    drx_update_kernel<float><<<nb(f.nv, 256), 256, 0, st>>>(f, grain, grain_prev, gid_new, first_drx_id, n_drx, drx_rot,
                                                            drx_class, tau0f, nsys, cnt);
  } else {
    const Fields<double>& f = *static_cast<const Fields<double>*>(fields);
    drx_count_kernel<double><<<nb(f.nv, 256), 256, 0, st>>>(f, grain, grain_prev, gid_new, first_drx_id, n_drx, cnt);
    drx_update_kernel<double><<<nb(f.nv, 256), 256, 0, st>>>(f, grain, grain_prev, gid_new, first_drx_id, n_drx,
                                                             drx_rot, drx_class, tau0f, nsys, cnt);
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

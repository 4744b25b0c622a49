/*
 * drx_oracle.c -- ORACLE (test infrastructure only; never linked into the
 * product).
 *
 * CPU restatement, in FP64, of the dynamic-recrystallisation step of
 * M-THEMES: grain-boundary indicator (Gradient_ExchangeGrainID,
 * src/constitutive.c:724-873 and src/evolution.c:816-829), nucleation
 * (NucleationCheckDRX, src/integrated.c:161-494) and the sparse
 * order-parameter Allen-Cahn relaxation (PF_XRX / Update_grid / Update_gID,
 * src/pf_xrx.c:6-66,895-1311,1469-1698), in the deterministic form this
 * build defines (the reference's sparse lists are mutated during the sweep
 * and share a global rho_avg table, so its result depends on sweep order):
 *
 *  - at most K order parameters per voxel, stored sorted by grain id;
 *  - the neighbourhood id set N(v) = ids with eta > 5e-3 in the 3x3x3 block
 *    (src/pf_xrx.c:937-973, EPSILON of src/PFgrid.h:49);
 *  - the stored-energy average of grain j at v is the mean of rho over the
 *    7x7x7 window voxels whose current grain id is j (src/pf_xrx.c:1052-1086),
 *    computed for every j in N(v) and every id held at v;
 *  - the explicit update of src/pf_xrx.c:1184-1233 for every j in N(v) when
 *    |N(v)| > 1, values <= 1e-4 dropped (src/pf_xrx.c:1207,1221); a copy when
 *    |N(v)| == 1; the K largest values kept;
 *  - grain id = argmax eta, ties to the smaller id (Update_gID,
 *    src/pf_xrx.c:11-66).
 * Nucleation: a grain-boundary voxel of a crystal phase whose total
 * dislocation density exceeds rho_nucleation nucleates with probability
 * nucleation_prob per step, drawn from a counter-based generator of
 * (seed, step, voxel); nuclei are numbered in voxel order and paint a
 * periodic disc |d|^2 <= r^2 (src/integrated.c:400), later nuclei over
 * earlier ones.
 *
 * Compiled with -ffp-contract=off: every floating-point operation is a
 * separately rounded IEEE operation in a fixed order, which the CUDA kernels
 * reproduce (-fmad=false) so FP64 grain maps can be compared bit for bit.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include "oracle.h"

#define PF_EPS 5.0e-3   /* EPSILON, src/PFgrid.h:49 */
#define PF_KEEP 1.0e-4  /* src/pf_xrx.c:1207,1221 */
#define MAXIDS 64

/* SplitMix64 finaliser of a (seed, counter) pair: uniform in (0, 1]. */
static uint64_t mix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ULL;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
  return x ^ (x >> 31);
}
double orc_uniform(uint64_t seed, uint64_t counter) {
  uint64_t h = mix64(seed * 0xD1342543DE82EF95ULL + mix64(counter));
  return (double)((h >> 11) + 1) * (1.0 / 9007199254740992.0);
}

/* PF_XRX coefficients (src/pf_xrx.c:1491-1498) with L_gb = width*dx. */
void orc_pf_coefficients(const mth_params* p, double* mcoef, double* kappa, double* mwell, double* edisl) {
  const double dx = p->pf_length_scale;
  const double lgb = p->pf_width_cells * dx;
  *mcoef = p->pf_time_step * 4.0 / 3.0 * p->m_gb / lgb;
  *kappa = 3.0 / 4.0 * p->e_gb * lgb / dx / dx;
  *mwell = 6 * p->e_gb / lgb;
  *edisl = p->stored_energy_scale * p->shear_modulus * p->burgers * p->burgers;
}

static inline long long vidx(const int* n, int x, int y, int z) {
  x = (x % n[0] + n[0]) % n[0];
  y = (y % n[1] + n[1]) % n[1];
  z = (z % n[2] + n[2]) % n[2];
  return ((long long)x * n[1] + y) * n[2] + z;
}

/* 1 where a face neighbour (periodic) belongs to another grain. */
void orc_gb_indicator(const int* n, const int* grain, unsigned char* gb) {
  for (int x = 0; x < n[0]; x++)
    for (int y = 0; y < n[1]; y++)
      for (int z = 0; z < n[2]; z++) {
        long long v = vidx(n, x, y, z);
        int g = grain[v];
        int b = (grain[vidx(n, x + 1, y, z)] != g) | (grain[vidx(n, x - 1, y, z)] != g) |
                (grain[vidx(n, x, y + 1, z)] != g) | (grain[vidx(n, x, y - 1, z)] != g) |
                (grain[vidx(n, x, y, z + 1)] != g) | (grain[vidx(n, x, y, z - 1)] != g);
        gb[v] = (unsigned char)b;
      }
}

long long orc_nucleation_sites(const int* n, const int* grain, const int* phase_crystal, const double* rho,
                               double rho_nuc, double prob, uint64_t seed, long long step, long long* sites,
                               long long cap) {
  const long long nv = (long long)n[0] * n[1] * n[2];
  unsigned char* gb = (unsigned char*)malloc(nv);
  orc_gb_indicator(n, grain, gb);
  long long k = 0;
  for (long long v = 0; v < nv; v++) {
    if (!gb[v] || !phase_crystal[v]) continue;
    if (!(rho[v] > rho_nuc)) continue;
    double u = orc_uniform(seed, (uint64_t)step * (uint64_t)nv + (uint64_t)v);
    if (u < prob) {
      if (k < cap) sites[k] = v;
      k++;
    }
  }
  free(gb);
  return k;
}

void orc_paint_nuclei(const int* n, int* grain, const long long* sites, int nn, int first_id, int radius) {
  const int r2 = radius * radius;
  for (int k = 0; k < nn; k++) {
    long long v = sites[k];
    int x0 = (int)(v / ((long long)n[1] * n[2])), y0 = (int)((v / n[2]) % n[1]), z0 = (int)(v % n[2]);
    for (int dx = -radius; dx <= radius; dx++)
      for (int dy = -radius; dy <= radius; dy++)
        for (int dz = -radius; dz <= radius; dz++)
          if (dx * dx + dy * dy + dz * dz <= r2) grain[vidx(n, x0 + dx, y0 + dy, z0 + dz)] = first_id + k;
  }
}

/* eta of grain id at voxel w (0 when absent) */
static inline double eta_of(const int* ids, const double* phi, const int* cnt, int K, long long w, int id) {
  for (int s = 0; s < cnt[w]; s++)
    if (ids[w * K + s] == id) return phi[w * K + s];
  return 0.0;
}

static void sorted_insert(int* list, int* nl, int id) {
  int i = 0;
  while (i < *nl && list[i] < id) i++;
  if (i < *nl && list[i] == id) return;
  if (*nl >= MAXIDS) return;
  for (int j = *nl; j > i; j--) list[j] = list[j - 1];
  list[i] = id;
  (*nl)++;
}

/* one explicit substep: (ids,phi,cnt) -> (ids2,phi2,cnt2); gid/rho: current
   grain ids and stored energy used by the window averages */
static void pf_substep(const int* n, int K, const int* ids, const double* phi, const int* cnt, int* ids2,
                       double* phi2, int* cnt2, const int* gid, const double* rho, double mcoef, double kappa,
                       double mwell, double edisl) {
  const long long nv = (long long)n[0] * n[1] * n[2];
#pragma omp parallel for schedule(dynamic, 256)
  for (long long v = 0; v < nv; v++) {
    const int x = (int)(v / ((long long)n[1] * n[2])), y = (int)((v / n[2]) % n[1]), z = (int)(v % n[2]);
    int nid[MAXIDS], nn = 0;
    for (int dx = -1; dx <= 1; dx++)
      for (int dy = -1; dy <= 1; dy++)
        for (int dz = -1; dz <= 1; dz++) {
          long long w = vidx(n, x + dx, y + dy, z + dz);
          for (int s = 0; s < cnt[w]; s++)
            if (phi[w * K + s] > PF_EPS) sorted_insert(nid, &nn, ids[w * K + s]);
        }
    if (nn <= 1) {
      cnt2[v] = cnt[v];
      for (int s = 0; s < K; s++) {
        ids2[v * K + s] = s < cnt[v] ? ids[v * K + s] : 0;
        phi2[v * K + s] = s < cnt[v] ? phi[v * K + s] : 0.0;
      }
      continue;
    }
    /* ids whose window average is needed: N(v) and the ids held at v */
    int uid[MAXIDS], nu = 0;
    for (int i = 0; i < nn; i++) sorted_insert(uid, &nu, nid[i]);
    for (int s = 0; s < cnt[v]; s++) sorted_insert(uid, &nu, ids[v * K + s]);
    /* window sums per id, in a fixed association: the 7x7 (y,z) patch of
       each x plane summed in (y,z) order, then the seven planes in x order */
    double wsum[MAXIDS];
    int wcnt[MAXIDS];
    for (int i = 0; i < nu; i++) { wsum[i] = 0.0; wcnt[i] = 0; }
    for (int dx = -3; dx <= 3; dx++) {
      double psum[MAXIDS];
      int pcnt[MAXIDS];
      for (int i = 0; i < nu; i++) { psum[i] = 0.0; pcnt[i] = 0; }
      for (int dy = -3; dy <= 3; dy++)
        for (int dz = -3; dz <= 3; dz++) {
          long long w = vidx(n, x + dx, y + dy, z + dz);
          const int g = gid[w];
          for (int i = 0; i < nu; i++)
            if (uid[i] == g) { psum[i] = psum[i] + rho[w]; pcnt[i]++; }
        }
      for (int i = 0; i < nu; i++) { wsum[i] = wsum[i] + psum[i]; wcnt[i] += pcnt[i]; }
    }
    double rbar[MAXIDS];
    for (int i = 0; i < nu; i++) rbar[i] = wcnt[i] > 0 ? wsum[i] / (double)wcnt[i] : 0.0;
    /* sums over the order parameters held at v (src/pf_xrx.c:1096-1104) */
    double sum_rex = 0.0, sum1 = 0.0, hdef = 0.0;
    for (int s = 0; s < cnt[v]; s++) {
      const int id = ids[v * K + s];
      int i = 0;
      while (i < nu && uid[i] != id) i++;
      if (i < nu && wcnt[i] > 0 && rbar[i] > 0.0) {
        const double e = phi[v * K + s];
        const double h = e * e * e * (10.0 - 15.0 * e + 6.0 * e * e);
        sum_rex = sum_rex + e * e;
        sum1 = sum1 + h;
        hdef = hdef + h * rbar[i];
      }
    }
    int kid[MAXIDS], nk = 0;
    double kval[MAXIDS];
    for (int a = 0; a < nn; a++) {
      const int id = nid[a];
      int i = 0;
      while (i < nu && uid[i] != id) i++;
      if (i == nu || !(rbar[i] > 0.0)) continue;
      const double c = eta_of(ids, phi, cnt, K, v, id);
      const double f_r = eta_of(ids, phi, cnt, K, vidx(n, x + 1, y, z), id);
      const double f_l = eta_of(ids, phi, cnt, K, vidx(n, x - 1, y, z), id);
      const double f_f = eta_of(ids, phi, cnt, K, vidx(n, x, y + 1, z), id);
      const double f_b = eta_of(ids, phi, cnt, K, vidx(n, x, y - 1, z), id);
      const double f_u = eta_of(ids, phi, cnt, K, vidx(n, x, y, z + 1), id);
      const double f_d = eta_of(ids, phi, cnt, K, vidx(n, x, y, z - 1), id);
      const double e_lu = eta_of(ids, phi, cnt, K, vidx(n, x - 1, y, z + 1), id);
      const double e_lf = eta_of(ids, phi, cnt, K, vidx(n, x - 1, y - 1, z), id);
      const double e_ld = eta_of(ids, phi, cnt, K, vidx(n, x - 1, y, z - 1), id);
      const double e_lb = eta_of(ids, phi, cnt, K, vidx(n, x - 1, y + 1, z), id);
      const double e_rd = eta_of(ids, phi, cnt, K, vidx(n, x + 1, y, z - 1), id);
      const double e_ru = eta_of(ids, phi, cnt, K, vidx(n, x + 1, y, z + 1), id);
      const double e_rf = eta_of(ids, phi, cnt, K, vidx(n, x + 1, y - 1, z), id);
      const double e_rb = eta_of(ids, phi, cnt, K, vidx(n, x + 1, y + 1, z), id);
      const double e_cuf = eta_of(ids, phi, cnt, K, vidx(n, x, y - 1, z + 1), id);
      const double e_cdb = eta_of(ids, phi, cnt, K, vidx(n, x, y + 1, z - 1), id);
      const double e_cub = eta_of(ids, phi, cnt, K, vidx(n, x, y + 1, z + 1), id);
      const double e_cdf = eta_of(ids, phi, cnt, K, vidx(n, x, y - 1, z - 1), id);
      /* laplacian(), src/pf_xrx.c:6-9: faces 0.5, edges 0.125, centre -4.5 */
      const double lap = 0.5 * (f_r + f_l + f_f + f_b + f_u + f_d) +
                         0.125 * (e_lu + e_lf + e_ld + e_lb + e_rd + e_ru + e_rf + e_rb + e_cuf + e_cdb + e_cub + e_cdf) -
                         4.5 * c;
      const double h = c * c * c * (10.0 - 15.0 * c + 6.0 * c * c);
      const double dh = c * c * (30.0 - 60.0 * c + 30.0 * c * c);
      const double drive = sum1 > 0.0 ? edisl * dh * ((sum1 - h) * rbar[i] - (hdef - h * rbar[i])) / (sum1 * sum1) : 0.0;
      const double val = c - mcoef * (mwell * (c * c * c - c + 3.0 * c * (sum_rex - c * c)) - kappa * lap + drive);
      if (val > PF_KEEP) { kid[nk] = id; kval[nk] = val; nk++; }
    }
    /* keep the K largest (ties to the smaller id), stored sorted by id */
    while (nk > K) {
      int m = 0;
      for (int a = 1; a < nk; a++)
        if (kval[a] < kval[m] || (kval[a] == kval[m] && kid[a] > kid[m])) m = a;
      for (int a = m; a < nk - 1; a++) { kid[a] = kid[a + 1]; kval[a] = kval[a + 1]; }
      nk--;
    }
    cnt2[v] = nk;
    for (int s = 0; s < K; s++) {
      ids2[v * K + s] = s < nk ? kid[s] : 0;
      phi2[v * K + s] = s < nk ? kval[s] : 0.0;
    }
  }
}

/* grain id = argmax eta, ties to the smaller id; a voxel that lost every
   order parameter keeps its id */
static void pf_argmax(long long nv, int K, const int* ids, const double* phi, const int* cnt, int* gid) {
  for (long long v = 0; v < nv; v++) {
    double best = 0.0;
    int g = gid[v];
    for (int s = 0; s < cnt[v]; s++)
      if (phi[v * K + s] > best) { best = phi[v * K + s]; g = ids[v * K + s]; }
    gid[v] = g;
  }
}

int orc_pf_relax(const mth_params* p, const int* n, const int* grain, const double* rho, int substeps, int K,
                 int* grain_out, int* ids_out, double* phi_out, int* cnt_out) {
  const long long nv = (long long)n[0] * n[1] * n[2];
  double mcoef, kappa, mwell, edisl;
  orc_pf_coefficients(p, &mcoef, &kappa, &mwell, &edisl);
  int *ids = (int*)calloc((size_t)nv * K, sizeof(int)), *ids2 = (int*)calloc((size_t)nv * K, sizeof(int));
  double *phi = (double*)calloc((size_t)nv * K, sizeof(double)), *phi2 = (double*)calloc((size_t)nv * K, sizeof(double));
  int *cnt = (int*)calloc(nv, sizeof(int)), *cnt2 = (int*)calloc(nv, sizeof(int));
  if (!ids || !ids2 || !phi || !phi2 || !cnt || !cnt2) return MTH_ERR_NOMEM;
  /* initial state: one order parameter per voxel (src/pf_xrx.c:1533-1578) */
  for (long long v = 0; v < nv; v++) {
    ids[v * K] = grain[v];
    phi[v * K] = 1.0;
    cnt[v] = 1;
    grain_out[v] = grain[v];
  }
  for (int s = 0; s < substeps; s++) {
    pf_substep(n, K, ids, phi, cnt, ids2, phi2, cnt2, grain_out, rho, mcoef, kappa, mwell, edisl);
    int* ti = ids; ids = ids2; ids2 = ti;
    double* tp = phi; phi = phi2; phi2 = tp;
    int* tc = cnt; cnt = cnt2; cnt2 = tc;
    pf_argmax(nv, K, ids, phi, cnt, grain_out);
  }
  if (ids_out) memcpy(ids_out, ids, sizeof(int) * (size_t)nv * K);
  if (phi_out) memcpy(phi_out, phi, sizeof(double) * (size_t)nv * K);
  if (cnt_out) memcpy(cnt_out, cnt, sizeof(int) * (size_t)nv);
  free(ids); free(ids2); free(phi); free(phi2); free(cnt); free(cnt2);
  return MTH_OK;
}

/* ------------------------------------------------ PF <-> FFT grid transfer
 * InterpolateGrid / InterpolateGID (src/integrated.c:621-760) and the
 * coarse-graining of gID_new in Update_microstructure
 * (src/integrated.c:821-860): node-based coordinates x = i/(N-1) on [0,1]
 * (x0 = 0), source cell index floor(x/dx) with dx = 1/(Ns-1), upper corner
 * clamped to the last node.  The reference aborts (PError 1203) when
 * rounding puts a destination node past the last source node; here the last
 * cell is used.  An axis of one node maps everything to node 0. */
static void axis_pos(int i, int nd, int ns, int* i0, int* i1, double* s) {
  if (nd < 2 || ns < 2) { *i0 = 0; *i1 = 0; *s = 0.0; return; }
  const double dxd = 1.0 / (nd - 1), dxs = 1.0 / (ns - 1);
  const double x = 0.0 + (double)i * dxd;
  int ix = (int)floor(x / dxs);
  if (ix > ns - 1) ix = ns - 1;
  if (ix < 0) ix = 0;
  *s = x / dxs - (double)ix;
  *i0 = ix;
  *i1 = ix + 1 < ns ? ix + 1 : ns - 1;
}

/* Integer field: value of the nearest of the eight corners of the source
 * cell, first minimum in the order 000,100,110,010,001,101,111,011
 * (TrilinearInterpolationINT, src/integrated.c:496-565). */
void orc_resample_nearest(const int* ns, const int* src, const int* nd, int* dst) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nd[0]; i++)
    for (int j = 0; j < nd[1]; j++)
      for (int k = 0; k < nd[2]; k++) {
        int x0, x1, y0, y1, z0, z1;
        double sx, sy, sz;
        axis_pos(i, nd[0], ns[0], &x0, &x1, &sx);
        axis_pos(j, nd[1], ns[1], &y0, &y1, &sy);
        axis_pos(k, nd[2], ns[2], &z0, &z1, &sz);
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
        for (int c = 1; c < 8; c++)
          if (dist[m] > dist[c]) m = c;
        dst[((long long)i * nd[1] + j) * nd[2] + k] = src[((long long)cx[m] * ns[1] + cy[m]) * ns[2] + cz[m]];
      }
}

/* Double field: trilinear interpolation (TrilinearInterpolation,
 * src/integrated.c:567-619), terms in the reference's order. */
void orc_resample_trilinear(const int* ns, const double* src, const int* nd, double* dst) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nd[0]; i++)
    for (int j = 0; j < nd[1]; j++)
      for (int k = 0; k < nd[2]; k++) {
        int x0, x1, y0, y1, z0, z1;
        double sx, sy, sz;
        axis_pos(i, nd[0], ns[0], &x0, &x1, &sx);
        axis_pos(j, nd[1], ns[1], &y0, &y1, &sy);
        axis_pos(k, nd[2], ns[2], &z0, &z1, &sz);
#define V(a, b, c) src[((long long)(a) * ns[1] + (b)) * ns[2] + (c)]
        dst[((long long)i * nd[1] + j) * nd[2] + k] =
            V(x0, y0, z0) * (1.0 - sx) * (1.0 - sy) * (1.0 - sz) + V(x1, y0, z0) * sx * (1.0 - sy) * (1.0 - sz) +
            V(x0, y1, z0) * sy * (1.0 - sx) * (1.0 - sz) + V(x0, y0, z1) * sz * (1.0 - sy) * (1.0 - sx) +
            V(x1, y0, z1) * sx * (1.0 - sy) * sz + V(x0, y1, z1) * sy * (1.0 - sx) * sz +
            V(x1, y1, z0) * sx * (1.0 - sz) * sy + V(x1, y1, z1) * sx * sy * sz;
#undef V
      }
}

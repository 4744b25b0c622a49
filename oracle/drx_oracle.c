/*
 * drx_oracle.c -- ORACLE (test infrastructure only; never linked into the
 * product).
 *
 * CPU restatement, in FP64, of the dynamic-recrystallisation step of
 * M-THEMES: grain-boundary indicator (Gradient_ExchangeGrainID,
 * src/constitutive.c:724-873 and src/evolution.c:816-829), nucleation
 * (NucleationCheckDRX, src/integrated.c:161-494), the sparse
 * order-parameter Allen-Cahn relaxation (PF_XRX / Update_grid / Update_gID,
 * src/pf_xrx.c:6-66,895-1311,1469-1698), restated statement by statement
 * (section "phase field" below), and the grid transfer of InterpolateGrid
 * (src/integrated.c:496-760).
 *
 * Nucleation: a grain-boundary voxel (the reference's indicator, which skips
 * the -z face) of a crystal phase whose dislocation density exceeds
 * rho_nucleation nucleates with probability nucleation_prob per step, drawn
 * from a counter-based generator of (seed, step, voxel) (the reference's
 * static branch is the case nucleation_prob = 1 with a uniform threshold);
 * nuclei are numbered in voxel order and paint every voxel within squared
 * distance nucleus_radius, without periodic images (src/integrated.c:400),
 * later nuclei over earlier ones.
 *
 * Pinned against the reference's own functions, run on crafted inputs by
 * oracle/refshim/drx_harness.cc (tests/golden/pf_*.npz, nucl_*.npz,
 * interp_*.npz).  Compiled with -ffp-contract=off: every floating-point
 * operation is a separately rounded IEEE operation in the reference's order,
 * which the CUDA kernels reproduce (-fmad=false).
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

/* Grain-boundary indicator of src/evolution.c:816-829 from the checks of
 * Gradient_ExchangeGrainID (src/constitutive.c:724-873), periodic: 1 where
 * the +x, -x, +y, -y or +z neighbour belongs to another grain.  The
 * reference's "-z" check compares with the -y neighbour
 * (src/constitutive.c:808,831,853), so a difference across the -z face alone
 * does not mark a voxel. */
void orc_gb_indicator(const int* n, const int* grain, unsigned char* gb) {
  for (int x = 0; x < n[0]; x++)
    for (int y = 0; y < n[1]; y++)
      for (int z = 0; z < n[2]; z++) {
        long long v = vidx(n, x, y, z);
        int g = grain[v];
        int b = (grain[vidx(n, x + 1, y, z)] != g) | (grain[vidx(n, x - 1, y, z)] != g) |
                (grain[vidx(n, x, y + 1, z)] != g) | (grain[vidx(n, x, y - 1, z)] != g) |
                (grain[vidx(n, x, y, z + 1)] != g);
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

void orc_paint_nuclei(const int* n, int* grain, const long long* sites, int nn, int first_id, int radius2) {
  /* src/integrated.c:397-402: every voxel whose squared distance to the
   * nucleus is <= nucleus_radius, without periodic images */
  int r = 0;
  while ((r + 1) * (r + 1) <= radius2) r++;
  for (int k = 0; k < nn; k++) {
    long long v = sites[k];
    int x0 = (int)(v / ((long long)n[1] * n[2])), y0 = (int)((v / n[2]) % n[1]), z0 = (int)(v % n[2]);
    for (int dx = -r; dx <= r; dx++)
      for (int dy = -r; dy <= r; dy++)
        for (int dz = -r; dz <= r; dz++) {
          const int x = x0 + dx, y = y0 + dy, z = z0 + dz;
          if (x < 0 || x >= n[0] || y < 0 || y >= n[1] || z < 0 || z >= n[2]) continue;
          if (dx * dx + dy * dy + dz * dz <= radius2) grain[vidx(n, x, y, z)] = first_id + k;
        }
  }
}

/* ------------------------------------------------------------ phase field
 * Literal restatement of PF_XRX / Update_grid / Update_gID
 * (src/pf_xrx.c:6-66,895-1311,1469-1698) for one rank, statement by
 * statement where the result depends on it:
 *  - the grid carries three halo layers per side (l = L + 6), refilled from
 *    the periodic interior after every sweep (boundary_conditions,
 *    src/pf_xrx.c:253-679): halo lists are copies, so reads of a halo do not
 *    change the interior voxel it mirrors;
 *  - each voxel holds an ordered list of (id, eta); lookups follow
 *    PFdata::operator[] (src/PFgrid.h:70-90): a missing id takes over the
 *    last entry when that entry is below EPSILON, else a (id, 0) entry is
 *    appended -- reads of neighbours and of the voxel itself do this too,
 *    during the sweep, on the grid being read;
 *  - the sweep runs x, y, z over the interior; a voxel holding more than one
 *    entry when the sweep reaches it is updated, one holding a single entry
 *    copies its values of the ids in N(v) (src/pf_xrx.c:1235-1240); N(v) =
 *    ids with eta > EPSILON over the 3x3x3 block in scan order
 *    (src/pf_xrx.c:937-973);
 *  - stored-energy averages over the 7x7x7 window use the grain map of the
 *    start of the call (GID of PF_XRX: only its halos are refreshed,
 *    src/pf_xrx.c:683-893) and the energy buffer, summed in window order per
 *    held entry (src/pf_xrx.c:1052-1086) and written to the caller's rho_avg
 *    table, from which ids not held at v read what earlier voxels left
 *    (written at src/pf_xrx.c:1079-1086, read at :1202-1214);
 *  - a recrystallised id (> init_gid) that passes 0.5 at a voxel sets that
 *    voxel's stored energy to 100 for the rest of the call (src/pf_xrx.c:
 *    1217-1219); the Laplacian adds its twelve edge terms in the order its
 *    parameters are bound at the call (src/pf_xrx.c:6-9 against :1193-1198);
 *  - grain id = first maximum of the list, 0 when every eta <= 0
 *    (src/pf_xrx.c:11-66).
 * The GPU computes the same sweep in parallel passes (drx.cu); tests require
 * both to agree bit for bit in FP64. */
#define PF_OCAP 24

typedef struct {
  int n;
  int id[PF_OCAP];
  double v[PF_OCAP];
} pf_list;

/* PFdata::operator[]: slot of id j, taking over a weak last entry or
 * appending; -1 (and *over set) when the list is full */
static int pf_slot(pf_list* l, int j, int* over) {
  for (int k = 0; k < l->n; k++)
    if (l->id[k] == j) return k;
  if (l->n > 0 && l->v[l->n - 1] < PF_EPS) {
    l->id[l->n - 1] = j;
    return l->n - 1;
  }
  if (l->n == PF_OCAP) { *over = 1; return -1; }
  l->id[l->n] = j;
  l->v[l->n] = 0.0;
  return l->n++;
}
static double pf_rd(pf_list* l, int j, int* over) {
  int k = pf_slot(l, j, over);
  return k < 0 ? 0.0 : l->v[k];
}
static void pf_wr(pf_list* l, int j, double val, int* over) {
  int k = pf_slot(l, j, over);
  if (k >= 0) l->v[k] = val;
}

typedef struct {
  int L[3], l[3];
  size_t np;
} pf_geom;
static inline size_t pf_at(const pf_geom* g, int x, int y, int z) {
  return ((size_t)x * g->l[1] + y) * g->l[2] + z;
}
static inline int pf_src(int x, int L) { return ((x - 3) % L + L) % L + 3; }
static inline int pf_interior(const pf_geom* g, int x, int y, int z) {
  return x >= 3 && x < g->l[0] - 3 && y >= 3 && y < g->l[1] - 3 && z >= 3 && z < g->l[2] - 3;
}
/* halo lists := copies of their periodic interior sources */
static void pf_fill_halos(const pf_geom* g, pf_list* gd, int* over) {
  for (int x = 0; x < g->l[0]; x++)
    for (int y = 0; y < g->l[1]; y++)
      for (int z = 0; z < g->l[2]; z++) {
        if (pf_interior(g, x, y, z)) continue;
        pf_list* d = &gd[pf_at(g, x, y, z)];
        const pf_list* s = &gd[pf_at(g, pf_src(x, g->L[0]), pf_src(y, g->L[1]), pf_src(z, g->L[2]))];
        d->n = 0;
        for (int k = 0; k < s->n; k++) pf_wr(d, s->id[k], s->v[k], over);
      }
}
/* mesh_extend: halos of the energy and grain-id buffers from the interior */
static void pf_fill_halo_scalars(const pf_geom* g, double* e, int* gid) {
  for (int x = 0; x < g->l[0]; x++)
    for (int y = 0; y < g->l[1]; y++)
      for (int z = 0; z < g->l[2]; z++) {
        if (pf_interior(g, x, y, z)) continue;
        const size_t s = pf_at(g, pf_src(x, g->L[0]), pf_src(y, g->L[1]), pf_src(z, g->L[2]));
        e[pf_at(g, x, y, z)] = e[s];
        gid[pf_at(g, x, y, z)] = gid[s];
      }
}

/* one sweep of Update_grid over gd into tmp */
static int pf_sweep(const pf_geom* g, pf_list* gd, pf_list* tmp, const int* GID, double* E, double* table,
                    int table_len, int init_gid, double mcoef, double kappa, double mwell, double edisl, int* over) {
  const int l0 = g->l[0], l1 = g->l[1], l2 = g->l[2];
  for (size_t i = 0; i < g->np; i++) tmp[i].n = 0;
  for (int x = 3; x < l0 - 3; x++)
    for (int y = 3; y < l1 - 3; y++)
      for (int z = 3; z < l2 - 3; z++) {
        const size_t me_at = pf_at(g, x, y, z);
        int nid[MAXIDS], nn = 0;
        for (int i = x - 1; i <= x + 1; i++)
          for (int j = y - 1; j <= y + 1; j++)
            for (int m = z - 1; m <= z + 1; m++) {
              const pf_list* d = &gd[pf_at(g, i, j, m)];
              for (int k = 0; k < d->n; k++)
                if (d->v[k] > PF_EPS) {
                  int a = 0;
                  while (a < nn && nid[a] != d->id[k]) a++;
                  if (a == nn) {
                    if (nn == MAXIDS) { *over = 1; continue; }
                    nid[nn++] = d->id[k];
                  }
                }
            }
        pf_list* me = &gd[me_at];
        pf_list* out = &tmp[me_at];
        const int NN = me->n;
        if (NN > 1) {
          double avg[PF_OCAP];
          int cnt[PF_OCAP];
          for (int k = 0; k < NN; k++) { avg[k] = 0.0; cnt[k] = 0; }
          for (int i = x - 3; i <= x + 3; i++)
            for (int j = y - 3; j <= y + 3; j++)
              for (int m = z - 3; m <= z + 3; m++) {
                const size_t p = pf_at(g, i, j, m);
                for (int k = 0; k < NN; k++)
                  if (GID[p] == me->id[k]) { avg[k] = avg[k] + E[p]; cnt[k]++; }
              }
          for (int k = 0; k < NN; k++) {
            const int ix = me->id[k] - 1;
            if (ix < 0 || ix >= table_len) return MTH_ERR_ARG;
            table[ix] = 0.0;
            if (cnt[k] > 0) table[ix] = avg[k] / (double)cnt[k];
          }
          double sum_rex = 0.0, sum1 = 0.0, hdef = 0.0;
          for (int k = 0; k < NN; k++)
            if (cnt[k] > 0 && avg[k] > 0.0) {
              const double e = me->v[k];
              sum_rex = sum_rex + e * e;
              sum1 = sum1 + e * e * e * (10.0 - 15.0 * e + 6.0 * e * e);
              hdef = hdef + (e * e * e * (10.0 - 15.0 * e + 6.0 * e * e)) * (avg[k] / (double)cnt[k]);
            }
          for (int a = 0; a < nn; a++) {
            const int id = nid[a];
            const double c = pf_rd(me, id, over);
            const double h = c * c * c * (10.0 - 15.0 * c + 6.0 * c * c);
            const double dh = c * c * (30.0 - 60.0 * c + 30.0 * c * c);
#define NB(a_, b_, c_) pf_rd(&gd[pf_at(g, x + (a_), y + (b_), z + (c_))], id, over)
            const double right = NB(1, 0, 0), left = NB(-1, 0, 0), front = NB(0, 1, 0), back = NB(0, -1, 0);
            const double up = NB(0, 0, 1), down = NB(0, 0, -1);
            const double lu = NB(-1, 0, 1), ld = NB(-1, 0, -1), lf = NB(-1, -1, 0), lb = NB(-1, 1, 0);
            const double cuf = NB(0, -1, 1), cub = NB(0, 1, 1), cdf = NB(0, -1, -1), cdb = NB(0, 1, -1);
            const double ru = NB(1, 0, 1), rdn = NB(1, 0, -1), rf = NB(1, -1, 0), rb = NB(1, 1, 0);
#undef NB
            const double lap = 0.5 * (right + left + front + back + up + down) +
                               0.125 * (cuf + cdf + cub + cdb + ld + lu + lf + lb + ru + rb + rdn + rf) - 4.5 * c;
            const int ix = id - 1;
            if (ix < 0 || ix >= table_len) return MTH_ERR_ARG;
            const double ra = table[ix];
            if (ra > 0.0) {
              const double val = c - mcoef * (mwell * (c * c * c - c + 3.0 * c * (sum_rex - c * c)) - kappa * lap +
                                              edisl * dh * ((sum1 - h) * ra - (hdef - h * ra)) / (sum1 * sum1));
              if (id > init_gid && c < 0.5 && val > 0.5) E[me_at] = 100.0;
              if (val > PF_KEEP) pf_wr(out, id, val, over);
            }
          }
        } else if (NN == 1) {
          for (int a = 0; a < nn; a++) {
            const double val = pf_rd(me, nid[a], over);
            pf_wr(out, nid[a], val, over);
          }
        }
      }
  pf_fill_halos(g, tmp, over);
  return MTH_OK;
}

int orc_pf_relax(const mth_params* p, const int* n, const int* grain, const double* rho, int substeps, int init_gid,
                 double* table, int table_len, int* grain_out, int* cnt_out, int* ids_out, double* phi_out,
                 int kmax) {
  pf_geom g;
  for (int i = 0; i < 3; i++) { g.L[i] = n[i]; g.l[i] = n[i] + 6; }
  g.np = (size_t)g.l[0] * g.l[1] * g.l[2];
  double mcoef, kappa, mwell, edisl;
  orc_pf_coefficients(p, &mcoef, &kappa, &mwell, &edisl);
  pf_list* gd = (pf_list*)calloc(g.np, sizeof(pf_list));
  pf_list* tmp = (pf_list*)calloc(g.np, sizeof(pf_list));
  int* GID = (int*)calloc(g.np, sizeof(int));
  double* E = (double*)calloc(g.np, sizeof(double));
  if (!gd || !tmp || !GID || !E) { free(gd); free(tmp); free(GID); free(E); return MTH_ERR_NOMEM; }
  int over = 0, st = MTH_OK;
  for (int x = 0; x < n[0]; x++)
    for (int y = 0; y < n[1]; y++)
      for (int z = 0; z < n[2]; z++) {
        const size_t v = ((size_t)x * n[1] + y) * n[2] + z, q = pf_at(&g, x + 3, y + 3, z + 3);
        pf_wr(&gd[q], grain[v], 1.0, &over);
        GID[q] = grain[v];
        E[q] = rho[v];
        grain_out[v] = grain[v];
      }
  pf_fill_halos(&g, gd, &over);
  pf_fill_halo_scalars(&g, E, GID);
  for (int s = 0; s < substeps && st == MTH_OK; s++) {
    st = pf_sweep(&g, gd, tmp, GID, E, table, table_len, init_gid, mcoef, kappa, mwell, edisl, &over);
    pf_list* t = gd; gd = tmp; tmp = t;
    for (int x = 0; x < n[0]; x++)
      for (int y = 0; y < n[1]; y++)
        for (int z = 0; z < n[2]; z++) {
          const pf_list* d = &gd[pf_at(&g, x + 3, y + 3, z + 3)];
          double best = 0.0;
          int id = 0;
          for (int k = 0; k < d->n; k++)
            if (best < d->v[k]) { best = d->v[k]; id = d->id[k]; }
          grain_out[((size_t)x * n[1] + y) * n[2] + z] = id;
        }
    pf_fill_halo_scalars(&g, E, GID);
  }
  if (st == MTH_OK && over) st = MTH_ERR_UNSUPPORTED;
  if (st == MTH_OK && cnt_out) {
    for (int x = 0; x < n[0]; x++)
      for (int y = 0; y < n[1]; y++)
        for (int z = 0; z < n[2]; z++) {
          const size_t v = ((size_t)x * n[1] + y) * n[2] + z;
          const pf_list* d = &gd[pf_at(&g, x + 3, y + 3, z + 3)];
          cnt_out[v] = d->n;
          for (int k = 0; k < kmax; k++) {
            if (ids_out) ids_out[v * kmax + k] = k < d->n ? d->id[k] : 0;
            if (phi_out) phi_out[v * kmax + k] = k < d->n ? d->v[k] : 0.0;
          }
          if (d->n > kmax) st = MTH_ERR_UNSUPPORTED;
        }
  }
  free(gd); free(tmp); free(GID); free(E);
  return st;
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

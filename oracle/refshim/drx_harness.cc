/*
 * drx_harness.cc -- drives the reference's own dynamic-recrystallisation
 * functions on crafted inputs, one case per process, to make golden vectors
 * for the oracle.  Linked by oracle/build_ref.sh with the reference's
 * translation units (src/pf_xrx.c compiled with MTH_PF_HOOK, see
 * mth_ref_prelude.h) into oracle/_ref/drx_ref.  Test infrastructure only.
 *
 *   drx_ref pf     IN OUT   PF_XRX (src/pf_xrx.c:1469-1698), NumPE = 1:
 *                           every substep's (id, eta) lists in stored
 *                           order, then gID_new and the rho_avg table
 *   drx_ref nucl   IN OUT   Gradient_ExchangeGrainID
 *                           (src/constitutive.c:724-873), the GB indicator
 *                           of src/evolution.c:816-829, and
 *                           NucleationCheckDRX (src/integrated.c:161-494)
 *                           with Nucl_Static_Flag = 1 (threshold kappa_drx)
 *   drx_ref interp IN OUT   InterpolateGrid (src/integrated.c:674-760):
 *                           grain ids by TrilinearInterpolationINT, rho_tot
 *                           by TrilinearInterpolation onto CellDim_pf
 *   drx_ref upd    IN OUT   Update_microstructure (src/integrated.c:801-1807)
 *                           on the mechanical grid, over a sequence of
 *                           relaxed grain maps: the grain map and the
 *                           membership counters gID_rex and growth after
 *                           each call (growth == 1 marks the voxels
 *                           src/evolution.c:1132-1145 resets)
 *
 * IN/OUT are flat little-endian binaries whose layout is written next to
 * each mode below (tests/golden/make_golden.py writes and reads them).
 * One process per case: Update_grid keeps its scratch grid in a
 * function-local static sized by its first call (src/pf_xrx.c:899).
 */
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include "evp.h"

void Gradient_ExchangeGrainID(void);

static FILE* g_out = nullptr;

template <typename T>
static std::vector<T> rd(FILE* f, size_t n) {
  std::vector<T> v(n);
  if (n && fread(v.data(), sizeof(T), n, f) != n) {
    fprintf(stderr, "drx_ref: short input\n");
    exit(2);
  }
  return v;
}
template <typename T>
static void wr(const T* p, size_t n) {
  if (n) fwrite(p, sizeof(T), n, g_out);
}

/* PF hook: the interior (x, y, z in [3, l-3)) of the grid just swapped in,
 * in data order: counts, then ids, then values */
void mth_ref_pf_after_substep(MthPFgrid3DBase& g, int l_x, int l_y, int l_z) {
  std::vector<int> cnt, ids;
  std::vector<double> val;
  for (int x = 3; x < l_x - 3; x++)
    for (int y = 3; y < l_y - 3; y++)
      for (int z = 3; z < l_z - 3; z++) {
        PFdata& d = g[x][y][z];
        cnt.push_back(d.nonzero());
        for (int k = 0; k < d.nonzero(); k++) {
          ids.push_back(d.index(k));
          val.push_back(d.value(k));
        }
      }
  int tot = (int)ids.size();
  wr(cnt.data(), cnt.size());
  wr(&tot, 1);
  wr(ids.data(), ids.size());
  wr(val.data(), val.size());
}

/* IN:  int32 L[3], steps, init_gid, n_avg, count;
 *      float64 E_gb, M_gb, mu, bb, alpha, pf_length_scale, pf_time_step;
 *      int32 gID[N]; float64 rho[N]; float64 rho_avg[n_avg]
 * OUT: per substep {int32 cnt[N]; int32 tot; int32 ids[tot]; float64 val[tot]};
 *      int32 gID_new[N]; float64 rho_avg[n_avg] */
static int run_pf(FILE* in) {
  std::vector<int> h = rd<int>(in, 7);
  std::vector<double> c = rd<double>(in, 7);
  const int L0 = h[0], L1 = h[1], L2 = h[2], steps = h[3], n_avg = h[5], count = h[6];
  const size_t n = (size_t)L0 * L1 * L2;
  init_gid = h[4];
  pf_length_scale = c[5];
  pf_time_step = c[6];
  std::vector<int> gid = rd<int>(in, n);
  std::vector<double> rho = rd<double>(in, n);
  std::vector<double> avg = rd<double>(in, (size_t)n_avg);
  std::vector<int> gnew(n, 0);
  PF_XRX(L0, L1, L2, 1, 0, c[0], c[1], c[2], c[3], c[4], gid.data(), rho.data(), steps, gnew.data(), count, 0,
         avg.data());
  wr(gnew.data(), n);
  wr(avg.data(), avg.size());
  return 0;
}

/* IN:  int32 dims[3], n_grains, nucleus_radius, step;
 *      int32 grain[N]; int32 phase[N] (1-based); float64 rho_s0[N];
 *      float64 kappa[N]; float64 rot[N*9] (crystal -> sample, row-major)
 * OUT: int32 n_new; int32 grain[N]; int32 gb[N]; float64 diff_rho[N];
 *      n_new x {int32 id; float64 t1, Phi, t2} (the new gID_list entries) */
static int run_nucl(FILE* in) {
  std::vector<int> h = rd<int>(in, 6);
  CellDim[0] = h[0]; CellDim[1] = h[1]; CellDim[2] = h[2];
  const int ng = h[3];
  nucleus_radius = h[4];
  const int step = h[5];
  const size_t n = (size_t)h[0] * h[1] * h[2];
  Nxyz = (int)n; lnx = h[0]; lxs = 0; lsize = (int)n; mpirank = 0; NumPE = 1;
  Nucl_Static_Flag = 1;
  std::vector<int> grain = rd<int>(in, n), phase = rd<int>(in, n);
  std::vector<double> rs = rd<double>(in, n), kap = rd<double>(in, n), rot = rd<double>(in, n * 9);
  static int nsys[2] = {NSYSMX, 0};
  nSYS = nsys;
  grain_f = grain.data();
  phase_f = phase.data();
  AllocMem(TranMat_xt2sa, n, ten2nd);
  for (size_t v = 0; v < n; v++)
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) TranMat_xt2sa[v][i][j] = rot[v * 9 + i * 3 + j];
  real** arr[5];
  for (int a = 0; a < 5; a++) {
    AllocMem(arr[a], n, real*);
    for (size_t v = 0; v < n; v++) arr[a][v] = (real*)calloc(NSYSMX, sizeof(real));
  }
  rho_s = arr[0]; rho_m = arr[1]; rho_g1 = arr[2]; rho_g2 = arr[3]; rho_g3 = arr[4];
  for (size_t v = 0; v < n; v++) rho_s[v][0] = rs[v];
  AllocMem(rho_tot, n, real);
  AllocMem(diff_rho, n, real);
  kappa_drx = kap.data();
  std::vector<double> kc(n, 1.0);
  GB_indicator = (int*)calloc(n, sizeof(int));
  gID_rex = (int*)calloc(n, sizeof(int));
  nuclei = (int*)calloc(n, sizeof(int));
  swap_check = (int*)calloc(n, sizeof(int));
  GB_type = (int*)calloc(n, sizeof(int));
  int** chk[3];
  for (int a = 0; a < 3; a++) {
    AllocMem(chk[a], n, int*);
    for (size_t v = 0; v < n; v++) chk[a][v] = (int*)calloc(2, sizeof(int));
  }
  GB_checkX = chk[0]; GB_checkY = chk[1]; GB_checkZ = chk[2];
  const size_t plane = (size_t)h[1] * h[2];
  local_pxpG_send = (int*)calloc(plane, sizeof(int));
  local_pxmG_send = (int*)calloc(plane, sizeof(int));
  local_pxpG_recv = (int*)calloc(plane, sizeof(int));
  local_pxmG_recv = (int*)calloc(plane, sizeof(int));
  gID_list.clear();
  for (int g = 1; g <= ng; g++) {
    G_Info e = {g, 0.0, 0.0, 0.0};
    gID_list.push_back(e);
  }
  Gradient_ExchangeGrainID();
  /* the GB indicator as src/evolution.c:816-829 forms it */
  for (size_t v = 0; v < n; v++) {
    int s = GB_checkX[v][0] + GB_checkX[v][1] + GB_checkY[v][0] + GB_checkY[v][1] + GB_checkZ[v][0] + GB_checkZ[v][1];
    GB_indicator[v] = s < 6 ? 1 : 0;
  }
  int nn = NucleationCheckDRX(step, kc.data(), 1.0);
  wr(&nn, 1);
  wr(grain_f, n);
  wr(GB_indicator, n);
  wr(diff_rho, n);
  for (size_t k = (size_t)ng; k < gID_list.size(); k++) {
    wr(&gID_list[k].ID, 1);
    wr(&gID_list[k].t1, 1);
    wr(&gID_list[k].Phi, 1);
    wr(&gID_list[k].t2, 1);
  }
  return 0;
}

/* IN:  int32 CellDim[3], CellDim_pf[3]; int32 grain[N]; float64 rho_tot[N]
 * OUT: int32 grain_pf[Npf]; float64 rho_pf[Npf] */
static int run_interp(FILE* in) {
  std::vector<int> h = rd<int>(in, 6);
  for (int i = 0; i < 3; i++) { CellDim[i] = h[i]; CellDim_pf[i] = h[3 + i]; }
  const size_t n = (size_t)h[0] * h[1] * h[2], npf = (size_t)h[3] * h[4] * h[5];
  Nxyz = (int)n; lnx = h[0]; lxs = 0; lsize = (int)n; mpirank = 0; NumPE = 1;
  std::vector<int> grain = rd<int>(in, n);
  std::vector<double> rt = rd<double>(in, n);
  grain_f = grain.data();
  rho_tot = rt.data();
  grain_f_drx = (int*)calloc(npf, sizeof(int));
  rho_tot_drx = (real*)calloc(npf, sizeof(real));
  InterpolateGrid();
  wr(grain_f_drx, npf);
  wr(rho_tot_drx, npf);
  return 0;
}

/* IN:  int32 dims[3], n_ids, n_calls; int32 ids[n_ids] (gID_list);
 *      int32 grain[N], gid_rex[N], growth[N] (state before the first call);
 *      n_calls x {int32 paint[N]; int32 gID_new[N]}: before each call the
 *      voxels with paint != 0 take that id and gID_rex = 1, as the nuclei
 *      NucleationCheckDRX paints (src/integrated.c:397-404)
 * OUT: n_calls x {int32 grain[N]; int32 gid_rex[N]; int32 growth[N]} */
static int run_upd(FILE* in) {
  std::vector<int> h = rd<int>(in, 5);
  CellDim[0] = h[0]; CellDim[1] = h[1]; CellDim[2] = h[2];
  const int n_ids = h[3], n_calls = h[4];
  const size_t n = (size_t)h[0] * h[1] * h[2];
  Nxyz = (int)n; lnx = h[0]; lxs = 0; lsize = (int)n; mpirank = 0; NumPE = 1;
  DRX_Interpolation_Flag = 0;
  std::vector<int> ids = rd<int>(in, (size_t)n_ids);
  std::vector<int> grain = rd<int>(in, n), rex = rd<int>(in, n), grow = rd<int>(in, n);
  std::vector<int> gnew(n), gfn(n);
  grain_f = grain.data();
  gID_rex = rex.data();
  growth = grow.data();
  gID_new = gnew.data();
  grain_f_new = gfn.data();
  GB_type = (int*)calloc(n, sizeof(int));
  int** chk[3];
  for (int a = 0; a < 3; a++) {
    AllocMem(chk[a], n, int*);
    for (size_t v = 0; v < n; v++) chk[a][v] = (int*)calloc(2, sizeof(int));
  }
  GB_checkX = chk[0]; GB_checkY = chk[1]; GB_checkZ = chk[2];
  const size_t plane = (size_t)h[1] * h[2];
  local_pxpG_send = (int*)calloc(plane, sizeof(int));
  local_pxmG_send = (int*)calloc(plane, sizeof(int));
  local_pxpG_recv = (int*)calloc(plane, sizeof(int));
  local_pxmG_recv = (int*)calloc(plane, sizeof(int));
  gID_list.clear();
  for (int k = 0; k < n_ids; k++) {
    G_Info e = {ids[k], 0.0, 0.0, 0.0};
    gID_list.push_back(e);
  }
  for (int call = 0; call < n_calls; call++) {
    std::vector<int> paint = rd<int>(in, n);
    for (size_t v = 0; v < n; v++)
      if (paint[v] != 0) {
        grain_f[v] = paint[v];
        gID_rex[v] = 1;
      }
    std::vector<int> g = rd<int>(in, n);
    memcpy(gID_new, g.data(), sizeof(int) * n);
    Update_microstructure();
    wr(grain_f, n);
    wr(gID_rex, n);
    wr(growth, n);
  }
  return 0;
}

int main(int argc, char** argv) {
  if (argc != 4) {
    fprintf(stderr, "usage: drx_ref pf|nucl|interp|upd IN OUT\n");
    return 2;
  }
  FILE* in = fopen(argv[2], "rb");
  g_out = fopen(argv[3], "wb");
  if (!in || !g_out) {
    fprintf(stderr, "drx_ref: cannot open files\n");
    return 2;
  }
  int rc = 2;
  if (!strcmp(argv[1], "pf")) rc = run_pf(in);
  else if (!strcmp(argv[1], "nucl")) rc = run_nucl(in);
  else if (!strcmp(argv[1], "interp")) rc = run_interp(in);
  else if (!strcmp(argv[1], "upd")) rc = run_upd(in);
  fclose(in);
  fclose(g_out);
  return rc;
}

/*
 * mth_io.c -- readers for the reference's three input files, in plain C.
 *
 *  - input.in namelist: GetNameList (src/io.c:96-164).  Lines starting with
 *    '#' or '\n' are skipped, the first token is the key, values follow
 *    separated by ", \t\n"; reading stops at the first line with no token;
 *    unknown keys are ignored; a key given twice keeps its first values.
 *  - .sx single-crystal file: PlasticInit (src/init.c:52-231), the same
 *    fixed line layout.  As in the reference, hself/hlat come from the last
 *    mode block of the file and the systems from the last selected mode.
 *  - voxel microstructure: InitMicroStruct (src/init.c:255-270), one line
 *    "phi1 Phi phi2 i j k grain phase" per voxel, z fastest, indices checked.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "../../include/mth.h"

typedef enum { K_I, K_R, K_S } ktype;
typedef struct {
  const char* name;
  ktype type;
  int len;
  void* ptr;
  int seen;
} key_t_;

/* values the EVPFFT/PF solve does not need but the namelist carries */
static int s_ntype[2], s_printctl[2], s_texflag, s_nuclr, s_celldim_pf[3], s_randseed;
static double s_el1[4], s_el2[4];
/* dislocation-density block (src/io.c:47-68): per-phase pairs, phase 1 kept */
static double s_a0[2], s_qslip[2], s_qbulk[2], s_cc[8][2], s_inter[6][2];

mth_status mth_read_namelist(const char* path, mth_params* p, char* slip1, char* slip2, char* ms, size_t cap) {
  if (!path || !p) return MTH_ERR_ARG;
  FILE* fp = fopen(path, "r");
  if (!fp) return MTH_ERR_IO;
  char sx1[200] = "", sx2[200] = "", msf[200] = "";
  double dummy_r;
  (void)dummy_r;
  key_t_ keys[] = {
      {"CellDim", K_I, 3, p->cell_dim, 0},
      {"N_phases", K_I, 1, &p->n_phases, 0},
      {"Type_phases", K_I, 2, s_ntype, 0},
      {"TimeStep", K_R, 1, &p->time_step, 0},
      {"N_steps", K_I, 1, &p->n_steps, 0},
      {"Update_Flag", K_I, 1, &p->update_flag, 0},
      {"Hard_Flag", K_I, 1, &p->hard_flag, 0},
      {"Tex_Flag", K_I, 1, &s_texflag, 0},
      {"IterMax", K_I, 1, &p->iter_max, 0},
      {"PrintControl", K_I, 2, s_printctl, 0},
      {"Err", K_R, 1, &p->err, 0},
      {"VelGrad_BC_Flag", K_I, 6, p->velgrad_bc_flag, 0},
      {"VelGrad_BC", K_R, 6, p->velgrad_bc, 0},
      {"Stress_BC_Flag", K_I, 6, p->stress_bc_flag, 0},
      {"Stress_BC", K_R, 6, p->stress_bc, 0},
      {"ElastBC", K_I, 1, &p->elast_bc, 0},
      {"ElastConst_PhaseI", K_R, 4, s_el1, 0},
      {"ElastConst_PhaseII", K_R, 4, s_el2, 0},
      {"Slip_PhaseI", K_S, 1, sx1, 0},
      {"Slip_PhaseII", K_S, 1, sx2, 0},
      {"initial_ms", K_S, 1, msf, 0},
      {"nucleus_radius", K_I, 1, &s_nuclr, 0},
      {"CellDim_pf", K_I, 3, s_celldim_pf, 0},
      {"RandSeed", K_I, 1, &s_randseed, 0},
      {"E_gb", K_R, 1, &p->e_gb, 0},
      {"M_gb", K_R, 1, &p->m_gb, 0},
      {"Scale_Fdeform", K_R, 1, &p->stored_energy_scale, 0},
      {"pf_length_scale", K_R, 1, &p->pf_length_scale, 0},
      {"pf_time_step", K_R, 1, &p->pf_time_step, 0},
      {"a0", K_R, 2, s_a0, 0},
      {"L0", K_R, 1, &p->dd_L0, 0},
      {"T__K", K_R, 1, &p->dd_T, 0},
      {"Q_slip", K_R, 2, s_qslip, 0},
      {"Q_bulk", K_R, 2, s_qbulk, 0},
      {"C_1", K_R, 2, s_cc[0], 0},
      {"C_2", K_R, 2, s_cc[1], 0},
      {"C_3", K_R, 2, s_cc[2], 0},
      {"C_4", K_R, 2, s_cc[3], 0},
      {"C_5", K_R, 2, s_cc[4], 0},
      {"C_6", K_R, 2, s_cc[5], 0},
      {"C_7", K_R, 2, s_cc[6], 0},
      {"C_8", K_R, 2, s_cc[7], 0},
      {"Selfinter", K_R, 2, s_inter[0], 0},
      {"Coplanar", K_R, 2, s_inter[1], 0},
      {"CrossSlip", K_R, 2, s_inter[2], 0},
      {"GlissileJunction", K_R, 2, s_inter[3], 0},
      {"HirthLock", K_R, 2, s_inter[4], 0},
      {"LomerCottrellLock", K_R, 2, s_inter[5], 0},
      {"rho_SSD_initial", K_R, 1, &p->dd_rho_ssd0, 0},
      {"D_0", K_R, 1, &p->dd_d0, 0},
  };
  const int nk = (int)(sizeof(keys) / sizeof(keys[0]));
  char buff[200];
  while (1) {
    if (!fgets(buff, 200, fp)) break;
    if (buff[0] == '#' || buff[0] == '\n') continue;
    char* save = NULL;
    char* tok = strtok_r(buff, " \t\n", &save);
    if (!tok) break;
    for (int k = 0; k < nk; k++) {
      if (strcmp(tok, keys[k].name) != 0) continue;
      if (keys[k].seen) break;
      keys[k].seen = 1;
      for (int j = 0; j < keys[k].len; j++) {
        char* t = strtok_r(NULL, ", \t\n", &save);
        if (!t) break;
        if (keys[k].type == K_I) ((int*)keys[k].ptr)[j] = (int)atol(t);
        else if (keys[k].type == K_R) ((double*)keys[k].ptr)[j] = atof(t);
        else { strncpy((char*)keys[k].ptr, t, 199); ((char*)keys[k].ptr)[199] = 0; }
      }
      break;
    }
  }
  fclose(fp);
  p->phase[0].type = s_ntype[0];
  p->phase[1].type = s_ntype[1];
  p->phase[0].c11 = s_el1[0]; p->phase[0].c12 = s_el1[1]; p->phase[0].c44 = s_el1[2];
  p->phase[1].c11 = s_el2[0]; p->phase[1].c12 = s_el2[1]; p->phase[1].c44 = s_el2[2];
  p->nucleus_radius = s_nuclr;
  if (s_randseed) p->seed = (uint64_t)s_randseed;
  for (int i = 0; i < 3; i++) p->pf_cell_dim[i] = s_celldim_pf[i];
  p->dd_a0 = s_a0[0];
  p->dd_q_slip = s_qslip[0];
  p->dd_q_bulk = s_qbulk[0];
  for (int k = 0; k < 8; k++) p->dd_c[k] = s_cc[k][0];
  for (int k = 0; k < 6; k++) p->dd_chi[k] = s_inter[k][0];
  p->dd_nu = s_el1[3];
  if (slip1 && cap) { strncpy(slip1, sx1, cap - 1); slip1[cap - 1] = 0; }
  if (slip2 && cap) { strncpy(slip2, sx2, cap - 1); slip2[cap - 1] = 0; }
  if (ms && cap) { strncpy(ms, msf, cap - 1); ms[cap - 1] = 0; }
  return MTH_OK;
}

static int gl(char* b, FILE* fp) { return fgets(b, 80, fp) != NULL; }

mth_status mth_read_sx(const char* path, mth_params* p, int iphase) {
  if (!path || !p || iphase < 0 || iphase >= MTH_NPH_MAX) return MTH_ERR_ARG;
  FILE* fp = fopen(path, "r");
  if (!fp) return MTH_ERR_IO;
  mth_phase* ph = &p->phase[iphase];
  char b[80] = {0};
  int n_modes_max = 0, n_modes = 0, imode[16];
  int ok = 1;
  ok &= gl(b, fp);                     /* header */
  ok &= gl(b, fp);                     /* XtalSys */
  ok &= gl(b, fp); ok &= gl(b, fp);
  ok &= gl(b, fp);                     /* XtalAxis */
  ok &= gl(b, fp); ok &= gl(b, fp);
  ok &= gl(b, fp); if (sscanf(b, "%d", &n_modes_max) != 1) ok = 0;
  ok &= gl(b, fp); ok &= gl(b, fp);
  ok &= gl(b, fp); if (sscanf(b, "%d", &n_modes) != 1) ok = 0;
  if (!ok || n_modes < 1 || n_modes > 16) { fclose(fp); return MTH_ERR_IO; }
  ok &= gl(b, fp); ok &= gl(b, fp);
  for (int i = 0; i < n_modes; i++) { ok &= gl(b, fp); if (sscanf(b, "%d", &imode[i]) != 1) ok = 0; }
  ok &= gl(b, fp);
  int nsmx = 0, isect = 0, matched_any = 0;
  double nrs = 0, gamd0 = 0, twsh = 0, t0f = 0, t0b = 0, t1 = 0, th0 = 0, th1 = 0, hs = 0, hl = 0;
  for (int i = 0; i < n_modes_max && ok; i++) {
    int mx = -1, match = 0;
    ok &= gl(b, fp);
    if (sscanf(b, "%*s %*s %d %*s", &mx) < 1) ok = 0;
    for (int j = 0; j < n_modes; j++) if (mx == imode[j]) { match = 1; break; }
    ok &= gl(b, fp); ok &= gl(b, fp);
    if (sscanf(b, "%d %lf %lf %lf %d", &nsmx, &nrs, &gamd0, &twsh, &isect) < 3) ok = 0;
    ok &= gl(b, fp); ok &= gl(b, fp);
    if (sscanf(b, "%lf %lf %lf %lf %lf", &t0f, &t0b, &t1, &th0, &th1) != 5) ok = 0;
    ok &= gl(b, fp); ok &= gl(b, fp);
    if (sscanf(b, "%lf %lf", &hs, &hl) != 2) ok = 0;
    ok &= gl(b, fp);
    if (!ok || nsmx < 1 || nsmx > MTH_NSYS_MAX) { ok = 0; break; }
    for (int j = 0; j < nsmx; j++) {
      ok &= gl(b, fp);
      if (match) {
        double* n = ph->bn[j];
        double* d = ph->bb[j];
        if (sscanf(b, "%lf %lf %lf %lf %lf %lf", &n[0], &n[1], &n[2], &d[0], &d[1], &d[2]) != 6) ok = 0;
      }
    }
    if (match) {
      matched_any = 1;
      ph->nsys = nsmx;
      ph->nrs = nrs; ph->gamd0 = gamd0;
      ph->tau0f = t0f; ph->tau0b = t0b; ph->tau1 = t1; ph->thet0 = th0; ph->thet1 = th1;
    }
  }
  fclose(fp);
  if (!ok || !matched_any) return MTH_ERR_IO;
  ph->hself = hs;   /* last block of the file, src/init.c:205-215 */
  ph->hlat = hl;
  return MTH_OK;
}

mth_status mth_read_microstructure(const char* path, const int cell_dim[3], int* grain, int* phase, double* euler) {
  if (!path || !cell_dim || !grain || !phase || !euler) return MTH_ERR_ARG;
  FILE* fp = fopen(path, "r");
  if (!fp) return MTH_ERR_IO;
  char b[80];
  long long idx = 0;
  for (int x = 0; x < cell_dim[0]; x++)
    for (int y = 0; y < cell_dim[1]; y++)
      for (int z = 0; z < cell_dim[2]; z++, idx++) {
        double e0, e1, e2;
        int ii, jj, kk, g, ph;
        if (!fgets(b, 80, fp) || sscanf(b, "%lf %lf %lf %d %d %d %d %d", &e0, &e1, &e2, &ii, &jj, &kk, &g, &ph) != 8) {
          fclose(fp);
          return MTH_ERR_IO;
        }
        long long id = ((long long)(ii - 1) * cell_dim[1] + jj - 1) * cell_dim[2] + kk - 1;
        if (id != idx) { fclose(fp); return MTH_ERR_IO; }
        grain[idx] = g;
        phase[idx] = ph;
        euler[3 * idx] = e0;
        euler[3 * idx + 1] = e1;
        euler[3 * idx + 2] = e2;
      }
  fclose(fp);
  return MTH_OK;
}

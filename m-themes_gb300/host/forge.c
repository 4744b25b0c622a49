/*
 * forge.c -- C driver with the shape of the reference's main (src/evp.c:7-32):
 * read the namelist given on the command line, set up, evolve N_steps
 * mechanical steps, tear down.  The solve goes through the C-ABI of
 * include/mth.h; the per-step scalars go to vm.out in the reference's columns
 * (TIME EVM EVMP DVM DVMP SVM SVM_1, src/init.c:497 and
 * src/evolution.c:1621-1625), and the macroscopic stress-strain curve (which
 * the reference keeps only in globals) to ss.out.  With --iout-every K the
 * elastic-strain and stress fields are written every K steps in the format
 * of WriteElsMPI / WriteSigMPI (src/io.c:322-437; the reference's print
 * block at src/evolution.c:1633-1648 writes the same two every 500 steps),
 * in the background while the next steps run.
 *
 * Usage: forge input.in [--mixed] [--iout-every K] [--dd | --dd-cu]
 * --dd runs the dislocation-density law (the reference's DD_BASED_FLAG build)
 * with the namelist's DD block and writes dd.out; --dd-cu also applies the
 * DD_CU switch of the shipped flags (fixed Cu elastic constants), which is
 * what the reference's test_run/ is run with.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "../../include/mth.h"

int main(int argc, char** argv) {
  if (argc < 2) {
    fprintf(stderr, "usage: %s input.in [--mixed] [--iout-every K] [--dd | --dd-cu]\n", argv[0]);
    return 2;
  }
  mth_params p;
  memset(&p, 0, sizeof(p));
  char sx1[256], sx2[256], ms[256];
  if (mth_read_namelist(argv[1], &p, sx1, sx2, ms, sizeof(sx1)) != MTH_OK) {
    fprintf(stderr, "Input file not found!\n");
    return 1;
  }
  int iout_every = 0;
  for (int i = 2; i < argc; i++) {
    if (!strcmp(argv[i], "--mixed")) p.precision = MTH_MIXED;
    else if (!strcmp(argv[i], "--iout-every") && i + 1 < argc) iout_every = atoi(argv[++i]);
    else if (!strcmp(argv[i], "--dd")) p.flow_law = 1;
    else if (!strcmp(argv[i], "--dd-cu")) p.flow_law = 2;   /* resolved after the .sx files are read */
  }
  if (p.n_phases >= 1 && p.phase[0].type == 0 && mth_read_sx(sx1, &p, 0) != MTH_OK) {
    fprintf(stderr, "cannot read %s\n", sx1);
    return 1;
  }
  if (p.n_phases == 2 && p.phase[1].type == 0 && mth_read_sx(sx2, &p, 1) != MTH_OK) {
    fprintf(stderr, "cannot read %s\n", sx2);
    return 1;
  }
  if (p.flow_law == 2) {
    /* the DD_CU switch of the reference's shipped flags: fixed Cu elastic
       constants replace input.in's (src/init.c:821-825) */
    p.flow_law = 1;
    p.phase[0].c11 = 241.1674 * 1000;
    p.phase[0].c12 = 89.1989 * 1000;
    p.phase[0].c44 = 151.9685 * 1000;
  }
  size_t nv = (size_t)p.cell_dim[0] * p.cell_dim[1] * p.cell_dim[2];
  int* grain = (int*)malloc(sizeof(int) * nv);
  int* phase = (int*)malloc(sizeof(int) * nv);
  double* euler = (double*)malloc(sizeof(double) * 3 * nv);
  if (!grain || !phase || !euler || mth_read_microstructure(ms, p.cell_dim, grain, phase, euler) != MTH_OK) {
    fprintf(stderr, "Error in reading microstructure data file %s\n", ms);
    return 1;
  }
  mth_ctx* ctx = NULL;
  mth_status s = mth_create(&p, &ctx);
  if (s == MTH_OK) s = mth_upload_microstructure(ctx, grain, phase, euler, nv);
  if (s != MTH_OK) {
    fprintf(stderr, "set-up failed (%d): %s\n", (int)s, mth_last_error());
    return 1;
  }
  FILE* vm = fopen("vm.out", "w");
  FILE* ss = fopen("ss.out", "w");
  FILE* dd = p.flow_law == 1 ? fopen("dd.out", "w") : NULL;
  fprintf(vm, "TIME\tEVM\tEVMP\tDVM\tDVMP\tSVM\tSVMSVM_1\n");
  if (dd) fprintf(dd, "TIME\tEVM\tDD_F\tDD_P\tDD_s\tDD_m\tDD_g\n");   /* src/init.c:499 */
  fprintf(ss, "STEP\tITER\tTIME\tE11\tE22\tE33\tS11\tS22\tS33\tERRS\tERRE\n");
  for (int istep = 0; istep < p.n_steps; istep++) {
    mth_step_report r;
    s = mth_step(ctx, &r);
    if (s != MTH_OK) {
      fprintf(stderr, "step %d failed (%d): %s\n", istep, (int)s, mth_last_error());
      break;
    }
    fprintf(vm, "%e\t%e\t%e\t%e\t%e\t%e\t%e\n", r.time, r.e_vm, r.evmp, r.d_vm, r.dvmp, r.s_vm, r.s_vm1);
    fprintf(ss, "%d\t%d\t%e\t%.9e\t%.9e\t%.9e\t%.9e\t%.9e\t%.9e\t%e\t%e\n", istep, r.iterations, r.time,
            r.disgrad_avg[0][0], r.disgrad_avg[1][1], r.disgrad_avg[2][2], r.sig_avg[0][0], r.sig_avg[1][1],
            r.sig_avg[2][2], r.err_s, r.err_e);
    if (dd) {   /* src/evolution.c:1566-1569 */
      fprintf(dd, "%e\t%e", r.time, r.e_vm);
      for (int k = 0; k < 7; k++) fprintf(dd, "\t%e", r.dd_avg[k]);
      fprintf(dd, "\n");
      fflush(dd);
    }
    fflush(vm);
    fflush(ss);
    if (iout_every > 0 && istep % iout_every == 0) {
      s = mth_write_iout(ctx, MTH_IOUT_ELS, "els", istep);
      if (s == MTH_OK) s = mth_write_iout(ctx, MTH_IOUT_SIG, "sig", istep);
      if (s != MTH_OK) {
        fprintf(stderr, "field files of step %d failed (%d): %s\n", istep, (int)s, mth_last_error());
        break;
      }
    }
  }
  if (s == MTH_OK) s = mth_iout_wait(ctx);
  if (s != MTH_OK) fprintf(stderr, "%s\n", mth_last_error());
  fclose(vm);
  fclose(ss);
  if (dd) fclose(dd);
  mth_destroy(ctx);
  free(grain);
  free(phase);
  free(euler);
  return s == MTH_OK ? 0 : 1;
}

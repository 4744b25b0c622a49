/*
 * oracle.h -- ORACLE (test infrastructure only).
 *
 * A CPU restatement, in plain C with OpenMP, of the reference algorithm for
 * the EVPFFT Green iteration with the power-law flow rule and Voce hardening
 * (M-THEMES src/evolution.c, src/constitutive.c, src/kinematics.c,
 * src/init.c).  It exists to check the CUDA product: only tests/, the smoke
 * check in __graft_entry__.py and the cpu_baseline / --impl reference legs of
 * bench.py may load it.  Nothing in the product links against it.
 */
#ifndef MTH_ORACLE_H
#define MTH_ORACLE_H
#include "../include/mth.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_ctx orc_ctx;

/* How the reference's out-of-bounds read SigDevAvg[3][3] in get_smacro
 * (src/evolution.c:531) is resolved: 0 -> the word reads as 0.0;
 * 1 -> it reads EpsAvg[1][0]; 2 -> it reads SigAvg1[0][0], the word found at
 * that address in the reference built here by oracle/build_ref.sh (g++ 13,
 * -O3: SigAvg1 is placed 96 bytes after SigDevAvg). */
enum { ORC_SVM_OOB_ZERO = 0, ORC_SVM_OOB_EPSAVG10 = 1, ORC_SVM_OOB_SIGAVG1_00 = 2 };

orc_ctx* orc_create(const mth_params* p, const int* grain, const int* phase,
                    const double* euler_deg, int nthreads, int svm_oob_mode,
                    int* status);
int  orc_step(orc_ctx* c, mth_step_report* rep);
int  orc_get_field(orc_ctx* c, int field, double* out);
int  orc_get_c066(orc_ctx* c, double* c066);   /* 36 doubles */
long long orc_second_backtracks(orc_ctx* c);   /* count of line searches that
                                                  reached the cubic branch */
void orc_destroy(orc_ctx* c);

/* Newton of UpdateStress for n independent voxels; same argument meaning as
 * mth_local_solve in include/mth.h. */
int orc_local_solve(const mth_params* p, const double c066[36], size_t n,
                    double* sig, const double* eps_p, const double* strain,
                    const double* rot, const double* crss, double* edot,
                    double* err, long long* newton_iters);

/* DRX restatement (oracle/drx_oracle.c). */
double orc_uniform(uint64_t seed, uint64_t counter);
void orc_pf_coefficients(const mth_params* p, double* mcoef, double* kappa, double* mwell, double* edisl);
void orc_gb_indicator(const int* n, const int* grain, unsigned char* gb);
long long orc_nucleation_sites(const int* n, const int* grain, const int* phase_crystal, const double* rho,
                               double rho_nuc, double prob, uint64_t seed, long long step, long long* sites,
                               long long cap);
void orc_paint_nuclei(const int* n, int* grain, const long long* sites, int nn, int first_id, int radius2);
/* PF_XRX on one rank: substeps sweeps from (grain, 1) per voxel; table is
 * the caller's rho_avg table (table_len entries, grain id g at g-1), read and
 * written as the reference does; init_gid: ids above it are recrystallised.
 * Outputs the grain map after the last substep and, when cnt_out is given,
 * every voxel's list in stored order (up to kmax entries, slot-major per
 * voxel: ids_out[v*kmax+k]). */
int orc_pf_relax(const mth_params* p, const int* n, const int* grain, const double* rho, int substeps, int init_gid,
                 double* table, int table_len, int* grain_out, int* cnt_out, int* ids_out, double* phi_out,
                 int kmax);

/* Transfer between the mechanical grid and a phase-field grid of another
 * size (InterpolateGrid, src/integrated.c:496-760): nearest-corner for
 * integer fields, trilinear for doubles; ns, nd: source / destination dims. */
void orc_resample_nearest(const int* ns, const int* src, const int* nd, int* dst);
void orc_resample_trilinear(const int* ns, const double* src, const int* nd, double* dst);

/* Complex FFT used by the oracle: in-place 3-D transform of an n0*n1*n2
 * array of interleaved (re,im) doubles, un-normalised, sign -1 forward,
 * +1 backward (FFTW 2.1.5 convention used at src/evolution.c:1367,1399). */
void orc_fft3d(double* data, int n0, int n1, int n2, int sign);

#ifdef __cplusplus
}
#endif
#endif

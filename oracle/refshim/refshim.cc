/*
 * refshim.cc -- single-rank MPI, FFTW-MPI and GSL stand-ins plus the hooks
 * that turn the reference build into a power-law/Voce run with a per-step
 * trace.  Compiled together with the reference's own sources by
 * oracle/build_ref.sh; output goes to oracle/_ref/ only.  Test
 * infrastructure: nothing in the product uses it.
 *
 * Hooks (installed by -D renames on the reference translation units, see
 * build_ref.sh; FFTW's own fftw_malloc_hook pads the FFT buffers):
 *   evp.c:       SetupJob  -> mth_ref_SetupJob  (adds the power-law CRSS
 *                state that the DD build does not allocate: crss, trial_tau,
 *                xkin, gamacum, as src/init.c:1148-1174 does without DD)
 *                DestroyJob -> mth_ref_DestroyJob (dumps final fields)
 *   evolution.c: StrainRate_Orowan -> StrainRate_eval (power law,
 *                src/evolution.c:10-18,116-125)
 *                DislocationEvolution -> mth_ref_after_step (Voce harden()
 *                where src/evolution.c:1574 has it commented out, then the
 *                trace line)
 *                AvgDislocation, Gradient_ShearRate, Gradient_Shear -> no-op
 *                VonMises -> mth_ref_VonMises (captures DisGradAvg_actual)
 */
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <cstdint>
#include "evp.h"

/* ------------------------------ MPI ------------------------------ */
struct mth_mpi_file { FILE* fp; long long disp; };
static MPI_Aint g_type_extent[256];
static int g_ntypes = 100;

static size_t type_size(MPI_Datatype t) {
  switch (t) {
    case MPI_INT: return sizeof(int);
    case MPI_DOUBLE: return sizeof(double);
    case MPI_FLOAT: return sizeof(float);
    case MPI_CHAR: return 1;
    default:
      if (t >= 100 && t < 256) return (size_t)g_type_extent[t];
      fprintf(stderr, "refshim: unknown MPI datatype %d\n", t);
      abort();
  }
}
extern "C" {
int MPI_Init(int*, char***) { return 0; }
int MPI_Finalize(void) { return 0; }
int MPI_Comm_size(MPI_Comm, int* n) { *n = 1; return 0; }
int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
int MPI_Barrier(MPI_Comm) { return 0; }
int MPI_Abort(MPI_Comm, int code) { fprintf(stderr, "refshim: MPI_Abort(%d)\n", code); exit(code ? code : 1); }
int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
  if (s != r) memmove(r, s, (size_t)n * type_size(t));
  return 0;
}
int MPI_Allgather(const void* s, int sc, MPI_Datatype st, void* r, int, MPI_Datatype, MPI_Comm) {
  memmove(r, s, (size_t)sc * type_size(st));
  return 0;
}
int MPI_Allgatherv(const void* s, int sc, MPI_Datatype st, void* r, const int*, const int* displs,
                   MPI_Datatype rt, MPI_Comm) {
  memmove((char*)r + (size_t)displs[0] * type_size(rt), s, (size_t)sc * type_size(st));
  return 0;
}
int MPI_Send(const void*, int, MPI_Datatype, int, int, MPI_Comm) {
  fprintf(stderr, "refshim: MPI_Send with one rank\n");
  abort();
}
int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*) {
  fprintf(stderr, "refshim: MPI_Recv with one rank\n");
  abort();
}
int MPI_Sendrecv(const void* sb, int sc, MPI_Datatype st, int, int, void* rb, int, MPI_Datatype, int, int,
                 MPI_Comm, MPI_Status*) {
  memmove(rb, sb, (size_t)sc * type_size(st));
  return 0;
}
int MPI_Address(void* p, MPI_Aint* a) { *a = (MPI_Aint)(intptr_t)p; return 0; }
int MPI_Type_struct(int count, int* bl, MPI_Aint* disps, MPI_Datatype* types, MPI_Datatype* out) {
  MPI_Aint ub = 0, al = 1;
  for (int i = 0; i < count; i++) {
    MPI_Aint sz = (MPI_Aint)type_size(types[i]);
    MPI_Aint e = disps[i] + bl[i] * sz;
    if (e > ub) ub = e;
    if (sz > al) al = sz;
  }
  ub = (ub + al - 1) / al * al;   /* padded to the largest member, as C structs are */
  if (g_ntypes >= 256) abort();
  g_type_extent[g_ntypes] = ub;
  *out = g_ntypes++;
  return 0;
}
int MPI_Type_commit(MPI_Datatype*) { return 0; }
int MPI_Type_extent(MPI_Datatype t, MPI_Aint* e) { *e = (MPI_Aint)type_size(t); return 0; }
int MPI_File_open(MPI_Comm, const char* name, int, MPI_Info, MPI_File* fh) {
  FILE* fp = fopen(name, "wb");
  if (!fp) return 1;
  *fh = new mth_mpi_file{fp, 0};
  return 0;
}
int MPI_File_set_view(MPI_File fh, long long disp, MPI_Datatype, MPI_Datatype, const char*, MPI_Info) {
  fh->disp = disp;
  fseek(fh->fp, (long)disp, SEEK_SET);
  return 0;
}
int MPI_File_write(MPI_File fh, const void* b, int n, MPI_Datatype t, MPI_Status*) {
  fwrite(b, type_size(t), (size_t)n, fh->fp);
  return 0;
}
int MPI_File_close(MPI_File* fh) {
  fclose((*fh)->fp);
  delete *fh;
  *fh = nullptr;
  return 0;
}

/* --------------------------- FFTW-MPI ---------------------------- */
struct mth_fftwnd_mpi_plan_s { fftwnd_plan p; int n[3]; int dir; };
static long long g_inverse_calls = 0;

fftwnd_mpi_plan fftw3d_mpi_create_plan(MPI_Comm, int nx, int ny, int nz, fftw_direction dir, int flags) {
  mth_fftwnd_mpi_plan_s* q = new mth_fftwnd_mpi_plan_s;
  q->p = (nx > 0 && ny > 0 && nz > 0) ? fftw3d_create_plan(nx, ny, nz, dir, flags | FFTW_IN_PLACE) : nullptr;
  q->n[0] = nx; q->n[1] = ny; q->n[2] = nz;
  q->dir = (int)dir;
  return q;
}
void fftwnd_mpi_local_sizes(fftwnd_mpi_plan p, int* lnx, int* lxs, int* lnyt, int* lyst, int* lsize) {
  *lnx = p->n[0]; *lxs = 0; *lnyt = p->n[1]; *lyst = 0;
  *lsize = p->n[0] * p->n[1] * p->n[2];
}
void fftwnd_mpi(fftwnd_mpi_plan p, int, fftw_complex* data, fftw_complex*, int) {
  if (p->dir == (int)FFTW_BACKWARD) g_inverse_calls++;
  fftwnd_one(p->p, data, nullptr);
}
void fftwnd_mpi_destroy_plan(fftwnd_mpi_plan p) {
  if (p->p) fftwnd_destroy_plan(p->p);
  delete p;
}

/* ------------------------------ GSL ------------------------------ */
static const gsl_rng_type g_type = {"mth-splitmix64"};
const gsl_rng_type* gsl_rng_default = &g_type;
unsigned long gsl_rng_default_seed = 0;
gsl_rng* gsl_rng_alloc(const gsl_rng_type*) {
  gsl_rng* r = new gsl_rng;
  const char* s = getenv("MTH_REF_SEED");
  r->seed = s ? strtoull(s, nullptr, 10) : 1ULL;
  r->counter = 0;
  return r;
}
void gsl_rng_free(gsl_rng* r) { delete r; }
static uint64_t splitmix(uint64_t x) {
  x += 0x9E3779B97F4A7C15ULL;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
  return x ^ (x >> 31);
}
double gsl_rng_uniform(gsl_rng* r) {
  uint64_t v = splitmix(r->seed * 0x632BE59BD9B4E019ULL + r->counter++);
  return (double)(v >> 11) * (1.0 / 9007199254740992.0);
}
double gsl_rng_uniform_pos(gsl_rng* r) {
  double u;
  do { u = gsl_rng_uniform(r); } while (u == 0.0);
  return u;
}
double gsl_ran_weibull(gsl_rng* r, double a, double b) {
  double u = gsl_rng_uniform_pos(r);
  return a * pow(-log(u), 1.0 / b);
}
}  /* extern "C" */

/* ----------------------------- hooks ----------------------------- */
static FILE* g_trace = nullptr;
static int g_vm_calls = 0;
static ten2nd g_disgrad_actual;
static long long g_inv_at_last_step = 0;

/* fftw_malloc with slack.  The displacement block of Evolution assigns
 * fft_data[pIDX] after its local_loop has finished (src/evolution.c:1598-1599),
 * when px, py and pz are one past their ranges: about one x-plane past the end
 * of the array.  Nothing reads that element; the slack takes the write, which
 * otherwise corrupts the heap and crashes some runs (the second step of
 * test_run/, 32^3 with 64 grains). */
static void* mth_ref_fftw_malloc(size_t n) {
  const size_t pad = n / 4 + 65536;
  void* p = malloc(n + pad);
  if (p) memset(p, 0, n + pad);
  return p;
}

void mth_ref_SetupJob(void) {
  fftw_malloc_hook = mth_ref_fftw_malloc;
  SetupJob();
  /* power-law CRSS state of the non-DD build (src/init.c:1148-1174) */
  AllocMem(gamacum, lsize, real);
  AllocMem(xkin, lsize, real*);
  AllocMem(trial_tau, lsize, real**);
  AllocMem(crss, lsize, real**);
  local_loop {
    AllocMem(xkin[pIDX], NSYSMX, real);
    AllocMem(trial_tau[pIDX], NSYSMX, real*);
    AllocMem(crss[pIDX], NSYSMX, real*);
    for (int i = 0; i < NSYSMX; i++) {
      AllocMem(trial_tau[pIDX][i], 2, real);
      AllocMem(crss[pIDX][i], 2, real);
    }
  }
  local_loop {
    gamacum[pIDX] = 0.0;
    int jph = phase_f[pIDX];
    if (Type_phases[jph - 1] == 0) {
      for (int i = 0; i < nSYS[jph - 1]; i++) {
        crss[pIDX][i][0] = tau[jph - 1][i][0];
        crss[pIDX][i][1] = tau[jph - 1][i][1];
        trial_tau[pIDX][i][0] = tau[jph - 1][i][0];
        trial_tau[pIDX][i][1] = tau[jph - 1][i][1];
        xkin[pIDX][i] = 0.0;
      }
    }
  }
  const char* tp = getenv("MTH_REF_TRACE");
  g_trace = fopen(tp ? tp : "mth_ref_trace.txt", "w");
  fprintf(g_trace, "# layout &SigDevAvg=%p &EpsAvg=%p &SigAvg=%p &SigAvg1=%p &EdotAvg=%p &VelGradAvg=%p\n",
          (void*)SigDevAvg, (void*)EpsAvg, (void*)SigAvg, (void*)SigAvg1, (void*)EdotAvg, (void*)VelGradAvg);
  fprintf(g_trace, "# C066");
  for (int i = 0; i < 6; i++) for (int j = 0; j < 6; j++) fprintf(g_trace, " %.17e", C066[i][j]);
  fprintf(g_trace, "\n");
  fflush(g_trace);
}

real mth_ref_VonMises(ten2nd t) {
  if ((g_vm_calls++ % 2) == 0) memcpy(g_disgrad_actual, t, sizeof(ten2nd));
  return VonMises(t);
}

void mth_ref_noop(void) {}

void mth_ref_after_step(int istep) {
  if (Hard_Flag == 1) harden();
  long long inv = g_inverse_calls - g_inv_at_last_step - (istep > 0 ? 3 : 0);
  g_inv_at_last_step = g_inverse_calls;
  const double* oob = &((const double*)SigDevAvg)[0] + 12;
  fprintf(g_trace, "%d %lld", istep, inv / 9);
  for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) fprintf(g_trace, " %.17e", SigAvg[i][j]);
  for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) fprintf(g_trace, " %.17e", g_disgrad_actual[i][j]);
  for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) fprintf(g_trace, " %.17e", EpsAvg[i][j]);
  for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) fprintf(g_trace, " %.17e", EdotAvg[i][j]);
  fprintf(g_trace, " %.17e %.17e %.17e %.17e %.17e %.17e %.17e\n", s_vm, s_vm1, e_vm, d_vm, Err_s, Err_e, *oob);
  fflush(g_trace);
}

/* Dislocation-density build: called where src/evolution.c:1565 calls
 * AvgDislocation(); writes the power-law trace line plus the dd.out averages
 * (src/evolution.c:1566-1569). */
void mth_ref_dd_after_step(void) {
  static int calls = 0;
  AvgDislocation();
  /* 9 inverse transforms per Green iteration, plus the 3 of the previous
     step's displacement block (src/evolution.c:1578-1607) */
  long long inv = g_inverse_calls - g_inv_at_last_step - (calls > 0 ? 3 : 0);
  g_inv_at_last_step = g_inverse_calls;
  const double* oob = &((const double*)SigDevAvg)[0] + 12;
  fprintf(g_trace, "%d %lld", calls++, inv / 9);
  for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) fprintf(g_trace, " %.17e", SigAvg[i][j]);
  for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) fprintf(g_trace, " %.17e", g_disgrad_actual[i][j]);
  for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) fprintf(g_trace, " %.17e", EpsAvg[i][j]);
  for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) fprintf(g_trace, " %.17e", EdotAvg[i][j]);
  fprintf(g_trace, " %.17e %.17e %.17e %.17e %.17e %.17e %.17e", s_vm, s_vm1, e_vm, d_vm, Err_s, Err_e, *oob);
  fprintf(g_trace, " %.17e %.17e %.17e %.17e %.17e %.17e %.17e\n", rho_F_avg, rho_P_avg, rho_s_avg, rho_m_avg,
          rho_g_avg, rho_dipole_avg, rho_forest_avg);
  fflush(g_trace);
}

static void dump(const char* dir, const char* name, const void* p, size_t bytes) {
  char path[512];
  snprintf(path, sizeof(path), "%s/%s.bin", dir, name);
  FILE* f = fopen(path, "wb");
  if (!f) return;
  fwrite(p, 1, bytes, f);
  fclose(f);
}

void mth_ref_DestroyJob(void) {
  const char* dir = getenv("MTH_REF_DUMP");
  if (dir) {
    size_t n = (size_t)lsize;
    dump(dir, "sig", Sig, n * sizeof(ten2nd));
    dump(dir, "eps", Eps, n * sizeof(ten2nd));
    dump(dir, "edot", Edot, n * sizeof(ten2nd));
    dump(dir, "disgrad", DisGrad, n * sizeof(ten2nd));
    dump(dir, "rot", TranMat_xt2sa, n * sizeof(ten2nd));
    double* cr = (double*)calloc(n * NSYSMX, sizeof(double));
    for (size_t v = 0; v < n; v++) {
      int jph = phase_f[v];
      if (Type_phases[jph - 1] == 0)
        for (int i = 0; i < nSYS[jph - 1]; i++) cr[v * NSYSMX + i] = crss[v][i][0];
    }
    dump(dir, "crss", cr, n * NSYSMX * sizeof(double));
    free(cr);
    dump(dir, "gamacum", gamacum, n * sizeof(double));
    if (getenv("MTH_REF_DD")) {
      double* rr = (double*)calloc(n * NSYSMX * 4, sizeof(double));
      for (size_t v = 0; v < n; v++)
        for (int i = 0; i < NSYSMX; i++) {
          rr[(v * 4 + 0) * NSYSMX + i] = rho_s[v][i];
          rr[(v * 4 + 1) * NSYSMX + i] = rho_g1[v][i];
          rr[(v * 4 + 2) * NSYSMX + i] = rho_g2[v][i];
          rr[(v * 4 + 3) * NSYSMX + i] = rho_g3[v][i];
        }
      dump(dir, "rho", rr, n * NSYSMX * 4 * sizeof(double));
      free(rr);
    }
  }
  if (g_trace) fclose(g_trace);
  DestroyJob();
}

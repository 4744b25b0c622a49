// capi.cu -- host orchestration and the extern "C" entry points of
// include/mth.h: context creation (SetupJob, src/init.c:727-1205), one
// mechanical step (the istep loop body of Evolution, src/evolution.c:
// 1319-1693, power-law path), field download and the batch local solve.
//
// The macroscopic bookkeeping of get_smacro (src/evolution.c:473-547), the
// error normalisation (src/evolution.c:1430-1455) and the end-of-step macro
// updates (src/evolution.c:1471-1535,1691-1693) run on the host in FP64 on
// the reduced sums that the kernels produce; everything per voxel or per
// wave vector runs on the GPU.
#include <algorithm>
#include "capi_internal.h"

static thread_local char g_err[512] = "";

mth_status set_err(mth_status s, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return s;
}


extern "C" const char* mth_version(void) { return "mth-gb300 0.1 (sm_103a)"; }
extern "C" const char* mth_last_error(void) { return g_err; }

// ------------------------------------------------------------ host math
namespace capi_host {

const double Bh[6][3][3] = {
    {{-RSQ2, 0, 0}, {0, RSQ2, 0}, {0, 0, 0}},
    {{-RSQ6, 0, 0}, {0, -RSQ6, 0}, {0, 0, 2. * RSQ6}},
    {{0, 0, 0}, {0, 0, RSQ2}, {0, RSQ2, 0}},
    {{0, 0, RSQ2}, {0, 0, 0}, {RSQ2, 0, 0}},
    {{0, RSQ2, 0}, {RSQ2, 0, 0}, {0, 0, 0}},
    {{RSQ3, 0, 0}, {0, RSQ3, 0}, {0, 0, RSQ3}}};

void t2v(const t33 t, double* v, int nv) {
  for (int i = 0; i < nv; i++) {
    double s = 0;
    for (int m = 0; m < 3; m++)
      for (int n = 0; n < 3; n++) s += t[m][n] * Bh[i][m][n];
    v[i] = s;
  }
}
void v2t(const double* v, t33 t, int nv) {
  for (int m = 0; m < 3; m++)
    for (int n = 0; n < 3; n++) {
      double s = 0;
      for (int i = 0; i < nv; i++) s += v[i] * Bh[i][m][n];
      t[m][n] = s;
    }
}
void m2t4(const double c[6][6], double* t /*81*/) {
  for (int m = 0; m < 3; m++)
    for (int n = 0; n < 3; n++)
      for (int k = 0; k < 3; k++)
        for (int l = 0; l < 3; l++) {
          double s = 0;
          for (int i = 0; i < 6; i++)
            for (int j = 0; j < 6; j++) s += c[i][j] * Bh[i][m][n] * Bh[j][k][l];
          t[((m * 3 + n) * 3 + k) * 3 + l] = s;
        }
}
// Gauss-Jordan inverse with partial pivoting; false if singular.
bool inv6(const double a[6][6], double out[6][6]) {
  double m[6][12];
  for (int i = 0; i < 6; i++)
    for (int j = 0; j < 12; j++) m[i][j] = j < 6 ? a[i][j] : (double)(j - 6 == i);
  for (int c = 0; c < 6; c++) {
    int p = c;
    for (int r = c + 1; r < 6; r++)
      if (fabs(m[r][c]) > fabs(m[p][c])) p = r;
    if (fabs(m[p][c]) < 1e-300) return false;
    if (p != c)
      for (int j = 0; j < 12; j++) { double t = m[p][j]; m[p][j] = m[c][j]; m[c][j] = t; }
    double id = 1.0 / m[c][c];
    for (int j = 0; j < 12; j++) m[c][j] *= id;
    for (int r = 0; r < 6; r++)
      if (r != c) {
        double f = m[r][c];
        if (f != 0.0)
          for (int j = 0; j < 12; j++) m[r][j] -= f * m[c][j];
      }
  }
  for (int i = 0; i < 6; i++)
    for (int j = 0; j < 6; j++) out[i][j] = m[i][j + 6];
  return true;
}
double von_mises(const t33 t) {
  double tr = t[0][0] + t[1][1] + t[2][2], vm = 0.0;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      double d = (t[i][j] + t[j][i]) / 2. - (double)(i == j) * tr / 3.0;
      vm += d * d;
    }
  return sqrt(2. / 3. * vm);
}
void voigt_to_full(const double* v, t33 m) {
  m[0][0] = v[0]; m[0][1] = v[5]; m[0][2] = v[4];
  m[1][0] = v[5]; m[1][1] = v[1]; m[1][2] = v[3];
  m[2][0] = v[4]; m[2][1] = v[3]; m[2][2] = v[2];
}
bool radix_ok(int n) {
  if (n < 2 || (n & 1)) return false;
  while (n % 2 == 0) n /= 2;
  while (n % 3 == 0) n /= 3;
  return n == 1;
}

// Phase constants: PlasticInit (src/init.c:52-231) normalisation of the slip
// vectors, Schmid tensors in crystal axes, hardening matrix and the
// tau1/thet checks; crystal-axes stiffness/compliance, diagonal in the LT
// basis for cubic symmetry.
mth_status fill_phase(const mth_phase& in, PhaseConst& ph) {
  memset(&ph, 0, sizeof(ph));
  ph.type = in.type;
  const double ev[6] = {in.c11 - in.c12, in.c11 - in.c12, 2 * in.c44, 2 * in.c44, 2 * in.c44, in.c11 + 2 * in.c12};
  for (int i = 0; i < 6; i++) {
    ph.c_xt[i] = ev[i];
    ph.s_xt[i] = ev[i] != 0.0 ? 1.0 / ev[i] : 0.0;
  }
  if (in.type != 0) return MTH_OK;
  if (in.nsys <= 0 || in.nsys > NSYS) return set_err(MTH_ERR_ARG, "nsys=%d out of range", in.nsys);
  for (int i = 0; i < 5; i++)
    if (!(ev[i] > 0)) return set_err(MTH_ERR_SINGULAR, "elastic constants not positive definite");
  double tau1 = in.tau1, thet0 = in.thet0, thet1 = in.thet1;
  if (thet0 < thet1) return set_err(MTH_ERR_ARG, "Initial hardening rate is lower than final hardening rate");
  if (tau1 < 1.e-6) { tau1 = 1.e-6; thet0 = thet1; }
  ph.nsys = in.nsys;
  ph.nrs = in.nrs;
  ph.gamd0 = in.gamd0;
  ph.tau0f = in.tau0f;
  ph.tau_back_minus_fwd = in.tau0b - in.tau0f;
  ph.tau1 = tau1;
  ph.thet0 = thet0;
  ph.thet1 = thet1;
  ph.nrs_int = (in.nrs == floor(in.nrs) && in.nrs >= 1 && in.nrs <= 64) ? (int)in.nrs : 0;
  if (!(in.tau0f > 0) || !(in.tau0b > 0)) return set_err(MTH_ERR_ARG, "CRSS must be positive");
  for (int j = 0; j < ph.nsys; j++) {
    double nn = sqrt(in.bn[j][0] * in.bn[j][0] + in.bn[j][1] * in.bn[j][1] + in.bn[j][2] * in.bn[j][2]);
    double nb = sqrt(in.bb[j][0] * in.bb[j][0] + in.bb[j][1] * in.bb[j][1] + in.bb[j][2] * in.bb[j][2]);
    if (!(nn > 0) || !(nb > 0)) return set_err(MTH_ERR_ARG, "zero slip vector in system %d", j);
    double dot = 0;
    for (int m = 0; m < 3; m++) {
      ph.bn[j][m] = in.bn[j][m] / nn;
      ph.bb[j][m] = in.bb[j][m] / nb;
      dot += ph.bn[j][m] * ph.bb[j][m];
    }
    if (dot > 1e-3) return set_err(MTH_ERR_ARG, "Slip systems is NOT orthogonal (system %d)", j);
    t33 a;
    for (int m = 0; m < 3; m++)
      for (int n = 0; n < 3; n++) a[m][n] = (ph.bn[j][m] * ph.bb[j][n] + ph.bn[j][n] * ph.bb[j][m]) / 2.0;
    t2v(a, ph.m_xt[j], 5);
  }
  for (int i = 0; i < ph.nsys; i++)
    for (int j = 0; j < ph.nsys; j++) ph.hard[i][j] = (i == j) ? in.hself : in.hlat;
  return MTH_OK;
}
}  // namespace capi_host


namespace capi_host {
int pkh(int i, int j) {
  if (i > j) { int t = i; i = j; j = t; }
  return i * 5 - (i * (i - 1)) / 2 + (j - i);
}
// Crystal->sample matrix of Bunge angles in degrees: the transpose of
// EulerToTransMatrix opt 2 (src/kinematics.c:221-232, src/init.c:273-278).
void euler_to_rot(const double* e, double R[9]) {
  const double d2r = 3.14159265359 / 180.;
  const double t1 = e[0] * d2r, p = e[1] * d2r, t2 = e[2] * d2r;
  const double ct1 = cos(t1), st1 = sin(t1), cph = cos(p), sph = sin(p), ct2 = cos(t2), st2 = sin(t2);
  double a[3][3];
  a[0][0] = ct1 * ct2 - st1 * st2 * cph;
  a[0][1] = st1 * ct2 + ct1 * st2 * cph;
  a[0][2] = st2 * sph;
  a[1][0] = -1.0 * ct1 * st2 - st1 * ct2 * cph;
  a[1][1] = -1.0 * st1 * st2 + ct1 * ct2 * cph;
  a[1][2] = ct2 * sph;
  a[2][0] = st1 * sph;
  a[2][1] = -1.0 * ct1 * sph;
  a[2][2] = cph;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) R[i * 3 + j] = a[j][i];
}
// Elastic-class row without the S066 part: C_gr and S_gr = C_gr^-1 of a
// cubic crystal at rotation R, Q^T diag(.) Q in the LT basis.
void class_row(const PhaseConst& ph, const double R[9], double* row) {
  double Q[25];
  rot_to_q<double>(R, Q);
  for (int i = 0; i < ETAB_W; i++) row[i] = 0.0;
  for (int i = 0; i < 5; i++)
    for (int j = i; j < 5; j++) {
      double c = 0, s = 0;
      for (int k = 0; k < 5; k++) {
        c += Q[k * 5 + i] * ph.c_xt[k] * Q[k * 5 + j];
        s += Q[k * 5 + i] * ph.s_xt[k] * Q[k * 5 + j];
      }
      row[ET_CGR + pkh(i, j)] = c;
      row[ET_SEL + pkh(i, j)] = s;
    }
  row[ET_CGR_HH] = ph.c_xt[5];
  row[ET_SEL_HH] = ph.s_xt[5];
}
// Smallest eigenvalue of a symmetric 5x5 matrix (cyclic Jacobi rotations
// until the off-diagonal part is negligible).
static double sym5_min_eig(double a[5][5]) {
  for (int sweep = 0; sweep < 50; sweep++) {
    double off = 0, diag = 0;
    for (int i = 0; i < 5; i++) {
      diag += a[i][i] * a[i][i];
      for (int j = i + 1; j < 5; j++) off += a[i][j] * a[i][j];
    }
    if (off <= 1e-30 * diag) break;
    for (int p = 0; p < 4; p++)
      for (int q = p + 1; q < 5; q++) {
        if (a[p][q] == 0.0) continue;
        const double th = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
        const double t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
        const double cs = 1.0 / sqrt(t * t + 1.0), sn = t * cs;
        for (int k = 0; k < 5; k++) {   // columns p, q
          const double akp = a[k][p], akq = a[k][q];
          a[k][p] = cs * akp - sn * akq;
          a[k][q] = sn * akp + cs * akq;
        }
        for (int k = 0; k < 5; k++) {   // rows p, q
          const double apk = a[p][k], aqk = a[q][k];
          a[p][k] = cs * apk - sn * aqk;
          a[q][k] = sn * apk + cs * aqk;
        }
      }
  }
  double m = a[0][0];
  for (int i = 1; i < 5; i++) m = std::min(m, a[i][i]);
  return m;
}
void class_row_add_s0(double* row, const double s066[6][6]) {
  double a[5][5];
  for (int i = 0; i < 5; i++)
    for (int j = i; j < 5; j++) {
      row[ET_STOT + pkh(i, j)] = s066[i][j] + row[ET_SEL + pkh(i, j)];
      a[i][j] = a[j][i] = row[ET_STOT + pkh(i, j)];
    }
  // the Hessian base of the local solve is Q (this block) Q^T with Q
  // orthogonal, so its smallest eigenvalue is this block's; kept 1e-6 low
  row[ET_STOT_MIN] = sym5_min_eig(a) * (1.0 - 1e-6);
}
}  // namespace capi_host

bool mth::make_plan(int n, FftPlan* p) {
  p->n = n;
  p->nst = 0;
  int m = n;
  while (m % 4 == 0) { p->radix[p->nst++] = 4; m /= 4; }
  while (m % 2 == 0) { p->radix[p->nst++] = 2; m /= 2; }
  while (m % 3 == 0) { p->radix[p->nst++] = 3; m /= 3; }
  return m == 1 && p->nst <= 8;
}

// ---------------------------------------------------------------- context

// (Re)builds the context's tensor maps with ks / kg kz columns per tile of the
// strided / Green passes; 0 or a width the passes are not compiled for takes
// the default.
void ctx_set_tiles(mth_ctx* c, int ks, int kg) {
  tma_destroy(c->tma);
  const FftGeom& g = c->geom;
  c->tma = c->mixed ? tma_create<float>(g, c->ff.sig, c->ff.strain, c->ff.wspin, static_cast<c2<float>*>(c->spec),
                                        static_cast<c2<float>*>(c->anti), ks, kg)
                    : tma_create<double>(g, c->fd.sig, c->fd.strain, c->fd.wspin, static_cast<c2<double>*>(c->spec),
                                         static_cast<c2<double>*>(c->anti), ks, kg);
}

void ctx_free(mth_ctx* c) {
  if (!c) return;
  iout_free(c->iout);
  cudaFree(c->fieldmem);
  cudaFree(c->spec);
  cudaFree(c->anti);
  cudaFree(c->skew_d);
  tma_destroy(c->tma);
  if (!c->in_batch) {
    cudaFree(c->err_d);
    cudaFree(c->red);
    cudaFree(c->add_d);
    cudaFree(c->live_d);
  }
  if (c->err_h) cudaFreeHost(c->err_h);
  if (c->add_h) cudaFreeHost(c->add_h);
  cudaFree(c->phase_d);
  cudaFree(c->grain_d);
  cudaFree(c->eclass_d);
  cudaFree(c->etab_d);
  cudaFree(c->etabf_d);
  cudaFree(c->partials);
  if (c->red_h) cudaFreeHost(c->red_h);
  cudaFree(c->bk_d);
  if (c->book_h) cudaFreeHost(c->book_h);
  for (int a = 0; a < 3; a++)
    for (int d = 0; d < 2; d++) cudaFree(c->tw[a][d]);
  if (c->st && !c->in_batch) cudaStreamDestroy(c->st);
  if (c->ev_pool) {
    for (cudaEvent_t e : *c->ev_pool) cudaEventDestroy(e);
    delete c->ev_pool;
  }
  delete c->ev_pending;
  delete c->etab_h;
  delete c->drx_rot_h;
  delete c->drx_class_h;
  cudaFree(c->drx_rot_d);
  cudaFree(c->drx_class_d);
  cudaFree(c->drx_cnt_d);
  pf_free(c->pff);
  pf_free(c->pfd);
  cudaFree(c->rho_d);
  cudaFree(c->rho_t);
  cudaFree(c->grain_prev_d);
  cudaFree(c->winner_d);
  cudaFree(c->sites_d);
  cudaFree(c->count_d);
  cudaFree(c->crystal_d);
  cudaFree(c->hist_d);
  cudaFree(c->gather_d);
  cudaFree(c->dl_d);
  cudaFree(c->grain_pf_d);
  cudaFree(c->rho_pf_d);
  cudaFree(c->rho_pf_t);
  cudaFree(c->gid_coarse_d);
  delete c->ddc;
  cudaFree(c->dd_mem);
  cudaFree(c->gb_d);
  delete c;
}

// ------------------------------------------------------------- profiling
static const char* k_names[K_NCLASS] = {"fft_z_r2c", "fft_y", "fft_x_green", "fft_z_c2r_strain", "newton",
                                        "reduce", "end_step", "spin_fft", "setup", "drx",
                                        "pf_relax", "adj_local", "adj_cg", "dislocation_density", "iter_book"};
const char* prof_class_name(int cls) { return cls >= 0 && cls < K_NCLASS ? k_names[cls] : "?"; }

void prof_begin(mth_ctx* c) {
  if (!c->prof_on) return;
  size_t i = c->ev_pending->size();
  if (c->ev_pool->size() < 2 * (i + 1)) {
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    c->ev_pool->push_back(a);
    c->ev_pool->push_back(b);
  }
  cudaEventRecord((*c->ev_pool)[2 * i], c->st);
}
void prof_end(mth_ctx* c, int cls, int kernels, double bytes) {
  c->prof_launch[cls] += kernels;
  c->prof_bytes[cls] += bytes;
  if (!c->prof_on) return;
  size_t i = c->ev_pending->size();
  cudaEventRecord((*c->ev_pool)[2 * i + 1], c->st);
  c->ev_pending->push_back(cls);
}
// after the stream has been synchronised
void prof_resolve(mth_ctx* c) {
  if (!c->ev_pending) return;
  for (size_t i = 0; i < c->ev_pending->size(); i++) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, (*c->ev_pool)[2 * i], (*c->ev_pool)[2 * i + 1]) == cudaSuccess)
      c->prof_ms[(*c->ev_pending)[i]] += ms;
  }
  c->ev_pending->clear();
}
// one launcher call of class cls issuing `kernels` kernels that move
// `bytes` algorithmic bytes

template <typename T>
static mth_status make_twiddles(int n, int sign, void** out) {
  std::vector<c2<T>> h(n);
  for (int k = 0; k < n; k++) {
    long double a = (long double)sign * 2.0L * 3.14159265358979323846264338327950288L * (long double)k / (long double)n;
    h[k].x = (T)cosl(a);
    h[k].y = (T)sinl(a);
  }
  CK(cudaMalloc(out, sizeof(c2<T>) * n));
  CK(cudaMemcpy(*out, h.data(), sizeof(c2<T>) * n, cudaMemcpyHostToDevice));
  return MTH_OK;
}

// Constants of the dislocation-density law for phase 1: b = a0/sqrt(2)
// (src/init.c:182), the shear modulus of src/init.c:826, kT and the reduced
// activation energies (src/constitutive.c:540, src/evp.h:81-86), the junction
// strengths (FCC junction type of each pair of systems from their geometry:
// self, coplanar, collinear, Hirth, and for 60-degree pairs glissile when
// the junction b_i -/+ b_j lies in one of the two planes, Lomer-Cottrell
// otherwise; for the system order of the FCC .sx files this is the matrix of
// InteractionStrengthMatrix, src/init.c:593-702) and the projections of
// src/init.c:1107-1126.
// The constants of the dislocation-density law for phase 1, folded in FP64
// (the reference evaluates the same products and quotients per voxel and
// system: StrainRate_Orowan src/constitutive.c:507-721, DislocationEvolution
// src/constitutive.c:1346-1520), with an FP32 copy for the mixed modes.
static void dd_constants(const mth_params& p, const PhaseConst& ph, DdConst& dc) {
  memset(&dc, 0, sizeof(dc));
  const mth_phase& in = p.phase[0];
  DdCoef<double>& k = dc.d;
  dc.nsys = ph.nsys;
  const double* c = p.dd_c;
  const double b = p.dd_a0 / sqrt(2.0);
  const double G = 0.1 * (in.c11 - in.c12 + 3 * in.c44) +
                   (0.5) * (5 * (in.c11 - in.c12) * in.c44) / (4 * in.c44 + 3 * (in.c11 - in.c12));
  const double kT = p.dd_T * 1.380658e-23 * (1.0 / 1.60217733e-19);   // eV
  const double j_in_ev = 0.62415063631;
  const double qslip = p.dd_q_slip * j_in_ev / kT;
  const double qbulk = p.dd_q_bulk * j_in_ev / kT;
  k.rm = 2.0 * kT / c[0] / c[1] / c[2] / G / (b * b * b) * 160.2177;
  k.tp = c[0] * G * b * 1.0e-3;
  k.tcut = (kT / j_in_ev) / c[1] / c[2] / b / b * 0.1;
  k.g0 = 1.0e-3 * 1.0e10 * c[1] * b * exp(-qslip);   // attempt frequency 1e10
  k.dip = sqrt(3.0) * G * b / 16.0 / 3.14159265359 / (1 - p.dd_nu);
  k.eps = 5.0e-3;
  k.c4 = c[3];
  k.c5 = c[4];
  k.c6 = c[5];
  k.ann = c[6] * 1.6 * 1E12 * 1E-9;
  k.clb = 4 * 1E12 * (p.dd_d0 / b);
  k.clb_h = b * b * b * 100 / (1.38 * p.dd_T);
  k.clb_0 = -1.0 - qbulk;
  k.gnd = 1.0 / b / p.dd_L0;
  const int ns = ph.nsys;
  for (int i = 0; i < ns; i++) {
    for (int m = 0; m < 5; m++) k.m[i][m] = ph.m_xt[i][m];
    for (int m = 0; m < 3; m++) k.bb[i][m] = ph.bb[i][m];
    k.bp[i][0] = ph.bb[i][1] * ph.bn[i][2] - ph.bb[i][2] * ph.bn[i][1];
    k.bp[i][1] = ph.bb[i][2] * ph.bn[i][0] - ph.bb[i][0] * ph.bn[i][2];
    k.bp[i][2] = ph.bb[i][0] * ph.bn[i][1] - ph.bb[i][1] * ph.bn[i][0];
  }
  auto dot3 = [](const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; };
  for (int i = 0; i < ns; i++)
    for (int j = 0; j < ns; j++) {
      const double* ni = ph.bn[i];
      const double* nj = ph.bn[j];
      const double* bi = ph.bb[i];
      const double* bj = ph.bb[j];
      double chi;
      if (i == j) chi = p.dd_chi[0];
      else if (fabs(fabs(dot3(ni, nj)) - 1.0) < 1e-6) chi = p.dd_chi[1];
      else if (fabs(fabs(dot3(bi, bj)) - 1.0) < 1e-6) chi = p.dd_chi[2];
      else if (fabs(dot3(bi, bj)) < 1e-6) chi = p.dd_chi[4];
      else {
        const double sg = dot3(bi, bj) > 0 ? 1.0 : -1.0;
        const double q[3] = {bi[0] - sg * bj[0], bi[1] - sg * bj[1], bi[2] - sg * bj[2]};
        chi = (fabs(dot3(q, ni)) < 1e-6 || fabs(dot3(q, nj)) < 1e-6) ? p.dd_chi[3] : p.dd_chi[5];
      }
      k.chi[i][j] = chi;
      const double sv[3] = {nj[1] * bj[2] - nj[2] * bj[1], nj[2] * bj[0] - nj[0] * bj[2], nj[0] * bj[1] - nj[1] * bj[0]};
      k.cs[i][j] = fabs(dot3(ni, sv));
      k.ss[i][j] = fabs(sqrt(fabs(1.0 - k.cs[i][j] * k.cs[i][j])));
      k.cg1[i][j] = fabs(dot3(ni, bj));
      k.sg1[i][j] = fabs(sqrt(fabs(1.0 - k.cg1[i][j] * k.cg1[i][j])));
      k.cg3[i][j] = fabs(dot3(ni, nj));
      k.sg3[i][j] = fabs(sqrt(fabs(1.0 - k.cg3[i][j] * k.cg3[i][j])));
    }
  // FP32 copy: every member is a double, in declaration order
  static_assert(sizeof(DdCoef<double>) == 2 * sizeof(DdCoef<float>), "DdCoef holds only T members");
  const double* src = reinterpret_cast<const double*>(&dc.d);
  float* dst = reinterpret_cast<float*>(&dc.f);
  for (size_t i = 0; i < sizeof(DdCoef<float>) / sizeof(float); i++) dst[i] = (float)src[i];
}

extern "C" mth_status mth_create(const mth_params* p, mth_ctx** out) {
  if (!p || !out) return set_err(MTH_ERR_ARG, "null argument");
  *out = nullptr;
  for (int i = 0; i < 3; i++)
    if (!radix_ok(p->cell_dim[i]) || p->cell_dim[i] > 512)
      return set_err(MTH_ERR_UNSUPPORTED, "CellDim[%d]=%d: each edge must be even, of the form 2^a 3^b, <= 512", i,
                     p->cell_dim[i]);
  if (p->n_phases < 1 || p->n_phases > MTH_NPH_MAX) return set_err(MTH_ERR_ARG, "N_phases=%d", p->n_phases);
  if (p->iter_max < 1) return set_err(MTH_ERR_ARG, "IterMax must be >= 1");
  if (!(p->time_step > 0)) return set_err(MTH_ERR_ARG, "TimeStep must be > 0");
  if (p->precision != MTH_FP64 && p->precision != MTH_MIXED && p->precision != MTH_MIXED_FAST &&
      p->precision != MTH_MIXED_ROOT64)
    return set_err(MTH_ERR_ARG, "precision");
  mth_ctx* c = new mth_ctx();
  memset(c, 0, sizeof(*c));
  c->p = *p;
  c->mixed = (p->precision == MTH_MIXED) ? 1 : (p->precision == MTH_MIXED_FAST) ? 2
             : (p->precision == MTH_MIXED_ROOT64) ? 3 : 0;
  for (int i = 0; i < 3; i++) c->n[i] = p->cell_dim[i];
  c->nv = (long long)c->n[0] * c->n[1] * c->n[2];
  c->wgt = 1.0 / (double)c->nv;
  for (int k = 0; k < p->n_phases; k++) {
    mth_status s = fill_phase(p->phase[k], c->nc.ph[k]);
    if (s) { delete c; return s; }
  }
  c->dd = p->flow_law == 1 ? 1 : 0;
  if (p->flow_law != 0 && p->flow_law != 1) { delete c; return set_err(MTH_ERR_ARG, "flow_law=%d", p->flow_law); }
  if (c->dd) {
    if (c->nc.ph[0].type != 0 || (p->n_phases == 2 && c->nc.ph[1].type == 0)) {
      delete c;
      return set_err(MTH_ERR_UNSUPPORTED, "dislocation-density law: phase 1 crystalline, phase 2 (if any) gas");
    }
    if (c->nc.ph[0].nsys != 12) {
      delete c;
      return set_err(MTH_ERR_UNSUPPORTED, "dislocation-density law: the 12 FCC {111}<110> systems (nsys=%d)",
                     c->nc.ph[0].nsys);
    }
    if (p->pf_substeps > 0) {
      delete c;
      return set_err(MTH_ERR_UNSUPPORTED, "dislocation-density law with phase-field DRX");
    }
    if (!(p->dd_a0 > 0) || !(p->dd_T > 0) || !(p->dd_L0 > 0) || !(p->dd_c[0] > 0) || !(p->dd_c[1] > 0) ||
        !(p->dd_c[2] > 0) || !(p->dd_nu < 1)) {
      delete c;
      return set_err(MTH_ERR_ARG, "dislocation-density parameters: a0, T__K, L0, C_1..C_3 > 0 and nu < 1");
    }
  }
  c->nc.dt = p->time_step;
  c->nc.ph1_only = (p->n_phases == 1 || c->nc.ph[1].type != 0) ? 1 : 0;
  c->nc.bound_stop = c->mixed ? 1 : 0;
  c->nc.tol = p->newton_tol > 0 ? p->newton_tol : (c->mixed ? 1e-6 : 1e-10);
  c->nc.itmax = p->newton_itmax > 0 ? p->newton_itmax : 500;
  // boundary conditions (src/init.c:861-900)
  double vb[6];
  for (int i = 0; i < 6; i++) {
    c->vbc[i] = p->velgrad_bc_flag[i];
    c->sbc[i] = p->stress_bc_flag[i];
    vb[i] = p->velgrad_bc[i] * c->vbc[i];
  }
  if (c->vbc[0] + c->vbc[1] + c->vbc[2] == 2) {
    delete c;
    return set_err(MTH_ERR_ARG, "Cannot enforce only two deviatoric components (Check input VelGrad_BC_Flag)");
  }
  for (int i = 0; i < 6; i++)
    if ((c->sbc[i] * c->vbc[i] != 0) || (c->sbc[i] + c->vbc[i] != 1)) {
      delete c;
      return set_err(MTH_ERR_ARG, "Check boundary conditions on strain rate and stress");
    }
  voigt_to_full(vb, c->udot);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      c->udot_s[i][j] = (c->udot[i][j] + c->udot[j][i]) / 2.;
      c->udot_a[i][j] = (c->udot[i][j] - c->udot[j][i]) / 2.;
    }
  {
    double d6[6];
    t33 dev;
    t2v(c->udot_s, d6, 6);
    v2t(d6, dev, 5);
    double s = 0;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) s += dev[i][j] * dev[i][j];
    c->d_vm = sqrt(2. / 3. * s);
  }
  c->creep = 0;
  for (int i = 0; i < 6; i++) c->creep += c->sbc[i];
  c->creep /= 6;
  if (c->creep) { delete c; return set_err(MTH_ERR_UNSUPPORTED, "all-stress (creep) boundary conditions"); }
  voigt_to_full(p->stress_bc, c->scauchy);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) c->disgrad_avg[i][j] = c->udot[i][j] * p->time_step;
  c->e_vm = c->d_vm * p->time_step;

  // geometry and plans
  FftGeom& g = c->geom;
  g.n0 = c->n[0]; g.n1 = c->n[1]; g.n2 = c->n[2];
  g.kz = g.n2 / 2 + 1;
  g.kzs = (g.kz + 1) & ~1;
  g.plane = c->nv;
  g.kplane = (long long)g.n0 * g.n1 * g.kzs;
  make_plan(g.n0, &g.px);
  make_plan(g.n1, &g.py);
  make_plan(g.n2, &g.pz);
  g.smem_budget = 100 * 1024;
  c->nblocks = (int)((c->nv + 255) / 256);
  c->ev_pool = new std::vector<cudaEvent_t>();
  c->ev_pending = new std::vector<int>();

  {
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess) { delete c; return set_err(MTH_ERR_CUDA, "cudaGetDeviceCount: %s", cudaGetErrorString(e)); }
    if (p->device < 0 || p->device >= ndev) { delete c; return set_err(MTH_ERR_ARG, "device %d of %d", p->device, ndev); }
    e = cudaSetDevice(p->device);
    if (e != cudaSuccess) { delete c; return set_err(MTH_ERR_CUDA, "cudaSetDevice: %s", cudaGetErrorString(e)); }
  }
  mth_status s = MTH_OK;
#define CKC(call)                                                                                  \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess) {                                                                       \
      s = set_err(e_ == cudaErrorMemoryAllocation ? MTH_ERR_NOMEM : MTH_ERR_CUDA, "%s: %s", #call, \
                  cudaGetErrorString(e_));                                                         \
      ctx_free(c);                                                                                 \
      return s;                                                                                    \
    }                                                                                              \
  } while (0)
  CKC(cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking));
  CKC(prepare_newton_kernels());
  // failure-path test hook: MTH_TEST_FAIL_TILE_WAIT=1 makes the tile passes'
  // first waits report a time-out (steps return MTH_ERR_TIMEOUT); every
  // context creation sets the device's hook from the environment
  {
    const char* probe = getenv("MTH_TEST_FAIL_TILE_WAIT");
    CKC(tma_set_wait_probe(probe && probe[0] == '1' ? 1 : 0));
  }
  const size_t esz = c->mixed ? sizeof(float) : sizeof(double);
  const long long P = c->nv;
  const int nplanes = 6 + 6 + 6 + 6 + 9 + 12 + 1 + 3;
  CKC(cudaMalloc(&c->fieldmem, esz * P * nplanes));
  CKC(cudaMalloc(&c->spec, 2 * esz * g.kplane * 6));
  CKC(cudaMalloc(&c->anti, 2 * esz * g.kplane * 3));
  // the padding column of the half spectra stays zero
  CKC(cudaMemset(c->spec, 0, 2 * esz * g.kplane * 6));
  CKC(cudaMemset(c->anti, 0, 2 * esz * g.kplane * 3));
  CKC(cudaMalloc(&c->phase_d, P));
  CKC(cudaMalloc(&c->grain_d, sizeof(int) * P));
  CKC(cudaMalloc(&c->eclass_d, sizeof(int) * P));
  CKC(cudaMalloc(&c->partials, sizeof(double) * 21 * c->nblocks));
  CKC(cudaMalloc(&c->red, sizeof(double) * 32));
  CKC(cudaMallocHost(&c->red_h, sizeof(double) * 32));
  CKC(cudaMalloc(&c->bk_d, sizeof(IterBook)));
  CKC(cudaMallocHost(&c->book_h, sizeof(int) * 4));
  c->book_h[3] = 1;   // source of the live flag's reset
  CKC(cudaMalloc(&c->err_d, sizeof(int)));
  CKC(cudaMemset(c->err_d, 0, sizeof(int)));
  CKC(cudaMallocHost(&c->err_h, sizeof(int)));
  *c->err_h = 0;
  CKC(cudaMalloc(&c->add_d, sizeof(double) * 8));
  CKC(cudaMemset(c->add_d, 0, sizeof(double) * 8));
  CKC(cudaMallocHost(&c->add_h, sizeof(double) * 8));
  CKC(cudaMalloc(&c->live_d, sizeof(int)));
  {
    const int one = 1;
    CKC(cudaMemcpy(c->live_d, &one, sizeof(int), cudaMemcpyHostToDevice));
  }
  auto carve = [&](auto* base, auto& f) {
    long long o = 0;
    f.sig = base + o; o += 6 * P;
    f.strain = base + o; o += 6 * P;
    f.epsp = base + o; o += 6 * P;
    f.edot = base + o; o += 6 * P;
    f.rot = base + o; o += 9 * P;
    f.crss = base + o; o += 12 * P;
    f.gamacum = base + o; o += P;
    f.wspin = base + o; o += 3 * P;
    f.ddc = nullptr;
    f.phase = c->phase_d;
    f.eclass = c->eclass_d;
    f.etab = nullptr;
    f.etabf = nullptr;
    f.nv = P;
  };
  if (c->mixed) carve(static_cast<float*>(c->fieldmem), c->ff);
  else carve(static_cast<double*>(c->fieldmem), c->fd);
  if (c->dd) {
    c->ddc = new DdConst;
    dd_constants(*p, c->nc.ph[0], *c->ddc);
    CKC(cudaMalloc(&c->dd_mem, esz * P * (7 * NSYS + 3 * NSYS)));
    CKC(cudaMalloc(&c->gb_d, P));
    auto carve_dd = [&](auto* base, auto& d, auto& f) {
      long long o = 0;
      d.rho_s = base + o; o += NSYS * P;
      d.g1 = base + o; o += NSYS * P;
      d.g2 = base + o; o += NSYS * P;
      d.g3 = base + o; o += NSYS * P;
      d.dipole = base + o; o += NSYS * P;
      d.forest = base + o; o += NSYS * P;
      d.gamdot = base + o; o += NSYS * P;
      f.ddc = base + o; o += 3 * NSYS * P;
      d.gb = c->gb_d;
    };
    if (c->mixed) carve_dd(static_cast<float*>(c->dd_mem), c->ddf, c->ff);
    else carve_dd(static_cast<double*>(c->dd_mem), c->ddd, c->fd);
  }
  // MTH_PDL=0: the iteration's kernels launched one after the other without
  // programmatic dependencies (for comparisons)
  {
    const char* pd = getenv("MTH_PDL");
    c->pdl = pd && pd[0] == '0' ? 0 : 1;
  }
  // MTH_HOST_BOOK=1: mth_step keeps the per-iteration bookkeeping on the
  // host (tests compare it with the device's, bit for bit)
  {
    const char* hb = getenv("MTH_HOST_BOOK");
    c->host_book = hb && hb[0] == '1';
  }
  {
    // MTH_FFT_TILES="ks,kg" picks the TMA passes' tile widths (tests cover
    // every compiled width); unset or unknown widths take the defaults
    int ks = 0, kg = 0;
    const char* tiles = getenv("MTH_FFT_TILES");
    if (tiles && sscanf(tiles, "%d,%d", &ks, &kg) != 2) ks = kg = 0;
    ctx_set_tiles(c, ks, kg);
  }
  CKC(cudaMalloc(&c->crystal_d, P));
  c->etab_h = new std::vector<double>();
  c->drx_rot_h = new std::vector<double>();
  c->drx_class_h = new std::vector<int>();
  c->drx = p->pf_substeps > 0;
  if (c->drx) {
    if (!(p->pf_length_scale > 0) || !(p->pf_time_step > 0) || !(p->pf_width_cells > 0) || !(p->m_gb >= 0) ||
        p->nucleus_radius < 0 || p->nucleus_radius > 256) {
      ctx_free(c);
      return set_err(MTH_ERR_ARG, "phase-field parameters");
    }
    c->pfc.mcoef = p->pf_time_step * 4.0 / 3.0 * p->m_gb / (p->pf_width_cells * p->pf_length_scale);
    c->pfc.kappa = 3.0 / 4.0 * p->e_gb * (p->pf_width_cells * p->pf_length_scale) / p->pf_length_scale / p->pf_length_scale;
    c->pfc.mwell = 6 * p->e_gb / (p->pf_width_cells * p->pf_length_scale);
    c->pfc.edisl = p->stored_energy_scale * p->shear_modulus * p->burgers * p->burgers;
    // phase-field grid: the mechanical one unless CellDim_pf names another
    const bool pf_zero = p->pf_cell_dim[0] == 0 && p->pf_cell_dim[1] == 0 && p->pf_cell_dim[2] == 0;
    for (int i = 0; i < 3; i++) c->npf[i] = pf_zero ? c->n[i] : p->pf_cell_dim[i];
    if (!pf_zero)
      for (int i = 0; i < 3; i++)
        if (c->npf[i] < 2 || c->npf[i] > 4096 || c->n[i] < 2) {
          ctx_free(c);
          return set_err(MTH_ERR_ARG, "pf_cell_dim must be 0 0 0 or >= 2 per axis (with cell_dim >= 2)");
        }
    c->pf_resample = c->npf[0] != c->n[0] || c->npf[1] != c->n[1] || c->npf[2] != c->n[2];
    c->nvpf = (long long)c->npf[0] * c->npf[1] * c->npf[2];
    const long long Q = c->nvpf;
    // the rho_avg table grows with the grain ids (drx_step)
    CKC(c->mixed ? pf_alloc(c->pff, c->npf, 0) : pf_alloc(c->pfd, c->npf, 0));
    if (c->pf_resample) {
      CKC(cudaMalloc(&c->grain_pf_d, sizeof(int) * Q));
      CKC(cudaMalloc(&c->rho_pf_d, sizeof(double) * Q));
      CKC(cudaMalloc(&c->rho_pf_t, esz * Q));
      CKC(cudaMalloc(&c->gid_coarse_d, sizeof(int) * P));
    }
    CKC(cudaMalloc(&c->rho_d, sizeof(double) * P));
    CKC(cudaMalloc(&c->rho_t, esz * P));
    CKC(cudaMalloc(&c->grain_prev_d, sizeof(int) * P));
    CKC(cudaMalloc(&c->winner_d, sizeof(int) * P));
    CKC(cudaMemset(c->winner_d, 0xff, sizeof(int) * P));
    CKC(cudaMalloc(&c->sites_d, sizeof(long long) * MAX_CANDIDATES));
    CKC(cudaMalloc(&c->count_d, sizeof(unsigned long long)));
    CKC(cudaMalloc(&c->gather_d, sizeof(double) * 9 * MAX_NUCLEI));
    c->hist_cap = (size_t)(P + MAX_NUCLEI);
    CKC(cudaMalloc(&c->hist_d, sizeof(unsigned long long) * c->hist_cap));
  }
  for (int a = 0; a < 3; a++)
    for (int d = 0; d < 2; d++) {
      mth_status t = c->mixed ? make_twiddles<float>(c->n[a], d == 0 ? -1 : 1, &c->tw[a][d])
                              : make_twiddles<double>(c->n[a], d == 0 ? -1 : 1, &c->tw[a][d]);
      if (t) { ctx_free(c); return t; }
    }
#undef CKC
  *out = c;
  return MTH_OK;
}


extern "C" mth_status mth_destroy(mth_ctx* c) {
  if (!c) return set_err(MTH_ERR_ARG, "null context");
  SETDEV(c);
  cudaStreamSynchronize(c->st);
  ctx_free(c);
  return MTH_OK;
}

// programmatic dependent launches along the iteration's kernels, outside a
// batch (whose graph keeps ordinary edges)
IterIn iter_in(const mth_ctx* c) { return IterIn{c->add_d, c->live_d, c->in_batch ? 0 : c->pdl}; }

// gated: the kernel follows the live flag (inside a batch graph)
mth_status launch_reduce(mth_ctx* c, int width, bool gated) {
  LAUNCH(K_REDUCE, 8.0 * width * (c->nblocks + 1),
         launch_reduce_partials(c->partials, c->nblocks, width, c->red, gated ? iter_in(c) : IterIn{nullptr, nullptr},
                                c->st));
  return MTH_OK;
}

mth_status reduce_to_host(mth_ctx* c, int width, double* out) {
  mth_status s = launch_reduce(c, width, false);
  if (s) return s;
  CK(cudaMemcpyAsync(c->red_h, c->red, sizeof(double) * width, cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(c->err_h, c->err_d, sizeof(int), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  prof_resolve(c);
  if (*c->err_h) return set_err(MTH_ERR_TIMEOUT, "a kernel timed out waiting for its tile copies");
  memcpy(out, c->red_h, sizeof(double) * width);
  return MTH_OK;
}

// (Re)upload the elastic class table in double and as a float copy; the
// stream is synchronised first so no kernel still reads the old tables.
static mth_status upload_class_table(mth_ctx* c, const std::vector<double>& rows) {
  CK(cudaStreamSynchronize(c->st));
  cudaFree(c->etab_d);
  cudaFree(c->etabf_d);
  c->etab_d = nullptr;
  c->etabf_d = nullptr;
  std::vector<float> rf(rows.size());
  for (size_t i = 0; i < rows.size(); i++) rf[i] = (float)rows[i];
  CK(cudaMalloc(&c->etab_d, sizeof(double) * rows.size()));
  CK(cudaMalloc(&c->etabf_d, sizeof(float) * rows.size()));
  CK(cudaMemcpy(c->etab_d, rows.data(), sizeof(double) * rows.size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(c->etabf_d, rf.data(), sizeof(float) * rows.size(), cudaMemcpyHostToDevice));
  c->ff.etab = c->etab_d;
  c->fd.etab = c->etab_d;
  c->ff.etabf = c->etabf_d;
  c->fd.etabf = c->etabf_d;
  return MTH_OK;
}

extern "C" mth_status mth_upload_microstructure(mth_ctx* c, const int* grain, const int* phase,
                                                const double* euler_deg, size_t n) {
  if (!c || !grain || !phase || !euler_deg) return set_err(MTH_ERR_ARG, "null argument");
  if ((long long)n != c->nv) return set_err(MTH_ERR_ARG, "n_voxels=%zu but CellDim gives %lld", n, c->nv);
  SETDEV(c);
  std::vector<uint8_t> ph(n);
  std::vector<int> ecl(n, 0);
  // elastic classes: voxels of equal phase and initial Euler angles share
  // C_gr (src/init.c:272-283); C066 is their voxel-weighted average
  std::map<std::tuple<int, double, double, double>, int> key2class;
  std::vector<double> rows;
  std::vector<long long> counts;
  long long nph1 = 0;
  int last_k = -1, last_key[1] = {0};
  double last_e[3] = {0, 0, 0};
  for (size_t v = 0; v < n; v++) {
    if (phase[v] < 1 || phase[v] > c->p.n_phases)
      return set_err(MTH_ERR_ARG, "voxel %zu has phase %d (N_phases=%d)", v, phase[v], c->p.n_phases);
    ph[v] = (uint8_t)(phase[v] - 1);
    if (phase[v] == 1) nph1++;
    const PhaseConst& pc = c->nc.ph[phase[v] - 1];
    if (pc.type != 0) continue;
    const double* e = euler_deg + 3 * v;
    if (!std::isfinite(e[0]) || !std::isfinite(e[1]) || !std::isfinite(e[2]))
      return set_err(MTH_ERR_ARG, "voxel %zu has a non-finite Euler angle", v);
    // consecutive voxels mostly lie in one grain: reuse the previous class
    if (last_k >= 0 && phase[v] == last_key[0] && e[0] == last_e[0] && e[1] == last_e[1] && e[2] == last_e[2]) {
      counts[last_k]++;
      ecl[v] = last_k;
      continue;
    }
    auto key = std::make_tuple(phase[v], e[0], e[1], e[2]);
    auto it = key2class.find(key);
    int k;
    if (it == key2class.end()) {
      k = (int)counts.size();
      key2class.emplace(key, k);
      counts.push_back(0);
      rows.resize(rows.size() + ETAB_W);
      double R[9];
      euler_to_rot(e, R);
      class_row(pc, R, &rows[(size_t)k * ETAB_W]);
    } else {
      k = it->second;
    }
    counts[k]++;
    ecl[v] = k;
    last_k = k;
    last_key[0] = phase[v];
    last_e[0] = e[0];
    last_e[1] = e[1];
    last_e[2] = e[2];
  }
  if (counts.empty()) return set_err(MTH_ERR_ARG, "no crystal voxel in the microstructure");
  memset(c->c066, 0, sizeof(c->c066));
  for (size_t k = 0; k < counts.size(); k++) {
    const double* r = &rows[k * ETAB_W];
    for (int i = 0; i < 5; i++)
      for (int j = 0; j < 5; j++) c->c066[i][j] += (double)counts[k] * r[ET_CGR + pkh(i, j)];
    c->c066[5][5] += (double)counts[k] * r[ET_CGR_HH];
  }
  for (int i = 0; i < 6; i++)
    for (int j = 0; j < 6; j++) c->c066[i][j] *= c->wgt;
  c->wgt_ph1 = (double)nph1 * c->wgt;
  c->adj_solid = ((size_t)nph1 == n && c->nc.ph[0].type == 0) ? 1 : 0;
  if (!inv6(c->c066, c->s066)) return set_err(MTH_ERR_SINGULAR, "reference stiffness C066 is singular");
  for (size_t k = 0; k < counts.size(); k++) class_row_add_s0(&rows[k * ETAB_W], c->s066);
  m2t4(c->c066, c->gc.c0);
  for (int i = 0; i < 6; i++)
    for (int j = 0; j < 6; j++) c->gc.s066[i * 6 + j] = c->s066[i][j];
  for (int i = 0; i < 81; i++) c->gc.c0f[i] = (float)c->gc.c0[i];
  for (int i = 0; i < 36; i++) c->gc.s066f[i] = (float)c->gc.s066[i];
  c->gc.elast_bc = c->p.elast_bc;
  m2t4(c->s066, c->s0_4);
  for (int i = 0; i < 5; i++)
    for (int j = 0; j < 5; j++) c->nc.s0dev[i * 5 + j] = c->s066[i][j];
  c->nc.s0hh = c->s066[5][5];
  c->nclass = (int)counts.size();
  *c->etab_h = rows;
  {
    std::vector<uint8_t> cry(n);
    int gmax = 0;
    for (size_t v = 0; v < n; v++) {
      cry[v] = c->nc.ph[phase[v] - 1].type == 0 ? 1 : 0;
      if (grain[v] > gmax) gmax = grain[v];
    }
    CK(cudaMemcpy(c->crystal_d, cry.data(), n, cudaMemcpyHostToDevice));
    c->first_drx_id = c->next_grain_id = gmax + 1;
    c->drx_rot_h->clear();
    c->drx_class_h->clear();
    c->tau0f = c->nc.ph[0].tau0f;
    c->nsys = c->nc.ph[0].nsys;
  }
  {
    mth_status s = upload_class_table(c, rows);
    if (s != MTH_OK) return s;
  }
  double* eul_d = nullptr;
  CK(cudaMalloc(&eul_d, sizeof(double) * 3 * n));
  CK(cudaMemcpyAsync(eul_d, euler_deg, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->phase_d, ph.data(), n, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->grain_d, grain, sizeof(int) * n, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->eclass_d, ecl.data(), sizeof(int) * n, cudaMemcpyHostToDevice, c->st));
  double d6[6];
  t2v(c->disgrad_avg, d6, 6);
  const void* f = c->mixed ? (const void*)&c->ff : (const void*)&c->fd;
  LAUNCH(K_SETUP, 0.0, launch_setup(c->mixed, c->nc, f, eul_d, d6, c->nblocks, c->st));
  if (c->dd) {
    // same-grain flags of the six face neighbours (Gradient_ExchangeGrainID,
    // src/constitutive.c:724-873; its -z flag compares with the -y neighbour)
    std::vector<uint8_t> gb(n);
    const int n0 = c->n[0], n1 = c->n[1], n2 = c->n[2];
    for (int x = 0; x < n0; x++)
      for (int y = 0; y < n1; y++)
        for (int z = 0; z < n2; z++) {
          const size_t v = ((size_t)x * n1 + y) * n2 + z;
          auto at = [&](int a, int b, int cz) { return grain[((size_t)a * n1 + b) * n2 + cz]; };
          const int g0 = grain[v];
          const int ym = at(x, (y + n1 - 1) % n1, z);
          gb[v] = (uint8_t)((g0 == at((x + 1) % n0, y, z)) | ((g0 == at((x + n0 - 1) % n0, y, z)) << 1) |
                            ((g0 == at(x, (y + 1) % n1, z)) << 2) | ((g0 == ym) << 3) |
                            ((g0 == at(x, y, (z + 1) % n2)) << 4) | ((g0 == ym) << 5));
        }
    CK(cudaMemcpyAsync(c->gb_d, gb.data(), n, cudaMemcpyHostToDevice, c->st));
    const void* dd = c->mixed ? (const void*)&c->ddf : (const void*)&c->ddd;
    LAUNCH(K_DD, 0.0, launch_dd_init(c->mixed, dd, c->phase_d, c->nv, c->p.dd_rho_ssd0, c->st));
    CK(cudaStreamSynchronize(c->st));   // gb is a local buffer
  }
  CK(cudaStreamSynchronize(c->st));
  prof_resolve(c);
  cudaFree(eul_d);
  if (c->skew_d) {
    const size_t esz = c->mixed ? sizeof(float) : sizeof(double);
    CK(cudaMemsetAsync(c->skew_d, 0, 3 * esz * c->nv, c->st));
    CK(cudaStreamSynchronize(c->st));
  }
  c->uploaded = 1;
  c->istep = 0;
  return MTH_OK;
}

template <typename T>
mth_status green_iteration(mth_ctx* c) {
  const IterIn it = iter_in(c);
  const FftGeom& g = c->geom;
  Fields<T>& f = *reinterpret_cast<Fields<T>*>(c->mixed ? (void*)&c->ff : (void*)&c->fd);
  c2<T>* spec = static_cast<c2<T>*>(c->spec);
  c2<T>* anti = static_cast<c2<T>*>(c->anti);
  auto tw = [&](int a, int d) { return static_cast<const c2<T>*>(c->tw[a][d]); };
  // algorithmic bytes: real plane = w*nv, complex spectrum plane = 2w*kplane
  const double w = sizeof(T), rp = w * (double)c->nv, kp = 2.0 * w * (double)g.n0 * g.n1 * g.kz;
  const bool tz = !c->tma_off && tma_has(c->tma, 0), ts = !c->tma_off && tma_has(c->tma, 1),
             tg = !c->tma_off && tma_has(c->tma, 2);
  const T scale = (T)(1.0 / (double)c->nv);
  LAUNCH(K_FFT_Z_R2C, 6 * rp + 6 * kp,
         tz ? tma_fft_z_r2c<T>(c->tma, g, tw(2, 0), it, c->err_d, c->st)
            : launch_fft_z_r2c<T>(g, f.sig, spec, 6, tw(2, 0), it, c->st));
  LAUNCH(K_FFT_Y, 12 * kp,
         ts ? tma_fft_strided<T>(c->tma, g, 0, -1, tw(1, 0), it, c->err_d, c->st)
            : launch_fft_strided<T>(g, spec, 6, 1, -1, tw(1, 0), it, c->st));
  LAUNCH(K_FFT_X_GREEN, 12 * kp + 6 * kp,
         tg ? tma_fft_x_green<T>(c->tma, g, c->gc, tw(0, 0), tw(0, 1), it, c->err_d, c->st)
            : launch_fft_x_green<T>(g, c->gc, spec, anti, tw(0, 0), tw(0, 1), it, c->st));
  LAUNCH(K_FFT_Y, 12 * kp,
         ts ? tma_fft_strided<T>(c->tma, g, 0, +1, tw(1, 1), it, c->err_d, c->st)
            : launch_fft_strided<T>(g, spec, 6, 1, +1, tw(1, 1), it, c->st));
  LAUNCH(K_FFT_Z_C2R, 6 * kp + 12 * rp,
         tz ? tma_fft_z_c2r<T>(c->tma, g, 0, tw(2, 1), scale, it, c->err_d, c->st)
            : launch_fft_z_c2r<T>(g, spec, f.strain, 6, tw(2, 1), scale, it, 1, c->st));
  // Newton: read sigma, strain, eps_p (18), rot (9), CRSS (12); write sigma, edot (12);
  // phase (1 B) and elastic class (4 B) per voxel
  LAUNCH(K_NEWTON, (18 + 9 + 12 + 12) * rp + 5.0 * (double)c->nv,
         launch_newton(c->mixed, c->nc, &f, c->partials, c->nblocks, it, c->st, c->dd));
  return MTH_OK;
}

template mth_status green_iteration<float>(mth_ctx* c);
template mth_status green_iteration<double>(mth_ctx* c);

template <typename T>
static mth_status spin_field(mth_ctx* c) {
  const FftGeom& g = c->geom;
  Fields<T>& f = *reinterpret_cast<Fields<T>*>(c->mixed ? (void*)&c->ff : (void*)&c->fd);
  c2<T>* anti = static_cast<c2<T>*>(c->anti);
  auto tw = [&](int a, int d) { return static_cast<const c2<T>*>(c->tw[a][d]); };
  const IterIn it{nullptr, nullptr};   // no uniform part; always live
  const double w = sizeof(T), rp = w * (double)c->nv, kp = 2.0 * w * (double)g.n0 * g.n1 * g.kz;
  const bool tz = !c->tma_off && tma_has(c->tma, 0), ts = !c->tma_off && tma_has(c->tma, 1);
  const T scale = (T)(1.0 / (double)c->nv);
  LAUNCH(K_SPIN, 6 * kp,
         ts ? tma_fft_strided<T>(c->tma, g, 2, +1, tw(0, 1), it, c->err_d, c->st)
            : launch_fft_strided<T>(g, anti, 3, 0, +1, tw(0, 1), it, c->st));
  LAUNCH(K_SPIN, 6 * kp,
         ts ? tma_fft_strided<T>(c->tma, g, 1, +1, tw(1, 1), it, c->err_d, c->st)
            : launch_fft_strided<T>(g, anti, 3, 1, +1, tw(1, 1), it, c->st));
  LAUNCH(K_SPIN, 3 * kp + 3 * rp,
         tz ? tma_fft_z_c2r<T>(c->tma, g, 1, tw(2, 1), scale, it, c->err_d, c->st)
            : launch_fft_z_c2r<T>(g, anti, f.wspin, 3, tw(2, 1), scale, it, 0, c->st));
  return MTH_OK;
}

// Reference stiffness after a change of the elastic classes: C066 as the
// voxel average of C_gr, S066, S0 (src/evolution.c:1200-1216); the Green
// operator keeps the initial C0 (src/init.c:1195).
static mth_status refresh_reference_medium(mth_ctx* c) {
  const int ncl = (int)(c->etab_h->size() / ETAB_W);
  if ((size_t)ncl > c->hist_cap) {
    CK(cudaStreamSynchronize(c->st));
    cudaFree(c->hist_d);
    c->hist_cap = (size_t)ncl * 2;
    CK(cudaMalloc(&c->hist_d, sizeof(unsigned long long) * c->hist_cap));
  }
  CK(cudaMemsetAsync(c->hist_d, 0, sizeof(unsigned long long) * ncl, c->st));
  LAUNCH(K_DRX, 5.0 * c->nv, launch_class_histogram(c->nv, c->crystal_d, c->eclass_d, c->hist_d, c->st));
  std::vector<unsigned long long> hist(ncl);
  CK(cudaMemcpyAsync(hist.data(), c->hist_d, sizeof(unsigned long long) * ncl, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  prof_resolve(c);
  std::vector<double>& rows = *c->etab_h;
  memset(c->c066, 0, sizeof(c->c066));
  for (int k = 0; k < ncl; k++) {
    const double* r = &rows[(size_t)k * ETAB_W];
    for (int i = 0; i < 5; i++)
      for (int j = 0; j < 5; j++) c->c066[i][j] += (double)hist[k] * r[ET_CGR + pkh(i, j)];
    c->c066[5][5] += (double)hist[k] * r[ET_CGR_HH];
  }
  for (int i = 0; i < 6; i++)
    for (int j = 0; j < 6; j++) c->c066[i][j] *= c->wgt;
  if (!inv6(c->c066, c->s066)) return set_err(MTH_ERR_SINGULAR, "reference stiffness C066 is singular after DRX");
  for (int k = 0; k < ncl; k++) class_row_add_s0(&rows[(size_t)k * ETAB_W], c->s066);
  m2t4(c->s066, c->s0_4);
  for (int i = 0; i < 5; i++)
    for (int j = 0; j < 5; j++) c->nc.s0dev[i * 5 + j] = c->s066[i][j];
  c->nc.s0hh = c->s066[5][5];
  {
    mth_status s = upload_class_table(c, rows);
    if (s != MTH_OK) return s;
  }
  c->nclass = ncl;
  return MTH_OK;
}

// Algorithmic HBM bytes of one phase-field relaxation of nv voxels with
// field element size ts: per substep the sparse state (PF_K ids and order
// parameters and a count per voxel) is read and written once, with the
// stored energy and the grain id of the voxel; neighbour and window reads are
// served from cache.
static double pf_relax_bytes(long long nv, size_t ts, int substeps) {
  const double state = PF_K * (4.0 + (double)ts) + 1.0;
  return (double)nv * (4.0 + state + (double)ts + substeps * (2.0 * state + (double)ts + 4.0));
}

mth_status pf_bad_status(unsigned bad) {
  return set_err(MTH_ERR_UNSUPPORTED,
                 "phase field beyond this build's capacities:%s%s%s%s", (bad & PF_BAD_LIST) ? " a voxel list over 16 entries;" : "",
                 (bad & PF_BAD_NEIGH) ? " over 32 ids in a 3x3x3 neighbourhood;" : "",
                 (bad & PF_BAD_ROW) ? " over 128 ids written by one row of voxels;" : "",
                 (bad & PF_BAD_TABLE) ? " a grain id outside the rho_avg table;" : "");
}

// Dynamic recrystallisation at the start of a mechanical step, the order of
// Evolution (src/evolution.c:850-1253): nucleation, phase-field relaxation,
// microstructure update, reset of recrystallised voxels, new reference
// medium.  Returns the number of nuclei.
static mth_status drx_step(mth_ctx* c, int* n_new) {
  *n_new = 0;
  const mth_params& p = c->p;
  const void* f = c->mixed ? (const void*)&c->ff : (const void*)&c->fd;
  const double es = c->mixed ? 4.0 : 8.0;   // bytes of a field element
  LAUNCH(K_DRX, (double)c->nv * (4 + 2 * es + 8),
         launch_drx_rho(c->mixed, f, p.rho0, p.rho_k, c->rho_d, c->rho_t, c->st));
  CK(cudaMemcpyAsync(c->grain_prev_d, c->grain_d, sizeof(int) * c->nv, cudaMemcpyDeviceToDevice, c->st));
  // nucleation
  CK(cudaMemsetAsync(c->count_d, 0, sizeof(unsigned long long), c->st));
  LAUNCH(K_DRX, (double)c->nv * (4 + 1 + 8), launch_nucleation_candidates(c->n, c->grain_d, c->crystal_d, c->rho_d, p.rho_nucleation,
                                                  p.nucleation_prob, p.seed, (uint64_t)c->istep * (uint64_t)c->nv,
                                                  c->sites_d, c->count_d, MAX_CANDIDATES, c->st));
  unsigned long long cnt = 0;
  CK(cudaMemcpyAsync(&cnt, c->count_d, sizeof(cnt), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  prof_resolve(c);
  if ((long long)cnt > MAX_CANDIDATES)
    return set_err(MTH_ERR_UNSUPPORTED, "%llu nucleation candidates in one step (limit %lld)", cnt, MAX_CANDIDATES);
  int nn = 0;
  if (cnt > 0) {
    std::vector<long long> sites(cnt);
    CK(cudaMemcpy(sites.data(), c->sites_d, sizeof(long long) * cnt, cudaMemcpyDeviceToHost));
    std::sort(sites.begin(), sites.end());
    nn = (int)std::min<unsigned long long>(cnt, (unsigned long long)MAX_NUCLEI);
    CK(cudaMemcpy(c->sites_d, sites.data(), sizeof(long long) * nn, cudaMemcpyHostToDevice));
    // each nucleus takes the current orientation of its parent voxel
    // (src/integrated.c:271-283): gather the rotations
    std::vector<double> R((size_t)nn * 9);
    const void* rot = c->mixed ? (const void*)c->ff.rot : (const void*)c->fd.rot;
    LAUNCH(K_DRX, 9.0 * nn * (8 + (c->mixed ? 4 : 8)),
           launch_gather_rot(c->mixed, rot, c->nv, c->sites_d, nn, c->gather_d, c->st));
    CK(cudaMemcpyAsync(R.data(), c->gather_d, sizeof(double) * 9 * nn, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    for (int k = 0; k < nn; k++) {
      const int cls = (int)(c->etab_h->size() / ETAB_W);
      c->etab_h->resize(c->etab_h->size() + ETAB_W);
      class_row(c->nc.ph[0], &R[(size_t)k * 9], &(*c->etab_h)[(size_t)cls * ETAB_W]);
      c->drx_rot_h->insert(c->drx_rot_h->end(), &R[(size_t)k * 9], &R[(size_t)k * 9] + 9);
      c->drx_class_h->push_back(cls);
    }
    LAUNCHN(K_DRX, 2, (double)c->nv * 8, launch_paint_nuclei(c->n, c->sites_d, nn, p.nucleus_radius, c->next_grain_id, c->winner_d,
                                           c->grain_d, c->st));
    c->next_grain_id += nn;
  }
  *n_new = nn;
  const int n_drx = c->next_grain_id - c->first_drx_id;
  if (n_drx == 0) return MTH_OK;
  // class table with the new rows (S066 part refreshed below)
  for (size_t k = 0; k < c->etab_h->size() / ETAB_W; k++) class_row_add_s0(&(*c->etab_h)[k * ETAB_W], c->s066);
  {
    mth_status s = upload_class_table(c, *c->etab_h);
    if (s != MTH_OK) return s;
  }
  if ((size_t)n_drx > c->drx_cap) {
    cudaFree(c->drx_rot_d);
    cudaFree(c->drx_class_d);
    cudaFree(c->drx_cnt_d);
    c->drx_cap = (size_t)n_drx * 2 + 64;
    CK(cudaMalloc(&c->drx_rot_d, sizeof(double) * 9 * c->drx_cap));
    CK(cudaMalloc(&c->drx_class_d, sizeof(int) * c->drx_cap));
    CK(cudaMalloc(&c->drx_cnt_d, sizeof(int) * 2 * c->drx_cap));
  }
  CK(cudaMemcpyAsync(c->drx_rot_d, c->drx_rot_h->data(), sizeof(double) * 9 * n_drx, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->drx_class_d, c->drx_class_h->data(), sizeof(int) * n_drx, cudaMemcpyHostToDevice, c->st));
  // phase-field relaxation from the painted grain map, on the PF grid
  // (grain ids and rho carried over first, src/evolution.c:1013-1018)
  const int* pf_grain = c->grain_d;
  const void* pf_rho = c->rho_t;
  if (c->pf_resample) {
    LAUNCH(K_DRX, (double)c->nvpf * 4 + (double)c->nv * 4,
           launch_resample_nearest(c->n, c->grain_d, c->npf, c->grain_pf_d, c->st));
    LAUNCH(K_DRX, (double)c->nvpf * (c->mixed ? 4 : 8) + (double)c->nv * 8,
           launch_resample_trilinear(c->n, c->rho_d, c->npf, c->rho_pf_t, c->mixed, c->st));
    pf_grain = c->grain_pf_d;
    pf_rho = c->rho_pf_t;
  }
  // PF_XRX's rho_avg table persists across mechanical steps (a global of the
  // reference); ids above the initial grains' are recrystallised (init_gid)
  int* gid_new;
  int pf_launches = 0;
  unsigned pf_bad = 0;
  const int init_gid = c->first_drx_id - 1;
  if (c->mixed) {
    CK(pf_table_reserve(c->pff, c->next_grain_id, c->st));
    LAUNCHN(K_PF, pf_launches, pf_relax_bytes(c->nvpf, sizeof(float), p.pf_substeps),
            launch_pf_relax<float>(c->npf, pf_grain, (const float*)pf_rho, p.pf_substeps, init_gid, c->pfc, c->pff,
                                   c->st, &pf_launches, &pf_bad));
    gid_new = c->pff.gid;
  } else {
    CK(pf_table_reserve(c->pfd, c->next_grain_id, c->st));
    LAUNCHN(K_PF, pf_launches, pf_relax_bytes(c->nvpf, sizeof(double), p.pf_substeps),
            launch_pf_relax<double>(c->npf, pf_grain, (const double*)pf_rho, p.pf_substeps, init_gid, c->pfc, c->pfd,
                                    c->st, &pf_launches, &pf_bad));
    gid_new = c->pfd.gid;
  }
  if (pf_bad) return pf_bad_status(pf_bad);
  if (c->pf_resample) {   // relaxed ids back to the mechanical grid (src/integrated.c:821-860)
    LAUNCH(K_DRX, (double)c->nvpf * 4 + (double)c->nv * 4,
           launch_resample_nearest(c->npf, gid_new, c->n, c->gid_coarse_d, c->st));
    gid_new = c->gid_coarse_d;
  }
  LAUNCHN(K_DRX, 2, (double)c->nv * 24,
          launch_drx_update(c->mixed, f, c->grain_d, c->grain_prev_d, gid_new, c->first_drx_id, n_drx, c->drx_rot_d,
                            c->drx_class_d, c->tau0f, c->nsys, c->drx_cnt_d, c->st));
  return refresh_reference_medium(c);
}

// A mechanical step in phases, shared by mth_step and the batch driver:
// step_begin (DRX, per-step flags, spin accumulator), then per Green
// iteration iter_add (host: the uniform strain increment of the iteration
// into add_h) / the iteration kernels / iter_finish (host: error norms and
// the macroscopic stress update from the reduced partial sums) while
// iter_more, and step_end (end-of-step updates and the report).
mth_status step_begin(mth_ctx* c) {
  c->it_nnew = 0;
  if (c->drx && c->istep > 0) {
    mth_status s = drx_step(c, &c->it_nnew);
    if (s) return s;
  }
  c->nc.flow_off = (c->istep == 0 && c->p.update_flag != 1) ? 1 : 0;
  if (c->dd) {
    // the step's passing stress, tau_0 + cutting stress and reference rate
    // per system, from the densities at the start of the step
    const void* dd = c->mixed ? (const void*)&c->ddf : (const void*)&c->ddd;
    const void* f = c->mixed ? (const void*)&c->ff : (const void*)&c->fd;
    const double w = c->mixed ? 4.0 : 8.0;
    LAUNCH(K_DD, (double)c->nv * w * (4 * NSYS + 3 * NSYS), launch_dd_prep(c->mixed, *c->ddc, dd, f, c->st));
  }
  // the step's bookkeeping: constants, then the state of a step's start
  IterBook& b = c->bk;
  memcpy(b.udot, c->udot, sizeof(t33));
  memcpy(b.scauchy, c->scauchy, sizeof(t33));
  memcpy(b.s0_4, c->s0_4, sizeof(b.s0_4));
  memcpy(b.vbc, c->vbc, sizeof(b.vbc));
  memcpy(b.sbc, c->sbc, sizeof(b.sbc));
  b.wgt = c->wgt;
  b.wgt_ph1 = c->wgt_ph1;
  b.dt = c->p.time_step;
  b.err = c->p.err;
  b.e_vm = c->e_vm;
  b.iter_max = c->p.iter_max;
  b.nan = 0;
  memset(b.ddg, 0, sizeof(b.ddg));
  memset(b.ddg_acum, 0, sizeof(b.ddg_acum));
  memset(b.ddg_applied, 0, sizeof(b.ddg_applied));
  const size_t esz = c->mixed ? sizeof(float) : sizeof(double);
  CK(cudaMemsetAsync(c->anti, 0, 2 * esz * c->geom.kplane * 3, c->st));
  c->bk.it_iter = 0;
  c->bk.it_nit = 0;
  c->bk.it_nbad = 0;
  c->bk.err_e = 2. * c->p.err;
  c->bk.err_s = 2. * c->p.err;
  return MTH_OK;
}

bool iter_more(const mth_ctx* c) { return book_more(c->bk); }

// uniform strain added this iteration: dDisGradAvg of the previous
// get_smacro, plus Udot dt on the first one (src/evolution.c:1319-1332)
void iter_add(mth_ctx* c) { book_add(c->bk, c->add_h); }

mth_status iter_finish(mth_ctx* c, const double* red) {
  if (!book_finish(c->bk, red, NPART))
    return set_err(MTH_ERR_NAN, "non-finite value in the Green iteration (step %d, iteration %d)", c->istep,
                   c->bk.it_iter);
  return MTH_OK;
}

mth_status step_end(mth_ctx* c, mth_step_report* rep) {
  const int istep = c->istep;
  const double dt = c->p.time_step;
  // end of step (src/evolution.c:1471-1546)
  t33 actual, vg;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      actual[i][j] = c->disgrad_avg[i][j] + c->bk.ddg_acum[i][j];
      vg[i][j] = (actual[i][j] - c->disgrad_avg_t[i][j]) / dt;
    }
  c->e_vm = von_mises(actual);
  c->d_vm = von_mises(vg);
  c->time_tot += dt;
  memcpy(c->disgrad_avg_t, actual, sizeof(t33));
  const int do_orient = (c->p.update_flag == 1 && istep > 1);
  const int do_harden = (c->p.hard_flag == 1);
  if (do_orient || c->skew_d) {
    mth_status s = c->mixed ? spin_field<float>(c) : spin_field<double>(c);
    if (s) return s;
  }
  // uniform part of the spin increment: Udot_a dt (applied rotation) plus the
  // antisymmetric part of the uniform grad-u added to the field this step,
  // Udot dt + the dDisGradAvg corrections applied before each iteration (the
  // correction of the last get_smacro enters DisGradAvg_actual only)
  double au[3];
  {
    t33 a;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++)
        a[i][j] = 2.0 * c->udot_a[i][j] * dt + 0.5 * (c->bk.ddg_applied[i][j] - c->bk.ddg_applied[j][i]);
    au[0] = a[2][1];
    au[1] = a[0][2];
    au[2] = a[1][0];
  }
  for (int i = 0; i < 3; i++) c->last_au[i] = au[i];
  const void* f = c->mixed ? (const void*)&c->ff : (const void*)&c->fd;
  if (c->skew_d) {
    // DisGrad's antisymmetric part: the step's uniform increment, the
    // antisymmetric part of Udot dt plus that of the applied corrections,
    // and the local part in wspin
    t33 w;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++)
        w[i][j] = c->udot_a[i][j] * dt + 0.5 * (c->bk.ddg_applied[i][j] - c->bk.ddg_applied[j][i]);
    const double u[3] = {w[2][1], w[0][2], w[1][0]};
    const double rp = (double)(c->mixed ? sizeof(float) : sizeof(double)) * (double)c->nv;
    const void* wspin = c->mixed ? (const void*)c->ff.wspin : (const void*)c->fd.wspin;
    LAUNCH(K_SPIN, 9 * rp, launch_disgrad_skew(c->mixed, wspin, c->skew_d, c->nv, u, c->st));
  }
  if (c->dd) {
    // shear rates at the converged stress, then DislocationEvolution (with
    // the shear-rate gradients from the third step on when Hard_Flag = 1,
    // src/evolution.c:1551-1565) on the rotation of the start of the step,
    // before the lattice rotation of end_step
    const void* dd = c->mixed ? (const void*)&c->ddf : (const void*)&c->ddd;
    const double w = c->mixed ? 4.0 : 8.0, nv = (double)c->nv;
    LAUNCH(K_DD, nv * w * (6 + 9 + 3 * NSYS + NSYS), launch_dd_gamdot(c->mixed, *c->ddc, dd, f, c->nc.flow_off, c->st));
    const int do_grad = (c->p.hard_flag == 1 && istep > 1) ? 1 : 0;
    LAUNCH(K_DD, nv * w * (6 + 9 + 7 * NSYS + 5 * NSYS) + nv,
           launch_dd_evolve(c->mixed, *c->ddc, dd, f, c->n, dt, do_grad, c->partials, c->st));
    double red[NPART_DD];
    mth_status s = reduce_to_host(c, NPART_DD, red);
    if (s) return s;
    for (int k = 0; k < NPART_DD; k++) c->dd_avg[k] = red[k] * c->wgt;
  }
  {
    // end-of-step bytes: eps_p RMW + edot (18), sigma (6), rot RMW (18), CRSS RMW (24), gamacum RMW (2), spin (3)
    const double rp = (double)(c->mixed ? sizeof(float) : sizeof(double)) * (double)c->nv;
    LAUNCH(K_END_STEP, (18 + 6 + 18 + 24 + 2 + 3) * rp + (double)c->nv,
           launch_end_step(c->mixed, c->nc, f, au, do_orient, do_harden, c->partials, c->nblocks, c->st, c->dd));
  }
  double red[NPART_END];
  mth_status s = reduce_to_host(c, NPART_END, red);
  if (s) return s;
  double e6[6], d6[6];
  t33 ea, da;
  for (int i = 0; i < 6; i++) { e6[i] = red[i] * c->wgt; d6[i] = red[6 + i] * c->wgt; }
  v2t(e6, ea, 6);
  v2t(d6, da, 6);
  double evmp = 0, dvmp = 0;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) { evmp += ea[i][j] * ea[i][j]; dvmp += da[i][j] * da[i][j]; }
  evmp = sqrt(2. / 3. * evmp);
  dvmp = sqrt(2. / 3. * dvmp);
  if (rep) {
    memset(rep, 0, sizeof(*rep));
    rep->step = istep;
    rep->iterations = c->bk.it_iter;
    rep->time = c->time_tot;
    memcpy(rep->sig_avg, c->bk.sig_avg, sizeof(t33));
    memcpy(rep->sig_avg_ph1, c->bk.sig_avg1, sizeof(t33));
    memcpy(rep->disgrad_avg, actual, sizeof(t33));
    memcpy(rep->eps_avg, ea, sizeof(t33));
    memcpy(rep->edot_avg, da, sizeof(t33));
    rep->e_vm = c->e_vm; rep->evmp = evmp; rep->d_vm = c->d_vm; rep->dvmp = dvmp;
    rep->s_vm = c->bk.s_vm; rep->s_vm1 = c->bk.s_vm1;
    rep->err_s = c->bk.err_s; rep->err_e = c->bk.err_e;
    rep->newton_iters = c->bk.it_nit;
    rep->newton_failed = c->bk.it_nbad;
    rep->n_new_grains = c->it_nnew;
    if (c->dd) memcpy(rep->dd_avg, c->dd_avg, sizeof(c->dd_avg));
  }
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) c->disgrad_avg[i][j] = c->disgrad_avg_t[i][j] + c->udot[i][j] * dt;
  c->istep++;
  return MTH_OK;
}

extern "C" mth_status mth_step(mth_ctx* c, mth_step_report* rep) {
  if (!c) return set_err(MTH_ERR_ARG, "null context");
  if (!c->uploaded) return set_err(MTH_ERR_STATE, "mth_step before mth_upload_microstructure");
  if (c->in_batch) return set_err(MTH_ERR_STATE, "context belongs to a batch: use mth_batch_step");
  SETDEV(c);
  mth_status s = step_begin(c);
  if (s) return s;
  // The iterations run with their bookkeeping on the device (book.cu): each
  // iteration's kernels, its reduction and the one-warp bookkeeping
  // kernel, which computes the next iteration's strain increment or drops
  // the live flag; the host queues groups of iterations and reads the flag
  // once per group, so the iterations follow one another without a host
  // round trip.  Iterations queued after the last one return at once.
  IterBook& b = c->bk;
  if (c->host_book) {
    // the same bookkeeping on the host after every iteration (test hook)
    while (iter_more(c)) {
      iter_add(c);
      CK(cudaMemcpyAsync(c->add_d, c->add_h, sizeof(double) * 6, cudaMemcpyHostToDevice, c->st));
      s = c->mixed ? green_iteration<float>(c) : green_iteration<double>(c);
      if (s) return s;
      double red[NPART];
      s = reduce_to_host(c, NPART, red);
      if (s) return s;
      s = iter_finish(c, red);
      if (s) return s;
    }
    return step_end(c, rep);
  }
  CK(cudaMemcpyAsync(c->bk_d, &b, sizeof(IterBook), cudaMemcpyHostToDevice, c->st));
  LAUNCH(K_BOOK, 0, launch_iter_book(c->bk_d, c->red, c->add_d, c->live_d, 1, c->st, 0));
  int queued = 0, group = 2;
  for (;;) {
    const int n = std::min(group, b.iter_max - queued);
    for (int k = 0; k < n; k++) {
      s = c->mixed ? green_iteration<float>(c) : green_iteration<double>(c);
      if (s) return s;
      s = launch_reduce(c, NPART, true);
      if (s) return s;
      LAUNCH(K_BOOK, 0, launch_iter_book(c->bk_d, c->red, c->add_d, c->live_d, 0, c->st, c->pdl));
    }
    queued += n;
    CK(cudaMemcpyAsync(&c->book_h[0], c->live_d, sizeof(int), cudaMemcpyDeviceToHost, c->st));
    CK(cudaMemcpyAsync(&c->book_h[1], &c->bk_d->nan, sizeof(int), cudaMemcpyDeviceToHost, c->st));
    CK(cudaMemcpyAsync(&c->book_h[2], &c->bk_d->it_iter, sizeof(int), cudaMemcpyDeviceToHost, c->st));
    CK(cudaMemcpyAsync(c->err_h, c->err_d, sizeof(int), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    prof_resolve(c);
    if (*c->err_h) return set_err(MTH_ERR_TIMEOUT, "a kernel timed out waiting for its tile copies");
    if (c->book_h[1])
      return set_err(MTH_ERR_NAN, "non-finite value in the Green iteration (step %d, iteration %d)", c->istep,
                     c->book_h[2]);
    if (!c->book_h[0] || queued >= b.iter_max) break;
    group = std::min(2 * group, 16);
  }
  CK(cudaMemcpyAsync(&b, c->bk_d, sizeof(IterBook), cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(c->live_d, &c->book_h[3], sizeof(int), cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  return step_end(c, rep);
}

// ------------------------------------------------------------- downloads
template <typename T>
static mth_status download(mth_ctx* c, int field, double* host) {
  const Fields<T>& f = *reinterpret_cast<const Fields<T>*>(c->mixed ? (void*)&c->ff : (void*)&c->fd);
  const long long P = c->nv;
  int nc;
  const T* src;
  switch (field) {
    case MTH_FIELD_SIG: src = f.sig; nc = 6; break;
    case MTH_FIELD_EPS: src = f.epsp; nc = 6; break;
    case MTH_FIELD_EDOT: src = f.edot; nc = 6; break;
    case MTH_FIELD_STRAIN:
    case MTH_FIELD_DISGRAD: src = f.strain; nc = 6; break;
    case MTH_FIELD_ROT: src = f.rot; nc = 9; break;
    case MTH_FIELD_CRSS: src = f.crss; nc = 12; break;
    case MTH_FIELD_GAMACUM: src = f.gamacum; nc = 1; break;
    case MTH_FIELD_RHO_SSD:
    case MTH_FIELD_RHO_GND: {
      if (!c->dd) return set_err(MTH_ERR_STATE, "dislocation densities exist with the dislocation-density law only");
      const DdFields<T>& d = *reinterpret_cast<const DdFields<T>*>(c->mixed ? (void*)&c->ddf : (void*)&c->ddd);
      src = field == MTH_FIELD_RHO_SSD ? d.rho_s : d.g1;   // g1, g2, g3 are consecutive planes
      nc = field == MTH_FIELD_RHO_SSD ? NSYS : 3 * NSYS;
      break;
    }
    default: return set_err(MTH_ERR_ARG, "field %d", field);
  }
  // converted to the host layout on the device, then one copy into the
  // caller's buffer (a pinned buffer gets the full copy bandwidth)
  const size_t out = (size_t)(nc == 6 ? 9 : nc) * P;
  if (c->dl_cap < out) {
    CK(cudaStreamSynchronize(c->st));
    cudaFree(c->dl_d);
    c->dl_d = nullptr;
    c->dl_cap = 0;
    CK(cudaMalloc(&c->dl_d, sizeof(double) * out));
    c->dl_cap = out;
  }
  if (field == MTH_FIELD_DISGRAD) CK(launch_disgrad_to_host(c->mixed, src, c->skew_d, P, c->dl_d, c->st));
  else CK(launch_to_host_layout(c->mixed, src, P, nc, nc == 6 ? 1 : 0, c->dl_d, c->st));
  CK(cudaMemcpyAsync(host, c->dl_d, sizeof(double) * out, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return MTH_OK;
}

extern "C" mth_status mth_download_field(mth_ctx* c, int field, double* host, size_t count) {
  if (!c || !host) return set_err(MTH_ERR_ARG, "null argument");
  if (!c->uploaded) return set_err(MTH_ERR_STATE, "no microstructure uploaded");
  SETDEV(c);
  if (field == MTH_FIELD_RHO) {
    if (count != (size_t)c->nv) return set_err(MTH_ERR_ARG, "count");
    if (!c->drx) return set_err(MTH_ERR_STATE, "rho is only kept when DRX is enabled (pf_substeps > 0)");
    const void* f = c->mixed ? (const void*)&c->ff : (const void*)&c->fd;
    CK(launch_drx_rho(c->mixed, f, c->p.rho0, c->p.rho_k, c->rho_d, c->rho_t, c->st));
    CK(cudaMemcpyAsync(host, c->rho_d, sizeof(double) * c->nv, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    return MTH_OK;
  }
  if (field == MTH_FIELD_GRAIN) {
    if (count != (size_t)c->nv) return set_err(MTH_ERR_ARG, "count");
    std::vector<int> h(c->nv);
    CK(cudaMemcpyAsync(h.data(), c->grain_d, sizeof(int) * c->nv, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    for (long long v = 0; v < c->nv; v++) host[v] = h[v];
    return MTH_OK;
  }
  if (field == MTH_FIELD_DISGRAD && !c->skew_d)
    return set_err(MTH_ERR_STATE, "DisGrad is kept only after mth_track_disgrad (before the first step)");
  const int ncomp = (field == MTH_FIELD_CRSS || field == MTH_FIELD_RHO_SSD) ? 12
                    : (field == MTH_FIELD_RHO_GND)                          ? 36
                    : (field == MTH_FIELD_GAMACUM || field == MTH_FIELD_RHO) ? 1
                                                                             : 9;
  if (count != (size_t)ncomp * c->nv) return set_err(MTH_ERR_ARG, "count=%zu, expected %lld", count, ncomp * c->nv);
  return c->mixed ? download<float>(c, field, host) : download<double>(c, field, host);
}

// The reference keeps the full displacement gradient DisGrad per voxel
// (src/evolution.c:1319-1405); here the strain planes hold its symmetric
// part, and the antisymmetric part (3 planes) is kept only on request.
extern "C" mth_status mth_track_disgrad(mth_ctx* c, int on) {
  if (!c) return set_err(MTH_ERR_ARG, "null context");
  if (c->in_batch) return set_err(MTH_ERR_STATE, "context belongs to a batch");
  SETDEV(c);
  if (!on) {
    if (c->skew_d) {
      CK(cudaStreamSynchronize(c->st));
      cudaFree(c->skew_d);
      c->skew_d = nullptr;
    }
    return MTH_OK;
  }
  if (!c->uploaded || c->istep != 0)
    return set_err(MTH_ERR_STATE, "mth_track_disgrad after mth_upload_microstructure and before the first step");
  if (c->skew_d) return MTH_OK;
  const size_t bytes = 3 * (c->mixed ? sizeof(float) : sizeof(double)) * (size_t)c->nv;
  void* planes = nullptr;
  CK(cudaMalloc(&planes, bytes));
  cudaError_t e = cudaMemsetAsync(planes, 0, bytes, c->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
  if (e != cudaSuccess) {
    cudaFree(planes);
    return set_err(MTH_ERR_CUDA, "clearing the DisGrad planes failed: %s", cudaGetErrorString(e));
  }
  c->skew_d = planes;   // kept only once cleared
  return MTH_OK;
}

// ------------------------------------------------------------- profiling
extern "C" mth_status mth_profile_enable(mth_ctx* c, int on) {
  if (!c) return set_err(MTH_ERR_ARG, "null context");
  SETDEV(c);
  CK(cudaStreamSynchronize(c->st));
  prof_resolve(c);
  c->prof_on = on ? 1 : 0;
  return MTH_OK;
}

extern "C" mth_status mth_profile_read(mth_ctx* c, mth_profile* out, int reset) {
  if (!c || !out) return set_err(MTH_ERR_ARG, "null argument");
  SETDEV(c);
  CK(cudaStreamSynchronize(c->st));
  prof_resolve(c);
  memset(out, 0, sizeof(*out));
  out->n_kernels = K_NCLASS;
  for (int k = 0; k < K_NCLASS; k++) {
    strncpy(out->name[k], k_names[k], 31);
    out->ms[k] = c->prof_ms[k];
    out->launches[k] = c->prof_launch[k];
    out->bytes[k] = c->prof_bytes[k];
    out->total_launches += c->prof_launch[k];
  }
  if (reset) {
    memset(c->prof_ms, 0, sizeof(c->prof_ms));
    memset(c->prof_launch, 0, sizeof(c->prof_launch));
    memset(c->prof_bytes, 0, sizeof(c->prof_bytes));
  }
  return MTH_OK;
}

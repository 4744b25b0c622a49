// capi_adjoint.cu -- host driver of the calibration adjoint (mth_adjoint).
#include "capi_internal.h"

// ------------------------------------------------------ calibration adjoint
// Forward sweep with stored states every K steps, then per mechanical step
// in reverse order: adj_pre (transposed end-of-step Jacobians, tangent
// stiffness, right-hand side), b = Q(C_t sigbar) + W^T(spin adjoint), CG on
// Q C_t mu = b, adj_post (explicit dependences of the local law).  The
// segment of steps between two stored states is recomputed before it is
// reversed; the last segment's snapshots come from the first sweep.
namespace {
struct HostCkpt {
  t33 disgrad_avg, disgrad_avg_t, sig_avg, sig_avg1;
  double e_vm, d_vm, s_vm, s_vm1, err_e, err_s, time_tot;
  int istep;
};
constexpr int CKPT_PLANES = 46;   // sig, strain, epsp, edot (6 each), rot 9, crss 12, gamacum 1
constexpr int SNAP_PLANES = 31;   // before the step: rot 9, crss 12, gamacum 1; after: sig 6, wspin 3
constexpr int ADJ_STATE_PLANES = 25;   // eps_p 6, CRSS 12, gamacum 1, rotation 3, later spin 3

struct FieldPtrs {
  char* sig; char* strain; char* epsp; char* edot; char* rot; char* crss; char* gam; char* wspin;
};
template <typename T>
FieldPtrs field_ptrs_of(Fields<T>& f) {
  return FieldPtrs{(char*)f.sig, (char*)f.strain, (char*)f.epsp, (char*)f.edot,
                   (char*)f.rot, (char*)f.crss, (char*)f.gamacum, (char*)f.wspin};
}

struct AdjRun {
  size_t esz = 0;
  long long P = 0;
  std::vector<void*> mem;
  char* ckpt = nullptr;
  char* snap = nullptr;
  double* st = nullptr;
  double* sigbar = nullptr;
  char* ct = nullptr;
  char* rhs = nullptr;
  char* spec9 = nullptr;
  char* mu = nullptr;
  char* r = nullptr;
  char* p = nullptr;
  char* ap = nullptr;
  char* tmp = nullptr;
  std::vector<HostCkpt> hck;
  ~AdjRun() {
    for (void* m : mem) cudaFree(m);
  }
  cudaError_t alloc(void** out, size_t bytes) {
    cudaError_t e = cudaMalloc(out, bytes ? bytes : 16);
    if (e == cudaSuccess) mem.push_back(*out);
    return e;
  }
};
}  // namespace

static FieldPtrs field_ptrs(mth_ctx* c) { return c->mixed ? field_ptrs_of(c->ff) : field_ptrs_of(c->fd); }

// state before step slot*K (device planes and host macro state)
static mth_status adj_save(mth_ctx* c, AdjRun& run, int slot) {
  const FieldPtrs f = field_ptrs(c);
  const size_t pl = run.esz * (size_t)run.P;
  char* d = run.ckpt + (size_t)slot * CKPT_PLANES * pl;
  CK(cudaMemcpyAsync(d, f.sig, 6 * pl, cudaMemcpyDeviceToDevice, c->st));
  CK(cudaMemcpyAsync(d + 6 * pl, f.strain, 6 * pl, cudaMemcpyDeviceToDevice, c->st));
  CK(cudaMemcpyAsync(d + 12 * pl, f.epsp, 6 * pl, cudaMemcpyDeviceToDevice, c->st));
  CK(cudaMemcpyAsync(d + 18 * pl, f.edot, 6 * pl, cudaMemcpyDeviceToDevice, c->st));
  CK(cudaMemcpyAsync(d + 24 * pl, f.rot, 9 * pl, cudaMemcpyDeviceToDevice, c->st));
  CK(cudaMemcpyAsync(d + 33 * pl, f.crss, 12 * pl, cudaMemcpyDeviceToDevice, c->st));
  CK(cudaMemcpyAsync(d + 45 * pl, f.gam, pl, cudaMemcpyDeviceToDevice, c->st));
  HostCkpt& h = run.hck[slot];
  memcpy(h.disgrad_avg, c->disgrad_avg, sizeof(t33));
  memcpy(h.disgrad_avg_t, c->disgrad_avg_t, sizeof(t33));
  memcpy(h.sig_avg, c->bk.sig_avg, sizeof(t33));
  memcpy(h.sig_avg1, c->bk.sig_avg1, sizeof(t33));
  h.e_vm = c->e_vm; h.d_vm = c->d_vm; h.s_vm = c->bk.s_vm; h.s_vm1 = c->bk.s_vm1;
  h.err_e = c->bk.err_e; h.err_s = c->bk.err_s; h.time_tot = c->time_tot; h.istep = c->istep;
  return MTH_OK;
}

static mth_status adj_restore(mth_ctx* c, AdjRun& run, int slot) {
  const FieldPtrs f = field_ptrs(c);
  const size_t pl = run.esz * (size_t)run.P;
  const char* d = run.ckpt + (size_t)slot * CKPT_PLANES * pl;
  CK(cudaMemcpyAsync(f.sig, d, 6 * pl, cudaMemcpyDeviceToDevice, c->st));
  CK(cudaMemcpyAsync(f.strain, d + 6 * pl, 6 * pl, cudaMemcpyDeviceToDevice, c->st));
  CK(cudaMemcpyAsync(f.epsp, d + 12 * pl, 6 * pl, cudaMemcpyDeviceToDevice, c->st));
  CK(cudaMemcpyAsync(f.edot, d + 18 * pl, 6 * pl, cudaMemcpyDeviceToDevice, c->st));
  CK(cudaMemcpyAsync(f.rot, d + 24 * pl, 9 * pl, cudaMemcpyDeviceToDevice, c->st));
  CK(cudaMemcpyAsync(f.crss, d + 33 * pl, 12 * pl, cudaMemcpyDeviceToDevice, c->st));
  CK(cudaMemcpyAsync(f.gam, d + 45 * pl, pl, cudaMemcpyDeviceToDevice, c->st));
  const HostCkpt& h = run.hck[slot];
  memcpy(c->disgrad_avg, h.disgrad_avg, sizeof(t33));
  memcpy(c->disgrad_avg_t, h.disgrad_avg_t, sizeof(t33));
  memcpy(c->bk.sig_avg, h.sig_avg, sizeof(t33));
  memcpy(c->bk.sig_avg1, h.sig_avg1, sizeof(t33));
  c->e_vm = h.e_vm; c->d_vm = h.d_vm; c->bk.s_vm = h.s_vm; c->bk.s_vm1 = h.s_vm1;
  c->bk.err_e = h.err_e; c->bk.err_s = h.err_s; c->time_tot = h.time_tot; c->istep = h.istep;
  return MTH_OK;
}

// one forward step with its snapshot in slot; records <sigma_33> and the step data
static mth_status adj_forward_step(mth_ctx* c, AdjRun& run, int slot, double* s33, AdjStepArgs* a) {
  const FieldPtrs f = field_ptrs(c);
  const size_t pl = run.esz * (size_t)run.P;
  char* d = run.snap + (size_t)slot * SNAP_PLANES * pl;
  const int istep = c->istep;
  if (slot >= 0) {
    CK(cudaMemcpyAsync(d, f.rot, 9 * pl, cudaMemcpyDeviceToDevice, c->st));
    CK(cudaMemcpyAsync(d + 9 * pl, f.crss, 12 * pl, cudaMemcpyDeviceToDevice, c->st));
    CK(cudaMemcpyAsync(d + 21 * pl, f.gam, pl, cudaMemcpyDeviceToDevice, c->st));
  }
  mth_step_report rep;
  mth_status s = mth_step(c, &rep);
  if (s) return s;
  if (slot >= 0) {
    CK(cudaMemcpyAsync(d + 22 * pl, f.sig, 6 * pl, cudaMemcpyDeviceToDevice, c->st));
    CK(cudaMemcpyAsync(d + 28 * pl, f.wspin, 3 * pl, cudaMemcpyDeviceToDevice, c->st));
  }
  *s33 = rep.sig_avg[2][2];
  for (int i = 0; i < 3; i++) a->au[i] = c->last_au[i];
  a->flow_off = c->nc.flow_off;
  a->do_orient = (c->p.update_flag == 1 && istep > 1) ? 1 : 0;
  a->do_harden = (c->p.hard_flag == 1) ? 1 : 0;
  a->seed = 0.0;
  return MTH_OK;
}

// out = Q(in) (nin = 6) or Q(in[0..5]) + W^T(in[6..8]) (nin = 9): the
// forward's z and y passes around the projection x pass
template <typename T>
static cudaError_t adj_project_launch(mth_ctx* c, AdjRun& run, const AdjProj& pj, const T* in, int nin, T* out) {
  const FftGeom& g = c->geom;
  c2<T>* sp = reinterpret_cast<c2<T>*>(run.spec9);
  auto tw = [&](int a, int d) { return static_cast<const c2<T>*>(c->tw[a][d]); };
  const IterIn none{nullptr, nullptr};
  cudaError_t e = launch_fft_z_r2c<T>(g, in, sp, nin, tw(2, 0), none, c->st);
  if (e == cudaSuccess) e = launch_fft_strided<T>(g, sp, nin, 1, -1, tw(1, 0), none, c->st);
  if (e == cudaSuccess) e = launch_adj_x_proj<T>(g, pj, sp, nin, tw(0, 0), tw(0, 1), c->st);
  if (e == cudaSuccess) e = launch_fft_strided<T>(g, sp, 6, 1, +1, tw(1, 1), none, c->st);
  if (e == cudaSuccess) e = launch_fft_z_c2r<T>(g, sp, out, 6, tw(2, 1), (T)(1.0 / (double)c->nv), none, 0, c->st);
  return e;
}
template <typename T>
static mth_status adj_project(mth_ctx* c, AdjRun& run, const AdjProj& pj, const T* in, int nin, T* out) {
  const FftGeom& g = c->geom;
  const double w = sizeof(T), rp = w * (double)c->nv, kp = 2.0 * w * (double)g.n0 * g.n1 * g.kz;
  LAUNCHN(K_ADJ_CG, 5, (nin + 6) * (rp + 2 * kp) + 2 * nin * kp, adj_project_launch<T>(c, run, pj, in, nin, out));
  return MTH_OK;
}

template <typename T>
static AdjViews<T> adj_views(mth_ctx* c, AdjRun& run, int slot) {
  const size_t P = (size_t)run.P;
  const T* d = reinterpret_cast<const T*>(run.snap) + (size_t)slot * SNAP_PLANES * P;
  AdjViews<T> v;
  v.nv = run.P;
  v.s_rot = d;
  v.s_crss = d + 9 * P;
  v.s_gam = d + 21 * P;
  v.s_sig = d + 22 * P;
  v.s_wspin = d + 28 * P;
  v.ep = run.st;
  v.tau = run.st + 6 * P;
  v.gam = run.st + 18 * P;
  v.phi = run.st + 19 * P;
  v.wnext = run.st + 22 * P;
  v.sigbar = run.sigbar;
  v.ct = reinterpret_cast<T*>(run.ct);
  v.rhs = reinterpret_cast<T*>(run.rhs);
  v.mu = reinterpret_cast<const T*>(run.mu);
  (void)c;
  return v;
}

template <typename T>
static mth_status adj_reverse_step(mth_ctx* c, AdjRun& run, int step, int slot, const AdjStepArgs& a,
                                   const AdjProj& pj, double tol, int itmax, double th[4], int* iters) {
  const long long P = run.P;
  const AdjViews<T> v = adj_views<T>(c, run, slot);
  const double w = sizeof(T);
  double red[4];
  LAUNCH(K_ADJ_LOCAL, (double)P * (31 * w + 25 * 8 * 2 + 6 * 8 + 16 * w + 9 * w + 8 * ETAB_W / 64.0),
         launch_adj_pre<T>(c->nc, a, v, c->eclass_d, c->etab_d, c->partials, c->st));
  mth_status s = reduce_to_host(c, 4, red);
  if (s) return s;
  for (int i = 0; i < 4; i++) {
    if (!std::isfinite(red[i]))
      return set_err(MTH_ERR_NAN, "adjoint: tangent stiffness not positive definite or non-finite value (step %d)",
                     step);
    th[i] += red[i];
  }
  T* mu = reinterpret_cast<T*>(run.mu);
  T* r = reinterpret_cast<T*>(run.r);
  T* p = reinterpret_cast<T*>(run.p);
  T* ap = reinterpret_cast<T*>(run.ap);
  T* tmp = reinterpret_cast<T*>(run.tmp);
  const T* ct = reinterpret_cast<const T*>(run.ct);
  const size_t b6 = sizeof(T) * 6 * (size_t)P;
  s = adj_project<T>(c, run, pj, reinterpret_cast<const T*>(run.rhs), 9, r);
  if (s) return s;
  CK(cudaMemsetAsync(mu, 0, b6, c->st));
  LAUNCH(K_ADJ_CG, 12.0 * w * P, launch_adj_dot<T>(r, r, P, c->partials, c->st));
  double rr0;
  s = reduce_to_host(c, 1, &rr0);
  if (s) return s;
  int it = 0;
  if (rr0 > 0.0) {
    CK(cudaMemcpyAsync(p, r, b6, cudaMemcpyDeviceToDevice, c->st));
    double rr = rr0, beta = 0.0;
    const double stop = tol * tol * rr0;
    for (; it < itmax;) {
      LAUNCH(K_ADJ_CG, (it ? 18.0 : 12.0) * w * P + 16.0 * w * P,
             launch_adj_ct_apply<T>(ct, p, r, beta, it > 0, tmp, P, c->st));
      s = adj_project<T>(c, run, pj, tmp, 6, ap);
      if (s) return s;
      LAUNCH(K_ADJ_CG, 12.0 * w * P, launch_adj_dot<T>(p, ap, P, c->partials, c->st));
      double pap;
      s = reduce_to_host(c, 1, &pap);
      if (s) return s;
      if (!(pap > 0.0))
        return set_err(MTH_ERR_NAN, "adjoint: projected tangent operator not positive (step %d, p.Ap=%g)", step, pap);
      const double alpha = rr / pap;
      LAUNCH(K_ADJ_CG, 36.0 * w * P, launch_adj_cg_update<T>(mu, r, p, ap, alpha, P, c->partials, c->st));
      double rn;
      s = reduce_to_host(c, 1, &rn);
      if (s) return s;
      it++;
      if (!std::isfinite(rn)) return set_err(MTH_ERR_NAN, "adjoint: non-finite CG residual");
      if (rn <= stop) break;
      beta = rn / rr;
      rr = rn;
    }
    if (it >= itmax)
      return set_err(MTH_ERR_NOT_CONVERGED, "adjoint: CG did not reach %g in %d iterations (step %d)", tol, itmax, step);
  }
  *iters = it;
  LAUNCH(K_ADJ_LOCAL, (double)P * (31 * w + 22 * 8 * 2 + 6 * 8 + 22 * w),
         launch_adj_post<T>(c->nc, a, v, c->partials, c->st));
  s = reduce_to_host(c, 4, red);
  if (s) return s;
  for (int i = 0; i < 4; i++) {
    if (!std::isfinite(red[i])) return set_err(MTH_ERR_NAN, "adjoint: non-finite parameter adjoint");
    th[i] += red[i];
  }
  return MTH_OK;
}

extern "C" mth_status mth_adjoint(mth_ctx* c, const mth_adjoint_opts* o, double* s33_out, mth_adjoint_result* res) {
  if (!c || !o || !res) return set_err(MTH_ERR_ARG, "null argument");
  if (!c->uploaded) return set_err(MTH_ERR_STATE, "mth_adjoint before mth_upload_microstructure");
  if (c->istep != 0) return set_err(MTH_ERR_STATE, "mth_adjoint needs a context at step 0 (it runs the forward solve)");
  if (c->in_batch) return set_err(MTH_ERR_STATE, "context belongs to a batch");
  if (c->skew_d) return set_err(MTH_ERR_STATE, "mth_adjoint on a context that tracks DisGrad (its replays would add to it)");
  if (o->n_steps < 1 || !o->target) return set_err(MTH_ERR_ARG, "n_steps >= 1 and a target curve are required");
  if (c->drx) return set_err(MTH_ERR_UNSUPPORTED, "adjoint with phase-field DRX");
  if (c->dd) return set_err(MTH_ERR_UNSUPPORTED, "adjoint of the dislocation-density law");
  if (!c->adj_solid) return set_err(MTH_ERR_UNSUPPORTED, "adjoint needs every voxel of phase 1 and crystalline");
  if (c->p.elast_bc != 1) return set_err(MTH_ERR_UNSUPPORTED, "adjoint needs ElastBC = 1");
  for (int a = 0; a < 6; a++) {
    if (c->vbc[a] + c->sbc[a] != 1)
      return set_err(MTH_ERR_UNSUPPORTED, "adjoint needs Stress_BC_Flag = 1 - VelGrad_BC_Flag (component %d)", a);
    if (c->vbc[a] == 0 && a >= 3)
      return set_err(MTH_ERR_UNSUPPORTED, "adjoint: stress-controlled shear component %d", a);
  }
  SETDEV(c);
  const int N = o->n_steps;
  const int K = o->checkpoint_every > 0 ? std::min(o->checkpoint_every, N) : std::min(10, N);
  const int nseg = (N + K - 1) / K;
  const int last0 = (nseg - 1) * K;
  const double tol = o->cg_tol > 0 ? o->cg_tol : (c->mixed ? 1e-5 : 1e-7);
  const int itmax = o->cg_itmax > 0 ? o->cg_itmax : 2000;
  AdjRun run;
  run.esz = c->mixed ? sizeof(float) : sizeof(double);
  run.P = c->nv;
  const size_t P = (size_t)c->nv, pl = run.esz * P;
  void* m;
  CK(run.alloc(&m, (size_t)(nseg + 1) * CKPT_PLANES * pl)); run.ckpt = (char*)m;
  CK(run.alloc(&m, (size_t)K * SNAP_PLANES * pl)); run.snap = (char*)m;
  CK(run.alloc(&m, sizeof(double) * ADJ_STATE_PLANES * P)); run.st = (double*)m;
  CK(run.alloc(&m, sizeof(double) * 6 * P)); run.sigbar = (double*)m;
  CK(run.alloc(&m, 16 * pl)); run.ct = (char*)m;
  CK(run.alloc(&m, 9 * pl)); run.rhs = (char*)m;
  CK(run.alloc(&m, 9 * 2 * run.esz * (size_t)c->geom.kplane)); run.spec9 = (char*)m;
  CK(run.alloc(&m, 6 * pl)); run.mu = (char*)m;
  CK(run.alloc(&m, 6 * pl)); run.r = (char*)m;
  CK(run.alloc(&m, 6 * pl)); run.p = (char*)m;
  CK(run.alloc(&m, 6 * pl)); run.ap = (char*)m;
  CK(run.alloc(&m, 6 * pl)); run.tmp = (char*)m;
  run.hck.resize(nseg + 1);
  // k = 0 block of the projection: stress-controlled diagonal components
  AdjProj pj;
  memset(&pj, 0, sizeof(pj));
  for (int a = 0; a < 3; a++) {
    if (c->vbc[a] != 0) continue;
    double e[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    e[a][a] = 1.0;
    double v6[6];
    cart_to_lt<double>(e, v6);
    for (int i = 0; i < 6; i++)
      for (int j = 0; j < 6; j++) pj.ps[i * 6 + j] += v6[i] * v6[j];
  }
  std::vector<double> s33(N);
  std::vector<AdjStepArgs> args(N);
  auto now = []() { return std::chrono::steady_clock::now(); };
  auto ms = [](std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
  };
  CK(cudaStreamSynchronize(c->st));
  const auto t0 = now();
  for (int n = 0; n < N; n++) {
    if (n % K == 0) {
      mth_status s = adj_save(c, run, n / K);
      if (s) return s;
    }
    mth_status s = adj_forward_step(c, run, n >= last0 ? n - last0 : -1, &s33[n], &args[n]);
    if (s) return s;
  }
  {
    mth_status s = adj_save(c, run, nseg);   // final state, put back at the end
    if (s) return s;
  }
  CK(cudaStreamSynchronize(c->st));
  const auto t1 = now();
  double J = 0;
  for (int n = 0; n < N; n++) J += (s33[n] - o->target[n]) * (s33[n] - o->target[n]);
  CK(cudaMemsetAsync(run.st, 0, sizeof(double) * ADJ_STATE_PLANES * P, c->st));
  double th[4] = {0, 0, 0, 0};
  long long cg_total = 0;
  int cg_max = 0, recomputed = 0;
  for (int seg = nseg - 1; seg >= 0; seg--) {
    const int n0 = seg * K, n1 = std::min(N, n0 + K);
    if (seg != nseg - 1) {
      mth_status s = adj_restore(c, run, seg);
      if (s) return s;
      for (int n = n0; n < n1; n++) {
        double s33r;
        AdjStepArgs ar;
        s = adj_forward_step(c, run, n - n0, &s33r, &ar);
        if (s) return s;
        recomputed++;
      }
    }
    for (int n = n1 - 1; n >= n0; n--) {
      AdjStepArgs a = args[n];
      a.seed = 2.0 * (s33[n] - o->target[n]) / (double)c->nv;
      int it = 0;
      mth_status s = c->mixed ? adj_reverse_step<float>(c, run, n, n - n0, a, pj, tol, itmax, th, &it)
                              : adj_reverse_step<double>(c, run, n, n - n0, a, pj, tol, itmax, th, &it);
      if (s) return s;
      cg_total += it;
      cg_max = std::max(cg_max, it);
    }
  }
  double gt;
  LAUNCH(K_ADJ_LOCAL, 8.0 * 12 * P, launch_adj_sum_tau(run.st + 6 * P, c->nc.ph[0].nsys, c->nv, c->partials, c->st));
  {
    mth_status s = reduce_to_host(c, 1, &gt);
    if (s) return s;
    s = adj_restore(c, run, nseg);
    if (s) return s;
  }
  CK(cudaStreamSynchronize(c->st));
  const auto t2 = now();
  memset(res, 0, sizeof(*res));
  res->misfit = J;
  res->grad[0] = gt;
  res->grad[1] = th[0];
  res->grad[2] = th[1];
  res->grad[3] = th[2];
  res->grad[4] = th[3];
  res->cg_iterations = cg_total;
  res->cg_iterations_max = cg_max;
  res->recomputed_steps = recomputed;
  res->forward_ms = ms(t0, t1);
  res->reverse_ms = ms(t1, t2);
  if (s33_out) memcpy(s33_out, s33.data(), sizeof(double) * N);
  return MTH_OK;
}


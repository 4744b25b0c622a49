// capi_arrays.cu -- entry points on caller arrays without a context: the
// phase-field relaxation and nucleation (mth_pf_relax, mth_nucleate) and the
// batch local solve (mth_local_solve, mth_local_solve_noalloc).
#include "capi_internal.h"

// ------------------------------------------------------ array-level DRX
template <typename T>
static mth_status pf_relax_arrays(const mth_params* p, const int* n, const int* grain, const double* rho, int substeps,
                                  int init_gid, double* rho_avg, int rho_avg_len, int* grain_out, int* ids_out,
                                  double* phi_out, int* cnt_out) {
  const long long nv = (long long)n[0] * n[1] * n[2];
  PfCoef co;
  const double lgb = p->pf_width_cells * p->pf_length_scale;
  co.mcoef = p->pf_time_step * 4.0 / 3.0 * p->m_gb / lgb;
  co.kappa = 3.0 / 4.0 * p->e_gb * lgb / p->pf_length_scale / p->pf_length_scale;
  co.mwell = 6 * p->e_gb / lgb;
  co.edisl = p->stored_energy_scale * p->shear_modulus * p->burgers * p->burgers;
  PfBuffers<T> b;
  int* g_d = nullptr;
  T* r_d = nullptr;
  std::vector<T> rt(nv), tab(rho_avg_len);
  for (long long v = 0; v < nv; v++) rt[v] = (T)rho[v];
  for (int i = 0; i < rho_avg_len; i++) tab[i] = (T)rho_avg[i];
  mth_status st = MTH_OK;
  cudaStream_t s = nullptr;
  int launches = 0;
  unsigned bad = 0;
  cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = pf_alloc(b, n, rho_avg_len);
  if (e == cudaSuccess) e = cudaMalloc(&g_d, sizeof(int) * nv);
  if (e == cudaSuccess) e = cudaMalloc(&r_d, sizeof(T) * nv);
  if (e == cudaSuccess) e = cudaMemcpyAsync(g_d, grain, sizeof(int) * nv, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(r_d, rt.data(), sizeof(T) * nv, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && rho_avg_len > 0)
    e = cudaMemcpyAsync(b.table, tab.data(), sizeof(T) * rho_avg_len, cudaMemcpyHostToDevice, s);
  // the table as the caller sized it: ids beyond rho_avg_len are flagged
  b.table_len = rho_avg_len < b.table_cap ? rho_avg_len : b.table_cap;
  if (e == cudaSuccess) e = launch_pf_relax<T>(n, g_d, r_d, substeps, init_gid, co, b, s, &launches, &bad);
  if (e == cudaSuccess) e = cudaMemcpyAsync(grain_out, b.gid, sizeof(int) * nv, cudaMemcpyDeviceToHost, s);
  std::vector<T> ph;
  std::vector<int> id;
  std::vector<uint8_t> cn;
  if (e == cudaSuccess && rho_avg_len > 0)
    e = cudaMemcpyAsync(tab.data(), b.table, sizeof(T) * rho_avg_len, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && ids_out) {
    id.resize((size_t)PF_K * nv);
    e = cudaMemcpyAsync(id.data(), b.ids[b.cur], sizeof(int) * PF_K * nv, cudaMemcpyDeviceToHost, s);
  }
  if (e == cudaSuccess && phi_out) {
    ph.resize((size_t)PF_K * nv);
    e = cudaMemcpyAsync(ph.data(), b.phi[b.cur], sizeof(T) * PF_K * nv, cudaMemcpyDeviceToHost, s);
  }
  if (e == cudaSuccess) {
    cn.resize(nv);
    e = cudaMemcpyAsync(cn.data(), b.cnt[b.cur], nv, cudaMemcpyDeviceToHost, s);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    st = set_err(e == cudaErrorMemoryAllocation ? MTH_ERR_NOMEM : MTH_ERR_CUDA, "phase-field relaxation: %s",
                 cudaGetErrorString(e));
  } else if (bad) {
    st = pf_bad_status(bad);
  } else {
    for (int i = 0; i < rho_avg_len; i++) rho_avg[i] = (double)tab[i];
    // lists voxel-major in stored order (the device keeps them slot-major)
    for (long long v = 0; v < nv; v++) {
      if (cnt_out) cnt_out[v] = cn[v];
      for (int k = 0; k < PF_K; k++) {
        const bool in = k < cn[v];
        if (ids_out) ids_out[v * PF_K + k] = in ? id[(size_t)k * nv + v] : 0;
        if (phi_out) phi_out[v * PF_K + k] = in ? (double)ph[(size_t)k * nv + v] : 0.0;
      }
    }
  }
  pf_free(b);
  cudaFree(g_d);
  cudaFree(r_d);
  if (s) cudaStreamDestroy(s);
  return st;
}

extern "C" mth_status mth_pf_relax(const mth_params* p, const int cell_dim[3], const int* grain, const double* rho,
                                   int substeps, int init_gid, double* rho_avg, int rho_avg_len, int* grain_out,
                                   int* ids_out, double* phi_out, int* cnt_out) {
  if (!p || !cell_dim || !grain || !rho || !grain_out || (rho_avg_len > 0 && !rho_avg))
    return set_err(MTH_ERR_ARG, "null argument");
  for (int i = 0; i < 3; i++)
    if (cell_dim[i] < 1) return set_err(MTH_ERR_ARG, "cell_dim");
  if (substeps < 0 || rho_avg_len < 0) return set_err(MTH_ERR_ARG, "substeps or rho_avg_len");
  if (!(p->pf_length_scale > 0) || !(p->pf_width_cells > 0)) return set_err(MTH_ERR_ARG, "phase-field parameters");
  CK(cudaSetDevice(p->device));
  return p->precision == MTH_FP64
             ? pf_relax_arrays<double>(p, cell_dim, grain, rho, substeps, init_gid, rho_avg, rho_avg_len, grain_out,
                                       ids_out, phi_out, cnt_out)
             : pf_relax_arrays<float>(p, cell_dim, grain, rho, substeps, init_gid, rho_avg, rho_avg_len, grain_out,
                                      ids_out, phi_out, cnt_out);
}

extern "C" mth_status mth_nucleate(const mth_params* p, const int cell_dim[3], int* grain, const int* phase,
                                   const double* rho, long long step, int first_id, long long* sites, long long cap,
                                   int* n_new) {
  if (!p || !cell_dim || !grain || !phase || !rho || !n_new) return set_err(MTH_ERR_ARG, "null argument");
  const long long nv = (long long)cell_dim[0] * cell_dim[1] * cell_dim[2];
  if (nv <= 0) return set_err(MTH_ERR_ARG, "cell_dim");
  std::vector<uint8_t> cry(nv);
  for (long long v = 0; v < nv; v++) {
    if (phase[v] < 1 || phase[v] > p->n_phases) return set_err(MTH_ERR_ARG, "phase of voxel %lld", v);
    cry[v] = p->phase[phase[v] - 1].type == 0;
  }
  CK(cudaSetDevice(p->device));
  int *g_d = nullptr, *w_d = nullptr;
  uint8_t* c_d = nullptr;
  double* r_d = nullptr;
  long long* s_d = nullptr;
  unsigned long long* n_d = nullptr;
  CK(cudaMalloc(&g_d, sizeof(int) * nv));
  CK(cudaMalloc(&w_d, sizeof(int) * nv));
  CK(cudaMalloc(&c_d, nv));
  CK(cudaMalloc(&r_d, sizeof(double) * nv));
  CK(cudaMalloc(&s_d, sizeof(long long) * MAX_CANDIDATES));
  CK(cudaMalloc(&n_d, sizeof(unsigned long long)));
  CK(cudaMemcpy(g_d, grain, sizeof(int) * nv, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(c_d, cry.data(), nv, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(r_d, rho, sizeof(double) * nv, cudaMemcpyHostToDevice));
  CK(cudaMemset(w_d, 0xff, sizeof(int) * nv));
  CK(cudaMemset(n_d, 0, sizeof(unsigned long long)));
  CK(launch_nucleation_candidates(cell_dim, g_d, c_d, r_d, p->rho_nucleation, p->nucleation_prob, p->seed,
                                  (uint64_t)step * (uint64_t)nv, s_d, n_d, MAX_CANDIDATES, nullptr));
  unsigned long long cnt = 0;
  CK(cudaMemcpy(&cnt, n_d, sizeof(cnt), cudaMemcpyDeviceToHost));
  mth_status st = MTH_OK;
  if ((long long)cnt > MAX_CANDIDATES) {
    st = set_err(MTH_ERR_UNSUPPORTED, "%llu nucleation candidates (limit %lld)", cnt, MAX_CANDIDATES);
  } else {
    std::vector<long long> sv(cnt);
    if (cnt) CK(cudaMemcpy(sv.data(), s_d, sizeof(long long) * cnt, cudaMemcpyDeviceToHost));
    std::sort(sv.begin(), sv.end());
    const int nn = (int)std::min<unsigned long long>(cnt, (unsigned long long)MAX_NUCLEI);
    if (nn) {
      CK(cudaMemcpy(s_d, sv.data(), sizeof(long long) * nn, cudaMemcpyHostToDevice));
      CK(launch_paint_nuclei(cell_dim, s_d, nn, p->nucleus_radius, first_id, w_d, g_d, nullptr));
      CK(cudaMemcpy(grain, g_d, sizeof(int) * nv, cudaMemcpyDeviceToHost));
    }
    for (long long k = 0; k < nn && k < cap && sites; k++) sites[k] = sv[k];
    *n_new = nn;
  }
  cudaFree(g_d); cudaFree(w_d); cudaFree(c_d); cudaFree(r_d); cudaFree(s_d); cudaFree(n_d);
  return st;
}

// ------------------------------------------------- allocation-free local solve
extern "C" mth_status mth_local_solve_noalloc(const mth_params* p, const double c066[36], size_t n, double* d_sig,
                                              const double* d_eps_p, const double* d_strain, const double* d_rot,
                                              const double* d_crss, double* d_edot, double* d_err,
                                              long long* newton_iters, void* stream) {
  if (!p || !c066 || !d_sig || !d_eps_p || !d_strain || !d_rot || !d_crss || !d_edot || !d_err)
    return set_err(MTH_ERR_ARG, "null argument");
  if (p->flow_law != 0) return set_err(MTH_ERR_UNSUPPORTED, "the array-level local solve runs the power law only");
  if (n > (size_t)noalloc_max_voxels())
    return set_err(MTH_ERR_ARG, "n=%zu exceeds the allocation-free limit of %lld voxels", n, noalloc_max_voxels());
  if (n == 0) {
    if (newton_iters) *newton_iters = 0;
    return MTH_OK;
  }
  NewtonConst nc;
  memset(&nc, 0, sizeof(nc));
  mth_status s = fill_phase(p->phase[0], nc.ph[0]);
  if (s) return s;
  if (p->phase[0].type != 0) return set_err(MTH_ERR_ARG, "phase 1 must be a crystal");
  double cm[6][6], sm[6][6];
  for (int i = 0; i < 6; i++)
    for (int j = 0; j < 6; j++) cm[i][j] = c066[i * 6 + j];
  if (!inv6(cm, sm)) return set_err(MTH_ERR_SINGULAR, "C066 singular");
  for (int i = 0; i < 5; i++)
    for (int j = 0; j < 5; j++) nc.s0dev[i * 5 + j] = sm[i][j];
  nc.s0hh = sm[5][5];
  nc.dt = p->time_step;
  nc.tol = p->newton_tol > 0 ? p->newton_tol : 1e-10;
  nc.itmax = p->newton_itmax > 0 ? p->newton_itmax : 500;
  // the solve runs with params->device current; the caller's current device
  // is restored on return
  int caller_dev = 0;
  CK(cudaGetDevice(&caller_dev));
  cudaError_t e = cudaSetDevice(p->device);
  if (e == cudaSuccess)
    e = launch_local_solve_noalloc(nc, (long long)n, d_sig, d_eps_p, d_strain, d_rot, d_crss, d_edot, d_err,
                                   newton_iters, static_cast<cudaStream_t>(stream));
  const cudaError_t e2 = cudaSetDevice(caller_dev);
  if (e == cudaSuccess) e = e2;
  if (e != cudaSuccess) return set_err(MTH_ERR_CUDA, "allocation-free local solve: %s", cudaGetErrorString(e));
  return MTH_OK;
}

// ------------------------------------------------------------ local solve
extern "C" mth_status mth_local_solve(const mth_params* p, const double c066[36], size_t n, double* sig,
                                      const double* eps_p, const double* strain, const double* rot,
                                      const double* crss, double* edot, double* err, long long* newton_iters) {
  if (!p || !c066 || !sig || !eps_p || !strain || !rot || !crss || !edot || !err)
    return set_err(MTH_ERR_ARG, "null argument");
  if (p->flow_law != 0) return set_err(MTH_ERR_UNSUPPORTED, "the array-level local solve runs the power law only");
  if (n == 0) {
    if (newton_iters) *newton_iters = 0;
    return MTH_OK;
  }
  NewtonConst nc;
  memset(&nc, 0, sizeof(nc));
  mth_status s = fill_phase(p->phase[0], nc.ph[0]);
  if (s) return s;
  if (p->phase[0].type != 0) return set_err(MTH_ERR_ARG, "phase 1 must be a crystal");
  double cm[6][6], sm[6][6];
  for (int i = 0; i < 6; i++)
    for (int j = 0; j < 6; j++) cm[i][j] = c066[i * 6 + j];
  if (!inv6(cm, sm)) return set_err(MTH_ERR_SINGULAR, "C066 singular");
  for (int i = 0; i < 5; i++)
    for (int j = 0; j < 5; j++) nc.s0dev[i * 5 + j] = sm[i][j];
  nc.s0hh = sm[5][5];
  nc.dt = p->time_step;
  nc.tol = p->newton_tol > 0 ? p->newton_tol : 1e-10;
  nc.itmax = p->newton_itmax > 0 ? p->newton_itmax : 500;
  CK(cudaSetDevice(p->device));
  cudaStream_t st;
  CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  double *ds, *de, *dst, *dr, *dc, *ded, *der;
  long long* dit;
  CK(cudaMalloc(&ds, sizeof(double) * 6 * n));
  CK(cudaMalloc(&de, sizeof(double) * 6 * n));
  CK(cudaMalloc(&dst, sizeof(double) * 6 * n));
  CK(cudaMalloc(&dr, sizeof(double) * 9 * n));
  CK(cudaMalloc(&dc, sizeof(double) * 12 * n));
  CK(cudaMalloc(&ded, sizeof(double) * 6 * n));
  CK(cudaMalloc(&der, sizeof(double) * 2 * n));
  CK(cudaMalloc(&dit, sizeof(long long) * n));
  CK(cudaMemcpyAsync(ds, sig, sizeof(double) * 6 * n, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(de, eps_p, sizeof(double) * 6 * n, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(dst, strain, sizeof(double) * 6 * n, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(dr, rot, sizeof(double) * 9 * n, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(dc, crss, sizeof(double) * 12 * n, cudaMemcpyHostToDevice, st));
  std::vector<double> rows(n * ETAB_W);
  for (size_t v = 0; v < n; v++) {
    class_row(nc.ph[0], rot + 9 * v, &rows[v * ETAB_W]);
    class_row_add_s0(&rows[v * ETAB_W], sm);
  }
  double* det;
  CK(cudaMalloc(&det, sizeof(double) * rows.size()));
  CK(cudaMemcpyAsync(det, rows.data(), sizeof(double) * rows.size(), cudaMemcpyHostToDevice, st));
  CK(launch_local_solve(nc, (long long)n, ds, de, dst, dr, dc, det, ded, der, dit, st));
  std::vector<long long> it(n);
  CK(cudaMemcpyAsync(sig, ds, sizeof(double) * 6 * n, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(edot, ded, sizeof(double) * 6 * n, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(err, der, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(it.data(), dit, sizeof(long long) * n, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  long long tot = 0;
  for (size_t v = 0; v < n; v++) tot += it[v];
  if (newton_iters) *newton_iters = tot;
  cudaFree(ds); cudaFree(de); cudaFree(dst); cudaFree(dr); cudaFree(dc); cudaFree(ded); cudaFree(der); cudaFree(dit);
  cudaFree(det);
  cudaStreamDestroy(st);
  return MTH_OK;
}


// capi_batch.cu -- batches of independent RVEs (mth_batch_*).
#include <algorithm>
#include "capi_internal.h"

// ------------------------------------------------------------ RVE batches
// n independent volumes (own parameters, microstructure and grid size) on
// one GPU.  Every member is an ordinary context whose stream, reduction
// slot, error flag, strain-increment and live flag live in the batch.  One
// Green iteration of the whole batch is one launch of a CUDA graph:
//   H2D (strain increments and live flags of all members)
//   -> per member, as parallel branches: its FFT passes, Newton, reduction
//   -> D2H (reduced sums and error flags of all members).
// A member that has converged keeps its branch but its live flag is 0, so
// its kernels return at once.  The graph is captured again when the Newton
// constants baked into its kernel parameters change (the first step runs
// with the flow rule off).  For each distinct grid size and precision the
// batch times the TMA and the shared-memory FFT passes once on a scratch
// volume and keeps the faster (cached for the process).
struct mth_batch {
  int n = 0;
  int device = 0;
  cudaStream_t st = nullptr;
  std::vector<mth_ctx*> rve;
  std::vector<cudaStream_t> branch;
  std::vector<cudaEvent_t> join;
  cudaEvent_t fork = nullptr;
  double* add_d = nullptr;
  int* live_d = nullptr;
  int* live_h = nullptr;
  double* red_d = nullptr;
  int* err_d = nullptr;
  int* err_h = nullptr;
  int* ctl_d = nullptr;   // iterations the step's loop ran, and whether it hit its bound
  int* ctl_h = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<NewtonConst> cap_nc;
};

namespace {
constexpr int BATCH_RED = 32;   // reduction slot of a member (doubles)

void batch_free(mth_batch* b) {
  if (!b) return;
  if (b->st) cudaStreamSynchronize(b->st);
  for (mth_ctx* c : b->rve) ctx_free(c);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  for (cudaStream_t s : b->branch) cudaStreamDestroy(s);
  for (cudaEvent_t e : b->join) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  cudaFree(b->add_d);
  cudaFree(b->live_d);
  cudaFree(b->red_d);
  cudaFree(b->err_d);
  cudaFree(b->ctl_d);
  if (b->ctl_h) cudaFreeHost(b->ctl_h);
  if (b->live_h) cudaFreeHost(b->live_h);
  if (b->err_h) cudaFreeHost(b->err_h);
  if (b->st) cudaStreamDestroy(b->st);
  delete b;
}

// FFT pass choice per (grid, precision): TMA or shared-memory passes, and
// the TMA passes' tile widths (kz columns per block of the strided and the
// Green pass)
struct PassChoice {
  int tma, ks, kg;
};
std::map<std::vector<int>, PassChoice>& tuned_passes() {
  static std::map<std::vector<int>, PassChoice> m;
  return m;
}

// Times Green iterations of a scratch volume with the parameters of p
// (single grain, no pores; at least 3 iterations and about 2^21
// voxel-iterations, at most 64 iterations) for each candidate: the
// shared-memory passes, the strided pass's three compiled tile widths, then
// the Green pass's three with the best strided width (the passes are
// separate kernels, so their times add).  The best of two timed runs after a
// warm-up run counts.
mth_status tune_passes(const mth_params& p, PassChoice* out) {
  std::vector<int> key = {p.cell_dim[0], p.cell_dim[1], p.cell_dim[2], p.precision};
  auto it = tuned_passes().find(key);
  if (it != tuned_passes().end()) { *out = it->second; return MTH_OK; }
  mth_ctx* c = nullptr;
  mth_status s = mth_create(&p, &c);
  if (s) return s;
  *out = {0, 0, 0};
  if (!tma_has(c->tma, 0) && !tma_has(c->tma, 1) && !tma_has(c->tma, 2)) {
    ctx_free(c);
    tuned_passes()[key] = *out;
    return MTH_OK;
  }
  const size_t nv = (size_t)c->nv;
  std::vector<int> grain(nv, 1), phase(nv, 1);
  std::vector<double> eul(3 * nv, 0.0);
  s = mth_upload_microstructure(c, grain.data(), phase.data(), eul.data(), nv);
  if (s) { ctx_free(c); return s; }
  c->add_h[0] = c->add_h[1] = c->add_h[2] = c->add_h[3] = c->add_h[4] = c->add_h[5] = 0.0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int its = (int)std::min<long long>(64, std::max<long long>(3, (1LL << 21) / std::max<long long>(1, c->nv)));
  auto time = [&](float* best) {
    *best = 3.4e38f;
    for (int rep = 0; rep < 3 && !s; rep++) {   // the first run warms up
      if (cudaEventRecord(e0, c->st) != cudaSuccess) { s = set_err(MTH_ERR_CUDA, "pass tuning"); break; }
      for (int k = 0; k < its && !s; k++) s = c->mixed ? green_iteration<float>(c) : green_iteration<double>(c);
      if (s) break;
      cudaEventRecord(e1, c->st);
      cudaStreamSynchronize(c->st);
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep && ms < *best) *best = ms;
    }
  };
  float t_smem = 0, t_best = 3.4e38f;
  c->tma_off = true;
  time(&t_smem);
  c->tma_off = false;
  int ks_def = 0, kg_def = 0;
  tma_tiles(c->tma, &ks_def, &kg_def);
  PassChoice best = {1, ks_def, kg_def};
  for (int pass = 1; pass <= 2 && !s; pass++)
    for (int i = 0; i < 3 && !s; i++) {
      const int w = tma_tile_choice(c->mixed, pass, i);
      PassChoice cand = pass == 1 ? PassChoice{1, w, kg_def} : PassChoice{1, best.ks, w};
      ctx_set_tiles(c, cand.ks, cand.kg);
      float t = 0;
      time(&t);
      if (!s && t < t_best) { t_best = t; best = cand; }
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (cudaStreamSynchronize(c->st) != cudaSuccess && !s) s = set_err(MTH_ERR_CUDA, "pass tuning failed");
  if (!s && *c->err_h) s = set_err(MTH_ERR_TIMEOUT, "pass tuning timed out");
  ctx_free(c);
  if (s) return s;
  *out = t_smem < t_best ? PassChoice{0, 0, 0} : best;
  tuned_passes()[key] = *out;
  return MTH_OK;
}

// The Green-iteration loop of a mechanical step of every member, as one
// graph: a while node whose body is one iteration of all members (each
// member's FFT passes, Newton, reduction and one-warp bookkeeping as a
// parallel branch, gated by its live flag) followed by a one-thread kernel
// that continues the loop while a member is live.  The bookkeeping kernels
// (book.cu) drop a member's flag when it is done, so one graph launch runs
// the step's iterations with no host round trip; the loop also ends on a
// tile-wait time-out and after `bound` iterations (an error).
__global__ void batch_more_kernel(cudaGraphConditionalHandle h, const int* __restrict__ live,
                                  const int* __restrict__ err, int n, int* __restrict__ ctl, int bound) {
  if (threadIdx.x != 0) return;
  int any = 0, bad = 0;
  for (int i = 0; i < n; i++) {
    any |= live[i];
    bad |= err[i];
  }
  const int it = ++ctl[0];
  if (any && it >= bound) ctl[1] = 1;
  cudaGraphSetConditional(h, (any && !bad && it < bound) ? 1u : 0u);
}

mth_status batch_capture(mth_batch* b) {
  if (b->exec) {
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
  const int n = b->n;
  int bound = 1;
  for (mth_ctx* c : b->rve) bound = std::max(bound, c->p.iter_max + 1);
  mth_status s = MTH_OK;
  auto ck = [&](cudaError_t e) {
    if (e != cudaSuccess && !s) s = set_err(MTH_ERR_CUDA, "batch graph capture: %s", cudaGetErrorString(e));
  };
  cudaGraph_t g = nullptr;
  CK(cudaGraphCreate(&g, 0));
  cudaGraphConditionalHandle h;
  ck(cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault));
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = h;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t loop = nullptr;
  if (!s) ck(cudaGraphAddNode(&loop, g, nullptr, nullptr, 0, &cp));
  cudaGraph_t body = s ? nullptr : cp.conditional.phGraph_out[0];
  if (!s) ck(cudaStreamBeginCaptureToGraph(b->st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  if (!s) {
    ck(cudaEventRecord(b->fork, b->st));
    for (int i = 0; i < n && !s; i++) {
      mth_ctx* c = b->rve[i];
      ck(cudaStreamWaitEvent(b->branch[i], b->fork, 0));
      const int prof = c->prof_on;
      c->prof_on = 0;
      c->st = b->branch[i];
      if (!s) s = c->mixed ? green_iteration<float>(c) : green_iteration<double>(c);
      if (!s) s = launch_reduce(c, NPART, true);
      if (!s) ck(launch_iter_book(c->bk_d, c->red, c->add_d, c->live_d, 0, c->st, 0));
      c->st = b->st;
      c->prof_on = prof;
      ck(cudaEventRecord(b->join[i], b->branch[i]));
      ck(cudaStreamWaitEvent(b->st, b->join[i], 0));
    }
    batch_more_kernel<<<1, 32, 0, b->st>>>(h, b->live_d, b->err_d, n, b->ctl_d, bound);
    ck(cudaGetLastError());
    cudaGraph_t out = nullptr;
    cudaError_t e = cudaStreamEndCapture(b->st, &out);
    if (!s && e != cudaSuccess) s = set_err(MTH_ERR_CUDA, "batch graph capture: %s", cudaGetErrorString(e));
  }
  if (!s) {
    cudaError_t e = cudaGraphInstantiate(&b->exec, g, 0);
    if (e != cudaSuccess) s = set_err(MTH_ERR_CUDA, "batch graph instantiate: %s", cudaGetErrorString(e));
  }
  cudaGraphDestroy(g);
  if (s) return s;
  b->cap_nc.resize(n);
  for (int i = 0; i < n; i++) b->cap_nc[i] = b->rve[i]->nc;
  return MTH_OK;
}
}  // namespace

extern "C" mth_status mth_batch_create(const mth_params* params, int n, mth_batch** out) {
  if (!params || !out || n <= 0) return set_err(MTH_ERR_ARG, "batch needs params, out and n > 0");
  *out = nullptr;
  for (int i = 0; i < n; i++) {
    if (params[i].device != params[0].device) return set_err(MTH_ERR_ARG, "batch members on different devices");
    if (params[i].pf_substeps > 0) return set_err(MTH_ERR_UNSUPPORTED, "recrystallisation in a batch member");
    if (params[i].flow_law != 0) return set_err(MTH_ERR_UNSUPPORTED, "dislocation-density law in a batch member");
  }
  mth_batch* b = new mth_batch();
  b->n = n;
  b->device = params[0].device;
  mth_status s = MTH_OK;
  auto ck = [&](cudaError_t e) {
    if (e != cudaSuccess && !s)
      s = set_err(e == cudaErrorMemoryAllocation ? MTH_ERR_NOMEM : MTH_ERR_CUDA, "batch: %s", cudaGetErrorString(e));
  };
  for (int i = 0; i < n && !s; i++) {
    mth_ctx* c = nullptr;
    s = mth_create(&params[i], &c);
    if (!s) b->rve.push_back(c);
  }
  if (!s) {
    ck(cudaSetDevice(b->device));
    ck(cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking));
    ck(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
    b->branch.resize(n, nullptr);
    b->join.resize(n, nullptr);
    for (int i = 0; i < n; i++) {
      ck(cudaStreamCreateWithFlags(&b->branch[i], cudaStreamNonBlocking));
      ck(cudaEventCreateWithFlags(&b->join[i], cudaEventDisableTiming));
    }
    ck(cudaMalloc(&b->add_d, sizeof(double) * 8 * n));
    ck(cudaMalloc(&b->live_d, sizeof(int) * n));
    ck(cudaMalloc(&b->red_d, sizeof(double) * BATCH_RED * n));
    ck(cudaMalloc(&b->err_d, sizeof(int) * n));
    ck(cudaMalloc(&b->ctl_d, sizeof(int) * 2));
    ck(cudaMallocHost(&b->ctl_h, sizeof(int) * 2));
    ck(cudaMallocHost(&b->live_h, sizeof(int) * n));
    ck(cudaMallocHost(&b->err_h, sizeof(int) * n));
  }
  if (!s) {
    ck(cudaMemset(b->add_d, 0, sizeof(double) * 8 * n));
    ck(cudaMemset(b->err_d, 0, sizeof(int) * n));
    memset(b->err_h, 0, sizeof(int) * n);
    for (int i = 0; i < n; i++) b->live_h[i] = 1;
    ck(cudaMemcpy(b->live_d, b->live_h, sizeof(int) * n, cudaMemcpyHostToDevice));
  }
  for (int i = 0; i < n && !s; i++) {
    mth_ctx* c = b->rve[i];
    PassChoice pc;
    s = tune_passes(params[i], &pc);
    if (s) break;
    c->tma_off = !pc.tma;
    if (pc.tma) ctx_set_tiles(c, pc.ks, pc.kg);
    ck(cudaStreamSynchronize(c->st));
    cudaStreamDestroy(c->st);
    cudaFree(c->red);
    cudaFree(c->err_d);
    cudaFree(c->add_d);
    cudaFree(c->live_d);
    c->st = b->st;
    c->red = b->red_d + (size_t)BATCH_RED * i;
    c->err_d = b->err_d + i;
    c->add_d = b->add_d + (size_t)8 * i;
    c->live_d = b->live_d + i;
    c->in_batch = true;
  }
  if (s) {
    batch_free(b);
    return s;
  }
  *out = b;
  return MTH_OK;
}

extern "C" mth_status mth_batch_passes(const mth_batch* b, int i, int* tma, int* kz_strided, int* kz_green) {
  if (!b || i < 0 || i >= b->n || !tma || !kz_strided || !kz_green) return set_err(MTH_ERR_ARG, "batch member %d", i);
  const mth_ctx* c = b->rve[i];
  *tma = c->tma_off ? 0 : (tma_has(c->tma, 0) || tma_has(c->tma, 1) || tma_has(c->tma, 2)) ? 1 : 0;
  *kz_strided = *kz_green = 0;
  if (*tma) tma_tiles(c->tma, kz_strided, kz_green);
  return MTH_OK;
}

extern "C" mth_status mth_batch_upload(mth_batch* b, int i, const int* grain, const int* phase, const double* euler_deg,
                                       size_t n_voxels) {
  if (!b || i < 0 || i >= b->n) return set_err(MTH_ERR_ARG, "batch member %d", i);
  return mth_upload_microstructure(b->rve[i], grain, phase, euler_deg, n_voxels);
}

extern "C" mth_status mth_batch_step(mth_batch* b, mth_step_report* reports) {
  if (!b) return set_err(MTH_ERR_ARG, "null batch");
  CK(cudaSetDevice(b->device));
  const int n = b->n;
  for (int i = 0; i < n; i++)
    if (!b->rve[i]->uploaded) return set_err(MTH_ERR_STATE, "batch member %d has no microstructure", i);
  for (int i = 0; i < n; i++) {
    mth_status s = step_begin(b->rve[i]);
    if (s) return s;
  }
  bool recapture = !b->exec;
  for (int i = 0; i < n && !recapture; i++)
    recapture = memcmp(&b->cap_nc[i], &b->rve[i]->nc, sizeof(NewtonConst)) != 0;
  if (recapture) {
    mth_status s = batch_capture(b);
    if (s) return s;
  }
  // each member's bookkeeping to the device and its first iteration's
  // increment (live flags set), then the step's iterations in one launch
  for (int i = 0; i < n; i++) {
    mth_ctx* c = b->rve[i];
    CK(cudaMemcpyAsync(c->bk_d, &c->bk, sizeof(IterBook), cudaMemcpyHostToDevice, b->st));
    CK(launch_iter_book(c->bk_d, c->red, c->add_d, c->live_d, 1, b->st, 0));
  }
  CK(cudaMemsetAsync(b->ctl_d, 0, sizeof(int) * 2, b->st));
  CK(cudaGraphLaunch(b->exec, b->st));
  CK(cudaMemcpyAsync(b->ctl_h, b->ctl_d, sizeof(int) * 2, cudaMemcpyDeviceToHost, b->st));
  CK(cudaMemcpyAsync(b->err_h, b->err_d, sizeof(int) * n, cudaMemcpyDeviceToHost, b->st));
  for (int i = 0; i < n; i++) {
    mth_ctx* c = b->rve[i];
    CK(cudaMemcpyAsync(&c->bk, c->bk_d, sizeof(IterBook), cudaMemcpyDeviceToHost, b->st));
    b->live_h[i] = 1;
  }
  CK(cudaMemcpyAsync(b->live_d, b->live_h, sizeof(int) * n, cudaMemcpyHostToDevice, b->st));
  CK(cudaStreamSynchronize(b->st));
  for (int i = 0; i < n; i++)
    if (b->err_h[i]) return set_err(MTH_ERR_TIMEOUT, "batch member %d: a kernel timed out waiting for its tile copies", i);
  if (b->ctl_h[1]) return set_err(MTH_ERR_CUDA, "batch: the iteration loop reached its bound");
  for (int i = 0; i < n; i++)
    if (b->rve[i]->bk.nan)
      return set_err(MTH_ERR_NAN, "batch member %d: non-finite value in the Green iteration (step %d, iteration %d)", i,
                     b->rve[i]->istep, b->rve[i]->bk.it_iter);
  for (int i = 0; i < n; i++) {
    mth_status s = step_end(b->rve[i], reports ? &reports[i] : nullptr);
    if (s) return s;
  }
  return MTH_OK;
}

extern "C" mth_status mth_batch_download_field(mth_batch* b, int i, int field, double* host, size_t n_values) {
  if (!b || i < 0 || i >= b->n) return set_err(MTH_ERR_ARG, "batch member %d", i);
  return mth_download_field(b->rve[i], field, host, n_values);
}

extern "C" mth_status mth_batch_destroy(mth_batch* b) {
  if (!b) return set_err(MTH_ERR_ARG, "null batch");
  cudaSetDevice(b->device);
  batch_free(b);
  return MTH_OK;
}


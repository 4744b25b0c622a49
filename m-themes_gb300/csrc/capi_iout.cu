// capi_iout.cu -- per-step field files in the reference's .iout layout (mth_write_iout,
// mth_iout_wait).
#include "capi_internal.h"

// ------------------------------------------------------ field files (.iout)
// The reference's writers (src/io.c:247-541) dump raw native values with
// MPI-IO, one file per component.  Here the fields are copied device to
// device at the call (ordered with the context's stream, so the next step
// cannot overwrite them first); a background thread copies the snapshot to
// pinned host memory on its own stream, converts and writes the files while
// the caller goes on stepping.
struct IoutWriter {
  std::thread th;
  int device = 0;
  cudaStream_t io = nullptr;
  cudaEvent_t snap = nullptr;
  void* stage_d = nullptr;
  size_t stage_cap = 0;
  void* stage_h = nullptr;
  size_t host_cap = 0;
  mth_status status = MTH_OK;
  char msg[512] = "";
};

// 48-byte record of WriteTextureMPI (src/io.c:480-487)
struct TexRecord {
  double angle[3];
  int coord[3];
  int jgr, jph, buff;
};
static_assert(sizeof(TexRecord) == 48, "texture record layout");

static void iout_join(IoutWriter* w) {
  if (w && w->th.joinable()) w->th.join();
}

void iout_free(IoutWriter* w) {
  if (!w) return;
  iout_join(w);
  cudaSetDevice(w->device);
  cudaFree(w->stage_d);
  if (w->stage_h) cudaFreeHost(w->stage_h);
  if (w->snap) cudaEventDestroy(w->snap);
  if (w->io) cudaStreamDestroy(w->io);
  delete w;
}

// matrix -> Bunge angles in degrees, EulerToTransMatrix opt 1
// (src/kinematics.c:186-215); a = sample->crystal matrix
static void rot_to_bunge(const double a[3][3], double out[3]) {
  const double pi = 3.14159265358979323846;
  double t1, ph, t2;
  ph = acos(a[2][2]);
  if (fabs(a[2][2]) > 0.9999) {
    t2 = 0.;
    t1 = atan2(a[0][1], a[0][0]);
  } else {
    const double sph = sin(ph);
    t1 = atan2(a[2][0] / sph, -1.0 * a[2][1] / sph);
    t2 = atan2(a[0][2] / sph, a[1][2] / sph);
  }
  out[0] = t1 * 180. / pi;
  out[1] = ph * 180. / pi;
  out[2] = t2 * 180. / pi;
}

static bool write_file(const std::string& name, const void* data, size_t bytes, char* msg) {
  FILE* f = fopen(name.c_str(), "wb");
  if (!f) { snprintf(msg, 512, "cannot open %s", name.c_str()); return false; }
  const size_t w = fwrite(data, 1, bytes, f);
  const bool ok = (w == bytes) && fclose(f) == 0;
  if (w != bytes) fclose(f);
  if (!ok) snprintf(msg, 512, "short write to %s", name.c_str());
  return ok;
}

template <typename T>
static void iout_work(IoutWriter* w, int kind, std::string prefix, int step, long long P, int n0, int n1, int n2,
                      size_t bytes) {
  w->status = MTH_OK;
  auto fail = [&](mth_status s, const char* m) {
    w->status = s;
    snprintf(w->msg, sizeof(w->msg), "%s", m);
  };
  if (cudaSetDevice(w->device) != cudaSuccess || cudaStreamWaitEvent(w->io, w->snap, 0) != cudaSuccess ||
      cudaMemcpyAsync(w->stage_h, w->stage_d, bytes, cudaMemcpyDeviceToHost, w->io) != cudaSuccess ||
      cudaStreamSynchronize(w->io) != cudaSuccess)
    return fail(MTH_ERR_CUDA, "field file copy failed");
  char sfx[32];
  snprintf(sfx, sizeof(sfx), "S%06d.iout", step);
  if (kind == MTH_IOUT_GRAIN) {
    if (!write_file(prefix + "_" + sfx, w->stage_h, sizeof(int) * P, w->msg)) w->status = MTH_ERR_IO;
    return;
  }
  if (kind == MTH_IOUT_TEXTURE) {
    const T* rot = static_cast<const T*>(w->stage_h);
    const int* grain = reinterpret_cast<const int*>(rot + 9 * P);
    const uint8_t* phase = reinterpret_cast<const uint8_t*>(grain + P);
    std::vector<TexRecord> rec(P);
    for (long long v = 0; v < P; v++) {
      double a[3][3];
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) a[i][j] = (double)rot[(j * 3 + i) * P + v];   // transpose: sample->crystal
      TexRecord& r = rec[v];
      rot_to_bunge(a, r.angle);
      r.coord[0] = (int)(v / ((long long)n1 * n2)) + 1;
      r.coord[1] = (int)((v / n2) % n1) + 1;
      r.coord[2] = (int)(v % n2) + 1;
      r.jgr = grain[v];
      r.jph = (int)phase[v] + 1;
      r.buff = 0;
    }
    (void)n0;
    if (!write_file(prefix + "_" + sfx, rec.data(), sizeof(TexRecord) * P, w->msg)) w->status = MTH_ERR_IO;
    return;
  }
  // components 11, 22, 33, 23, 13, 12 (src/io.c:292-305, 404-418) of a
  // symmetric tensor, or of DisGrad: the strain's plus the antisymmetric
  // planes (W21, W02, W10), W23 = -W21, W13 = W02, W12 = -W10
  const T* a = static_cast<const T*>(w->stage_h);
  const T* b = kind == MTH_IOUT_ELS ? a + 6 * P : nullptr;   // ELS: strain - plastic strain
  const T* sk = kind == MTH_IOUT_DISGRAD ? a + 6 * P : nullptr;
  static const int ci[6][2] = {{0, 0}, {1, 1}, {2, 2}, {1, 2}, {0, 2}, {0, 1}};
  std::vector<double> comp((size_t)6 * P);
  for (long long v = 0; v < P; v++) {
    double s6[6];
    t33 t;
    for (int i = 0; i < 6; i++) s6[i] = (double)a[i * P + v] - (b ? (double)b[i * P + v] : 0.0);
    v2t(s6, t, 6);
    for (int c = 0; c < 6; c++) comp[c * P + v] = t[ci[c][0]][ci[c][1]];
    if (sk) {
      comp[3 * P + v] -= (double)sk[v];
      comp[4 * P + v] += (double)sk[P + v];
      comp[5 * P + v] -= (double)sk[2 * P + v];
    }
  }
  for (int c = 0; c < 6; c++) {
    if (!write_file(prefix + "_" + std::to_string(c + 1) + "_" + sfx, comp.data() + c * P, sizeof(double) * P,
                    w->msg)) {
      w->status = MTH_ERR_IO;
      return;
    }
  }
}

template <typename T>
static mth_status iout_start(mth_ctx* c, int kind, const char* prefix, int step) {
  const Fields<T>& f = *reinterpret_cast<const Fields<T>*>(c->mixed ? (void*)&c->ff : (void*)&c->fd);
  const long long P = c->nv;
  const size_t w = sizeof(T);
  size_t bytes;
  switch (kind) {
    case MTH_IOUT_SIG: case MTH_IOUT_EPS: case MTH_IOUT_EDOT: bytes = 6 * P * w; break;
    case MTH_IOUT_ELS: bytes = 12 * P * w; break;
    case MTH_IOUT_DISGRAD: bytes = 9 * P * w; break;
    case MTH_IOUT_GRAIN: bytes = sizeof(int) * P; break;
    case MTH_IOUT_TEXTURE: bytes = 9 * P * w + sizeof(int) * P + P; break;
    default: return set_err(MTH_ERR_ARG, "iout kind %d", kind);
  }
  if (!c->iout) {
    c->iout = new IoutWriter();
    c->iout->device = c->p.device;
    CK(cudaStreamCreateWithFlags(&c->iout->io, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&c->iout->snap, cudaEventDisableTiming));
  }
  IoutWriter* wr = c->iout;
  iout_join(wr);   // one write in flight: its staging buffers are reused
  if (wr->stage_cap < bytes) {
    cudaFree(wr->stage_d);
    wr->stage_d = nullptr;
    wr->stage_cap = 0;
    CK(cudaMalloc(&wr->stage_d, bytes));
    wr->stage_cap = bytes;
  }
  if (wr->host_cap < bytes) {
    if (wr->stage_h) cudaFreeHost(wr->stage_h);
    wr->stage_h = nullptr;
    wr->host_cap = 0;
    CK(cudaMallocHost(&wr->stage_h, bytes));
    wr->host_cap = bytes;
  }
  char* d = static_cast<char*>(wr->stage_d);
  auto snap = [&](const void* src, size_t n) -> cudaError_t {
    cudaError_t e = cudaMemcpyAsync(d, src, n, cudaMemcpyDeviceToDevice, c->st);
    d += n;
    return e;
  };
  switch (kind) {
    case MTH_IOUT_SIG: CK(snap(f.sig, 6 * P * w)); break;
    case MTH_IOUT_EPS: CK(snap(f.epsp, 6 * P * w)); break;
    case MTH_IOUT_EDOT: CK(snap(f.edot, 6 * P * w)); break;
    case MTH_IOUT_ELS: CK(snap(f.strain, 6 * P * w)); CK(snap(f.epsp, 6 * P * w)); break;
    case MTH_IOUT_DISGRAD: CK(snap(f.strain, 6 * P * w)); CK(snap(c->skew_d, 3 * P * w)); break;
    case MTH_IOUT_GRAIN: CK(snap(c->grain_d, sizeof(int) * P)); break;
    case MTH_IOUT_TEXTURE:
      CK(snap(f.rot, 9 * P * w));
      CK(snap(c->grain_d, sizeof(int) * P));
      CK(snap(c->phase_d, (size_t)P));
      break;
  }
  CK(cudaEventRecord(wr->snap, c->st));
  wr->th = std::thread(iout_work<T>, wr, kind, std::string(prefix), step, P, c->n[0], c->n[1], c->n[2], bytes);
  return MTH_OK;
}

extern "C" mth_status mth_write_iout(mth_ctx* c, int kind, const char* prefix, int step) {
  if (!c || !prefix) return set_err(MTH_ERR_ARG, "null argument");
  if (!c->uploaded) return set_err(MTH_ERR_STATE, "no microstructure uploaded");
  if (kind < MTH_IOUT_SIG || kind > MTH_IOUT_DISGRAD) return set_err(MTH_ERR_ARG, "iout kind %d", kind);
  if (kind == MTH_IOUT_DISGRAD && !c->skew_d)
    return set_err(MTH_ERR_STATE, "DisGrad is kept only after mth_track_disgrad (before the first step)");
  SETDEV(c);
  if (c->iout) {   // report a failure of the previous write before starting the next
    iout_join(c->iout);
    if (c->iout->status) {
      const mth_status s = c->iout->status;
      c->iout->status = MTH_OK;
      return set_err(s, "%s", c->iout->msg);
    }
  }
  return c->mixed ? iout_start<float>(c, kind, prefix, step) : iout_start<double>(c, kind, prefix, step);
}

extern "C" mth_status mth_iout_wait(mth_ctx* c) {
  if (!c) return set_err(MTH_ERR_ARG, "null context");
  if (!c->iout) return MTH_OK;
  iout_join(c->iout);
  if (c->iout->status) {
    const mth_status s = c->iout->status;
    c->iout->status = MTH_OK;
    return set_err(s, "%s", c->iout->msg);
  }
  return MTH_OK;
}


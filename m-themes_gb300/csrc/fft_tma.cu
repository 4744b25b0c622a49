// fft_tma.cu -- TMA-staged FFT passes of one Green iteration for the line
// lengths with compile-time plans (16, 32, 48, 64, 96, 128, 256).
//
// Same passes and results as fft_green.cu (src/evolution.c:1361-1405), laid
// out for GB300:
//   * every tile moves between HBM and shared memory with the tensor memory
//     accelerator (cp.async.bulk.tensor loads completing on an mbarrier,
//     bulk-group stores), so a block has its whole tile in flight at once
//     and no register round trip;
//   * the 1-D transforms run in place: each Stockham stage reads its
//     butterfly inputs into registers, synchronises, and writes the outputs
//     back into the same tile, which halves the shared memory of a two-buffer
//     Stockham and raises the number of resident blocks;
//   * the y and x passes take one spectrum component per block (the Green
//     pass needs all six at a wave vector and takes them together);
//   * the z passes transform a real line of N points as an N/2-point complex
//     line (even samples real, odd samples imaginary) plus the split step of
//     the real FFT, so the tile read by TMA is the complex input as it lies.
// Waits on the mbarrier are bounded (about one second); on time-out the
// block raises the error flag the host reads after the iteration.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cstdio>
#include <cstring>
#include "mth_common.cuh"
#include "mth_internal.h"
#include "green_op.cuh"
#include "fft_core.cuh"

namespace mth {

// ------------------------------------------------------------ TMA helpers
namespace {

constexpr unsigned long long WAIT_NS = 1000000000ULL;   // bounded mbarrier wait

__device__ __forceinline__ uint32_t sh(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* b) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sh(b)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(sh(b)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity) {
  const unsigned long long t0 = gtimer();
  while (true) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(sh(b)), "r"(parity)
        : "memory");
    if (ok) return true;
    if (gtimer() - t0 > WAIT_NS) return false;
  }
}

__device__ __forceinline__ void tma_load3(void* dst, const CUtensorMap* m, int x, int y, int z, uint64_t* b) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(sh(dst)),
      "l"(reinterpret_cast<uint64_t>(m)), "r"(x), "r"(y), "r"(z), "r"(sh(b))
      : "memory");
}
__device__ __forceinline__ void tma_load4(void* dst, const CUtensorMap* m, int x, int y, int z, int w, uint64_t* b) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"(sh(dst)),
      "l"(reinterpret_cast<uint64_t>(m)), "r"(x), "r"(y), "r"(z), "r"(w), "r"(sh(b))
      : "memory");
}
__device__ __forceinline__ void tma_store3(const CUtensorMap* m, const void* src, int x, int y, int z) {
  asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%2, %3, %4}], [%1];" ::"l"(
                   reinterpret_cast<uint64_t>(m)),
               "r"(sh(src)), "r"(x), "r"(y), "r"(z)
               : "memory");
}
__device__ __forceinline__ void tma_store4(const CUtensorMap* m, const void* src, int x, int y, int z, int w) {
  asm volatile("cp.async.bulk.tensor.4d.global.shared::cta.tile.bulk_group [%0, {%2, %3, %4, %5}], [%1];" ::"l"(
                   reinterpret_cast<uint64_t>(m)),
               "r"(sh(src)), "r"(x), "r"(y), "r"(z), "r"(w)
               : "memory");
}
__device__ __forceinline__ void tma_store_commit_wait() {
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}
// generic-proxy writes to shared memory visible to the following TMA store
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Failure-path test hook (tma_set_wait_probe): when set, every block's first
// wait reports a time-out at once; the drain wait below still waits for the
// real copies, so nothing is left in flight and the kernels return normally.
__device__ int g_tile_wait_probe = 0;

// Thread 0 has issued the loads that complete on bar; all threads learn
// whether they arrived.  On time-out the error flag is raised, the copies
// still in flight get a second bounded wait, and false is returned.
__device__ __forceinline__ bool block_wait_loads(uint64_t* bar, int* ok_s, int* err) {
  if (threadIdx.x == 0) {
    bool ok = g_tile_wait_probe ? false : mbar_wait(bar, 0);
    if (!ok) {
      atomicOr(err, 1);
      mbar_wait(bar, 0);
    }
    *ok_s = ok ? 1 : 0;
  }
  __syncthreads();
  return *ok_s != 0;
}

// ---------------------------------------------------- in-place tile FFT
// NG groups of QN lines of N points; element e of line (g, q) sits at
// d[g*GS + q + e*ES].  Work item w: q = w % QN fastest, then the butterfly
// index j, then the group, so a warp reads consecutive addresses.  Stage s
// of radix R maps element j + r*N/R (times W^(k r), k = j mod Ns) to
// (j/Ns)*Ns*R + k + r*Ns (Stockham autosort); inputs go through registers so
// the stage is done in place.  Twiddles W_N^i = tw[i*TWM] (table of N*TWM
// points, the sign of the transform).
// RMAX: the largest radix of a stage.  Measured at 128^3 (FP32, 200
// launches of each pass): the y pass 11.0 / 9.9 / 9.0 ms and the x + Green
// pass 12.2 / 11.8 / 11.1 ms with RMAX 4 / 8 / 16; the z passes 7.1 / 7.1 /
// 8.1 ms (r2c) and 8.1 / 8.2 / 9.0 ms (c2r), where a 16-point stage leaves
// half of the threads without a butterfly.
//
// Between stages the tile is held swizzled: complex element i of the tile
// sits at i ^ ((i / B) % B), B = the elements of one 128-byte row of shared
// memory (16 complex floats, 8 complex doubles).  Within each aligned group
// of B elements this permutes the slots by the group's index, so the
// strided stage writes of a warp (a butterfly's R outputs R elements apart
// between neighbouring threads: all threads of a warp on two slots for
// R = 8 in the z passes) spread over the row's slots.  The first stage
// reads and the last stage writes the dense tile the tensor copies move.
// SWZ (per pass): the z and x + Green passes (their stage writes conflict);
// the strided passes' dense tiles are conflict-free already (their warps
// write 16 consecutive columns), where the swizzle measured 2 % slower.
// At 128^3 (FP32, 300 launches of each pass): z R2C 9.4 against 10.7 ms,
// z C2R 11.1 against 12.3 ms, x + Green 15.8 against 16.6 ms.
template <typename T, bool SW>
__device__ __forceinline__ int tile_slot(int i) {
  constexpr int B = 128 / (int)sizeof(c2<T>);
  if constexpr (SW) return i ^ ((i / B) & (B - 1));
  else return i;
}
template <typename T, int N, int QN, int ES, int GS, int NG, int TWM, int SG, int NT, int RMAX, bool SWZ, int S = 0,
          int NS = 1>
__device__ __forceinline__ void tile_fft(c2<T>* d, const c2<T>* __restrict__ tw) {
  constexpr int NST = tl_nst(N, RMAX);
  if constexpr (S < NST) {
    constexpr bool SWI = SWZ && S > 0, SWO = SWZ && S + 1 < NST;
    constexpr int R = tl_radix(N, S, RMAX);
    constexpr int NB = N / R;
    constexpr int TWS = N / (NS * R);
    constexpr int TOTAL = NG * NB * QN;
    constexpr int IPT = (TOTAL + NT - 1) / NT;
    c2<T> v[IPT][R];
#pragma unroll
    for (int i = 0; i < IPT; i++) {
      const int w = threadIdx.x + i * NT;
      if (TOTAL % NT == 0 || w < TOTAL) {
        const int q = w % QN, t = w / QN;
        const int j = t % NB, g = t / NB;
        const int k = j % NS;
        const int base = g * GS + q;
#pragma unroll
        for (int r = 0; r < R; r++) {
          c2<T> x = d[tile_slot<T, SWI>(base + (j + r * NB) * ES)];
          if (r && NS > 1) x = cmul<T>(x, __ldg(&tw[k * r * TWS * TWM]));
          v[i][r] = x;
        }
      }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < IPT; i++) {
      const int w = threadIdx.x + i * NT;
      if (TOTAL % NT == 0 || w < TOTAL) {
        const int q = w % QN, t = w / QN;
        const int j = t % NB, g = t / NB;
        const int k = j % NS;
        butterfly<T, R>(v[i], SG);
        const int base = g * GS + q;
        const int idxD = (j / NS) * NS * R + k;
#pragma unroll
        for (int r = 0; r < R; r++) d[tile_slot<T, SWO>(base + (idxD + r * NS) * ES)] = v[i][r];
      }
    }
    __syncthreads();
    tile_fft<T, N, QN, ES, GS, NG, TWM, SG, NT, RMAX, SWZ, S + 1, NS * R>(d, tw);
  }
}

constexpr int NT = 256;   // threads per block of every TMA pass
constexpr int RMAX_Z = 8;     // largest radix: z passes
constexpr int RMAX_S = 16;    // strided (y, x) and Green passes

}  // namespace

// Tile parameters, shared with the host launchers.
template <typename T> __host__ __device__ constexpr int cw() { return (int)(sizeof(c2<T>) / 8); }   // 8-byte words per complex
// default kz columns per tile of the strided passes (128^3, FP32: 32 columns
// 8.3 ms against 9.0 ms (16) and 10.8 ms (8) for 400 launches)
template <typename T> __host__ __device__ constexpr int kb_strided() { return sizeof(T) == 4 ? 32 : 4; }
template <typename T> __host__ __device__ constexpr int kb_green() { return sizeof(T) == 4 ? 4 : 2; }
// lines per z-pass tile: about `elems` complex points (lines x N/2).  At
// 128^3 (FP32, 300 launches): R2C 9.4 ms with 2048 (32 lines), 9.5 ms with
// 1024, 10.6 ms with 4096; C2R + strain 9.9 ms with 1024 (16 lines), 11.1 ms
// with 2048, 12.9 ms with 4096 (its tile holds the spectrum rows, the work
// lines and the real field, so the smaller tile doubles the blocks per SM).
constexpr int ZR_ELEMS = 2048, ZC_ELEMS = 1024;
template <typename T> __host__ __device__ constexpr int lb_z(int n, int elems) {
  int lb = elems / (n / 2);
  int p = 8;
  while (p * 2 <= lb && p < 64) p *= 2;
  if (sizeof(T) == 8 && p > 8) p /= 2;
  return p;
}

// ------------------------------------------------------------- z passes
// r2c: one block = LB consecutive (x,y) lines of one stress component.
template <typename T, int N, int LB>
__global__ void __launch_bounds__(NT) fft_zr_tma_kernel(const __grid_constant__ CUtensorMap mreal,
                                                        const __grid_constant__ CUtensorMap mspec,
                                                        const c2<T>* __restrict__ tw, IterIn it, int* err) {
  if (!is_live(it)) return;
  constexpr int M = N / 2, KZ = M + 1, KZS = (KZ + 1) & ~1;
  extern __shared__ __align__(1024) unsigned char smraw[];
  __shared__ uint64_t bar;
  __shared__ int ok_s;
  c2<T>* A = reinterpret_cast<c2<T>*>(smraw);        // LB x M complex = LB x N real
  c2<T>* C = A + ((LB * M + 15) & ~15);              // LB x KZS output rows
  const int line0 = blockIdx.x * LB, comp = blockIdx.y;
  if (threadIdx.x == 0) {
    mbar_init(&bar);
    mbar_expect(&bar, (uint32_t)(LB * N * sizeof(T)));
    tma_load3(A, &mreal, 0, line0, comp, &bar);
  }
  if (!block_wait_loads(&bar, &ok_s, err)) return;
  tile_fft<T, M, 1, 1, M, LB, 2, -1, NT, RMAX_Z, true>(A, tw);
  // split step: X_k = (Z_k + conj Z_{M-k})/2 - i W_N^k (Z_k - conj Z_{M-k})/2
  for (int idx = threadIdx.x; idx < LB * KZS; idx += NT) {
    const int l = idx / KZS, k = idx - l * KZS;
    c2<T> X = mk<T>(0, 0);
    if (k < KZ) {
      const c2<T> z = A[l * M + (k % M)], zm = A[l * M + ((M - k) % M)];
      const c2<T> e = mk<T>((T)0.5 * (z.x + zm.x), (T)0.5 * (z.y - zm.y));   // (Z + conj Zm)/2
      const c2<T> o = mk<T>((T)0.5 * (z.x - zm.x), (T)0.5 * (z.y + zm.y));   // (Z - conj Zm)/2
      const c2<T> wo = cmul<T>(__ldg(&tw[k]), o);
      X = mk<T>(e.x + wo.y, e.y - wo.x);   // e - i wo
    }
    C[l * KZS + k] = X;
  }
  fence_async_smem();
  __syncthreads();
  if (threadIdx.x == 0) {
    tma_store3(&mspec, C, 0, line0, comp);
    tma_store_commit_wait();
  }
}

// c2r fused with the strain update (MODE 1: field += Re(.)*scale + add[c];
// MODE 0: field = Re(.)*scale + add[c]).  The imaginary parts of X_0 and
// X_{N/2} are dropped, as the real part of the reference's complex inverse.
template <typename T, int N, int LB, int MODE>
__global__ void __launch_bounds__(NT) fft_zc_tma_kernel(const __grid_constant__ CUtensorMap mspec,
                                                        const __grid_constant__ CUtensorMap mreal,
                                                        const c2<T>* __restrict__ tw, T scale, IterIn it, int* err) {
  if (!is_live(it)) return;
  constexpr int M = N / 2, KZS = (M + 2) & ~1;
  extern __shared__ __align__(1024) unsigned char smraw[];
  __shared__ uint64_t bar;
  __shared__ int ok_s;
  c2<T>* S = reinterpret_cast<c2<T>*>(smraw);        // LB x KZS spectrum rows
  c2<T>* A = S + ((LB * KZS + 15) & ~15);            // LB x M work
  T* F = reinterpret_cast<T*>(A + ((LB * M + 15) & ~15));   // LB x N real field
  const int line0 = blockIdx.x * LB, comp = blockIdx.y;
  if (threadIdx.x == 0) {
    mbar_init(&bar);
    mbar_expect(&bar, (uint32_t)(LB * KZS * sizeof(c2<T>) + (MODE ? LB * N * sizeof(T) : 0)));
    tma_load3(S, &mspec, 0, line0, comp, &bar);
    if (MODE) tma_load3(F, &mreal, 0, line0, comp, &bar);
  }
  if (!block_wait_loads(&bar, &ok_s, err)) return;
  // merge step: Z_k = (X_k + conj X_{M-k}) + i W_N^-k (X_k - conj X_{M-k})
  for (int idx = threadIdx.x; idx < LB * M; idx += NT) {
    const int l = idx / M, k = idx - l * M;
    c2<T> x = S[l * KZS + k], xm = S[l * KZS + (M - k)];
    if (k == 0) { x.y = 0; xm.y = 0; }
    const c2<T> e = mk<T>(x.x + xm.x, x.y - xm.y);
    const c2<T> o = cmul<T>(__ldg(&tw[k]), mk<T>(x.x - xm.x, x.y + xm.y));
    A[l * M + k] = mk<T>(e.x - o.y, e.y + o.x);   // e + i o
  }
  __syncthreads();
  tile_fft<T, M, 1, 1, M, LB, 2, +1, NT, RMAX_Z, true>(A, tw);
  const T ad = it.add ? (T)it.add[comp] : (T)0;
  for (int idx = threadIdx.x; idx < LB * N; idx += NT) {
    const int l = idx / N, z = idx - l * N;
    const c2<T> a = A[l * M + (z >> 1)];
    const T v = ((z & 1) ? a.y : a.x) * scale + ad;
    F[idx] = MODE ? F[idx] + v : v;
  }
  fence_async_smem();
  __syncthreads();
  if (threadIdx.x == 0) {
    tma_store3(&mreal, F, 0, line0, comp);
    tma_store_commit_wait();
  }
}

// ------------------------------------------------------- strided passes
// One block: KB consecutive kz columns of one component at one outer index,
// lines of L points along y (axis 1) or x (axis 0).
template <typename T, int L, int KB, int SG>
__global__ void __launch_bounds__(NT) fft_s_tma_kernel(const __grid_constant__ CUtensorMap m, int axis,
                                                       const c2<T>* __restrict__ tw, IterIn it, int* err) {
  if (!is_live(it)) return;
  extern __shared__ __align__(1024) unsigned char smraw[];
  __shared__ uint64_t bar;
  __shared__ int ok_s;
  c2<T>* D = reinterpret_cast<c2<T>*>(smraw);   // L x KB
  const int x0 = blockIdx.x * KB * cw<T>(), outer = blockIdx.y, comp = blockIdx.z;
  const int c1 = axis == 1 ? 0 : outer, c2i = axis == 1 ? outer : 0;
  if (threadIdx.x == 0) {
    mbar_init(&bar);
    mbar_expect(&bar, (uint32_t)(L * KB * sizeof(c2<T>)));
    tma_load4(D, &m, x0, c1, c2i, comp, &bar);
  }
  if (!block_wait_loads(&bar, &ok_s, err)) return;
  tile_fft<T, L, KB, KB, 0, 1, 1, SG, NT, RMAX_S, false>(D, tw);
  fence_async_smem();
  __syncthreads();
  if (threadIdx.x == 0) {
    tma_store4(&m, D, x0, c1, c2i, comp);
    tma_store_commit_wait();
  }
}

// x pass fused with Gamma0: six stress components forward along x, Delta =
// Gamma0 : sigma-hat at every wave vector of the tile, antisymmetric part
// added to the spin accumulator tile, inverse along x.  One block: fixed y,
// KB consecutive kz.
// resident blocks per SM the Green pass asks registers for: up to
// MTH_XG_CAP in FP32, no more than its shared-memory tile lets fit (228 KB
// per SM).  128^3, 300 launches: 15.5 ms with 5 (48 registers), 16.1 ms
// with 4 (64), 16.9 ms with 6 (40)
#ifndef MTH_XG_CAP
#define MTH_XG_CAP 5
#endif
template <typename T, int L, int KB>
constexpr int xg_min_blocks() {
  constexpr long fit = 228L * 1024 / (9L * L * KB * (long)sizeof(c2<T>) + 2048);
  return sizeof(T) == 8 || fit < 1 ? 1 : fit > MTH_XG_CAP ? MTH_XG_CAP : (int)fit;
}

template <typename T, int L, int KB>
__global__ void __launch_bounds__(NT, xg_min_blocks<T, L, KB>()) fft_xg_tma_kernel(const GreenConst gc, const __grid_constant__ CUtensorMap mspec,
                                                        const __grid_constant__ CUtensorMap manti, int n1, int n2,
                                                        int kz, const c2<T>* __restrict__ twf,
                                                        const c2<T>* __restrict__ twi, IterIn it, int* err) {
  if (!is_live(it)) return;
  constexpr int SLAB = L * KB;
  extern __shared__ __align__(1024) unsigned char smraw[];
  __shared__ uint64_t bar;
  __shared__ int ok_s;
  c2<T>* D = reinterpret_cast<c2<T>*>(smraw);   // 6 x L x KB
  c2<T>* Aq = D + 6 * SLAB;                     // 3 x L x KB
  const int k0 = blockIdx.x * KB, y = blockIdx.y;
  const int x0 = k0 * cw<T>();
  if (threadIdx.x == 0) {
    mbar_init(&bar);
    mbar_expect(&bar, (uint32_t)(9 * SLAB * sizeof(c2<T>)));
#pragma unroll
    for (int c = 0; c < 6; c++) tma_load4(D + c * SLAB, &mspec, x0, y, 0, c, &bar);
#pragma unroll
    for (int c = 0; c < 3; c++) tma_load4(Aq + c * SLAB, &manti, x0, y, 0, c, &bar);
  }
  if (!block_wait_loads(&bar, &ok_s, err)) return;
  tile_fft<T, L, KB, KB, SLAB, 6, 1, -1, NT, RMAX_S, true>(D, twf);
  for (int idx = threadIdx.x; idx < SLAB; idx += NT) {
    const int kk = idx % KB, kx = idx / KB;
    if (k0 + kk >= kz) continue;
    c2<T> s[6], a[3];
#pragma unroll
    for (int c = 0; c < 6; c++) s[c] = D[c * SLAB + idx];
    green_point<T>(gc, kx, y, k0 + kk, L, n1, n2, s, a);
#pragma unroll
    for (int c = 0; c < 6; c++) D[c * SLAB + idx] = s[c];
#pragma unroll
    for (int c = 0; c < 3; c++) Aq[c * SLAB + idx] = cadd<T>(Aq[c * SLAB + idx], a[c]);
  }
  __syncthreads();
  tile_fft<T, L, KB, KB, SLAB, 6, 1, +1, NT, RMAX_S, true>(D, twi);
  fence_async_smem();
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int c = 0; c < 6; c++) tma_store4(&mspec, D + c * SLAB, x0, y, 0, c);
#pragma unroll
    for (int c = 0; c < 3; c++) tma_store4(&manti, Aq + c * SLAB, x0, y, 0, c);
    tma_store_commit_wait();
  }
}

// ------------------------------------------------------------ host side
static bool ct_size(int n) {
  switch (n) {
    case 16: case 32: case 48: case 64: case 96: case 128: case 256: return true;
    default: return false;
  }
}

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// rank-r tiled map, element type dt of esz bytes; dims/box innermost first,
// strides in bytes for dims 1..r-1
static bool encode(CUtensorMap* m, CUtensorMapDataType dt, int rank, void* base, const cuuint64_t* dims,
                   const cuuint64_t* strides, const cuuint32_t* box) {
  PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
  if (!fn) return false;
  cuuint32_t es[5] = {1, 1, 1, 1, 1};
  return fn(m, dt, (cuuint32_t)rank, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

struct TmaMaps {
  CUtensorMap real_sig, real_strain, real_wspin;   // z passes, real fields
  CUtensorMap spec_z, spec_zc, anti_z;             // z passes, half spectra (R2C / C2R tiles)
  CUtensorMap spec_y, anti_y, anti_x;              // strided passes
  CUtensorMap spec_g, anti_g;                      // Green x pass
  bool z, s, g;                                    // passes with maps
  int ks, kg;                                      // kz columns per tile: strided passes, Green pass
};

// Tile widths (kz columns per block) the strided and Green passes are
// compiled for; tma_create falls back to the default for any other value.
template <typename T>
bool tile_ok_strided(int k) {
  return sizeof(T) == 4 ? (k == 8 || k == 16 || k == 32) : (k == 2 || k == 4 || k == 8);
}
template <typename T>
bool tile_ok_green(int k) {
  return sizeof(T) == 4 ? (k == 2 || k == 4 || k == 8) : (k == 1 || k == 2 || k == 4);
}

template <typename T>
TmaMaps* tma_create(const FftGeom& g, T* sig, T* strain, T* wspin, c2<T>* spec, c2<T>* anti, int ks, int kg) {
  TmaMaps* t = new TmaMaps();
  memset(t, 0, sizeof(*t));
  t->ks = tile_ok_strided<T>(ks) ? ks : kb_strided<T>();
  t->kg = tile_ok_green<T>(kg) ? kg : kb_green<T>();
  if (!ct_size(g.n0) || !ct_size(g.n1) || !ct_size(g.n2) || !encode_fn()) return t;
  const CUtensorMapDataType rt = sizeof(T) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
  const CUtensorMapDataType wt = CU_TENSOR_MAP_DATA_TYPE_FLOAT64;   // spectra in 8-byte words
  const cuuint64_t C = (cuuint64_t)cw<T>(), cb = sizeof(c2<T>), ws = sizeof(T);
  const cuuint64_t lines = (cuuint64_t)g.n0 * g.n1;
  const int lbr = lb_z<T>(g.n2, ZR_ELEMS), lbc = lb_z<T>(g.n2, ZC_ELEMS);
  bool ok = true;
  // z passes: real [c][line][z] and spectrum [c][line][kzs]; boxes of the
  // R2C tile (stress in, spectrum out) and of the C2R tile (spectra in,
  // strain and spin fields in and out)
  if ((cuuint64_t)g.kzs * C <= 256) {
    cuuint64_t d6[3] = {(cuuint64_t)g.n2, lines, 6}, d3[3] = {(cuuint64_t)g.n2, lines, 3};
    cuuint64_t st[2] = {g.n2 * ws, (cuuint64_t)g.plane * ws};
    cuuint32_t bxr[3] = {(cuuint32_t)g.n2, (cuuint32_t)lbr, 1}, bxc[3] = {(cuuint32_t)g.n2, (cuuint32_t)lbc, 1};
    ok = ok && encode(&t->real_sig, rt, 3, sig, d6, st, bxr) && encode(&t->real_strain, rt, 3, strain, d6, st, bxc) &&
         encode(&t->real_wspin, rt, 3, wspin, d3, st, bxc);
    cuuint64_t k6[3] = {(cuuint64_t)g.kzs * C, lines, 6}, k3[3] = {(cuuint64_t)g.kzs * C, lines, 3};
    cuuint64_t ks[2] = {(cuuint64_t)g.kzs * cb, (cuuint64_t)g.kplane * cb};
    cuuint32_t kbr[3] = {(cuuint32_t)(g.kzs * C), (cuuint32_t)lbr, 1}, kbc[3] = {(cuuint32_t)(g.kzs * C), (cuuint32_t)lbc, 1};
    ok = ok && encode(&t->spec_z, wt, 3, spec, k6, ks, kbr) && encode(&t->spec_zc, wt, 3, spec, k6, ks, kbc) &&
         encode(&t->anti_z, wt, 3, anti, k3, ks, kbc);
    t->z = ok;
  }
  // strided and Green passes: [c][x][y][kzs] as 4-D
  {
    cuuint64_t k6[4] = {(cuuint64_t)g.kzs * C, (cuuint64_t)g.n1, (cuuint64_t)g.n0, 6};
    cuuint64_t k3[4] = {(cuuint64_t)g.kzs * C, (cuuint64_t)g.n1, (cuuint64_t)g.n0, 3};
    cuuint64_t st[3] = {(cuuint64_t)g.kzs * cb, (cuuint64_t)g.n1 * g.kzs * cb, (cuuint64_t)g.kplane * cb};
    const cuuint32_t ks = (cuuint32_t)(t->ks * C), kg = (cuuint32_t)(t->kg * C);
    cuuint32_t by[4] = {ks, (cuuint32_t)g.n1, 1, 1}, bxs[4] = {ks, 1, (cuuint32_t)g.n0, 1};
    cuuint32_t bg[4] = {kg, 1, (cuuint32_t)g.n0, 1};
    bool s_ok = encode(&t->spec_y, wt, 4, spec, k6, st, by) && encode(&t->anti_y, wt, 4, anti, k3, st, by) &&
                encode(&t->anti_x, wt, 4, anti, k3, st, bxs);
    bool g_ok = encode(&t->spec_g, wt, 4, spec, k6, st, bg) && encode(&t->anti_g, wt, 4, anti, k3, st, bg);
    t->s = s_ok;
    t->g = g_ok;
  }
  return t;
}

cudaError_t tma_set_wait_probe(int on) { return cudaMemcpyToSymbol(g_tile_wait_probe, &on, sizeof(int)); }

void tma_destroy(TmaMaps* t) { delete t; }
bool tma_has(const TmaMaps* t, int pass) { return t && (pass == 0 ? t->z : pass == 1 ? t->s : t->g); }
int tma_tile_choice(bool fp32, int pass, int i) {
  static const int w[2][2][3] = {{{2, 4, 8}, {1, 2, 4}}, {{8, 16, 32}, {2, 4, 8}}};
  return w[fp32 ? 1 : 0][pass == 1 ? 0 : 1][i];
}
void tma_tiles(const TmaMaps* t, int* ks, int* kg) {
  *ks = t ? t->ks : 0;
  *kg = t ? t->kg : 0;
}

static size_t zr_smem(int n, int lb, size_t cb) {
  const int M = n / 2, KZS = (M + 2) & ~1;
  return cb * (size_t)(((lb * M + 15) & ~15) + lb * KZS);
}
static size_t zc_smem(int n, int lb, size_t cb) {
  const int M = n / 2, KZS = (M + 2) & ~1;
  return cb * (size_t)(((lb * KZS + 15) & ~15) + ((lb * M + 15) & ~15) + lb * M);
}

template <typename T, int N>
static cudaError_t zr_launch(const TmaMaps* t, int ncomp, long long lines, const c2<T>* tw, const IterIn& it,
                             int* err, cudaStream_t st) {
  constexpr int LB = lb_z<T>(N, ZR_ELEMS);
  const size_t sm = zr_smem(N, LB, sizeof(c2<T>));
  auto k = fft_zr_tma_kernel<T, N, LB>;
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  dim3 grid((unsigned)((lines + LB - 1) / LB), ncomp);
  return launch_chain(k, grid, dim3(NT), sm, st, it.pdl, t->real_sig, t->spec_z, tw, it, err);
}

template <typename T, int N>
static cudaError_t zc_launch(const CUtensorMap& ms, const CUtensorMap& mr, int ncomp, long long lines,
                             const c2<T>* tw, T scale, const IterIn& it, int mode, int* err, cudaStream_t st) {
  constexpr int LB = lb_z<T>(N, ZC_ELEMS);
  const size_t sm = zc_smem(N, LB, sizeof(c2<T>));
  dim3 grid((unsigned)((lines + LB - 1) / LB), ncomp);
  if (mode) {
    auto k = fft_zc_tma_kernel<T, N, LB, 1>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    return launch_chain(k, grid, dim3(NT), sm, st, it.pdl, ms, mr, tw, scale, it, err);
  } else {
    auto k = fft_zc_tma_kernel<T, N, LB, 0>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    return launch_chain(k, grid, dim3(NT), sm, st, it.pdl, ms, mr, tw, scale, it, err);
  }
}

template <typename T, int L, int KB>
static cudaError_t s_launch(const CUtensorMap& m, int axis, int ncomp, int nouter, int kzs, int sign,
                            const c2<T>* tw, const IterIn& it, int* err, cudaStream_t st) {
  const size_t sm = (size_t)L * KB * sizeof(c2<T>);
  dim3 grid((kzs + KB - 1) / KB, nouter, ncomp);
  if (sign < 0) {
    auto k = fft_s_tma_kernel<T, L, KB, -1>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    return launch_chain(k, grid, dim3(NT), sm, st, it.pdl, m, axis, tw, it, err);
  }
  auto k = fft_s_tma_kernel<T, L, KB, +1>;
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  return launch_chain(k, grid, dim3(NT), sm, st, it.pdl, m, axis, tw, it, err);
}

template <typename T, int L, int KB>
static cudaError_t g_launch(const TmaMaps* t, const FftGeom& g, const GreenConst& gc, const c2<T>* twf,
                            const c2<T>* twi, const IterIn& it, int* err, cudaStream_t st) {
  const size_t sm = (size_t)9 * L * KB * sizeof(c2<T>);
  auto k = fft_xg_tma_kernel<T, L, KB>;
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  dim3 grid((g.kzs + KB - 1) / KB, g.n1);
  return launch_chain(k, grid, dim3(NT), sm, st, it.pdl, gc, t->spec_g, t->anti_g, g.n1, g.n2, g.kz, twf, twi, it,
                      err);
}

// the compiled tile widths: FP32 strided 8/16/32, Green 2/4/8; FP64 strided
// 2/4/8, Green 1/2/4 (index 0/1/2 of each list)
template <typename T, int L>
static cudaError_t s_dispatch(const TmaMaps* t, const CUtensorMap& m, int axis, int ncomp, int nouter, int kzs, int sign,
                              const c2<T>* tw, const IterIn& it, int* err, cudaStream_t st) {
  constexpr int A = sizeof(T) == 4 ? 8 : 2;
  if (t->ks == A) return s_launch<T, L, A>(m, axis, ncomp, nouter, kzs, sign, tw, it, err, st);
  if (t->ks == 2 * A) return s_launch<T, L, 2 * A>(m, axis, ncomp, nouter, kzs, sign, tw, it, err, st);
  if (t->ks == 4 * A) return s_launch<T, L, 4 * A>(m, axis, ncomp, nouter, kzs, sign, tw, it, err, st);
  return cudaErrorInvalidValue;
}
template <typename T, int L>
static cudaError_t g_dispatch(const TmaMaps* t, const FftGeom& g, const GreenConst& gc, const c2<T>* twf,
                              const c2<T>* twi, const IterIn& it, int* err, cudaStream_t st) {
  constexpr int A = sizeof(T) == 4 ? 2 : 1;
  if (t->kg == A) return g_launch<T, L, A>(t, g, gc, twf, twi, it, err, st);
  if (t->kg == 2 * A) return g_launch<T, L, 2 * A>(t, g, gc, twf, twi, it, err, st);
  if (t->kg == 4 * A) return g_launch<T, L, 4 * A>(t, g, gc, twf, twi, it, err, st);
  return cudaErrorInvalidValue;
}

#define MTH_TMA_SIZES(X) X(16) X(32) X(48) X(64) X(96) X(128) X(256)

template <typename T>
cudaError_t tma_fft_z_r2c(const TmaMaps* t, const FftGeom& g, const c2<T>* tw, const IterIn& it, int* err,
                          cudaStream_t st) {
  const long long lines = (long long)g.n0 * g.n1;
  switch (g.n2) {
#define MTH_CASE(N) case N: return zr_launch<T, N>(t, 6, lines, tw, it, err, st);
    MTH_TMA_SIZES(MTH_CASE)
#undef MTH_CASE
    default: return cudaErrorInvalidValue;
  }
}

// which = 0: stress spectrum -> strain field (mode 1); 1: spin spectrum ->
// spin field (mode 0)
template <typename T>
cudaError_t tma_fft_z_c2r(const TmaMaps* t, const FftGeom& g, int which, const c2<T>* tw, T scale, const IterIn& it,
                          int* err, cudaStream_t st) {
  const long long lines = (long long)g.n0 * g.n1;
  const CUtensorMap& ms = which ? t->anti_z : t->spec_zc;
  const CUtensorMap& mr = which ? t->real_wspin : t->real_strain;
  const int ncomp = which ? 3 : 6, mode = which ? 0 : 1;
  switch (g.n2) {
#define MTH_CASE(N) case N: return zc_launch<T, N>(ms, mr, ncomp, lines, tw, scale, it, mode, err, st);
    MTH_TMA_SIZES(MTH_CASE)
#undef MTH_CASE
    default: return cudaErrorInvalidValue;
  }
}

// which = 0: stress spectrum along y; 1: spin spectrum along y; 2: spin
// spectrum along x
template <typename T>
cudaError_t tma_fft_strided(const TmaMaps* t, const FftGeom& g, int which, int sign, const c2<T>* tw,
                            const IterIn& it, int* err, cudaStream_t st) {
  const CUtensorMap& m = which == 0 ? t->spec_y : which == 1 ? t->anti_y : t->anti_x;
  const int axis = which == 2 ? 0 : 1;
  const int L = axis == 1 ? g.n1 : g.n0, nouter = axis == 1 ? g.n0 : g.n1;
  const int ncomp = which == 0 ? 6 : 3;
  switch (L) {
#define MTH_CASE(N) case N: return s_dispatch<T, N>(t, m, axis, ncomp, nouter, g.kzs, sign, tw, it, err, st);
    MTH_TMA_SIZES(MTH_CASE)
#undef MTH_CASE
    default: return cudaErrorInvalidValue;
  }
}

template <typename T>
cudaError_t tma_fft_x_green(const TmaMaps* t, const FftGeom& g, const GreenConst& gc, const c2<T>* twf,
                            const c2<T>* twi, const IterIn& it, int* err, cudaStream_t st) {
  switch (g.n0) {
#define MTH_CASE(N) case N: return g_dispatch<T, N>(t, g, gc, twf, twi, it, err, st);
    MTH_TMA_SIZES(MTH_CASE)
#undef MTH_CASE
    default: return cudaErrorInvalidValue;
  }
}

#define INST(T)                                                                                                    \
  template TmaMaps* tma_create<T>(const FftGeom&, T*, T*, T*, c2<T>*, c2<T>*, int, int);                       \
  template cudaError_t tma_fft_z_r2c<T>(const TmaMaps*, const FftGeom&, const c2<T>*, const IterIn&, int*,        \
                                        cudaStream_t);                                                             \
  template cudaError_t tma_fft_z_c2r<T>(const TmaMaps*, const FftGeom&, int, const c2<T>*, T, const IterIn&, int*, \
                                        cudaStream_t);                                                             \
  template cudaError_t tma_fft_strided<T>(const TmaMaps*, const FftGeom&, int, int, const c2<T>*, const IterIn&,   \
                                          int*, cudaStream_t);                                                     \
  template cudaError_t tma_fft_x_green<T>(const TmaMaps*, const FftGeom&, const GreenConst&, const c2<T>*,         \
                                          const c2<T>*, const IterIn&, int*, cudaStream_t);
INST(float)
INST(double)
#undef INST

}  // namespace mth

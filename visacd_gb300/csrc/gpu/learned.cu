// Learned plane proposer: a per-point MLP over sampled visibility edges,
// max-pooled over the edges, then an MLP head that emits 16 planes.
//
//   x (7 features, zero-padded to 16) -> 64 -> 128 -> 256   shared per-edge
//   layers, ReLU; max over the 2048 sampled edges -> 256 -> 128 -> 64 (ReLU)
//   -> 64 = 16 planes x (normal xyz, offset).
//
// Operands are BF16 and products accumulate in FP32 on the tensor cores
// (mma.sync m16n8k16 from shared-memory tiles filled by cp.async); FP32 master
// weights are updated by Adam. Forward, backward, loss and update are this
// file's kernels: no library GEMM is called. Weight gradients are split over
// the contraction and the partial tiles are summed in a fixed order, so a
// training run is deterministic.
//
// The proposer has no counterpart in the reference. It stands in for the random
// draw of candidate planes (lib/src/process.cpp:28-72) in the split search; the
// exact scoring kernel still ranks its proposals and the host driver falls
// back to the full candidate draw when a probe says the proposals are worse.
#include <cuda_bf16.h>

#include <cstring>
#include <random>

#include "common.cuh"

using vgpu::DevBuf;
using vgpu::ensure;
using bf16 = __nv_bfloat16;

namespace {

constexpr int kPts = VISACD_LP_POINTS;  // sampled edges per part
constexpr int kIn = 16;                 // padded input width
constexpr int kFeat = VISACD_LP_FEATURES;
constexpr int kPlanes = VISACD_LP_PLANES;
constexpr int kLayers = 6;
constexpr int kK[kLayers] = {16, 64, 128, 256, 128, 64};
constexpr int kN[kLayers] = {64, 128, 256, 128, 64, 64};
constexpr int kFanIn[kLayers] = {kFeat, 64, 128, 256, 128, 64};

struct Offsets {
  int w[kLayers], b[kLayers], total;
};
constexpr Offsets make_offsets() {
  Offsets o{};
  int at = 0;
  for (int l = 0; l < kLayers; ++l) {
    o.w[l] = at;
    at += kK[l] * kN[l];
    o.b[l] = at;
    at += kN[l];
  }
  o.total = at;
  return o;
}
constexpr Offsets kOff = make_offsets();
static_assert(kOff.total == 87744, "parameter count");

// ---------------------------------------------------------------------------
// Tensor-core GEMM: C[m][n] = sum_k A(m,k) B(k,n).
//   AK: A(m,k) = A[m*lda + k] (K contiguous), else A[k*lda + m].
//   BK: B(k,n) = B[n*ldb + k] (K contiguous), else B[k*ldb + n].
// 64x64 output tile per CTA, 32-deep K slices double-buffered in shared memory,
// 4 warps of 32x32 (2 x 4 mma tiles). blockIdx.z selects a contraction chunk
// [z*kchunk, (z+1)*kchunk); with more than one chunk the epilogue stores
// partial tiles at C + z*M*ldc (summed later in order).
// Host-checked preconditions: the contiguous extent of every operand is a
// multiple of 8 elements and every base / leading dimension is 16-byte aligned,
// so each 16-byte chunk is either wholly inside or wholly outside the matrix.
// ---------------------------------------------------------------------------
enum Epi : int { kEpiBiasReluBf16 = 0, kEpiBiasF32, kEpiMaskBf16, kEpiStoreF32 };

constexpr int kTM = 64, kTN = 64, kTK = 32;
constexpr int kPadK = kTK + 8;   // K-contiguous tile row: 40 bf16 = 80 B
constexpr int kPadMN = kTM + 8;  // MN-contiguous tile row: 72 bf16 = 144 B
constexpr int kTileElems = (kTM * kPadK > kTK * kPadMN) ? kTM * kPadK : kTK * kPadMN;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, bool valid) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src),
               "r"(valid ? 16 : 0));
}
__device__ __forceinline__ void ldsm_x4(uint32_t addr, uint32_t (&r)[4]) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(addr));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t addr, uint32_t (&r)[4]) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(addr));
}
__device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4], uint32_t b0,
                                         uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Load one operand tile (rows x cols of the stored layout) into shared memory.
// K-contiguous: 64 rows (m or n) x 32 k; MN-contiguous: 32 rows (k) x 64 cols.
template <bool KC>
__device__ __forceinline__ void load_tile(bf16* s, const bf16* __restrict__ g, int ld, int mn0,
                                          int mn_end, int k0, int k_end, int tid) {
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const int c = tid + i * 128;
    if (KC) {
      const int row = c >> 2, kc = (c & 3) * 8;
      const int gm = mn0 + row, gk = k0 + kc;
      const bool ok = gm < mn_end && gk < k_end;
      cp_async16(smem_u32(s + row * kPadK + kc), ok ? g + (size_t)gm * ld + gk : g, ok);
    } else {
      const int row = c >> 3, mc = (c & 7) * 8;
      const int gk = k0 + row, gm = mn0 + mc;
      const bool ok = gk < k_end && gm < mn_end;
      cp_async16(smem_u32(s + row * kPadMN + mc), ok ? g + (size_t)gk * ld + gm : g, ok);
    }
  }
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&h);
}

template <bool AK, bool BK, int EPI>
__global__ void __launch_bounds__(128) lp_gemm_kernel(const bf16* __restrict__ A, int lda,
                                                      const bf16* __restrict__ B, int ldb, void* C,
                                                      int ldc, int M, int N, int K, int kchunk,
                                                      const float* __restrict__ bias,
                                                      const bf16* __restrict__ R, int ldr) {
  __shared__ __align__(128) bf16 sA[2][kTileElems];
  __shared__ __align__(128) bf16 sB[2][kTileElems];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int m0 = blockIdx.x * kTM, n0 = blockIdx.y * kTN;
  const int kbeg = blockIdx.z * kchunk;
  const int kend = min(K, kbeg + kchunk);
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;

  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.f;

  const int nk = (kend - kbeg + kTK - 1) / kTK;
  if (nk > 0) {
    load_tile<AK>(sA[0], A, lda, m0, M, kbeg, kend, tid);
    load_tile<BK>(sB[0], B, ldb, n0, N, kbeg, kend, tid);
    asm volatile("cp.async.commit_group;\n" ::);
  }
  for (int it = 0; it < nk; ++it) {
    const int st = it & 1;
    if (it + 1 < nk) {
      const int kn = kbeg + (it + 1) * kTK;
      load_tile<AK>(sA[st ^ 1], A, lda, m0, M, kn, kend, tid);
      load_tile<BK>(sB[st ^ 1], B, ldb, n0, N, kn, kend, tid);
      asm volatile("cp.async.commit_group;\n" ::);
      asm volatile("cp.async.wait_group 1;\n" ::);
    } else {
      asm volatile("cp.async.wait_group 0;\n" ::);
    }
    __syncthreads();
    const bf16* a_s = sA[st];
    const bf16* b_s = sB[st];
#pragma unroll
    for (int kk = 0; kk < kTK; kk += 16) {
      uint32_t af[2][4], bfr[2][4];
#pragma unroll
      for (int mt = 0; mt < 2; ++mt) {
        const int mb = wm + mt * 16;
        if (AK) {
          const int row = mb + (lane & 7) + ((lane >> 3) & 1) * 8;
          const int col = kk + (lane >> 4) * 8;
          ldsm_x4(smem_u32(a_s + row * kPadK + col), af[mt]);
        } else {
          const int row = kk + (lane & 7) + (lane >> 4) * 8;
          const int col = mb + ((lane >> 3) & 1) * 8;
          ldsm_x4_t(smem_u32(a_s + row * kPadMN + col), af[mt]);
        }
      }
#pragma unroll
      for (int np = 0; np < 2; ++np) {
        const int nb = wn + np * 16;
        if (BK) {
          const int row = nb + (lane & 7) + (lane >> 4) * 8;
          const int col = kk + ((lane >> 3) & 1) * 8;
          ldsm_x4(smem_u32(b_s + row * kPadK + col), bfr[np]);
        } else {
          const int row = kk + (lane & 7) + ((lane >> 3) & 1) * 8;
          const int col = nb + (lane >> 4) * 8;
          ldsm_x4_t(smem_u32(b_s + row * kPadMN + col), bfr[np]);
        }
      }
#pragma unroll
      for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt)
          mma_bf16(acc[mt][nt], af[mt], bfr[nt >> 1][(nt & 1) * 2], bfr[nt >> 1][(nt & 1) * 2 + 1]);
    }
    __syncthreads();
  }

  // Epilogue: lane holds rows g, g+8 and columns 2t, 2t+1 of each 16x8 tile.
  const int g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
      const int n = n0 + wn + nt * 8 + 2 * t;
      if (n >= N) continue;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int m = m0 + wm + mt * 16 + g + h * 8;
        if (m >= M) continue;
        float v0 = acc[mt][nt][2 * h], v1 = acc[mt][nt][2 * h + 1];
        if (EPI == kEpiBiasReluBf16) {
          v0 += bias[n];
          v1 += bias[n + 1];
          v0 = v0 > 0.f ? v0 : 0.f;  // +0 for non-positive (pooling compares bit patterns)
          v1 = v1 > 0.f ? v1 : 0.f;
          *reinterpret_cast<uint32_t*>(static_cast<bf16*>(C) + (size_t)m * ldc + n) = pack_bf16(v0, v1);
        } else if (EPI == kEpiMaskBf16) {
          const __nv_bfloat162 r = *reinterpret_cast<const __nv_bfloat162*>(R + (size_t)m * ldr + n);
          v0 = __bfloat162float(r.x) > 0.f ? v0 : 0.f;
          v1 = __bfloat162float(r.y) > 0.f ? v1 : 0.f;
          *reinterpret_cast<uint32_t*>(static_cast<bf16*>(C) + (size_t)m * ldc + n) = pack_bf16(v0, v1);
        } else {
          if (EPI == kEpiBiasF32) {
            v0 += bias[n];
            v1 += bias[n + 1];
          }
          float* out = static_cast<float*>(C) + (size_t)blockIdx.z * M * ldc + (size_t)m * ldc + n;
          *reinterpret_cast<float2*>(out) = make_float2(v0, v1);
        }
      }
    }
}

// ---------------------------------------------------------------------------
// Blackwell tensor-core path of the forward per-edge layers (tcgen05):
// Y = relu(X W^T + b), X [M x K], W [N x K], K in {16, 64, 128}, N in
// {64, 128, 256}, accumulators in tensor memory. Persistent CTAs (4 warps)
// walk 128-row tiles of X:
//  * W is copied once into shared memory, X tiles are double-buffered with
//    cp.async; both in the canonical K-major no-swizzle layout: 8-row x
//    16-byte core matrices, core (row group g, k group j) at
//    ((j * groups) + g) * 128 bytes (stride 128 B between row groups = SBO,
//    groups * 128 B between k groups = LBO);
//  * two accumulators of N tensor-memory columns: thread 0 issues the
//    tcgen05.mma chain (M = 128, N, K = 16 each, BF16 -> FP32) of tile i + 1
//    and commits it to that accumulator's mbarrier while the four warps read
//    tile i back with tcgen05.ld (32 lanes x 16 columns per load), add the
//    bias, apply ReLU and store BF16;
//  * every mbarrier wait has an iteration limit (status bit on expiry).
// The dynamic shared memory (160 KB) leaves room for any stride reading of
// the W and X regions.
// ---------------------------------------------------------------------------
constexpr int kTcM = 128;
constexpr int kTcSmem = 160 * 1024;
constexpr int kTcW = 0, kTcX0 = 64 * 1024, kTcX1 = 96 * 1024, kTcBar = 128 * 1024;

__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

__device__ __forceinline__ bool tc_wait(uint32_t bar_addr, uint32_t parity) {
  for (int it = 0; it < (1 << 24); ++it) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar_addr), "r"(parity));
    if (ok) return true;
  }
  return false;
}

// cp.async of one 128-row X tile into the core-matrix layout (rows past M: zeros).
__device__ __forceinline__ void tc_load_x(unsigned char* buf, const bf16* __restrict__ X, int M, int K, int row0,
                                          int tid) {
  const int kg = K / 8, ag = kTcM / 8;
  for (int c = tid; c < kTcM * kg; c += 128) {
    const int r = c / kg, j = c % kg;
    const bool ok = row0 + r < M;
    cp_async16(smem_u32(buf + ((j * ag) + (r >> 3)) * 128 + (r & 7) * 16),
               ok ? X + (size_t)(row0 + r) * K + j * 8 : X, ok);
  }
  asm volatile("cp.async.commit_group;\n" ::);
}

__global__ void __launch_bounds__(128, 1) lp_gemm_tc_kernel(const bf16* __restrict__ X, int M, int K,
                                                           const bf16* __restrict__ W, int N,
                                                           const float* __restrict__ bias, bf16* __restrict__ Y,
                                                           uint32_t* __restrict__ status) {
  extern __shared__ __align__(1024) unsigned char smem[];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int ntiles = (M + kTcM - 1) / kTcM;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + kTcBar);  // two mbarriers
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + kTcBar + 32);
  const uint32_t s_base = smem_u32(smem);
  const uint32_t bar0 = smem_u32(&bar[0]), bar1 = smem_u32(&bar[1]);
  const int kg = K / 8, ag = kTcM / 8, bg = N / 8;
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar0));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar1));
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::);
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tslot)),
                 "r"(2 * N));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
  }
  // W once, then the first X tile.
  for (int c = tid; c < N * kg; c += 128) {
    const int r = c / kg, j = c % kg;
    cp_async16(smem_u32(smem + kTcW + ((j * bg) + (r >> 3)) * 128 + (r & 7) * 16), W + (size_t)r * K + j * 8, true);
  }
  int t0 = blockIdx.x;
  if (t0 < ntiles) tc_load_x(smem + kTcX0, X, M, K, t0 * kTcM, tid);
  else asm volatile("cp.async.commit_group;\n" ::);
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(tslot);
  const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
                         ((uint32_t)(kTcM >> 4) << 24);
  // MMA chain of local tile i (buffer and accumulator i % 2) by thread 0.
  auto issue = [&](int i) {
    if (tid == 0) {
      const uint32_t xb = s_base + ((i & 1) ? kTcX1 : kTcX0);
      const uint32_t acc = tmem + (uint32_t)((i & 1) * N);
      for (int s = 0; s < K / 16; ++s) {
        const uint64_t ad = tc_desc(xb + s * 2 * ag * 128, ag * 128, 128);
        const uint64_t bd = tc_desc(s_base + kTcW + s * 2 * bg * 128, bg * 128, 128);
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(acc),
            "l"(ad), "l"(bd), "r"(idesc), "r"(s > 0 ? 1 : 0));
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
          (i & 1) ? bar1 : bar0));
    }
  };
  bool ok = true;
  // tile 0 of this CTA: wait for its data, issue, prefetch tile 1
  asm volatile("cp.async.wait_group 0;\n" ::);
  asm volatile("fence.proxy.async.shared::cta;\n" ::);
  __syncthreads();
  const int nlocal = t0 < ntiles ? (ntiles - 1 - t0) / gridDim.x + 1 : 0;
  if (nlocal > 0) issue(0);
  if (nlocal > 1) tc_load_x(smem + kTcX1, X, M, K, (t0 + gridDim.x) * kTcM, tid);
  for (int i = 0; i < nlocal && ok; ++i) {
    // start tile i + 1 while tile i drains
    if (i + 1 < nlocal) {
      asm volatile("cp.async.wait_group 0;\n" ::);
      asm volatile("fence.proxy.async.shared::cta;\n" ::);
      asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
      __syncthreads();
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
      issue(i + 1);
    }
    // tile i's MMAs done: its buffer is free for tile i + 2
    ok = tc_wait((i & 1) ? bar1 : bar0, (uint32_t)((i >> 1) & 1));
    if (!ok) break;
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
    if (i + 2 < nlocal) tc_load_x(smem + ((i & 1) ? kTcX1 : kTcX0), X, M, K, (t0 + (i + 2) * gridDim.x) * kTcM, tid);
    const int row = (t0 + i * gridDim.x) * kTcM + warp * 32 + lane;
    const uint32_t acc = tmem + (uint32_t)((i & 1) * N);
    for (int c0 = 0; c0 < N; c0 += 16) {
      uint32_t r[16];
      const uint32_t taddr = acc + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::);
      if (row < M) {
        uint32_t o[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          float v0 = __uint_as_float(r[2 * k]) + bias[c0 + 2 * k];
          float v1 = __uint_as_float(r[2 * k + 1]) + bias[c0 + 2 * k + 1];
          v0 = v0 > 0.f ? v0 : 0.f;
          v1 = v1 > 0.f ? v1 : 0.f;
          o[k] = pack_bf16(v0, v1);
        }
        uint4* dst = reinterpret_cast<uint4*>(Y + (size_t)row * N + c0);
        dst[0] = make_uint4(o[0], o[1], o[2], o[3]);
        dst[1] = make_uint4(o[4], o[5], o[6], o[7]);
      }
    }
    // the accumulator of tile i is read before tile i + 2 reuses it
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::);
  }
  if (!ok) {
    if (tid == 0) atomicOr(status, vgpu::kStatusMbarrierTimeout);
    // MMAs possibly still in flight get a second bounded wait on both barriers
    tc_wait(bar0, 0);
    tc_wait(bar1, 0);
  }
  asm volatile("cp.async.wait_group 0;\n" ::);
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::);
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(2 * N));
}

// Sum of `parts` partial arrays of `count` floats, in order, into out.
__global__ void lp_sum_parts_kernel(const float* __restrict__ parts, int nparts, int count,
                                    float* __restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int p = 0; p < nparts; ++p) s += parts[(size_t)p * count + i];
    out[i] = s;
  }
}

// Column sums of a bf16 [rows x cols] matrix: block j sums rows
// [j*per, (j+1)*per) of column threadIdx.x into part[j*cols + c].
__global__ void lp_colsum_kernel(const bf16* __restrict__ X, int rows, int cols, int per,
                                 float* __restrict__ part) {
  const int c = threadIdx.x;
  if (c >= cols) return;
  const int r0 = blockIdx.x * per, r1 = min(rows, r0 + per);
  float s = 0.f;
  for (int r = r0; r < r1; ++r) s += __bfloat162float(X[(size_t)r * cols + c]);
  part[(size_t)blockIdx.x * cols + c] = s;
}

// ---------------------------------------------------------------------------
// Features of the sampled edges, in the part's normalised frame
// x' = (x - center) / scale: midpoint (3), unit direction with its largest
// component made positive (3), length (1). Sample s takes edge
// floor(s * E / 2048) when E >= 2048, else edge s mod E.
// ---------------------------------------------------------------------------
__global__ void lp_features_kernel(const float* __restrict__ pts, const uint32_t* __restrict__ edges,
                                   int64_t E, int32_t n, float cx, float cy, float cz, float inv_s,
                                   float* __restrict__ out_f32, bf16* __restrict__ out_bf16,
                                   uint32_t* __restrict__ status) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= kPts) return;
  const int64_t e = E >= kPts ? ((int64_t)s * E) / kPts : (int64_t)(s % E);
  uint32_t i = edges[2 * e], j = edges[2 * e + 1];
  float f[kFeat] = {0, 0, 0, 0, 0, 0, 0};
  if (i < (uint32_t)n && j < (uint32_t)n) {
    const float px = pts[3 * i], py = pts[3 * i + 1], pz = pts[3 * i + 2];
    const float qx = pts[3 * j], qy = pts[3 * j + 1], qz = pts[3 * j + 2];
    f[0] = (0.5f * (px + qx) - cx) * inv_s;
    f[1] = (0.5f * (py + qy) - cy) * inv_s;
    f[2] = (0.5f * (pz + qz) - cz) * inv_s;
    float dx = qx - px, dy = qy - py, dz = qz - pz;
    const float len = sqrtf(dx * dx + dy * dy + dz * dz);
    if (len > 0.f) {
      dx /= len;
      dy /= len;
      dz /= len;
      const float ax = fabsf(dx), ay = fabsf(dy), az = fabsf(dz);
      const float big = (ax >= ay && ax >= az) ? dx : (ay >= az ? dy : dz);
      if (big < 0.f) {
        dx = -dx;
        dy = -dy;
        dz = -dz;
      }
      f[3] = dx;
      f[4] = dy;
      f[5] = dz;
    }
    f[6] = len * inv_s;
  } else {
    atomicOr(status, vgpu::kStatusWorkOverrun);
  }
  if (out_f32)
    for (int k = 0; k < kFeat; ++k) out_f32[(size_t)s * kFeat + k] = f[k];
  if (out_bf16)
    for (int k = 0; k < kIn; ++k) out_bf16[(size_t)s * kIn + k] = __float2bfloat16_rn(k < kFeat ? f[k] : 0.f);
}

// Host features [rows x 7] (float32) -> padded bf16 input rows [rows x 16].
__global__ void lp_pack_input_kernel(const float* __restrict__ f, int64_t rows, bf16* __restrict__ x) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows * kIn) return;
  const int64_t r = i / kIn;
  const int k = (int)(i % kIn);
  x[i] = __float2bfloat16_rn(k < kFeat ? f[r * kFeat + k] : 0.f);
}

// Max over each part's 2048 rows of A3 [B*2048 x 256] (values >= +0). The key
// orders by value, then by the lower row: (bits << 32) | ~row.
__global__ void lp_pool_kernel(const bf16* __restrict__ A3, unsigned long long* __restrict__ key) {
  const int b = blockIdx.x, chunk = blockIdx.y, c = threadIdx.x;
  const int r0 = chunk * (kPts / 8);
  float best = -1.f;
  int arg = r0;
  for (int r = r0; r < r0 + kPts / 8; ++r) {
    const float v = __bfloat162float(A3[((size_t)b * kPts + r) * 256 + c]);
    if (v > best) {
      best = v;
      arg = r;
    }
  }
  const uint32_t bits = __float_as_uint(best > 0.f ? best : 0.f);
  atomicMax(&key[b * 256 + c], ((unsigned long long)bits << 32) | (0xFFFFFFFFu - (uint32_t)arg));
}

__global__ void lp_pool_finish_kernel(const unsigned long long* __restrict__ key, int count,
                                      float* __restrict__ G, bf16* __restrict__ Gb,
                                      int32_t* __restrict__ arg) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const unsigned long long k = key[i];
  const float v = __uint_as_float((uint32_t)(k >> 32));
  G[i] = v;
  Gb[i] = __float2bfloat16_rn(v);
  const uint32_t r = 0xFFFFFFFFu - (uint32_t)(k & 0xFFFFFFFFu);
  arg[i] = (int32_t)(r < (uint32_t)kPts ? r : 0u);  // every key is set by lp_pool_kernel
}

// Head output [B x 64] -> planes [B x 16 x 4]: unit normal and offset.
__global__ void lp_planes_kernel(const float* __restrict__ Z, int B, float* __restrict__ planes) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B * kPlanes) return;
  const float* z = Z + (size_t)i * 4;
  const float r = sqrtf(z[0] * z[0] + z[1] * z[1] + z[2] * z[2]) + 1e-12f;
  planes[4 * i] = z[0] / r;
  planes[4 * i + 1] = z[1] / r;
  planes[4 * i + 2] = z[2] / r;
  planes[4 * i + 3] = z[3];
}

// Set loss per part: for label planes l (unit normal n_l, offset d_l, weight
// w_l) and proposals q (normalised n_q, offset d_q),
//   D(q,l) = min over s = +-1 of |s n_q - n_l|^2 + (s d_q - d_l)^2
//   loss = sum_l w_l min_q D(q,l) / sum_l w_l + lambda/16 sum_q min_l D(q,l).
// Writes dZ (bf16, already divided by B) and the part's loss.
constexpr float kLambda = 0.1f;
__global__ void lp_loss_kernel(const float* __restrict__ Z, const float* __restrict__ labels,
                               const float* __restrict__ lw, int B, int L,
                               bf16* __restrict__ dZ, float* __restrict__ loss) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const float* z = Z + (size_t)b * 64;
  float nh[kPlanes][3], d[kPlanes], r[kPlanes], gn[kPlanes][3], gd[kPlanes];
  for (int q = 0; q < kPlanes; ++q) {
    r[q] = sqrtf(z[4 * q] * z[4 * q] + z[4 * q + 1] * z[4 * q + 1] + z[4 * q + 2] * z[4 * q + 2]) + 1e-12f;
    for (int a = 0; a < 3; ++a) nh[q][a] = z[4 * q + a] / r[q];
    d[q] = z[4 * q + 3];
    gn[q][0] = gn[q][1] = gn[q][2] = gd[q] = 0.f;
  }
  const float* lab = labels + (size_t)b * L * 4;
  const float* w = lw + (size_t)b * L;
  float wsum = 0.f;
  for (int l = 0; l < L; ++l) wsum += w[l];
  const float inv_w = wsum > 0.f ? 1.f / wsum : 0.f;
  float total = 0.f;
  auto dist = [&](int q, int l, float& sgn) {
    const float c = nh[q][0] * lab[4 * l] + nh[q][1] * lab[4 * l + 1] + nh[q][2] * lab[4 * l + 2];
    const float dp = d[q] - lab[4 * l + 3], dm = -d[q] - lab[4 * l + 3];
    const float Dp = 2.f - 2.f * c + dp * dp, Dm = 2.f + 2.f * c + dm * dm;
    sgn = Dp <= Dm ? 1.f : -1.f;
    return Dp <= Dm ? Dp : Dm;
  };
  // dD/dn_q = -2 s n_l ; dD/dd_q = 2 (d_q - s d_l)
  auto add_grad = [&](int q, int l, float sgn, float coef) {
    for (int a = 0; a < 3; ++a) gn[q][a] += coef * (-2.f * sgn * lab[4 * l + a]);
    gd[q] += coef * 2.f * (d[q] - sgn * lab[4 * l + 3]);
  };
  for (int l = 0; l < L; ++l) {
    if (w[l] <= 0.f) continue;
    int best = 0;
    float bs = 1.f, bd = 3.4e38f;
    for (int q = 0; q < kPlanes; ++q) {
      float s;
      const float D = dist(q, l, s);
      if (D < bd) {
        bd = D;
        best = q;
        bs = s;
      }
    }
    total += w[l] * inv_w * bd;
    add_grad(best, l, bs, w[l] * inv_w);
  }
  for (int q = 0; q < kPlanes; ++q) {
    int best = -1;
    float bs = 1.f, bd = 3.4e38f;
    for (int l = 0; l < L; ++l) {
      if (w[l] <= 0.f) continue;
      float s;
      const float D = dist(q, l, s);
      if (D < bd) {
        bd = D;
        best = l;
        bs = s;
      }
    }
    if (best < 0) continue;
    total += kLambda / kPlanes * bd;
    add_grad(q, best, bs, kLambda / kPlanes);
  }
  loss[b] = total;
  const float scale = 1.f / (float)B;
  for (int q = 0; q < kPlanes; ++q) {
    // through n_hat = n / |n|: dn = (g - n_hat (n_hat . g)) / |n|
    const float dotg = nh[q][0] * gn[q][0] + nh[q][1] * gn[q][1] + nh[q][2] * gn[q][2];
    for (int a = 0; a < 3; ++a)
      dZ[(size_t)b * 64 + 4 * q + a] = __float2bfloat16_rn(scale * (gn[q][a] - nh[q][a] * dotg) / r[q]);
    dZ[(size_t)b * 64 + 4 * q + 3] = __float2bfloat16_rn(scale * gd[q]);
  }
}

// Gradient through the max-pool: dZ3 is zero except at each (part, channel)'s
// arg-max row, where it carries dG when the pooled value is positive. Also the
// layer-3 bias gradient sum_b dG*[G>0] (float32).
__global__ void lp_pool_backward_kernel(const float* __restrict__ G, const float* __restrict__ dG,
                                        const int32_t* __restrict__ arg, int B,
                                        bf16* __restrict__ dZ3, float* __restrict__ db3) {
  const int c = threadIdx.x;
  float s = 0.f;
  for (int b = 0; b < B; ++b) {
    const int i = b * 256 + c;
    if (G[i] > 0.f) {
      dZ3[((size_t)b * kPts + arg[i]) * 256 + c] = __float2bfloat16_rn(dG[i]);
      s += dG[i];
    }
  }
  db3[c] = s;
}

__global__ void lp_adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                               float* __restrict__ v, bf16* __restrict__ pb, int count, float lr,
                               float bc1, float bc2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float gi = g[i];
  const float mi = 0.9f * m[i] + 0.1f * gi;
  const float vi = 0.999f * v[i] + 0.001f * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float pi = p[i] - lr * (mi * bc1) / (sqrtf(vi * bc2) + 1e-8f);
  p[i] = pi;
  pb[i] = __float2bfloat16_rn(pi);
}

__global__ void lp_to_bf16_kernel(const float* __restrict__ p, int count, bf16* __restrict__ pb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) pb[i] = __float2bfloat16_rn(p[i]);
}

// The proposals back in the part's input frame. The network sees (x - c) / s,
// so n . (x - c) / s + d' = 0 gives d = s d' - n . c, in FP64 in this order
// (explicit round-to-nearest, no contraction): the planes are the same on
// every path that asks for them.
__global__ void lp_frame_kernel(const float* __restrict__ pl, float cx, float cy, float cz, float s,
                                double* __restrict__ out) {
  const int q = threadIdx.x;
  if (q >= kPlanes) return;
  const double nx = pl[4 * q], ny = pl[4 * q + 1], nz = pl[4 * q + 2];
  const double nc = __dadd_rn(__dadd_rn(__dmul_rn(nx, (double)cx), __dmul_rn(ny, (double)cy)),
                              __dmul_rn(nz, (double)cz));
  out[4 * q] = nx;
  out[4 * q + 1] = ny;
  out[4 * q + 2] = nz;
  out[4 * q + 3] = __dsub_rn(__dmul_rn((double)s, (double)pl[4 * q + 3]), nc);
}

}  // namespace

struct visacd_lp {
  visacd_ctx* ctx = nullptr;
  int max_batch = 0;
  bool tcgen05 = false;  // forward per-edge layers on the tcgen05 path (on after create)
  int64_t step = 0;
  DevBuf params, params_bf16, grads, adam_m, adam_v;
  DevBuf x0, a1, a2, a3, poolkey, g, gb, arg, a4, a5, z6;
  DevBuf dz6, dz5, dz4, dg, dz3, dz2, dz1;
  DevBuf parts, labels, lw, loss, feats, planes, pts, edges, frame;
  template <class F>
  void each_buf(F f) {
    for (DevBuf* b : {&params, &params_bf16, &grads, &adam_m, &adam_v, &x0, &a1, &a2, &a3, &poolkey, &g, &gb,
                      &arg, &a4, &a5, &z6, &dz6, &dz5, &dz4, &dg, &dz3, &dz2, &dz1, &parts, &labels, &lw,
                      &loss, &feats, &planes, &pts, &edges, &frame})
      f(*b);
  }
};

namespace {

template <class T>
T* P(DevBuf& b) {
  return reinterpret_cast<T*>(b.p);
}

bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

// One GEMM launch (see lp_gemm_kernel) with its precondition checks.
template <bool AK, bool BK, int EPI>
int gemm(visacd_lp* lp, const bf16* A, int lda, const bf16* B, int ldb, void* C, int ldc, int M,
         int N, int K, int kchunk = 0, const float* bias = nullptr, const bf16* R = nullptr,
         int ldr = 0) {
  visacd_ctx* ctx = lp->ctx;
  VCHECK(M > 0 && N > 0 && K > 0, VISACD_ERR_INVALID_ARG, "lp gemm: empty shape");
  VCHECK((AK ? K : M) % 8 == 0 && (BK ? K : N) % 8 == 0 && N % 2 == 0 && ldc % 2 == 0,
         VISACD_ERR_INVALID_ARG, "lp gemm: contiguous extents must be multiples of 8");
  VCHECK(lda % 8 == 0 && ldb % 8 == 0 && aligned16(A) && aligned16(B), VISACD_ERR_INVALID_ARG,
         "lp gemm: operands must be 16-byte aligned");
  if (kchunk <= 0) kchunk = K;
  VCHECK(kchunk == K || kchunk % kTK == 0, VISACD_ERR_INVALID_ARG, "lp gemm: chunk must be a multiple of 32");
  const int splits = (K + kchunk - 1) / kchunk;
  VCHECK(splits == 1 || EPI == kEpiStoreF32, VISACD_ERR_INVALID_ARG, "lp gemm: split needs f32 parts");
  dim3 grid((M + kTM - 1) / kTM, (N + kTN - 1) / kTN, splits);
  VLAUNCH(ctx, vgpu::kKLpGemm, grid, 128, 0, (lp_gemm_kernel<AK, BK, EPI>), A, lda, B, ldb, C, ldc,
          M, N, K, kchunk, bias, R, ldr);
  return VISACD_OK;
}

// dW[N x K] = dZ^T X over `rows` rows, split over the rows and summed in order.
int weight_grad(visacd_lp* lp, const bf16* dZ, int N, const bf16* X, int K, int rows, float* out) {
  visacd_ctx* ctx = lp->ctx;
  const int tiles = ((N + kTM - 1) / kTM) * ((K + kTN - 1) / kTN);
  int splits = std::max(1, std::min((2 * ctx->sm_count + tiles - 1) / tiles, (rows + kTK - 1) / kTK));
  int kchunk = (rows + splits - 1) / splits;
  kchunk = (kchunk + kTK - 1) / kTK * kTK;
  splits = (rows + kchunk - 1) / kchunk;
  VCHECK(lp->parts.cap >= (size_t)splits * N * K * sizeof(float), VISACD_ERR_INVALID_ARG,
         "lp: partial-sum buffer too small");
  VTRY((gemm<false, false, kEpiStoreF32>(lp, dZ, N, X, K, lp->parts.p, K, N, K, rows, kchunk)));
  VLAUNCH(ctx, vgpu::kKLpMisc, vgpu::grid_for((int64_t)N * K, 256, 1024), 256, 0, lp_sum_parts_kernel,
          P<float>(lp->parts), splits, N * K, out);
  return VISACD_OK;
}

// db[N] = column sums of dZ [rows x N], in a fixed order.
int bias_grad(visacd_lp* lp, const bf16* dZ, int rows, int N, float* out) {
  visacd_ctx* ctx = lp->ctx;
  const int per = 512;
  const int blocks = (rows + per - 1) / per;
  VCHECK(lp->parts.cap >= (size_t)blocks * N * sizeof(float), VISACD_ERR_INVALID_ARG,
         "lp: partial-sum buffer too small");
  VLAUNCH(ctx, vgpu::kKLpMisc, blocks, N, 0, lp_colsum_kernel, dZ, rows, N, per, P<float>(lp->parts));
  VLAUNCH(ctx, vgpu::kKLpMisc, vgpu::grid_for(N, 256, 64), 256, 0, lp_sum_parts_kernel,
          P<float>(lp->parts), blocks, N, out);
  return VISACD_OK;
}

int alloc_batch(visacd_lp* lp, int B) {
  if (B <= lp->max_batch) return VISACD_OK;
  const size_t rows = (size_t)B * kPts;
  VTRY(ensure(lp->x0, rows * kIn * 2));
  VTRY(ensure(lp->a1, rows * 64 * 2));
  VTRY(ensure(lp->a2, rows * 128 * 2));
  VTRY(ensure(lp->a3, rows * 256 * 2));
  VTRY(ensure(lp->poolkey, (size_t)B * 256 * 8));
  VTRY(ensure(lp->g, (size_t)B * 256 * 4));
  VTRY(ensure(lp->gb, (size_t)B * 256 * 2));
  VTRY(ensure(lp->arg, (size_t)B * 256 * 4));
  VTRY(ensure(lp->a4, (size_t)B * 128 * 2));
  VTRY(ensure(lp->a5, (size_t)B * 64 * 2));
  VTRY(ensure(lp->z6, (size_t)B * 64 * 4));
  VTRY(ensure(lp->planes, (size_t)B * kPlanes * 4 * 4));
  lp->max_batch = B;
  return VISACD_OK;
}

int alloc_train(visacd_lp* lp, int B) {
  const size_t rows = (size_t)B * kPts;
  VTRY(ensure(lp->dz6, (size_t)B * 64 * 2));
  VTRY(ensure(lp->dz5, (size_t)B * 64 * 2));
  VTRY(ensure(lp->dz4, (size_t)B * 128 * 2));
  VTRY(ensure(lp->dg, (size_t)B * 256 * 4));
  VTRY(ensure(lp->dz3, rows * 256 * 2));
  VTRY(ensure(lp->dz2, rows * 128 * 2));
  VTRY(ensure(lp->dz1, rows * 64 * 2));
  VTRY(ensure(lp->loss, (size_t)B * 4));
  // Partial sums of the split weight gradients (at most 2 x SMs + tiles chunks
  // of <= 64 x 64 tiles... bounded by (2 * SMs + 8) * 256 * 128 floats is more
  // than enough) and of the bias column sums (rows / 512 blocks x 256).
  // Sized once here: a reallocation between stream-ordered launches would free
  // memory a queued kernel still uses.
  const size_t wparts = (size_t)(2 * lp->ctx->sm_count + 8) * 4096 * 8;
  const size_t bparts = (rows / 512 + 1) * 256;
  VTRY(ensure(lp->parts, std::max(wparts, bparts) * sizeof(float)));
  return VISACD_OK;
}

// Forward pass over x0 (B parts): fills a1..a3, g/gb/arg, a4, a5, z6.
int forward(visacd_lp* lp, int B) {
  visacd_ctx* ctx = lp->ctx;
  const int M = B * kPts;
  const bf16* W = P<bf16>(lp->params_bf16);
  const float* Pf = P<float>(lp->params);
  if (lp->tcgen05) {
    const bf16* xin[3] = {P<bf16>(lp->x0), P<bf16>(lp->a1), P<bf16>(lp->a2)};
    bf16* yout[3] = {P<bf16>(lp->a1), P<bf16>(lp->a2), P<bf16>(lp->a3)};
    const int tiles = (M + kTcM - 1) / kTcM;
    const int grid = std::max(1, std::min(tiles, ctx->sm_count));
    for (int l = 0; l < 3; ++l)
      VLAUNCH(ctx, vgpu::kKLpGemm, grid, 128, kTcSmem, lp_gemm_tc_kernel, xin[l], M, kK[l], W + kOff.w[l], kN[l],
              Pf + kOff.b[l], yout[l], ctx->d_status);
  } else {
    VTRY((gemm<true, true, kEpiBiasReluBf16>(lp, P<bf16>(lp->x0), kIn, W + kOff.w[0], kIn, lp->a1.p, 64, M,
                                             64, kIn, 0, Pf + kOff.b[0])));
    VTRY((gemm<true, true, kEpiBiasReluBf16>(lp, P<bf16>(lp->a1), 64, W + kOff.w[1], 64, lp->a2.p, 128, M,
                                             128, 64, 0, Pf + kOff.b[1])));
    VTRY((gemm<true, true, kEpiBiasReluBf16>(lp, P<bf16>(lp->a2), 128, W + kOff.w[2], 128, lp->a3.p, 256,
                                             M, 256, 128, 0, Pf + kOff.b[2])));
  }
  VCUDA(cudaMemsetAsync(lp->poolkey.p, 0, (size_t)B * 256 * 8, ctx->stream));
  VLAUNCH(ctx, vgpu::kKLpPool, dim3(B, 8), 256, 0, lp_pool_kernel, P<bf16>(lp->a3),
          P<unsigned long long>(lp->poolkey));
  VLAUNCH(ctx, vgpu::kKLpPool, vgpu::grid_for(B * 256, 256, 1 << 20), 256, 0, lp_pool_finish_kernel,
          P<unsigned long long>(lp->poolkey), B * 256, P<float>(lp->g), P<bf16>(lp->gb),
          P<int32_t>(lp->arg));
  VTRY((gemm<true, true, kEpiBiasReluBf16>(lp, P<bf16>(lp->gb), 256, W + kOff.w[3], 256, lp->a4.p, 128,
                                           B, 128, 256, 0, Pf + kOff.b[3])));
  VTRY((gemm<true, true, kEpiBiasReluBf16>(lp, P<bf16>(lp->a4), 128, W + kOff.w[4], 128, lp->a5.p, 64,
                                           B, 64, 128, 0, Pf + kOff.b[4])));
  VTRY((gemm<true, true, kEpiBiasF32>(lp, P<bf16>(lp->a5), 64, W + kOff.w[5], 64, lp->z6.p, 64, B, 64,
                                      64, 0, Pf + kOff.b[5])));
  return VISACD_OK;
}

// Loss and backward pass after forward(): fills grads (overwritten).
int backward(visacd_lp* lp, int B, int L) {
  visacd_ctx* ctx = lp->ctx;
  const int M = B * kPts;
  const bf16* W = P<bf16>(lp->params_bf16);
  float* G = P<float>(lp->grads);
  VLAUNCH(ctx, vgpu::kKLpLoss, vgpu::grid_for(B, 64, 1 << 20), 64, 0, lp_loss_kernel, P<float>(lp->z6),
          P<float>(lp->labels), P<float>(lp->lw), B, L, P<bf16>(lp->dz6), P<float>(lp->loss));
  // head
  VTRY(weight_grad(lp, P<bf16>(lp->dz6), 64, P<bf16>(lp->a5), 64, B, G + kOff.w[5]));
  VTRY(bias_grad(lp, P<bf16>(lp->dz6), B, 64, G + kOff.b[5]));
  VTRY((gemm<true, false, kEpiMaskBf16>(lp, P<bf16>(lp->dz6), 64, W + kOff.w[5], 64, lp->dz5.p, 64, B,
                                        64, 64, 0, nullptr, P<bf16>(lp->a5), 64)));
  VTRY(weight_grad(lp, P<bf16>(lp->dz5), 64, P<bf16>(lp->a4), 128, B, G + kOff.w[4]));
  VTRY(bias_grad(lp, P<bf16>(lp->dz5), B, 64, G + kOff.b[4]));
  VTRY((gemm<true, false, kEpiMaskBf16>(lp, P<bf16>(lp->dz5), 64, W + kOff.w[4], 128, lp->dz4.p, 128, B,
                                        128, 64, 0, nullptr, P<bf16>(lp->a4), 128)));
  VTRY(weight_grad(lp, P<bf16>(lp->dz4), 128, P<bf16>(lp->gb), 256, B, G + kOff.w[3]));
  VTRY(bias_grad(lp, P<bf16>(lp->dz4), B, 128, G + kOff.b[3]));
  VTRY((gemm<true, false, kEpiStoreF32>(lp, P<bf16>(lp->dz4), 128, W + kOff.w[3], 256, lp->dg.p, 256, B,
                                        256, 128)));
  // max-pool
  VCUDA(cudaMemsetAsync(lp->dz3.p, 0, (size_t)M * 256 * 2, ctx->stream));
  VLAUNCH(ctx, vgpu::kKLpPool, 1, 256, 0, lp_pool_backward_kernel, P<float>(lp->g), P<float>(lp->dg),
          P<int32_t>(lp->arg), B, P<bf16>(lp->dz3), G + kOff.b[2]);
  // shared per-edge layers
  VTRY(weight_grad(lp, P<bf16>(lp->dz3), 256, P<bf16>(lp->a2), 128, M, G + kOff.w[2]));
  VTRY((gemm<true, false, kEpiMaskBf16>(lp, P<bf16>(lp->dz3), 256, W + kOff.w[2], 128, lp->dz2.p, 128, M,
                                        128, 256, 0, nullptr, P<bf16>(lp->a2), 128)));
  VTRY(weight_grad(lp, P<bf16>(lp->dz2), 128, P<bf16>(lp->a1), 64, M, G + kOff.w[1]));
  VTRY(bias_grad(lp, P<bf16>(lp->dz2), M, 128, G + kOff.b[1]));
  VTRY((gemm<true, false, kEpiMaskBf16>(lp, P<bf16>(lp->dz2), 128, W + kOff.w[1], 64, lp->dz1.p, 64, M,
                                        64, 128, 0, nullptr, P<bf16>(lp->a1), 64)));
  VTRY(weight_grad(lp, P<bf16>(lp->dz1), 64, P<bf16>(lp->x0), kIn, M, G + kOff.w[0]));
  VTRY(bias_grad(lp, P<bf16>(lp->dz1), M, 64, G + kOff.b[0]));
  return VISACD_OK;
}

int upload_batch(visacd_lp* lp, const float* feats, int B, const float* labels, const float* lw, int L) {
  visacd_ctx* ctx = lp->ctx;
  VTRY(alloc_batch(lp, B));
  const size_t fbytes = (size_t)B * kPts * kFeat * 4;
  VTRY(ensure(lp->feats, fbytes));
  VCUDA(cudaMemcpyAsync(lp->feats.p, feats, fbytes, cudaMemcpyHostToDevice, ctx->stream));
  const int64_t rows = (int64_t)B * kPts;
  VLAUNCH(ctx, vgpu::kKLpFeatures, vgpu::grid_for(rows * kIn, 256, 1 << 30), 256, 0, lp_pack_input_kernel,
          P<float>(lp->feats), rows, P<bf16>(lp->x0));
  if (labels) {
    VTRY(alloc_train(lp, B));
    VTRY(ensure(lp->labels, (size_t)B * L * 16));
    VTRY(ensure(lp->lw, (size_t)B * L * 4));
    VCUDA(cudaMemcpyAsync(lp->labels.p, labels, (size_t)B * L * 16, cudaMemcpyHostToDevice, ctx->stream));
    VCUDA(cudaMemcpyAsync(lp->lw.p, lw, (size_t)B * L * 4, cudaMemcpyHostToDevice, ctx->stream));
  }
  return VISACD_OK;
}

int upload_part(visacd_ctx* ctx, visacd_lp* lp, const float* points, int32_t n, const uint32_t* edges,
                int64_t E) {
  VCHECK(points && edges && n > 0 && E > 0, VISACD_ERR_INVALID_ARG, "lp: empty part");
  VTRY(ensure(lp->pts, (size_t)n * 12));
  VTRY(ensure(lp->edges, (size_t)E * 8));
  VCUDA(cudaMemcpyAsync(lp->pts.p, points, (size_t)n * 12, cudaMemcpyHostToDevice, ctx->stream));
  VCUDA(cudaMemcpyAsync(lp->edges.p, edges, (size_t)E * 8, cudaMemcpyHostToDevice, ctx->stream));
  return VISACD_OK;
}

}  // namespace

extern "C" int visacd_lp_param_count(void) { return kOff.total; }

extern "C" int visacd_lp_create(visacd_ctx* ctx, const float* params, uint32_t seed, visacd_lp** out) {
  VCHECK(ctx && out, VISACD_ERR_INVALID_ARG, "lp_create: null argument");
  VCUDA(cudaSetDevice(ctx->device));
  visacd_lp* lp = new visacd_lp();
  lp->ctx = ctx;
  ctx->lps.push_back(lp);
  lp->each_buf([&](DevBuf& b) { b.stream = ctx->stream; });
  const size_t pb = (size_t)kOff.total * 4;
  int rc = VISACD_OK;
  auto fail = [&](int code) {
    visacd_lp_destroy(lp);
    return code;
  };
  for (DevBuf* b : {&lp->params, &lp->grads, &lp->adam_m, &lp->adam_v})
    if ((rc = ensure(*b, pb)) != VISACD_OK) return fail(rc);
  if ((rc = ensure(lp->params_bf16, pb / 2)) != VISACD_OK) return fail(rc);
  std::vector<float> init;
  if (!params) {
    // He-uniform weights over the real fan-in (the input's zero padding gets
    // zero weights), zero biases.
    init.assign(kOff.total, 0.f);
    std::mt19937 eng(seed);
    for (int l = 0; l < kLayers; ++l) {
      const float a = std::sqrt(6.f / kFanIn[l]) * (l == kLayers - 1 ? 0.5f : 1.f);
      std::uniform_real_distribution<float> u(-a, a);
      for (int r = 0; r < kN[l]; ++r)
        for (int k = 0; k < kK[l]; ++k) init[kOff.w[l] + r * kK[l] + k] = k < kFanIn[l] ? u(eng) : 0.f;
    }
    params = init.data();
  }
  cudaError_t e = cudaMemcpyAsync(lp->params.p, params, pb, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(lp->adam_m.p, 0, pb, ctx->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(lp->adam_v.p, 0, pb, ctx->stream);
  if (e != cudaSuccess) {
    vgpu::set_error("lp_create: %s", cudaGetErrorString(e));
    return fail(VISACD_ERR_CUDA);
  }
  // The forward per-edge layers run on tcgen05 (tensor memory) by default.
  if ((e = cudaFuncSetAttribute(lp_gemm_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem)) !=
      cudaSuccess) {
    vgpu::set_error("lp_create: %s", cudaGetErrorString(e));
    return fail(VISACD_ERR_CUDA);
  }
  lp->tcgen05 = true;
  lp_to_bf16_kernel<<<(kOff.total + 255) / 256, 256, 0, ctx->stream>>>(P<float>(lp->params), kOff.total,
                                                                      P<bf16>(lp->params_bf16));
  if ((rc = vgpu::after_launch(ctx, "lp_to_bf16_kernel")) != VISACD_OK) return fail(rc);
  if ((e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess) {
    vgpu::set_error("lp_create: %s", cudaGetErrorString(e));
    return fail(VISACD_ERR_CUDA);
  }
  *out = lp;
  return VISACD_OK;
}

extern "C" int visacd_lp_destroy(visacd_lp* lp) {
  if (!lp) return VISACD_OK;
  if (lp->ctx) {
    auto& v = lp->ctx->lps;
    v.erase(std::remove(v.begin(), v.end(), lp), v.end());
    vgpu::lp_detach(lp);
  }
  delete lp;
  return VISACD_OK;
}

extern "C" int visacd_lp_get_params(visacd_lp* lp, float* out) {
  VCHECK(lp && out, VISACD_ERR_INVALID_ARG, "lp_get_params: null argument");
  VCHECK(lp->ctx, VISACD_ERR_INVALID_ARG, "lp_get_params: the proposer's context was destroyed");
  VCUDA(cudaMemcpyAsync(out, lp->params.p, (size_t)kOff.total * 4, cudaMemcpyDeviceToHost, lp->ctx->stream));
  VCUDA(vgpu::stream_wait(lp->ctx));
  return VISACD_OK;
}

extern "C" int visacd_lp_features(visacd_lp* lp, const float* points, int32_t n, const uint32_t* edges,
                                  int64_t E, const float* center, float scale, float* feats_out) {
  VCHECK(lp && center && feats_out && scale > 0.f, VISACD_ERR_INVALID_ARG, "lp_features: bad argument");
  VCHECK(lp->ctx, VISACD_ERR_INVALID_ARG, "lp_features: the proposer's context was destroyed");
  visacd_ctx* ctx = lp->ctx;
  VCUDA(cudaSetDevice(ctx->device));
  VTRY(upload_part(ctx, lp, points, n, edges, E));
  VTRY(ensure(lp->feats, (size_t)kPts * kFeat * 4));
  VLAUNCH(ctx, vgpu::kKLpFeatures, kPts / 256, 256, 0, lp_features_kernel, P<float>(lp->pts),
          P<uint32_t>(lp->edges), E, n, center[0], center[1], center[2], 1.f / scale, P<float>(lp->feats),
          (bf16*)nullptr, ctx->d_status);
  VCUDA(cudaMemcpyAsync(feats_out, lp->feats.p, (size_t)kPts * kFeat * 4, cudaMemcpyDeviceToHost,
                        ctx->stream));
  return vgpu::check_status(ctx, "lp_features");
}

extern "C" int visacd_lp_forward(visacd_lp* lp, const float* feats, int32_t B, float* planes_out) {
  VCHECK(lp && feats && planes_out && B > 0, VISACD_ERR_INVALID_ARG, "lp_forward: bad argument");
  VCHECK(lp->ctx, VISACD_ERR_INVALID_ARG, "lp_forward: the proposer's context was destroyed");
  visacd_ctx* ctx = lp->ctx;
  VCUDA(cudaSetDevice(ctx->device));
  VTRY(upload_batch(lp, feats, B, nullptr, nullptr, 0));
  VTRY(forward(lp, B));
  VLAUNCH(ctx, vgpu::kKLpLoss, vgpu::grid_for(B * kPlanes, 128, 1 << 20), 128, 0, lp_planes_kernel,
          P<float>(lp->z6), B, P<float>(lp->planes));
  VCUDA(cudaMemcpyAsync(planes_out, lp->planes.p, (size_t)B * kPlanes * 16, cudaMemcpyDeviceToHost,
                        ctx->stream));
  VCUDA(vgpu::stream_wait(ctx));
  return VISACD_OK;
}

namespace vgpu {

visacd_ctx* lp_context(visacd_lp* lp) { return lp->ctx; }

void lp_detach(visacd_lp* lp) {
  cudaSetDevice(lp->ctx->device);
  lp->each_buf([](DevBuf& b) { release(b); });
  cudaStreamSynchronize(lp->ctx->stream);
  lp->ctx = nullptr;
}

int lp_propose_device(visacd_lp* lp, const float* d_pts, int32_t n, const uint32_t* d_edges, int64_t E,
                      const float* center, float scale, double* d_planes) {
  VCHECK(lp && d_pts && d_edges && center && d_planes && n > 0 && E > 0 && scale > 0.f,
         VISACD_ERR_INVALID_ARG, "lp_propose: bad argument");
  visacd_ctx* ctx = lp->ctx;
  VTRY(alloc_batch(lp, 1));
  VLAUNCH(ctx, kKLpFeatures, kPts / 256, 256, 0, lp_features_kernel, d_pts, d_edges, E, n, center[0],
          center[1], center[2], 1.f / scale, (float*)nullptr, P<bf16>(lp->x0), ctx->d_status);
  VTRY(forward(lp, 1));
  VLAUNCH(ctx, kKLpLoss, 1, 32, 0, lp_planes_kernel, P<float>(lp->z6), 1, P<float>(lp->planes));
  VLAUNCH(ctx, kKLpMisc, 1, 32, 0, lp_frame_kernel, P<float>(lp->planes), center[0], center[1], center[2],
          scale, d_planes);
  return VISACD_OK;
}

}  // namespace vgpu

extern "C" int visacd_lp_propose(visacd_lp* lp, const float* points, int32_t n, const uint32_t* edges,
                                 int64_t E, const float* center, float scale, double* planes_out) {
  VCHECK(lp && center && planes_out && scale > 0.f, VISACD_ERR_INVALID_ARG, "lp_propose: bad argument");
  VCHECK(lp->ctx, VISACD_ERR_INVALID_ARG, "lp_propose: the proposer's context was destroyed");
  visacd_ctx* ctx = lp->ctx;
  VCUDA(cudaSetDevice(ctx->device));
  VTRY(upload_part(ctx, lp, points, n, edges, E));
  VTRY(ensure(lp->frame, (size_t)kPlanes * 32));
  VTRY(vgpu::lp_propose_device(lp, P<float>(lp->pts), n, P<uint32_t>(lp->edges), E, center, scale,
                               P<double>(lp->frame)));
  double* h = nullptr;
  VTRY(vgpu::pinned(ctx, (size_t)kPlanes * 32, (void**)&h));
  VCUDA(cudaMemcpyAsync(h, lp->frame.p, (size_t)kPlanes * 32, cudaMemcpyDeviceToHost, ctx->stream));
  VCUDA(vgpu::stream_wait(ctx));
  // The read-back shares the pinned staging area with the status check: copy
  // it out first.
  std::memcpy(planes_out, h, (size_t)kPlanes * 32);
  return vgpu::check_status(ctx, "lp_propose");
}

extern "C" int visacd_lp_grads(visacd_lp* lp, const float* feats, const float* labels, const float* lw,
                               int32_t B, int32_t L, float* grads_out, float* loss_out) {
  VCHECK(lp && feats && labels && lw && B > 0 && L > 0, VISACD_ERR_INVALID_ARG, "lp_grads: bad argument");
  VCHECK(lp->ctx, VISACD_ERR_INVALID_ARG, "lp_grads: the proposer's context was destroyed");
  visacd_ctx* ctx = lp->ctx;
  VCUDA(cudaSetDevice(ctx->device));
  VTRY(upload_batch(lp, feats, B, labels, lw, L));
  VTRY(forward(lp, B));
  VTRY(backward(lp, B, L));
  std::vector<float> loss(B);
  VCUDA(cudaMemcpyAsync(loss.data(), lp->loss.p, (size_t)B * 4, cudaMemcpyDeviceToHost, ctx->stream));
  if (grads_out)
    VCUDA(cudaMemcpyAsync(grads_out, lp->grads.p, (size_t)kOff.total * 4, cudaMemcpyDeviceToHost,
                          ctx->stream));
  VCUDA(vgpu::stream_wait(ctx));
  if (loss_out) {
    double s = 0;
    for (float v : loss) s += v;
    *loss_out = (float)(s / B);
  }
  return VISACD_OK;
}

extern "C" int visacd_lp_train_step(visacd_lp* lp, const float* feats, const float* labels,
                                    const float* lw, int32_t B, int32_t L, float lr, float* loss_out) {
  VTRY(visacd_lp_grads(lp, feats, labels, lw, B, L, nullptr, loss_out));
  visacd_ctx* ctx = lp->ctx;
  lp->step += 1;
  const float bc1 = 1.f / (1.f - std::pow(0.9f, (float)lp->step));
  const float bc2 = 1.f / (1.f - std::pow(0.999f, (float)lp->step));
  VLAUNCH(ctx, vgpu::kKLpAdam, (kOff.total + 255) / 256, 256, 0, lp_adam_kernel, P<float>(lp->params),
          P<float>(lp->grads), P<float>(lp->adam_m), P<float>(lp->adam_v), P<bf16>(lp->params_bf16),
          kOff.total, lr, bc1, bc2);
  return VISACD_OK;
}

extern "C" int visacd_lp_set_tcgen05(visacd_lp* lp, int enable) {
  VCHECK(lp, VISACD_ERR_INVALID_ARG, "lp_set_tcgen05: null proposer");
  VCHECK(lp->ctx, VISACD_ERR_INVALID_ARG, "lp_set_tcgen05: the proposer's context was destroyed");
  if (enable) {
    VCUDA(cudaSetDevice(lp->ctx->device));
    VCUDA(cudaFuncSetAttribute(lp_gemm_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem));
  }
  lp->tcgen05 = enable != 0;
  return VISACD_OK;
}

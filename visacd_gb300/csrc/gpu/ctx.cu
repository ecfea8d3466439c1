// Context lifetime, error strings, grow-only buffers, launch timing, and the two
// generic device primitives the kernels share: an exclusive scan and a stable
// LSD radix sort (own kernels; no CUB/Thrust on the product path).
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <atomic>
#include <mutex>

#include "common.cuh"
#include "bvh.cuh"

namespace vgpu {

static thread_local char g_err[1024] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int ensure(DevBuf& b, size_t bytes) {
  if (bytes <= b.cap && b.p) return VISACD_OK;
  if (b.p) {
    if (b.stream)
      cudaFreeAsync(b.p, b.stream);
    else
      cudaFree(b.p);
    b.p = nullptr;
    b.cap = 0;
  }
  size_t want = bytes + bytes / 4;
  if (want < 256) want = 256;
  want = (want + 255) & ~size_t(255);
  cudaError_t e = b.stream ? cudaMallocAsync(&b.p, want, b.stream) : cudaMalloc(&b.p, want);
  if (e != cudaSuccess) {
    cudaGetLastError();
    b.p = nullptr;
    set_error("cudaMalloc(%zu) failed: %s", want, cudaGetErrorString(e));
    return VISACD_ERR_NO_MEMORY;
  }
  b.cap = want;
  return VISACD_OK;
}

void release(DevBuf& b) {
  if (b.p) {
    if (b.stream)
      cudaFreeAsync(b.p, b.stream);
    else
      cudaFree(b.p);
  }
  b.p = nullptr;
  b.cap = 0;
}

int keep_pool_cached(int device) {
  static std::mutex mu;
  static bool done[64] = {false};
  std::lock_guard<std::mutex> lock(mu);
  if (device < 0 || device >= 64 || done[device]) return VISACD_OK;
  cudaMemPool_t pool;
  cudaError_t e = cudaDeviceGetDefaultMemPool(&pool, device);
  if (e == cudaSuccess) {
    uint64_t threshold = UINT64_MAX;
    e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold);
  }
  if (e != cudaSuccess) {
    set_error("default memory pool setup: %s", cudaGetErrorString(e));
    return VISACD_ERR_CUDA;
  }
  done[device] = true;
  return VISACD_OK;
}

static const char* kNames[kKCount] = {
    "point_stats",   "pack_edges",     "score_planes", "score_recheck_fp64",
    "score_finish",  "tri_prep",       "morton",       "radix_hist",
    "radix_scan",    "radix_scatter",  "karras_build", "aabb_fit",
    "node_layout",   "vis_prep",       "visibility",   "bitset_popc",
    "scan_blocks",   "scan_top",       "scan_add",     "bitset_emit",
    "clip",          "clip_resolve",   "face_hausdorff", "hd_bound",
    "hd_query",      "hd_head",        "lp_features",
    "lp_gemm",       "lp_pool",        "lp_loss",      "lp_adam",
    "lp_misc",       "sdf_remesh",     "sdf_dist",     "sdf_cross",
    "hull_dist",     "seg_tri",        "candidates",
    "lp_refine",     "lp_split",       "grid_near",    "grid_edt",
    "grid_final",    "vis_walk",       "convex_hull",
    "misc"};

const char* kernel_name(int id) { return (id >= 0 && id < kKCount) ? kNames[id] : "?"; }

static cudaEvent_t take_event(visacd_ctx* ctx) {
  if (!ctx->event_pool.empty()) {
    cudaEvent_t e = ctx->event_pool.back();
    ctx->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  if (cudaEventCreate(&e) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return e;
}

void timing_begin(visacd_ctx* ctx, int kernel, cudaEvent_t* a) {
  (void)kernel;
  *a = nullptr;
  if (!ctx->timing) return;
  *a = take_event(ctx);
  if (*a) cudaEventRecord(*a, ctx->stream);
}

int timing_end(visacd_ctx* ctx, int kernel, cudaEvent_t a) {
  if (!ctx->timing || !a) return VISACD_OK;
  cudaEvent_t b = take_event(ctx);
  if (!b) return VISACD_OK;
  VCUDA(cudaEventRecord(b, ctx->stream));
  ctx->pending.push_back({kernel, a, b});
  return VISACD_OK;
}

int after_launch(visacd_ctx* ctx, const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("launch of %s failed: %s", what, cudaGetErrorString(e));
    return VISACD_ERR_CUDA;
  }
  ctx->launches++;
  return VISACD_OK;
}

int pinned(visacd_ctx* ctx, size_t bytes, void** out) {
  if (bytes > ctx->h_pinned_cap) {
    if (ctx->h_pinned) cudaFreeHost(ctx->h_pinned);
    ctx->h_pinned = nullptr;
    ctx->h_pinned_cap = 0;
    size_t want = bytes < 4096 ? 4096 : bytes + bytes / 4;
    cudaError_t e = cudaMallocHost(&ctx->h_pinned, want);
    if (e != cudaSuccess) {
      cudaGetLastError();
      set_error("cudaMallocHost(%zu) failed: %s", want, cudaGetErrorString(e));
      return VISACD_ERR_NO_MEMORY;
    }
    ctx->h_pinned_cap = want;
  }
  *out = ctx->h_pinned;
  return VISACD_OK;
}

int Stager::reserve(size_t total_bytes, int arrays) {
  const size_t need = total_bytes + 64 * (size_t)(arrays + 1);
  VCUDA(stream_wait(ctx_));
  if (need > ctx_->h_upload_cap) {
    if (ctx_->h_upload) cudaFreeHost(ctx_->h_upload);
    ctx_->h_upload = nullptr;
    ctx_->h_upload_cap = 0;
    const size_t want = need + need / 4;
    cudaError_t e = cudaMallocHost(&ctx_->h_upload, want);
    if (e != cudaSuccess) {
      cudaGetLastError();
      set_error("cudaMallocHost(%zu) failed: %s", want, cudaGetErrorString(e));
      return VISACD_ERR_NO_MEMORY;
    }
    ctx_->h_upload_cap = want;
  }
  used_ = 0;
  cap_ = need;
  return VISACD_OK;
}

int Stager::put(void* dst, const void* src, size_t bytes) {
  if (bytes == 0) return VISACD_OK;
  VCHECK(used_ + bytes <= cap_, VISACD_ERR_INVALID_ARG, "upload larger than reserved");
  char* h = static_cast<char*>(ctx_->h_upload) + used_;
  std::memcpy(h, src, bytes);
  VCUDA(cudaMemcpyAsync(dst, h, bytes, cudaMemcpyHostToDevice, ctx_->stream));
  used_ += (bytes + 63) & ~size_t(63);
  return VISACD_OK;
}

int Stager::copy(void* dst, size_t bytes) {
  VCHECK(bytes <= cap_, VISACD_ERR_INVALID_ARG, "upload larger than reserved");
  if (bytes) VCUDA(cudaMemcpyAsync(dst, ctx_->h_upload, bytes, cudaMemcpyHostToDevice, ctx_->stream));
  return VISACD_OK;
}

int check_status(visacd_ctx* ctx, const char* what) {
  uint32_t* h = nullptr;
  VTRY(pinned(ctx, 64, (void**)&h));
  VCUDA(cudaMemcpyAsync(h, ctx->d_status, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
  VCUDA(stream_wait(ctx));
  return status_result(ctx, h[0], what);
}

int status_result(visacd_ctx* ctx, uint32_t s, const char* what) {
  if (s) {
    VCUDA(cudaMemsetAsync(ctx->d_status, 0, sizeof(uint32_t), ctx->stream));
    set_error("%s: device status 0x%x (traversal overrun=%d, stack overflow=%d, recheck "
              "overflow=%d, mbarrier timeout=%d, work overrun=%d)",
              what, s, !!(s & kStatusTraversalOverrun), !!(s & kStatusStackOverflow),
              !!(s & kStatusRecheckOverflow), !!(s & kStatusMbarrierTimeout),
              !!(s & kStatusWorkOverrun));
    return VISACD_ERR_DEVICE;
  }
  return VISACD_OK;
}

// ---------------------------------------------------------------------------
// Exclusive scan u32 -> u64 (three phases: block sums, top scan, add).
// ---------------------------------------------------------------------------
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ uint64_t block_exclusive_scan_u64(uint64_t v, uint64_t* total) {
  __shared__ uint64_t warp_sums[kScanThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint64_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint64_t w = lane < kScanThreads / 32 ? warp_sums[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint64_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < kScanThreads / 32) warp_sums[lane] = w;
  }
  __syncthreads();
  uint64_t before = warp ? warp_sums[warp - 1] : 0;
  *total = warp_sums[kScanThreads / 32 - 1];
  __syncthreads();
  return before + x - v;
}

__global__ void scan_blocks_kernel(const uint32_t* __restrict__ in, int64_t n,
                                   uint64_t* __restrict__ block_sums) {
  int64_t base = (int64_t)blockIdx.x * kScanTile;
  uint64_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    int64_t i = base + (int64_t)k * kScanThreads + threadIdx.x;
    if (i < n) s += in[i];
  }
  uint64_t total;
  block_exclusive_scan_u64(s, &total);
  if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

__global__ void scan_top_kernel(uint64_t* __restrict__ block_sums, int64_t nb) {
  uint64_t carry = 0;
  for (int64_t start = 0; start < nb; start += kScanThreads) {
    int64_t i = start + threadIdx.x;
    uint64_t v = i < nb ? block_sums[i] : 0;
    uint64_t total;
    uint64_t ex = block_exclusive_scan_u64(v, &total);
    if (i < nb) block_sums[i] = carry + ex;
    carry += total;
  }
  if (threadIdx.x == 0) block_sums[nb] = carry;
}

__global__ void scan_add_kernel(const uint32_t* __restrict__ in, int64_t n,
                                const uint64_t* __restrict__ block_sums,
                                uint64_t* __restrict__ out, int64_t nb) {
  // Each thread owns kScanItems consecutive elements.
  int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  uint32_t v[kScanItems];
  uint64_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    int64_t i = base + k;
    v[k] = i < n ? in[i] : 0u;
    s += v[k];
  }
  uint64_t total;
  uint64_t ex = block_exclusive_scan_u64(s, &total) + block_sums[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    int64_t i = base + k;
    if (i < n) out[i] = ex;
    ex += v[k];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) out[n] = block_sums[nb];
}

// Small scans (up to kScanSingle elements) in one launch: one block walks
// the tiles in order with a running carry.
constexpr int64_t kScanSingle = 4 * kScanTile;

__global__ void scan_single_kernel(const uint32_t* __restrict__ in, int64_t n, uint64_t* __restrict__ out) {
  uint64_t carry = 0;
  for (int64_t t0 = 0; t0 < n; t0 += kScanTile) {
    const int64_t base = t0 + (int64_t)threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint64_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
      const int64_t i = base + k;
      v[k] = i < n ? in[i] : 0u;
      s += v[k];
    }
    uint64_t total;
    uint64_t ex = block_exclusive_scan_u64(s, &total) + carry;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
      const int64_t i = base + k;
      if (i < n) out[i] = ex;
      ex += v[k];
    }
    carry += total;
  }
  if (threadIdx.x == 0) out[n] = carry;
}

int exclusive_scan_u32_to_u64(visacd_ctx* ctx, const uint32_t* in, uint64_t* out, int64_t n) {
  if (n <= kScanSingle) {
    VLAUNCH(ctx, kKScanAdd, 1, kScanThreads, 0, scan_single_kernel, in, n, out);
    return VISACD_OK;
  }
  int64_t nb = (n + kScanTile - 1) / kScanTile;
  if (nb < 1) nb = 1;
  VCHECK(nb < (1ll << 31), VISACD_ERR_INVALID_ARG, "scan too large: %lld", (long long)n);
  VTRY(ensure_slot(ctx, kSlotScanScratch, (size_t)(nb + 1) * sizeof(uint64_t)));
  uint64_t* bs = slot<uint64_t>(ctx, kSlotScanScratch);
  VLAUNCH(ctx, kKScanBlocks, (unsigned)nb, kScanThreads, 0, scan_blocks_kernel, in, n, bs);
  VLAUNCH(ctx, kKScanTop, 1, kScanThreads, 0, scan_top_kernel, bs, nb);
  VLAUNCH(ctx, kKScanAdd, (unsigned)nb, kScanThreads, 0, scan_add_kernel, in, n, bs, out, nb);
  return VISACD_OK;
}

// ---------------------------------------------------------------------------
// Stable LSD radix sort, 8-bit digits.
// ---------------------------------------------------------------------------
constexpr int kSortThreads = 256;
constexpr int kSortRounds = 8;
constexpr int kSortTile = kSortThreads * kSortRounds;

__global__ void radix_hist_kernel(const uint64_t* __restrict__ keys, int32_t n, int shift,
                                  uint32_t* __restrict__ hist, int nblocks) {
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  int64_t base = (int64_t)blockIdx.x * kSortTile;
  for (int r = 0; r < kSortRounds; ++r) {
    int64_t i = base + (int64_t)r * kSortThreads + threadIdx.x;
    if (i < n) atomicAdd(&h[(keys[i] >> shift) & 0xffu], 1u);
  }
  __syncthreads();
  hist[(int64_t)threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

__global__ void radix_scatter_kernel(const uint64_t* __restrict__ keys,
                                     const uint32_t* __restrict__ vals, int32_t n, int shift,
                                     const uint64_t* __restrict__ offsets, int nblocks,
                                     uint64_t* __restrict__ keys_out,
                                     uint32_t* __restrict__ vals_out) {
  __shared__ uint32_t cnt[kSortThreads / 32][256];
  __shared__ uint64_t base_off[256];
  __shared__ uint32_t round_total[256];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  base_off[threadIdx.x] = offsets[(int64_t)threadIdx.x * nblocks + blockIdx.x];
  int64_t tile = (int64_t)blockIdx.x * kSortTile;
  for (int r = 0; r < kSortRounds; ++r) {
#pragma unroll
    for (int w = 0; w < kSortThreads / 32; ++w) cnt[w][threadIdx.x] = 0;
    __syncthreads();
    int64_t i = tile + (int64_t)r * kSortThreads + threadIdx.x;
    bool valid = i < n;
    uint64_t k = valid ? keys[i] : 0;
    uint32_t v = valid ? vals[i] : 0;
    uint32_t digit = (uint32_t)(k >> shift) & 0xffu;
    unsigned active = __ballot_sync(0xffffffffu, valid);
    unsigned rank = 0;
    if (valid) {
      unsigned peers = __match_any_sync(active, digit);
      unsigned lower = peers & ((1u << lane) - 1u);
      rank = __popc(lower);
      if (lower == 0) cnt[warp][digit] = __popc(peers);
    }
    __syncthreads();
    {
      uint32_t run = 0;
#pragma unroll
      for (int w = 0; w < kSortThreads / 32; ++w) {
        uint32_t c = cnt[w][threadIdx.x];
        cnt[w][threadIdx.x] = run;
        run += c;
      }
      round_total[threadIdx.x] = run;
    }
    __syncthreads();
    if (valid) {
      uint64_t pos = base_off[digit] + cnt[warp][digit] + rank;
      keys_out[pos] = k;
      vals_out[pos] = v;
    }
    __syncthreads();
    base_off[threadIdx.x] += round_total[threadIdx.x];
    __syncthreads();
  }
}

// Small inputs (n <= kSmallSort) in one CTA: bitonic sort in shared memory of
// (key restricted to key_bits, input position), which is exactly the order of
// the stable LSD radix sort below, in one launch instead of 5 per key byte.
constexpr int kSmallSort = 512;  // above it the one-CTA LSD sort is faster (a 4096-key bitonic sort took ~49 us)
constexpr size_t kSmallSortSmem = (size_t)kSmallSort * 16;

__global__ void __launch_bounds__(1024) small_sort_kernel(uint64_t* __restrict__ keys, uint32_t* __restrict__ vals,
                                                          int n, uint64_t mask) {
  extern __shared__ __align__(16) unsigned char sm[];
  uint64_t* K = reinterpret_cast<uint64_t*>(sm);
  uint32_t* V = reinterpret_cast<uint32_t*>(sm + (size_t)kSmallSort * 8);
  uint32_t* Pos = reinterpret_cast<uint32_t*>(sm + (size_t)kSmallSort * 12);
  int n2 = 1;
  while (n2 < n) n2 <<= 1;
  for (int i = threadIdx.x; i < n2; i += blockDim.x) {
    if (i < n) {
      K[i] = keys[i];
      V[i] = vals[i];
    } else {
      K[i] = ~0ull;
      V[i] = 0;
    }
    Pos[i] = (uint32_t)i;
  }
  __syncthreads();
  for (int k = 2; k <= n2; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < n2; i += blockDim.x) {
        const int ixj = i ^ j;
        if (ixj > i) {
          // pads (position >= n) order after every real element
          const uint64_t ka = Pos[i] < (uint32_t)n ? (K[i] & mask) : ~0ull;
          const uint64_t kb = Pos[ixj] < (uint32_t)n ? (K[ixj] & mask) : ~0ull;
          const bool gt = ka > kb || (ka == kb && Pos[i] > Pos[ixj]);
          const bool asc = (i & k) == 0;
          if (gt == asc) {
            const uint64_t tk = K[i];
            K[i] = K[ixj];
            K[ixj] = tk;
            const uint32_t tv = V[i];
            V[i] = V[ixj];
            V[ixj] = tv;
            const uint32_t tp = Pos[i];
            Pos[i] = Pos[ixj];
            Pos[ixj] = tp;
          }
        }
      }
      __syncthreads();
    }
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    keys[i] = K[i];
    vals[i] = V[i];
  }
}

// Mid-size inputs (kSmallSort < n <= kMidSort) in one CTA: the same stable
// LSD passes over 8-bit digits as below, all in one launch instead of three
// launches per pass. Warp w owns the contiguous run [w C, (w + 1) C) of the input; per
// pass, per-warp digit counts give every (digit, warp) its output offset
// (digit-major, warp-minor), and each warp scatters its run in order, 32 keys
// at a time with match-any ranks (the next 32 loaded while one group is
// placed), so the order is stable. Keys and values ping-pong between the two
// buffer pairs in global memory (L2), plain loads only (the data changes
// between passes within the launch).
constexpr int kMidSort = 32768;
constexpr int kMidDigitBits = 8;  // 10-bit digits measured slower (per-pass fixed cost)
constexpr int kMidDigits = 1 << kMidDigitBits;
constexpr size_t kMidSortSmem = (size_t)32 * kMidDigits * 4 + 32 * 4;

__global__ void __launch_bounds__(1024) mid_sort_kernel(uint64_t* keys, uint32_t* vals, uint64_t* keys_alt,
                                                        uint32_t* vals_alt, int n, int passes) {
  extern __shared__ __align__(16) uint32_t ms_smem[];
  uint32_t* cnt = ms_smem;                          // [32][kMidDigits]
  uint32_t* wsum = ms_smem + 32 * kMidDigits;       // [32]
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int chunk = (n + 31) / 32;
  const int b0 = min(n, warp * chunk), b1 = min(n, b0 + chunk);
  const unsigned lt = (1u << lane) - 1u;
  uint64_t* ks = keys;
  uint32_t* vs = vals;
  uint64_t* kd = keys_alt;
  uint32_t* vd = vals_alt;
  uint32_t* my = cnt + warp * kMidDigits;
  for (int p = 0; p < passes; ++p) {
    const int shift = kMidDigitBits * p;
    for (int d = lane; d < kMidDigits; d += 32) my[d] = 0;
    __syncwarp();
    for (int i = b0 + lane; i < b1; i += 32)
      atomicAdd(&my[(uint32_t)(ks[i] >> shift) & (kMidDigits - 1)], 1u);
    __syncthreads();
    // Digit totals, then their exclusive scan (thread d holds digit d).
    constexpr int kDigitWarps = kMidDigits / 32;
    const int d = threadIdx.x;
    uint32_t tot = 0, incl = 0;
    if (warp < kDigitWarps) {
      for (int w = 0; w < 32; ++w) tot += cnt[w * kMidDigits + d];
      incl = tot;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
      }
      if (lane == 31) wsum[warp] = incl;
    }
    __syncthreads();
    if (warp == 0) {
      const uint32_t x = lane < kDigitWarps ? wsum[lane] : 0u;
      uint32_t xi = x;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, xi, o);
        if (lane >= o) xi += y;
      }
      if (lane < kDigitWarps) wsum[lane] = xi - x;
    }
    __syncthreads();
    if (warp < kDigitWarps) {
      uint32_t run = wsum[warp] + incl - tot;
      for (int w = 0; w < 32; ++w) {
        const uint32_t c = cnt[w * kMidDigits + d];
        cnt[w * kMidDigits + d] = run;
        run += c;
      }
    }
    __syncthreads();
    uint64_t kn = 0;
    uint32_t vn = 0;
    if (b0 + lane < b1) {
      kn = ks[b0 + lane];
      vn = vs[b0 + lane];
    }
    for (int base = b0; base < b1; base += 32) {
      const int i = base + lane;
      const bool valid = i < b1;
      const uint64_t k = kn;
      const uint32_t v = vn;
      if (i + 32 < b1) {
        kn = ks[i + 32];
        vn = vs[i + 32];
      }
      const uint32_t digit = valid ? ((uint32_t)(k >> shift) & (kMidDigits - 1)) : 0xffffffffu;
      const unsigned peers = __match_any_sync(0xffffffffu, digit);
      if (valid) {
        const uint32_t pos = my[digit] + __popc(peers & lt);
        kd[pos] = k;
        vd[pos] = v;
      }
      __syncwarp();
      if (valid && (peers & lt) == 0) my[digit] += __popc(peers);
      __syncwarp();
    }
    __syncthreads();
    uint64_t* kt = ks;
    ks = kd;
    kd = kt;
    uint32_t* vt = vs;
    vs = vd;
    vd = vt;
  }
  if (ks != keys) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      keys[i] = ks[i];
      vals[i] = vs[i];
    }
  }
}

int radix_sort_u64(visacd_ctx* ctx, uint64_t* keys, uint32_t* vals, uint64_t* keys_alt,
                   uint32_t* vals_alt, int32_t n, int key_bits) {
  if (n <= 1) return VISACD_OK;
  if (n <= kSmallSort) {
    static std::atomic<bool> attr_set[64];
    if (ctx->device < 0 || ctx->device >= 64 || !attr_set[ctx->device].load()) {
      VCUDA(cudaFuncSetAttribute(small_sort_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kSmallSortSmem));
      if (ctx->device >= 0 && ctx->device < 64) attr_set[ctx->device].store(true);
    }
    const uint64_t mask = key_bits >= 64 ? ~0ull : ((1ull << key_bits) - 1);
    VLAUNCH(ctx, kKSortScatter, 1, 1024, kSmallSortSmem, small_sort_kernel, keys, vals, n, mask);
    return VISACD_OK;
  }
  if (n <= kMidSort) {
    static std::atomic<bool> mid_attr_set[64];
    if (ctx->device < 0 || ctx->device >= 64 || !mid_attr_set[ctx->device].load()) {
      VCUDA(cudaFuncSetAttribute(mid_sort_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kMidSortSmem));
      if (ctx->device >= 0 && ctx->device < 64) mid_attr_set[ctx->device].store(true);
    }
    VLAUNCH(ctx, kKSortScatter, 1, 1024, kMidSortSmem, mid_sort_kernel, keys, vals, keys_alt, vals_alt, n,
            (key_bits + kMidDigitBits - 1) / kMidDigitBits);
    return VISACD_OK;
  }
  int nblocks = (int)((n + kSortTile - 1) / kSortTile);
  size_t hist_n = (size_t)256 * nblocks;
  VTRY(ensure_slot(ctx, kSlotSortHist, hist_n * sizeof(uint32_t) + (hist_n + 1) * sizeof(uint64_t) + 16));
  uint32_t* hist = slot<uint32_t>(ctx, kSlotSortHist);
  uint64_t* offs = reinterpret_cast<uint64_t*>(
      (reinterpret_cast<uintptr_t>(hist + hist_n) + 15) & ~uintptr_t(15));
  uint64_t *ksrc = keys, *kdst = keys_alt;
  uint32_t *vsrc = vals, *vdst = vals_alt;
  int passes = (key_bits + 7) / 8;
  for (int p = 0; p < passes; ++p) {
    int shift = 8 * p;
    VLAUNCH(ctx, kKSortHist, nblocks, kSortThreads, 0, radix_hist_kernel, ksrc, n, shift, hist,
            nblocks);
    VTRY(exclusive_scan_u32_to_u64(ctx, hist, offs, (int64_t)hist_n));
    VLAUNCH(ctx, kKSortScatter, nblocks, kSortThreads, 0, radix_scatter_kernel, ksrc, vsrc, n,
            shift, offs, nblocks, kdst, vdst);
    uint64_t* kt = ksrc; ksrc = kdst; kdst = kt;
    uint32_t* vt = vsrc; vsrc = vdst; vdst = vt;
  }
  if (ksrc != keys) {
    VCUDA(cudaMemcpyAsync(keys, ksrc, (size_t)n * sizeof(uint64_t), cudaMemcpyDeviceToDevice,
                          ctx->stream));
    VCUDA(cudaMemcpyAsync(vals, vsrc, (size_t)n * sizeof(uint32_t), cudaMemcpyDeviceToDevice,
                          ctx->stream));
  }
  return VISACD_OK;
}

}  // namespace vgpu

// ---------------------------------------------------------------------------
// C ABI: errors and context.
// ---------------------------------------------------------------------------
using namespace vgpu;

extern "C" const char* visacd_last_error(void) { return g_err; }
extern "C" int visacd_abi_version(void) { return VISACD_ABI_VERSION; }

extern "C" int visacd_ctx_create(int device, void* cuda_stream, visacd_ctx** out) {
  VCHECK(out != nullptr, VISACD_ERR_INVALID_ARG, "visacd_ctx_create: out is NULL");
  *out = nullptr;
  int ndev = 0;
  VCUDA(cudaGetDeviceCount(&ndev));
  VCHECK(device >= 0 && device < ndev, VISACD_ERR_INVALID_ARG,
         "visacd_ctx_create: device %d out of range (%d devices)", device, ndev);
  VCUDA(cudaSetDevice(device));
  visacd_ctx* ctx = new visacd_ctx();
  ctx->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) {
    delete ctx;
    set_error("device %d: %s", device, cudaGetErrorString(e));
    return VISACD_ERR_CUDA;
  }
  if (cuda_stream) {
    ctx->stream = (cudaStream_t)cuda_stream;
  } else {
    e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      delete ctx;
      set_error("cudaStreamCreate: %s", cudaGetErrorString(e));
      return VISACD_ERR_CUDA;
    }
    ctx->own_stream = true;
  }
  e = cudaEventCreateWithFlags(&ctx->wait_event, cudaEventBlockingSync | cudaEventDisableTiming);
  if (e != cudaSuccess) {
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    set_error("cudaEventCreate: %s", cudaGetErrorString(e));
    return VISACD_ERR_CUDA;
  }
  e = cudaMalloc(&ctx->d_status, 256);
  if (e == cudaSuccess) e = cudaMemset(ctx->d_status, 0, 256);
  if (e != cudaSuccess) {
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    cudaEventDestroy(ctx->wait_event);
    delete ctx;
    set_error("status word allocation: %s", cudaGetErrorString(e));
    return VISACD_ERR_NO_MEMORY;
  }
  ctx->times.resize(kKCount);
  for (int i = 0; i < kKCount; ++i) ctx->times[i].name = kernel_name(i);
  for (int i = 0; i < kSlotCount; ++i) ctx->buf[i].stream = ctx->stream;
  if (keep_pool_cached(device) != VISACD_OK) {
    visacd_ctx_destroy(ctx);
    return VISACD_ERR_CUDA;
  }
  *out = ctx;
  return VISACD_OK;
}

extern "C" int visacd_ctx_destroy(visacd_ctx* ctx) {
  if (!ctx) return VISACD_OK;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  // BVHs still alive lose their device memory with their context.
  for (visacd_bvh* b : ctx->bvhs) bvh_detach(b);
  ctx->bvhs.clear();
  if (ctx->grid_tex) cudaDestroyTextureObject(ctx->grid_tex);
  if (ctx->grid_arr) cudaFreeArray(ctx->grid_arr);
  ctx->grid_tex = 0;
  ctx->grid_arr = nullptr;
  // So do proposers: destroying one afterwards only frees its host side.
  for (visacd_lp* lp : ctx->lps) lp_detach(lp);
  ctx->lps.clear();
  for (int i = 0; i < kSlotCount; ++i) release(ctx->buf[i]);
  cudaStreamSynchronize(ctx->stream);
  if (ctx->d_status) cudaFree(ctx->d_status);
  if (ctx->h_pinned) cudaFreeHost(ctx->h_pinned);
  if (ctx->h_upload) cudaFreeHost(ctx->h_upload);
  for (auto& p : ctx->pending) {
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  for (auto e : ctx->event_pool) cudaEventDestroy(e);
  if (ctx->wait_event) cudaEventDestroy(ctx->wait_event);
  if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return VISACD_OK;
}

extern "C" int visacd_ctx_synchronize(visacd_ctx* ctx) {
  VCHECK(ctx, VISACD_ERR_INVALID_ARG, "null context");
  VCUDA(stream_wait(ctx));
  return VISACD_OK;
}

extern "C" int visacd_ctx_set_blocking_wait(visacd_ctx* ctx, int enable) {
  VCHECK(ctx, VISACD_ERR_INVALID_ARG, "null context");
  ctx->blocking_wait = enable != 0;
  return VISACD_OK;
}

extern "C" int visacd_ctx_set_timing(visacd_ctx* ctx, int enable) {
  VCHECK(ctx, VISACD_ERR_INVALID_ARG, "null context");
  ctx->timing = enable != 0;
  return VISACD_OK;
}

static int drain_pending(visacd_ctx* ctx) {
  if (ctx->pending.empty()) return VISACD_OK;
  VCUDA(stream_wait(ctx));
  for (auto& p : ctx->pending) {
    float ms = 0.f;
    VCUDA(cudaEventElapsedTime(&ms, p.a, p.b));
    ctx->times[p.kernel].ms += ms;
    ctx->times[p.kernel].launches += 1;
    ctx->event_pool.push_back(p.a);
    ctx->event_pool.push_back(p.b);
  }
  ctx->pending.clear();
  return VISACD_OK;
}

extern "C" int visacd_ctx_reset_times(visacd_ctx* ctx) {
  VCHECK(ctx, VISACD_ERR_INVALID_ARG, "null context");
  VTRY(drain_pending(ctx));
  for (auto& t : ctx->times) {
    t.ms = 0.0;
    t.launches = 0;
  }
  return VISACD_OK;
}

extern "C" int visacd_ctx_kernel_times(visacd_ctx* ctx, const char** names, double* total_ms,
                                       int64_t* launches, int capacity, int* n_kernels) {
  VCHECK(ctx, VISACD_ERR_INVALID_ARG, "null context");
  VTRY(drain_pending(ctx));
  int n = 0;
  for (auto& t : ctx->times) {
    if (t.launches == 0) continue;
    if (n < capacity) {
      if (names) names[n] = t.name;
      if (total_ms) total_ms[n] = t.ms;
      if (launches) launches[n] = t.launches;
    }
    ++n;
  }
  if (n_kernels) *n_kernels = n;
  return VISACD_OK;
}

extern "C" int64_t visacd_ctx_launch_count(const visacd_ctx* ctx) { return ctx ? ctx->launches : 0; }
extern "C" int visacd_ctx_sm_count(const visacd_ctx* ctx) { return ctx ? ctx->sm_count : 0; }

extern "C" int visacd_radix_sort_pairs(visacd_ctx* ctx, uint64_t* keys, uint32_t* vals, int32_t n, int key_bits) {
  VCHECK(ctx && (n == 0 || (keys && vals)), VISACD_ERR_INVALID_ARG, "radix_sort_pairs: null argument");
  VCHECK(n >= 0 && key_bits >= 1 && key_bits <= 64, VISACD_ERR_INVALID_ARG, "radix_sort_pairs: bad size");
  if (key_bits < 64)
    for (int32_t i = 0; i < n; ++i)
      VCHECK(!(keys[i] >> key_bits), VISACD_ERR_INVALID_ARG, "radix_sort_pairs: key %d has bits above key_bits",
             (int)i);
  if (n <= 1) return VISACD_OK;
  VCUDA(cudaSetDevice(ctx->device));
  uint64_t* d = nullptr;
  VCUDA(cudaMallocAsync((void**)&d, (size_t)n * 24, ctx->stream));
  uint64_t *k0 = d, *k1 = d + n;
  uint32_t *v0 = reinterpret_cast<uint32_t*>(d + 2 * (size_t)n), *v1 = v0 + n;
  cudaError_t e = cudaMemcpyAsync(k0, keys, (size_t)n * 8, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(v0, vals, (size_t)n * 4, cudaMemcpyHostToDevice, ctx->stream);
  int rc = e == cudaSuccess ? radix_sort_u64(ctx, k0, v0, k1, v1, n, key_bits) : VISACD_ERR_CUDA;
  if (rc == VISACD_OK) {
    e = cudaMemcpyAsync(keys, k0, (size_t)n * 8, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(vals, v0, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream);
    if (e != cudaSuccess) rc = VISACD_ERR_CUDA;
  }
  cudaFreeAsync(d, ctx->stream);
  const cudaError_t w = cudaStreamSynchronize(ctx->stream);
  if (rc == VISACD_OK && (e != cudaSuccess || w != cudaSuccess)) {
    set_error("radix_sort_pairs: %s", cudaGetErrorString(e != cudaSuccess ? e : w));
    rc = VISACD_ERR_CUDA;
  }
  return rc;
}

extern "C" int visacd_set_blocking_sync(int device, int blocking) {
  VCUDA(cudaSetDevice(device));
  VCUDA(cudaSetDeviceFlags(blocking ? cudaDeviceScheduleBlockingSync : cudaDeviceScheduleAuto));
  return VISACD_OK;
}

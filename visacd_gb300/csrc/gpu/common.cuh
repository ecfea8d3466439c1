// Shared plumbing of the sm_103a library: error reporting, the context object,
// grow-only device buffers and per-kernel CUDA-event timing.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <unordered_map>
#include <vector>

#include "visacd_gpu.h"

namespace vgpu {

void set_error(const char* fmt, ...);

#define VCUDA(call)                                                                     \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess) {                                                            \
      vgpu::set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                      __LINE__);                                                        \
      return e_ == cudaErrorMemoryAllocation ? VISACD_ERR_NO_MEMORY : VISACD_ERR_CUDA;  \
    }                                                                                   \
  } while (0)

#define VCHECK(cond, code, ...)   \
  do {                            \
    if (!(cond)) {                \
      vgpu::set_error(__VA_ARGS__); \
      return (code);              \
    }                             \
  } while (0)

#define VTRY(expr)          \
  do {                      \
    int rc_ = (expr);       \
    if (rc_ != VISACD_OK) { \
      return rc_;           \
    }                       \
  } while (0)

// Device status word bits, set by kernels whose bounded loops ran out.
enum : uint32_t {
  kStatusTraversalOverrun = 1u << 0,
  kStatusStackOverflow = 1u << 1,
  kStatusRecheckOverflow = 1u << 2,
  kStatusMbarrierTimeout = 1u << 3,
  kStatusWorkOverrun = 1u << 4,
};

struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
  cudaStream_t stream = nullptr;  // owner's stream: allocations are stream-ordered on it
};

// Grow-only device buffer: reallocates (without preserving contents) only when
// the request exceeds the current capacity; capacities round up to 1.25x.
// Buffers with a stream use the stream-ordered allocator (cudaMallocAsync /
// cudaFreeAsync from the device's default pool, which keeps freed memory
// cached), so growing one context's buffer never waits for other streams.
int ensure(DevBuf& b, size_t bytes);
void release(DevBuf& b);
// Keep memory freed to the device's default pool cached in the pool (release
// threshold = unlimited) for the life of the process. Idempotent.
int keep_pool_cached(int device);

struct KernelTime {
  const char* name;
  double ms = 0.0;
  int64_t launches = 0;
};

}  // namespace vgpu

// Named buffer slots owned by a context.
enum CtxSlot {
  kSlotPoints = 0,
  kSlotMask,
  kSlotPlanes,
  kSlotEdgesIn,
  kSlotEdgePack,
  kSlotScoreQ,
  kSlotScores,
  kSlotRecheck,
  kSlotPointStats,
  kSlotVisKeys,
  kSlotVisKeysAlt,
  kSlotVisPerm,
  kSlotVisPermAlt,
  kSlotVisRank,
  kSlotBitset,
  kSlotWordCounts,
  kSlotWordOffsets,
  kSlotEdgesOut,
  kSlotScanScratch,
  kSlotSortHist,
  kSlotCounters,
  kSlotBuildVerts,
  kSlotBuildTris,
  kSlotTmpVerts,
  kSlotTmpTris,
  kSlotVisRowTiles,
  kSlotClip,
  kSlotHausdorff,
  kSlotSdf,
  kSlotSdfOut,
  kSlotSdfTris,
  kSlotHull,
  kSlotSegTri,
  kSlotCandidates,
  kSlotCandLinks,
  kSlotVisMulti,
  kSlotLearned,
  kSlotFreeGrid,
  kSlotVisCleared,
  kSlotConvexHull,
  kSlotCount
};

struct visacd_ctx {
  int device = 0;
  int sm_count = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  bool blocking_wait = false;        // host waits block (no spinning): see stream_wait
  cudaEvent_t wait_event = nullptr;  // blocking-sync event for those waits
  vgpu::DevBuf buf[kSlotCount];
  uint32_t* d_status = nullptr;      // device status word
  void* h_pinned = nullptr;          // small pinned staging area
  size_t h_pinned_cap = 0;
  void* h_upload = nullptr;          // pinned upload buffer (Stager)
  size_t h_upload_cap = 0;
  int64_t launches = 0;
  int64_t last_n_edges = 0;
  bool timing = false;
  int vis_variant_override = -1;                  // forced launch shape, -1 = tuned/default
  std::unordered_map<uint32_t, int> vis_tuned;    // shape class -> autotuned variant
  int score_k_override = 0;                       // forced planes per scoring thread, 0 = tuned/default
  std::unordered_map<uint32_t, int> score_tuned;  // scoring shape class -> autotuned planes per thread
  visacd_clip_result clip_out{};                  // last clip result (device-resident)
  std::vector<visacd_bvh*> bvhs;                  // live BVHs built on this context
  std::vector<visacd_lp*> lps;                    // live proposers made on this context
  // The last free-space grid's 3D array and texture, kept when its BVH goes
  // so that the next grid of the same size reuses them (no allocation and no
  // wait for the walks still queued on this context's stream).
  cudaArray_t grid_arr = nullptr;
  cudaTextureObject_t grid_tex = 0;
  int grid_dims[3] = {0, 0, 0};
  bool vis_trace = true;                          // free-space walks before the cage BVH
  int64_t last_vis_certified = 0, last_vis_trace_steps = 0;  // of the last visibility call
  int clip_nv = 0;
  int32_t sdf_nv = 0, sdf_nt = 0;                 // last SDF remesh result (device-resident)
  void* clip_ptrs[7] = {nullptr};
  // Per-kernel timing: events recorded around each launch when timing is on.
  struct Pending {
    int kernel;
    cudaEvent_t a, b;
  };
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> event_pool;
  std::vector<vgpu::KernelTime> times;
};

namespace vgpu {

// Kernel ids for timing (index into a static name table).
enum KernelId {
  kKPointStats = 0,
  kKPackEdges,
  kKScore,
  kKScoreRecheck,
  kKScoreFinish,
  kKTriPrep,
  kKMorton,
  kKSortHist,
  kKSortScan,
  kKSortScatter,
  kKKarras,
  kKFit,
  kKNodeLayout,
  kKVisPrep,
  kKVisibility,
  kKBitPopc,
  kKScanBlocks,
  kKScanTop,
  kKScanAdd,
  kKBitEmit,
  kKClip,
  kKClipResolve,
  kKHausdorff,
  kKHausdorffBound,
  kKHausdorffQuery,
  kKHausdorffHead,
  kKLpFeatures,
  kKLpGemm,
  kKLpPool,
  kKLpLoss,
  kKLpAdam,
  kKLpMisc,
  kKSdf,
  kKSdfDist,
  kKSdfCross,
  kKHullDist,
  kKSegTri,
  kKCandidates,
  kKLpRefine,
  kKLpSplit,
  kKGridNear,
  kKGridEdt,
  kKGridFinal,
  kKVisWalk,
  kKConvexHull,
  kKMisc,
  kKCount
};
const char* kernel_name(int id);

// Launch bookkeeping: call before and after each launch on ctx->stream.
void timing_begin(visacd_ctx* ctx, int kernel, cudaEvent_t* a);
int timing_end(visacd_ctx* ctx, int kernel, cudaEvent_t a);

// Check cudaGetLastError after a launch and update the launch counter.
int after_launch(visacd_ctx* ctx, const char* what);

// Read back and clear the device status word; returns VISACD_ERR_DEVICE with a
// message when any bit is set. Synchronizes the context stream.
int check_status(visacd_ctx* ctx, const char* what);
// The same for a status word the caller already read back (with its own
// results, in one wait): clears the device word when it is set.
int status_result(visacd_ctx* ctx, uint32_t status, const char* what);

// Pinned host staging of at least `bytes`.
int pinned(visacd_ctx* ctx, size_t bytes, void** out);

// Host-to-device uploads of one call through the context's pinned upload
// buffer: a host memcpy into pinned memory, then an asynchronous DMA from it,
// so contexts driven by several host threads do not contend on the driver's
// pageable-copy staging. reserve(total) first waits for the context stream
// (the previous call's DMAs may still read the buffer) and grows it; put()
// places each array at the next 64-byte boundary.
class Stager {
 public:
  explicit Stager(visacd_ctx* ctx) : ctx_(ctx) {}
  int reserve(size_t total_bytes, int arrays);
  int put(void* dst, const void* src, size_t bytes);
  // The pinned buffer itself (after reserve): filled in the device layout and
  // sent with one copy.
  char* host() { return static_cast<char*>(ctx_->h_upload); }
  int copy(void* dst, size_t bytes);

 private:
  visacd_ctx* ctx_;
  size_t used_ = 0, cap_ = 0;
};

template <class T>
inline T* slot(visacd_ctx* ctx, int s) {
  return reinterpret_cast<T*>(ctx->buf[s].p);
}
inline int ensure_slot(visacd_ctx* ctx, int s, size_t bytes) { return ensure(ctx->buf[s], bytes); }

// True when every p[0..n) lies in [0, bound) (host side, branch-free so the
// argument checks of the entry points stay cheap on large inputs).
inline bool indices_in_range(const int32_t* p, int64_t n, int64_t bound) {
  if (n <= 0) return true;
  if (bound <= 0) return false;
  const uint32_t b = bound > INT32_MAX ? 0xffffffffu : (uint32_t)bound;
  uint32_t bad = 0;
  for (int64_t k = 0; k < n; ++k) bad |= (uint32_t)((uint32_t)p[k] >= b);
  return bad == 0;
}

// Wait for the context's stream. By default the host thread spins (lowest
// latency for one caller); with blocking_wait it sleeps on a blocking-sync
// event, which leaves the cores to the other host threads when many
// contexts share the machine (process_batch workers).
inline cudaError_t stream_wait(visacd_ctx* ctx) {
  if (ctx->blocking_wait && ctx->wait_event) {
    cudaError_t e = cudaEventRecord(ctx->wait_event, ctx->stream);
    return e != cudaSuccess ? e : cudaEventSynchronize(ctx->wait_event);
  }
  return cudaStreamSynchronize(ctx->stream);
}

inline unsigned grid_for(int64_t n, int block, int64_t cap) {
  int64_t g = (n + block - 1) / block;
  if (g < 1) g = 1;
  if (g > cap) g = cap;
  return (unsigned)g;
}

// Bits per axis of the Morton codes that order n primitives: about 4 bits
// finer than the mean spacing (the orders only shape the BVHs and the pair
// tiles, never a result), at least 10 and at most 21, so the radix sort runs
// ceil(3 bits / 8) passes (4 up to about 2^21 primitives).
inline int morton_bits(int64_t n) {
  int len = 0;
  while (len < 62 && (int64_t(1) << len) <= n) ++len;
  const int b = (len + 2) / 3 + 4;
  return b < 10 ? 10 : (b > 21 ? 21 : b);
}

// Exclusive scan of n uint32 counts into uint64 offsets (device), total also
// written to offsets[n]. Uses ctx scan scratch.
int exclusive_scan_u32_to_u64(visacd_ctx* ctx, const uint32_t* in, uint64_t* out, int64_t n);

// Stable LSD radix sort of (key, value) pairs on the device. key_bits selects
// how many low bits of the key take part (multiple of 8). Results land in
// keys/vals (the alt buffers are scratch of the same size).
int radix_sort_u64(visacd_ctx* ctx, uint64_t* keys, uint32_t* vals, uint64_t* keys_alt,
                   uint32_t* vals_alt, int32_t n, int key_bits);

// Plane scoring on device pointers without a host wait (score.cu): the call's
// status word and FP64 queue demand are left in device memory.
int score_planes_device_async(visacd_ctx* ctx, const float* d_planes, int32_t P, const float* d_pts,
                              int32_t N, const uint32_t* d_edges, int64_t E, double* d_scores,
                              unsigned rcap, const unsigned** d_status, const unsigned** d_recheck_count);
unsigned score_recheck_capacity(int32_t P, int64_t E);

// The learned proposer on a part already on the device (learned.cu): f32
// points, edge pairs, the part's frame (centre, half extent). Writes its 16
// planes, FP64 in the input frame, to d_planes (16 x 4 doubles) without a
// host wait.
visacd_ctx* lp_context(visacd_lp* lp);
// Releases a proposer's device memory and unbinds it from its context (on
// context destruction; the host side stays until visacd_lp_destroy).
void lp_detach(visacd_lp* lp);
int lp_propose_device(visacd_lp* lp, const float* d_pts, int32_t n, const uint32_t* d_edges, int64_t E,
                      const float* center, float scale, double* d_planes);

}  // namespace vgpu

// Launch helper: times the launch when ctx timing is on, checks the launch.
#define VLAUNCH(ctx, kid, grid, block, smem, kernel, ...)                 \
  do {                                                                    \
    cudaEvent_t ev_a_ = nullptr;                                          \
    vgpu::timing_begin((ctx), (kid), &ev_a_);                             \
    kernel<<<(grid), (block), (smem), (ctx)->stream>>>(__VA_ARGS__);      \
    VTRY(vgpu::after_launch((ctx), #kernel));                             \
    VTRY(vgpu::timing_end((ctx), (kid), ev_a_));                          \
  } while (0)

// Plane scoring: score[p] = sum of |e| over visibility edges e that plane p cuts
// strictly (both endpoints farther than eps = 1e-6f on opposite sides).
//
// Reference semantics: lib/cuda/plane_intersections.cu:7-67 (one thread per
// (plane, edge), FP32 side test with eps, float atomicAdd of the FP32 length).
//
// GB300 design:
//  * pack_edges gathers each edge's two endpoints once into a 32-byte record
//    {x1,x2,y1,y2 | z1,z2,q,0} so the hot loop reads coalesced, pre-paired
//    operands for packed FP32x2 FMAs. q is the FP32 edge length (IEEE ops, no
//    contraction) quantized to 2^qexp, qexp chosen from the largest |coordinate|
//    so that q < 2^24 and a 256-edge block sums in 32 bits.
//  * score_planes keeps 1..8 planes per thread in registers (coefficients
//    duplicated into f32x2 pairs) and streams 512-edge blocks into shared memory
//    with cp.async.bulk (TMA bulk copy) + mbarrier, double-buffered (256-edge blocks). Every
//    thread of the CTA reads the same edge (shared-memory broadcast).
//  * The FP32 plane value carries an a-priori rounding bound B_p (Higham,
//    3 nested FMAs: |err| <= 3u * (|a|X + |b|Y + |c|Z + |d|)). Per (plane, edge
//    block) the kernel accumulates the certain crossings (both sides beyond
//    eps + B) and flags the block when some pair comes within the band
//    [eps - B, eps + B] (score_edge_block); a flagged block is queued and
//    score_recheck re-decides its band pairs in FP64 — the same FP64
//    evaluation the oracle uses — so classification equals the FP64 oracle's.
//  * Sums are integers (order independent), so scores are deterministic.
#include <cstring>
#include <vector>

#include "score_device.cuh"

namespace vgpu {

template <int K>
__global__ void __launch_bounds__(kScoreThreads, (K <= 4 ? 3 : 2))
    score_planes_kernel(const float4* __restrict__ planes, int32_t P,
                        const EdgeRec* __restrict__ recs, int64_t E, int64_t blocks_per_cta,
                        const unsigned* __restrict__ stats,
                        unsigned long long* __restrict__ score_q, uint2* __restrict__ recheck,
                        unsigned* __restrict__ recheck_count, unsigned recheck_cap,
                        unsigned* __restrict__ status) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  EdgeRec* buf = reinterpret_cast<EdgeRec*>(smem_raw);  // 2 x kEdgeBlock records
  unsigned long long* tot =
      reinterpret_cast<unsigned long long*>(smem_raw + 2 * kEdgeBlock * sizeof(EdgeRec));
  __shared__ __align__(8) uint64_t bars[2];

  const int tid = threadIdx.x;
  const int64_t n_blocks_total = (E + kEdgeBlock - 1) / kEdgeBlock;
  const int64_t b_begin = (int64_t)blockIdx.x * blocks_per_cta;
  int64_t b_end = b_begin + blocks_per_cta;
  if (b_end > n_blocks_total) b_end = n_blocks_total;
  const int nb = (int)(b_end > b_begin ? b_end - b_begin : 0);
  const int plane_base = blockIdx.y * (kScoreThreads * K);

  PlaneAcc pa[K];
  uint32_t acc[K], dmin[K];
#pragma unroll
  for (int k = 0; k < K; ++k) {
    int p = plane_base + k * kScoreThreads + tid;
    float4 pl = p < P ? planes[p]
                      : make_float4(__int_as_float(0x7fc00000), __int_as_float(0x7fc00000),
                                    __int_as_float(0x7fc00000), __int_as_float(0x7fc00000));
    pa[k] = plane_acc(pl, stats);
    acc[k] = 0u;
    dmin[k] = 0xffffffffu;
    tot[k * kScoreThreads + tid] = 0ull;
  }
  if (nb == 0) return;

  if (tid == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (tid == 0) {
    int64_t e0 = b_begin * kEdgeBlock;
    int64_t cnt = E - e0 < kEdgeBlock ? E - e0 : kEdgeBlock;
    bulk_load(buf, recs + e0, (unsigned)(cnt * sizeof(EdgeRec)), &bars[0]);
  }

  bool failed = false;
  for (int it = 0; it < nb; ++it) {
    const int cur = it & 1;
    if (tid == 0 && it + 1 < nb) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      int64_t e0 = (b_begin + it + 1) * kEdgeBlock;
      int64_t cnt = E - e0 < kEdgeBlock ? E - e0 : kEdgeBlock;
      bulk_load(buf + (cur ^ 1) * kEdgeBlock, recs + e0, (unsigned)(cnt * sizeof(EdgeRec)),
                &bars[cur ^ 1]);
    }
    bool ok = mbar_wait(&bars[cur], (unsigned)((it >> 1) & 1));
    if (__syncthreads_or(!ok)) {
      failed = true;
      break;
    }
    const int64_t e0 = (b_begin + it) * kEdgeBlock;
    const int cnt = (int)(E - e0 < kEdgeBlock ? E - e0 : kEdgeBlock);
    const ulonglong2* s = reinterpret_cast<const ulonglong2*>(buf + cur * kEdgeBlock);
    score_edge_block<K>(s, cnt, pa, acc, dmin);
    // Close the block: certain sums go to the total; blocks that may hold band
    // pairs are queued for the FP64 re-decision and contribute nothing here.
#pragma unroll
    for (int k = 0; k < K; ++k) {
      int p = plane_base + k * kScoreThreads + tid;
      if (dmin[k] > pa[k].wbits) {
        tot[k * kScoreThreads + tid] += acc[k];
      } else if (p < P) {
        unsigned idx = atomicAdd(recheck_count, 1u);
        if (idx < recheck_cap) {
          recheck[idx] = make_uint2((unsigned)p, (unsigned)(b_begin + it));
        } else {
          atomicOr(status, kStatusRecheckOverflow);
        }
      }
      acc[k] = 0u;
      dmin[k] = 0xffffffffu;
    }
    __syncthreads();
  }
  if (failed) {
    if (tid == 0) atomicOr(status, kStatusMbarrierTimeout);
    return;
  }
#pragma unroll
  for (int k = 0; k < K; ++k) {
    int p = plane_base + k * kScoreThreads + tid;
    unsigned long long t = tot[k * kScoreThreads + tid];
    if (p < P && t) atomicAdd(&score_q[p], t);
  }
}

// One warp per queued (plane, edge block): certain pairs are taken from the
// same FP32 evaluation as the main kernel, band pairs are decided in FP64.
__global__ void score_recheck_kernel(const float4* __restrict__ planes,
                                     const EdgeRec* __restrict__ recs, int64_t E,
                                     const unsigned* __restrict__ stats,
                                     const uint2* __restrict__ recheck,
                                     const unsigned* __restrict__ recheck_count,
                                     unsigned recheck_cap,
                                     unsigned long long* __restrict__ score_q) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  unsigned n = *recheck_count;
  if (n > recheck_cap) n = recheck_cap;
  const double eps = (double)kSideEps;
  for (int64_t r = warp; r < n; r += nwarps) {
    uint2 rec = recheck[r];
    float4 pl = planes[rec.x];
    float nlo, nhi;
    plane_thresholds(pl, stats, nlo, nhi);
    int64_t e0 = (int64_t)rec.y * kEdgeBlock;
    int64_t e1 = e0 + kEdgeBlock < E ? e0 + kEdgeBlock : E;
    unsigned long long sum = 0;
    for (int64_t e = e0 + lane; e < e1; e += 32) {
      EdgeRec er = recs[e];
      float v1 = fmaf(pl.x, er.x1, fmaf(pl.y, er.y1, fmaf(pl.z, er.z1, pl.w)));
      float v2 = fmaf(pl.x, er.x2, fmaf(pl.y, er.y2, fmaf(pl.z, er.z2, pl.w)));
      float sv = fmaxf(fminf(v1, v2), -fmaxf(v1, v2));
      if (sv < nhi) {
        sum += er.q;
      } else if (sv < nlo) {
        double w1 = side_value64(pl, er.x1, er.y1, er.z1);
        double w2 = side_value64(pl, er.x2, er.y2, er.z2);
        bool cross = (w1 > eps && w2 < -eps) || (w1 < -eps && w2 > eps);
        if (cross) sum += er.q;
      }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if (lane == 0 && sum) atomicAdd(&score_q[rec.x], sum);
  }
}

// Scores in float64 (exact: integer sum times a power of two) and the first
// index of the maximum. When the call's status word says that some work was
// lost (a bulk-copy wait that timed out, or a full FP64 re-decision queue),
// every score is NaN and the arg-max is -2, so a caller that reads only the
// device outputs still sees the failure.
__global__ void score_finish_kernel(const unsigned long long* __restrict__ score_q, int32_t P,
                                    const unsigned* __restrict__ stats,
                                    const unsigned* __restrict__ status, double* __restrict__ out,
                                    float* __restrict__ out_f32, int* __restrict__ argmax) {
  unsigned cmax = max(stats[0], max(stats[1], stats[2]));
  int qexp = quantum_exp_from_cmax_bits(cmax);
  const bool lost = (*status & (kStatusMbarrierTimeout | kStatusRecheckOverflow)) != 0u;
  unsigned long long best = 0;
  int best_i = P > 0 ? 0 : -1;
  for (int p = threadIdx.x; p < P; p += blockDim.x) {
    unsigned long long v = score_q[p];
    double s = lost ? __longlong_as_double(0x7ff8000000000000ll) : ldexp((double)v, qexp);
    if (out) out[p] = s;
    if (out_f32) out_f32[p] = (float)s;
    if (v > best || (v == best && p < best_i)) {
      best = v;
      best_i = p;
    }
  }
  __shared__ unsigned long long sv[1024];
  __shared__ int si[1024];
  sv[threadIdx.x] = best;
  si[threadIdx.x] = best_i;
  __syncthreads();
  for (int o = blockDim.x / 2; o; o >>= 1) {
    if ((int)threadIdx.x < o) {
      unsigned long long v2 = sv[threadIdx.x + o];
      int i2 = si[threadIdx.x + o];
      if (v2 > sv[threadIdx.x] || (v2 == sv[threadIdx.x] && i2 >= 0 && i2 < si[threadIdx.x])) {
        sv[threadIdx.x] = v2;
        si[threadIdx.x] = i2;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    argmax[0] = lost ? -2 : si[0];
    argmax[1] = qexp;
  }
}

// Device-side workspace layout inside kSlotCounters.
struct ScoreCounters {
  unsigned stats[4];                 // max |x|, |y|, |z| (float bits)
  unsigned recheck_count;
  unsigned status;                   // this call's kStatus* bits
  unsigned pad0[2];
  unsigned long long skipped;
  int argmax[2];                     // argmax, qexp
};

// Shape class of a scoring call: log2 buckets of P and E.
static uint32_t score_shape_class(int32_t P, int64_t E) {
  auto lg = [](int64_t x) { int r = 0; while (x > 1) { x >>= 1; ++r; } return r; };
  return (uint32_t)lg(P) | ((uint32_t)lg(E) << 8);
}

static int planes_per_thread(int32_t P);

// Planes per thread of a call: forced, autotuned for its shape class, or the
// default rule.
static int choose_score_k(visacd_ctx* ctx, int32_t P, int64_t E) {
  if (ctx->score_k_override) return ctx->score_k_override;
  auto it = ctx->score_tuned.find(score_shape_class(P, E));
  if (it != ctx->score_tuned.end()) return it->second;
  return planes_per_thread(P);
}

static int planes_per_thread(int32_t P) {
  if (P > 4 * kScoreThreads * 152 / 2) return 8;
  if (P > 2 * kScoreThreads * 4) return 4;
  if (P > kScoreThreads * 2) return 2;
  return 1;
}

template <int K>
static int launch_score(visacd_ctx* ctx, const float4* planes, int32_t P, const EdgeRec* recs,
                        int64_t E, const unsigned* stats, unsigned long long* sq, uint2* rq,
                        unsigned* rcount, unsigned rcap, unsigned* status) {
  const int per_cta = kScoreThreads * K;
  const int groups = (P + per_cta - 1) / per_cta;
  const int64_t nblocks = (E + kEdgeBlock - 1) / kEdgeBlock;
  // Aim for ~4 CTAs per SM in total (3 resident for K <= 4, 2 for K = 8, so
  // the edge slices keep every SM busy to the end); each CTA streams a
  // contiguous run of blocks.
  int64_t target_ctas = 4LL * ctx->sm_count;
  int64_t slices = (target_ctas + groups - 1) / groups;
  if (slices > nblocks) slices = nblocks;
  if (slices < 1) slices = 1;
  int64_t per = (nblocks + slices - 1) / slices;
  slices = (nblocks + per - 1) / per;
  size_t smem = 2 * kEdgeBlock * sizeof(EdgeRec) + (size_t)K * kScoreThreads * 8;
  static bool configured[9] = {false};
  if (!configured[K]) {
    VCUDA(cudaFuncSetAttribute(score_planes_kernel<K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem));
    configured[K] = true;
  }
  dim3 grid((unsigned)slices, (unsigned)groups);
  VLAUNCH(ctx, kKScore, grid, kScoreThreads, smem, score_planes_kernel<K>, planes, P, recs, E, per,
          stats, sq, rq, rcount, rcap, status);
  return VISACD_OK;
}

// Core of every scoring entry point. All pointers are device pointers.
static int score_device(visacd_ctx* ctx, const float* d_planes, int32_t P, const float* d_pts,
                        int32_t N, const uint32_t* d_edges, int64_t E, double* d_scores,
                        float* d_scores_f32, ScoreCounters** d_counters_out, unsigned rcap) {
  VTRY(ensure_slot(ctx, kSlotCounters, sizeof(ScoreCounters)));
  ScoreCounters* cnt = slot<ScoreCounters>(ctx, kSlotCounters);
  *d_counters_out = cnt;
  VCUDA(cudaMemsetAsync(cnt, 0, sizeof(ScoreCounters), ctx->stream));
  VTRY(ensure_slot(ctx, kSlotScoreQ, (size_t)(P > 0 ? P : 1) * sizeof(unsigned long long)));
  unsigned long long* sq = slot<unsigned long long>(ctx, kSlotScoreQ);
  if (P > 0) VCUDA(cudaMemsetAsync(sq, 0, (size_t)P * sizeof(unsigned long long), ctx->stream));
  if (N > 0) {
    VLAUNCH(ctx, kKPointStats, grid_for(N, 256, 4LL * ctx->sm_count), 256, 0, point_stats_kernel,
            d_pts, N, cnt->stats);
  }
  if (E > 0 && P > 0) {
    VTRY(ensure_slot(ctx, kSlotEdgePack, (size_t)E * sizeof(EdgeRec)));
    EdgeRec* recs = slot<EdgeRec>(ctx, kSlotEdgePack);
    VLAUNCH(ctx, kKPackEdges, grid_for(E, 256, 8LL * ctx->sm_count), 256, 0, pack_edges_kernel,
            d_pts, N, d_edges, E, cnt->stats, recs, &cnt->skipped);
    VTRY(ensure_slot(ctx, kSlotRecheck, (size_t)rcap * sizeof(uint2)));
    uint2* rq = slot<uint2>(ctx, kSlotRecheck);
    const float4* pl = reinterpret_cast<const float4*>(d_planes);
    int K = choose_score_k(ctx, P, E);
    switch (K) {
      case 8: VTRY(launch_score<8>(ctx, pl, P, recs, E, cnt->stats, sq, rq, &cnt->recheck_count, rcap, &cnt->status)); break;
      case 4: VTRY(launch_score<4>(ctx, pl, P, recs, E, cnt->stats, sq, rq, &cnt->recheck_count, rcap, &cnt->status)); break;
      case 2: VTRY(launch_score<2>(ctx, pl, P, recs, E, cnt->stats, sq, rq, &cnt->recheck_count, rcap, &cnt->status)); break;
      default: VTRY(launch_score<1>(ctx, pl, P, recs, E, cnt->stats, sq, rq, &cnt->recheck_count, rcap, &cnt->status)); break;
    }
    VLAUNCH(ctx, kKScoreRecheck, 2 * ctx->sm_count, 256, 0, score_recheck_kernel, pl, recs, E,
            cnt->stats, rq, &cnt->recheck_count, rcap, sq);
  }
  VLAUNCH(ctx, kKScoreFinish, 1, 1024, 0, score_finish_kernel, sq, P, cnt->stats, &cnt->status,
          d_scores, d_scores_f32, cnt->argmax);
  return VISACD_OK;
}

static unsigned recheck_capacity(int32_t P, int64_t E) {
  int64_t nblocks = (E + kEdgeBlock - 1) / kEdgeBlock;
  int64_t all = (int64_t)P * nblocks;
  int64_t cap = all / 128;
  if (cap < (1 << 20)) cap = 1 << 20;
  if (cap > all) cap = all;
  if (cap < 1) cap = 1;
  if (cap > (1LL << 30)) cap = 1LL << 30;
  return (unsigned)cap;
}

// Device-pointer scoring without a host wait, for callers that read the
// outcome later: the call's status word (kStatus* bits; a full FP64 queue or a
// timed-out wait) and its queue demand stay in device memory.
int score_planes_device_async(visacd_ctx* ctx, const float* d_planes, int32_t P, const float* d_pts,
                              int32_t N, const uint32_t* d_edges, int64_t E, double* d_scores,
                              unsigned rcap, const unsigned** d_status, const unsigned** d_recheck_count) {
  ScoreCounters* cnt = nullptr;
  VTRY(score_device(ctx, d_planes, P, d_pts, N, d_edges, E, d_scores, nullptr, &cnt, rcap));
  *d_status = &cnt->status;
  *d_recheck_count = &cnt->recheck_count;
  return VISACD_OK;
}

unsigned score_recheck_capacity(int32_t P, int64_t E) { return recheck_capacity(P, E); }

int score_planes_impl(visacd_ctx* ctx, const float* planes, int32_t P, const float* points,
                      int32_t N, const uint32_t* edges, int64_t E, int device_ptrs,
                      double* scores, float* scores_f32, visacd_score_stats* stats) {
  VCHECK(ctx, VISACD_ERR_INVALID_ARG, "score_planes: null context");
  VCHECK(P >= 0 && N >= 0 && E >= 0, VISACD_ERR_INVALID_ARG, "score_planes: negative size");
  VCHECK(P == 0 || planes, VISACD_ERR_INVALID_ARG, "score_planes: planes is NULL");
  VCHECK(N == 0 || points, VISACD_ERR_INVALID_ARG, "score_planes: points is NULL");
  VCHECK(E == 0 || edges, VISACD_ERR_INVALID_ARG, "score_planes: edges is NULL");
  VCHECK(E < (1LL << 40), VISACD_ERR_INVALID_ARG, "score_planes: too many edges");
  VCUDA(cudaSetDevice(ctx->device));
  const float *d_planes = planes, *d_pts = points;
  const uint32_t* d_edges = edges;
  double* d_scores = scores;
  float* d_scores_f32 = scores_f32;
  if (!device_ptrs) {
    VTRY(ensure_slot(ctx, kSlotPlanes, (size_t)(P > 0 ? P : 1) * 16));
    VTRY(ensure_slot(ctx, kSlotPoints, (size_t)(N > 0 ? N : 1) * 12));
    VTRY(ensure_slot(ctx, kSlotEdgesIn, (size_t)(E > 0 ? E : 1) * 8));
    VTRY(ensure_slot(ctx, kSlotScores, (size_t)(P > 0 ? P : 1) * 8));
    Stager up(ctx);
    VTRY(up.reserve((size_t)P * 16 + (size_t)N * 12 + (size_t)E * 8, 3));
    if (P) VTRY(up.put(ctx->buf[kSlotPlanes].p, planes, (size_t)P * 16));
    if (N) VTRY(up.put(ctx->buf[kSlotPoints].p, points, (size_t)N * 12));
    if (E) VTRY(up.put(ctx->buf[kSlotEdgesIn].p, edges, (size_t)E * 8));
    d_planes = slot<float>(ctx, kSlotPlanes);
    d_pts = slot<float>(ctx, kSlotPoints);
    d_edges = slot<uint32_t>(ctx, kSlotEdgesIn);
    d_scores = slot<double>(ctx, kSlotScores);
    d_scores_f32 = nullptr;
  }
  unsigned rcap = recheck_capacity(P, E);
  ScoreCounters* cnt = nullptr;
  VTRY(score_device(ctx, d_planes, P, d_pts, N, d_edges, E, d_scores, d_scores_f32, &cnt, rcap));
  if (!device_ptrs || stats) {
    // Counters, the context's status word and (host mode) the scores in one wait.
    ScoreCounters* h = nullptr;
    const size_t o_st = (sizeof(ScoreCounters) + 15) & ~size_t(15);
    VTRY(pinned(ctx, o_st + 16, (void**)&h));
    uint32_t* hst = reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(h) + o_st);
    auto read_back = [&]() -> int {
      VCUDA(cudaMemcpyAsync(h, cnt, sizeof(ScoreCounters), cudaMemcpyDeviceToHost, ctx->stream));
      VCUDA(cudaMemcpyAsync(hst, ctx->d_status, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
      if (!device_ptrs && P)
        VCUDA(cudaMemcpyAsync(scores, d_scores, (size_t)P * 8, cudaMemcpyDeviceToHost, ctx->stream));
      VCUDA(stream_wait(ctx));
      return VISACD_OK;
    };
    VTRY(read_back());
    ScoreCounters hc = *h;
    if (hc.recheck_count > rcap && !(hc.status & kStatusMbarrierTimeout)) {
      // The FP64 queue overflowed: rerun with room for every queued block.
      rcap = hc.recheck_count;
      VTRY(score_device(ctx, d_planes, P, d_pts, N, d_edges, E, d_scores, d_scores_f32, &cnt, rcap));
      VTRY(read_back());
      hc = *h;
    }
    VCHECK(!(hc.status & (kStatusMbarrierTimeout | kStatusRecheckOverflow)), VISACD_ERR_DEVICE,
           "score_planes: device status 0x%x (bulk-copy wait timed out or FP64 queue full)",
           hc.status);
    VTRY(status_result(ctx, *hst, "score_planes"));
    if (stats) {
      stats->quantum_exp = hc.argmax[1];
      stats->argmax = hc.argmax[0];
      stats->band_blocks = hc.recheck_count;
      stats->skipped_edges = (int64_t)hc.skipped;
    }
  }
  return VISACD_OK;
}

}  // namespace vgpu

using namespace vgpu;

extern "C" int visacd_score_planes(visacd_ctx* ctx, const float* planes, int32_t P,
                                   const float* points, int32_t N, const uint32_t* edges,
                                   int64_t E, int device_ptrs, double* scores,
                                   visacd_score_stats* stats) {
  return score_planes_impl(ctx, planes, P, points, N, edges, E, device_ptrs, scores, nullptr,
                           stats);
}

extern "C" int visacd_ctx_set_score_k(visacd_ctx* ctx, int k) {
  VCHECK(ctx, VISACD_ERR_INVALID_ARG, "set_score_k: null context");
  VCHECK(k == 0 || k == 1 || k == 2 || k == 4 || k == 8, VISACD_ERR_INVALID_ARG,
         "set_score_k: %d is not 0, 1, 2, 4 or 8", k);
  ctx->score_k_override = k;
  return VISACD_OK;
}

extern "C" int visacd_autotune_scoring(visacd_ctx* ctx, const float* planes, int32_t P, const float* points,
                                       int32_t N, const uint32_t* edges, int64_t E, int device_ptrs,
                                       int* best_k, double* ms_per_k) {
  VCHECK(ctx, VISACD_ERR_INVALID_ARG, "autotune_scoring: null context");
  const int saved_override = ctx->score_k_override;
  const bool saved_timing = ctx->timing;
  static const int kKs[4] = {1, 2, 4, 8};
  int best = 0;
  double best_ms = 1e300;
  int rc = VISACD_OK;
  std::vector<double> scores((size_t)(P > 0 ? P : 1));
  for (int v = 0; v < 4 && rc == VISACD_OK; ++v) {
    ctx->score_k_override = kKs[v];
    double ms = 0.0;
    for (int rep = 0; rep < 2 && rc == VISACD_OK; ++rep) {
      ctx->timing = true;
      rc = visacd_ctx_reset_times(ctx);
      // Device pointers get a device score buffer (the context's), host
      // pointers a host one.
      double* out = scores.data();
      if (rc == VISACD_OK && device_ptrs) {
        rc = ensure_slot(ctx, kSlotScores, (size_t)(P > 0 ? P : 1) * 8);
        out = slot<double>(ctx, kSlotScores);
      }
      if (rc == VISACD_OK)
        rc = score_planes_impl(ctx, planes, P, points, N, edges, E, device_ptrs, out, nullptr, nullptr);
      const char* names[64];
      double t[64];
      int64_t cnt[64];
      int nk = 0;
      if (rc == VISACD_OK) rc = visacd_ctx_kernel_times(ctx, names, t, cnt, 64, &nk);
      ms = 0.0;
      for (int k = 0; k < nk && k < 64; ++k)
        if (strcmp(names[k], kernel_name(kKScore)) == 0 || strcmp(names[k], kernel_name(kKScoreRecheck)) == 0)
          ms += t[k];
    }
    if (ms_per_k) ms_per_k[v] = ms;
    if (ms < best_ms) {
      best_ms = ms;
      best = kKs[v];
    }
  }
  ctx->score_k_override = saved_override;
  ctx->timing = saved_timing;
  visacd_ctx_reset_times(ctx);
  if (rc != VISACD_OK) return rc;
  ctx->score_tuned[score_shape_class(P, E)] = best;
  if (best_k) *best_k = best;
  return VISACD_OK;
}

// ---------------------------------------------------------------------------
// Drop-in replacement of the reference host wrapper
// (lib/cuda/plane_intersections.cu:71-133): host pointers, synchronous, float
// scores, no status return. Runs on a process-wide context on device 0.
// ---------------------------------------------------------------------------
#include <mutex>
#include <vector>

namespace vgpu {
visacd_ctx* default_ctx() {
  static std::once_flag once;
  static visacd_ctx* ctx = nullptr;
  std::call_once(once, [] {
    if (visacd_ctx_create(0, nullptr, &ctx) != VISACD_OK) ctx = nullptr;
  });
  return ctx;
}
}  // namespace vgpu

extern "C" void classify_and_rate_planes(const float* planes, const float* points,
                                         const unsigned int* edges, float* scores,
                                         int numPlanes, int numPoints, int numEdges) {
  if (numPlanes <= 0) return;
  for (int p = 0; p < numPlanes; ++p) scores[p] = 0.f;
  visacd_ctx* ctx = vgpu::default_ctx();
  if (!ctx) return;
  std::vector<double> s((size_t)numPlanes, 0.0);
  int rc = score_planes_impl(ctx, planes, numPlanes, points, numPoints < 0 ? 0 : numPoints,
                             edges, numEdges < 0 ? 0 : numEdges, 0, s.data(), nullptr, nullptr);
  if (rc != VISACD_OK) return;
  for (int p = 0; p < numPlanes; ++p) scores[p] = (float)s[p];
}

// ---------------------------------------------------------------------------
// Allocation-free plane scoring.
//
// For callers that must not allocate device or host memory from inside this
// library: code that runs under a caller-owned memory budget (a fixed arena
// reserved at start-up, a real-time loop where cudaMalloc's implicit device
// synchronisation and unbounded latency are not allowed), or code that is not
// allowed to touch the allocator at all while other work owns the device.
// Inputs and outputs are the caller's device buffers; every byte of scratch
// (packed edge records, integer score accumulators, the FP64 re-decision
// queue, counters) lives in one file-scope device array that the library image
// reserves on every GPU that loads it, until the process exits.
//
// Limits: E <= 65536 edges and P <= 4096 planes (10,518,784 bytes of scratch).
// The queue holds every (plane, edge block) pair, so it cannot overflow.
// All calls share the array and it keeps the previous call's contents: the
// accumulators and counters are cleared on the stream at the start of each
// call, and calls whose work overlaps on the GPU (different streams, or
// different host threads) race on it — serialise them.
// ---------------------------------------------------------------------------
namespace vgpu {

constexpr int64_t kNoAllocMaxEdges = 65536;
constexpr int32_t kNoAllocMaxPlanes = 4096;
constexpr int64_t kNoAllocMaxBlocks = kNoAllocMaxEdges / kEdgeBlock;
constexpr size_t kNoAllocCountersBytes = 256;
constexpr size_t kNoAllocScoreQBytes = (size_t)kNoAllocMaxPlanes * 8;
constexpr size_t kNoAllocPackBytes = (size_t)kNoAllocMaxEdges * sizeof(EdgeRec);
constexpr size_t kNoAllocQueueBytes = (size_t)kNoAllocMaxPlanes * kNoAllocMaxBlocks * sizeof(uint2);
constexpr size_t kNoAllocBytes =
    kNoAllocCountersBytes + kNoAllocScoreQBytes + kNoAllocPackBytes + kNoAllocQueueBytes;
static_assert(sizeof(ScoreCounters) <= kNoAllocCountersBytes, "counters must fit");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// Device address of the scratch array, looked up once per device with that
// device current (in host code the symbol is only a host-side stand-in).
static unsigned char* noalloc_scratch_ptr(int device, int* rc) {
  static std::mutex mu;
  static unsigned char* ptrs[64] = {nullptr};
  std::lock_guard<std::mutex> lock(mu);
  if (device < 0 || device >= 64) {
    set_error("score_planes_noalloc: device %d out of range", device);
    *rc = VISACD_ERR_INVALID_ARG;
    return nullptr;
  }
  if (!ptrs[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
      set_error("score_planes_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
      *rc = VISACD_ERR_CUDA;
      return nullptr;
    }
    ptrs[device] = static_cast<unsigned char*>(p);
  }
  *rc = VISACD_OK;
  return ptrs[device];
}

static int noalloc_sm_count(int device) {
  int sm = 0;
  if (cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) sm = 0;
  return sm > 0 ? sm : 1;
}

template <int K>
static int noalloc_launch_score(cudaStream_t st, int sm_count, const float4* planes, int32_t P,
                                const EdgeRec* recs, int64_t E, const unsigned* stats,
                                unsigned long long* sq, uint2* rq, unsigned* rcount, unsigned rcap,
                                unsigned* status) {
  const int per_cta = kScoreThreads * K;
  const int groups = (P + per_cta - 1) / per_cta;
  const int64_t nblocks = (E + kEdgeBlock - 1) / kEdgeBlock;
  int64_t slices = (4LL * sm_count + groups - 1) / groups;
  if (slices > nblocks) slices = nblocks;
  if (slices < 1) slices = 1;
  int64_t per = (nblocks + slices - 1) / slices;
  slices = (nblocks + per - 1) / per;
  size_t smem = 2 * kEdgeBlock * sizeof(EdgeRec) + (size_t)K * kScoreThreads * 8;
  VCUDA(cudaFuncSetAttribute(score_planes_kernel<K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem));
  score_planes_kernel<K><<<dim3((unsigned)slices, (unsigned)groups), kScoreThreads, smem, st>>>(
      planes, P, recs, E, per, stats, sq, rq, rcount, rcap, status);
  VCUDA(cudaGetLastError());
  return VISACD_OK;
}

}  // namespace vgpu

extern "C" int visacd_score_planes_noalloc(const float* d_planes, int32_t P, const float* d_points,
                                           int32_t N, const uint32_t* d_edges, int64_t E,
                                           double* d_scores, int32_t* d_argmax,
                                           void* cuda_stream) {
  using namespace vgpu;
  VCHECK(P >= 0 && N >= 0 && E >= 0, VISACD_ERR_INVALID_ARG, "score_planes_noalloc: negative size");
  VCHECK(P <= kNoAllocMaxPlanes, VISACD_ERR_CAPACITY,
         "score_planes_noalloc: P = %d planes exceeds the allocation-free limit of %d", P,
         kNoAllocMaxPlanes);
  VCHECK(E <= kNoAllocMaxEdges, VISACD_ERR_CAPACITY,
         "score_planes_noalloc: E = %lld edges exceeds the allocation-free limit of %lld",
         (long long)E, (long long)kNoAllocMaxEdges);
  VCHECK(P == 0 || (d_planes && d_scores), VISACD_ERR_INVALID_ARG,
         "score_planes_noalloc: planes or scores is NULL");
  VCHECK(N == 0 || d_points, VISACD_ERR_INVALID_ARG, "score_planes_noalloc: points is NULL");
  VCHECK(E == 0 || d_edges, VISACD_ERR_INVALID_ARG, "score_planes_noalloc: edges is NULL");
  int device = 0;
  VCUDA(cudaGetDevice(&device));
  int rc = VISACD_OK;
  unsigned char* base = noalloc_scratch_ptr(device, &rc);
  if (!base) return rc;
  cudaStream_t st = (cudaStream_t)cuda_stream;
  ScoreCounters* cnt = reinterpret_cast<ScoreCounters*>(base);
  unsigned long long* sq = reinterpret_cast<unsigned long long*>(base + kNoAllocCountersBytes);
  EdgeRec* recs = reinterpret_cast<EdgeRec*>(base + kNoAllocCountersBytes + kNoAllocScoreQBytes);
  uint2* rq = reinterpret_cast<uint2*>(base + kNoAllocCountersBytes + kNoAllocScoreQBytes +
                                       kNoAllocPackBytes);
  // The call's status word is part of the counters block, cleared below.
  unsigned* status = &cnt->status;
  VCUDA(cudaMemsetAsync(base, 0, kNoAllocCountersBytes + (size_t)(P > 0 ? P : 1) * 8, st));
  const int sm = noalloc_sm_count(device);
  if (N > 0) {
    point_stats_kernel<<<grid_for(N, 256, 4LL * sm), 256, 0, st>>>(d_points, N, cnt->stats);
    VCUDA(cudaGetLastError());
  }
  if (E > 0 && P > 0) {
    pack_edges_kernel<<<grid_for(E, 256, 8LL * sm), 256, 0, st>>>(d_points, N, d_edges, E,
                                                                   cnt->stats, recs, &cnt->skipped);
    VCUDA(cudaGetLastError());
    const unsigned rcap = (unsigned)((int64_t)P * ((E + kEdgeBlock - 1) / kEdgeBlock));
    const float4* pl = reinterpret_cast<const float4*>(d_planes);
    switch (planes_per_thread(P)) {
      case 8: VTRY(noalloc_launch_score<8>(st, sm, pl, P, recs, E, cnt->stats, sq, rq, &cnt->recheck_count, rcap, status)); break;
      case 4: VTRY(noalloc_launch_score<4>(st, sm, pl, P, recs, E, cnt->stats, sq, rq, &cnt->recheck_count, rcap, status)); break;
      case 2: VTRY(noalloc_launch_score<2>(st, sm, pl, P, recs, E, cnt->stats, sq, rq, &cnt->recheck_count, rcap, status)); break;
      default: VTRY(noalloc_launch_score<1>(st, sm, pl, P, recs, E, cnt->stats, sq, rq, &cnt->recheck_count, rcap, status)); break;
    }
    score_recheck_kernel<<<2 * sm, 256, 0, st>>>(pl, recs, E, cnt->stats, rq, &cnt->recheck_count,
                                                 rcap, sq);
    VCUDA(cudaGetLastError());
  }
  score_finish_kernel<<<1, 1024, 0, st>>>(sq, P, cnt->stats, status, d_scores, nullptr,
                                          cnt->argmax);
  VCUDA(cudaGetLastError());
  if (d_argmax) {
    VCUDA(cudaMemcpyAsync(d_argmax, cnt->argmax, sizeof(int32_t), cudaMemcpyDeviceToDevice, st));
  }
  return VISACD_OK;
}

// Batched visibility + plane scoring: every pending part of uneven size in one
// launch sequence, captured once as a CUDA graph and replayed.
//
// Per part (set up once per batch): its points, Morton vertex order, triangular
// tile rows, part and cage BVHs, candidate planes, and the FP32 rounding
// statistics of its points. One run is a fixed kernel sequence whose sizes
// come from device memory, so the sequence is graph-capturable:
//  1. batch_visibility: persistent warps pull global tile ids; a tile id maps
//     to (part, tile) by binary search over per-part tile offsets; the packet
//     traversal and segment tests are the single-part kernel's (traverse.cuh);
//     results land in one concatenated bitset, each part on a word boundary.
//  2. popcount / exclusive scan / emit over the whole bitset: the edges of part
//     p are the contiguous range [word offsets of p] of the scan (row-major).
//  3. batch_part_prep (one CTA): per-part edge counts and 256-edge-aligned
//     record offsets (a scan over parts).
//  4. batch_pack + batch_score<K>: the scoring kernel of score.cu with the part
//     looked up per CTA (grid = parts x plane groups); FP64 band re-decision
//     through a shared queue; per-part argmax.
#include "score_device.cuh"
#include "traverse.cuh"

namespace vgpu {

struct BatchPart {
  const float* pts;
  int n;
  int ntr, ntc;
  const uint32_t* perm;
  const unsigned long long* row_start;
  unsigned long long tile_begin;
  const float4* self_nodes;
  const float4* self_tris;
  int self_nt;
  const float4* cage_nodes;
  const float4* cage_tris;
  int cage_nt;
  unsigned long long word_begin;
  unsigned long long nwords;
  int plane_begin;
  int P;
  unsigned stats[4];  // max |x|, |y|, |z| of the part's points (float bits)
};

struct BatchDyn {  // per part, written during a run
  unsigned long long edge_begin, n_edges;
  unsigned long long rec_begin, n_blocks;
};

struct BatchCounters {
  unsigned long long work;
  unsigned recheck_count;
  unsigned pad;
};

// ---- 1. visibility over all parts -----------------------------------------
template <int TR>
__global__ void __launch_bounds__(kVisThreads, 6)
    batch_visibility_kernel(const BatchPart* __restrict__ parts, int n_parts,
                            const unsigned long long* __restrict__ part_tile_start,
                            unsigned long long total_tiles, uint32_t* __restrict__ bitset,
                            BatchCounters* __restrict__ cnt, unsigned* __restrict__ status) {
  constexpr int TC = 32 / TR;
  const int lane = threadIdx.x & 31;
  unsigned rechecks = 0, status_bits = 0, visits = 0, tri_tests = 0;
  for (int guard = 0; guard < (1 << 30); ++guard) {
    unsigned long long w = 0;
    if (lane == 0) w = atomicAdd(&cnt->work, 1ull);
    w = __shfl_sync(0xffffffffu, w, 0);
    if (w >= total_tiles) break;
    int lo = 0, hi = n_parts - 1;
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (part_tile_start[mid] <= w) lo = mid; else hi = mid - 1;
    }
    const BatchPart& P = parts[lo];
    const unsigned long long lw = w - P.tile_begin;
    int64_t rlo = 0, rhi = P.ntr - 1;
    while (rlo < rhi) {
      int64_t mid = (rlo + rhi + 1) >> 1;
      if (P.row_start[mid] <= lw) rlo = mid; else rhi = mid - 1;
    }
    const int64_t tr = rlo;
    const int64_t tc = (tr * TR) / TC + (int64_t)(lw - P.row_start[tr]);
    const int64_t a = tr * TR + lane / TC, b = tc * TC + lane % TC;
    const bool valid = a < b && b < P.n;
    uint32_t i = 0, j = 0;
    float3 p = make_float3(0.f, 0.f, 0.f), q = make_float3(0.f, 0.f, 0.f);
    if (valid) {
      uint32_t oi = P.perm[a], oj = P.perm[b];
      i = min(oi, oj);
      j = max(oi, oj);
      p = make_float3(P.pts[3 * (int64_t)i], P.pts[3 * (int64_t)i + 1], P.pts[3 * (int64_t)i + 2]);
      q = make_float3(P.pts[3 * (int64_t)j], P.pts[3 * (int64_t)j + 1], P.pts[3 * (int64_t)j + 2]);
    }
    Seg s;
    make_seg(s, p, q, (int)i, (int)j);
    bool active = valid && seg_len(s) > 0.f;
    if (!__ballot_sync(0xffffffffu, active)) continue;
    // The cage first; the self test only for segments that leave it.
    s.exclude = false;
    const bool cage_hit = packet_any_hit(P.cage_nodes, P.cage_tris, P.cage_nt, s, P.pts, active,
                                         rechecks, status_bits, visits, tri_tests);
    active = active && cage_hit;
    s.exclude = true;
    const bool self_hit = packet_any_hit(P.self_nodes, P.self_tris, P.self_nt, s, P.pts, active,
                                         rechecks, status_bits, visits, tri_tests);
    if (active && !self_hit) {
      const int64_t k = row_start(i, P.n) + (int64_t)(j - i - 1);
      atomicOr(&bitset[P.word_begin + (k >> 5)], 1u << (k & 31));
    }
  }
  status_bits = __reduce_or_sync(0xffffffffu, status_bits);
  if (lane == 0 && status_bits) atomicOr(status, status_bits);
}

// ---- 2. compaction --------------------------------------------------------
__global__ void batch_popc_kernel(const uint32_t* __restrict__ bits, int64_t nw, uint32_t* __restrict__ counts) {
  for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < nw; w += (int64_t)gridDim.x * blockDim.x)
    counts[w] = __popc(bits[w]);
}

__global__ void batch_emit_kernel(const BatchPart* __restrict__ parts, int n_parts,
                                  const unsigned long long* __restrict__ part_word_start,
                                  const uint32_t* __restrict__ bits, int64_t nw,
                                  const uint64_t* __restrict__ off, uint32_t* __restrict__ edges,
                                  unsigned long long edge_cap, unsigned* __restrict__ status) {
  for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < nw; w += (int64_t)gridDim.x * blockDim.x) {
    uint32_t m = bits[w];
    if (!m) continue;
    int lo = 0, hi = n_parts - 1;
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (part_word_start[mid] <= (unsigned long long)w) lo = mid; else hi = mid - 1;
    }
    const int64_t n = parts[lo].n;
    const int64_t k0 = (w - (int64_t)parts[lo].word_begin) * 32;
    uint64_t o = off[w];
    double b2 = (double)(2 * n - 1);
    double disc = b2 * b2 - 8.0 * (double)k0;
    int64_t i = (int64_t)((b2 - sqrt(disc > 0 ? disc : 0.0)) * 0.5);
    if (i < 0) i = 0;
    if (i > n - 2) i = n - 2;
    while (i > 0 && row_start(i, n) > k0) --i;
    while (i + 1 <= n - 2 && row_start(i + 1, n) <= k0) ++i;
    while (m) {
      int bpos = __ffs(m) - 1;
      m &= m - 1;
      int64_t k = k0 + bpos;
      while (i + 1 <= n - 2 && row_start(i + 1, n) <= k) ++i;
      int64_t j = k - row_start(i, n) + i + 1;
      if (o < edge_cap) {
        edges[2 * o] = (uint32_t)i;
        edges[2 * o + 1] = (uint32_t)j;
      } else {
        atomicOr(status, kStatusWorkOverrun);
      }
      ++o;
    }
  }
}

// ---- 3. per-part edge ranges and record offsets (one CTA) -----------------
__global__ void batch_part_prep_kernel(const BatchPart* __restrict__ parts, int n_parts,
                                       const uint64_t* __restrict__ off, BatchDyn* __restrict__ dyn) {
  __shared__ unsigned long long carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < n_parts; base += blockDim.x) {
    const int p = base + threadIdx.x;
    unsigned long long nb = 0, eb = 0, ne = 0;
    if (p < n_parts) {
      eb = off[parts[p].word_begin];
      ne = off[parts[p].word_begin + parts[p].nwords] - eb;
      nb = (ne + 255) / 256;
    }
    // Block-wide exclusive scan of nb (blockDim.x <= 1024).
    __shared__ unsigned long long sc[1024];
    sc[threadIdx.x] = nb;
    __syncthreads();
    for (int o = 1; o < (int)blockDim.x; o <<= 1) {
      unsigned long long v = threadIdx.x >= (unsigned)o ? sc[threadIdx.x - o] : 0;
      __syncthreads();
      sc[threadIdx.x] += v;
      __syncthreads();
    }
    const unsigned long long incl = sc[threadIdx.x];
    if (p < n_parts) {
      dyn[p].edge_begin = eb;
      dyn[p].n_edges = ne;
      dyn[p].rec_begin = (carry + incl - nb) * 256;
      dyn[p].n_blocks = nb;
    }
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry += incl;
    __syncthreads();
  }
}

// ---- 4. packing and scoring -------------------------------------------------
__global__ void batch_pack_kernel(const BatchPart* __restrict__ parts, const BatchDyn* __restrict__ dyn,
                                  const uint32_t* __restrict__ edges, EdgeRec* __restrict__ recs,
                                  unsigned long long rec_cap, int per_part_blocks) {
  const int p = blockIdx.x / per_part_blocks, sub = blockIdx.x % per_part_blocks;
  const BatchPart& P = parts[p];
  const BatchDyn d = dyn[p];
  const unsigned cmax = max(P.stats[0], max(P.stats[1], P.stats[2]));
  const int qexp = quantum_exp_from_cmax_bits(cmax);
  const unsigned long long padded = d.n_blocks * 256;
  for (unsigned long long e = (unsigned long long)sub * blockDim.x + threadIdx.x; e < padded;
       e += (unsigned long long)per_part_blocks * blockDim.x) {
    EdgeRec r;
    r.pad = 0;
    r.x1 = r.x2 = r.y1 = r.y2 = r.z1 = r.z2 = 0.f;
    r.q = 0;
    if (e < d.n_edges) {
      const uint32_t i = edges[2 * (d.edge_begin + e)], j = edges[2 * (d.edge_begin + e) + 1];
      const float* a = P.pts + 3 * (int64_t)i;
      const float* b = P.pts + 3 * (int64_t)j;
      float len = edge_len32(__fsub_rn(b[0], a[0]), __fsub_rn(b[1], a[1]), __fsub_rn(b[2], a[2]));
      r.x1 = a[0]; r.x2 = b[0]; r.y1 = a[1]; r.y2 = b[1]; r.z1 = a[2]; r.z2 = b[2];
      r.q = __float2uint_rn(ldexpf(len, -qexp));
    }
    if (d.rec_begin + e < rec_cap) recs[d.rec_begin + e] = r;
  }
}

template <int K>
__global__ void __launch_bounds__(kScoreThreads, (K <= 4 ? 2 : 1))
    batch_score_kernel(const BatchPart* __restrict__ parts, const BatchDyn* __restrict__ dyn,
                       const float4* __restrict__ planes, const EdgeRec* __restrict__ recs,
                       unsigned long long* __restrict__ score_q, uint2* __restrict__ recheck,
                       unsigned* __restrict__ recheck_count, unsigned recheck_cap, int groups,
                       unsigned* __restrict__ status) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  EdgeRec* buf = reinterpret_cast<EdgeRec*>(smem_raw);
  unsigned long long* tot =
      reinterpret_cast<unsigned long long*>(smem_raw + 2 * kEdgeBlock * sizeof(EdgeRec));
  __shared__ __align__(8) uint64_t bars[2];
  const int tid = threadIdx.x;
  const int part = blockIdx.x / groups, grp = blockIdx.x % groups;
  const BatchPart& Pp = parts[part];
  const BatchDyn d = dyn[part];
  const int nb = (int)d.n_blocks;
  const int64_t blk0 = (int64_t)(d.rec_begin / kEdgeBlock);
  const int plane_base = grp * kScoreThreads * K;
  PlaneAcc pa[K];
  uint32_t acc[K], dmin[K];
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const int lp = plane_base + k * kScoreThreads + tid;
    float4 pl = lp < Pp.P ? planes[Pp.plane_begin + lp]
                          : make_float4(__int_as_float(0x7fc00000), __int_as_float(0x7fc00000),
                                        __int_as_float(0x7fc00000), __int_as_float(0x7fc00000));
    pa[k] = plane_acc(pl, Pp.stats);
    acc[k] = 0u;
    dmin[k] = 0xffffffffu;
    tot[k * kScoreThreads + tid] = 0ull;
  }
  if (nb == 0 || plane_base >= Pp.P) return;
  if (tid == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (tid == 0) bulk_load(buf, recs + blk0 * kEdgeBlock, kEdgeBlock * sizeof(EdgeRec), &bars[0]);
  bool failed = false;
  for (int it = 0; it < nb; ++it) {
    const int cur = it & 1;
    if (tid == 0 && it + 1 < nb) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      bulk_load(buf + (cur ^ 1) * kEdgeBlock, recs + (blk0 + it + 1) * kEdgeBlock,
                kEdgeBlock * sizeof(EdgeRec), &bars[cur ^ 1]);
    }
    bool ok = mbar_wait(&bars[cur], (unsigned)((it >> 1) & 1));
    if (__syncthreads_or(!ok)) {
      failed = true;
      break;
    }
    const ulonglong2* sm = reinterpret_cast<const ulonglong2*>(buf + cur * kEdgeBlock);
    score_edge_block<K>(sm, kEdgeBlock, pa, acc, dmin);
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int lp = plane_base + k * kScoreThreads + tid;
      if (dmin[k] > pa[k].wbits) {
        tot[k * kScoreThreads + tid] += acc[k];
      } else if (lp < Pp.P) {
        const int gp = Pp.plane_begin + lp;
        unsigned idx = atomicAdd(recheck_count, 1u);
        if (idx < recheck_cap) recheck[idx] = make_uint2((unsigned)gp, (unsigned)(blk0 + it));
        else atomicOr(status, kStatusRecheckOverflow);
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
    const int lp = plane_base + k * kScoreThreads + tid;
    unsigned long long t = tot[k * kScoreThreads + tid];
    if (lp < Pp.P && t) atomicAdd(&score_q[Pp.plane_begin + lp], t);
  }
}

// FP64 re-decision of queued (plane, block) pairs; the part of a plane is
// found from the part plane offsets.
__global__ void batch_recheck_kernel(const BatchPart* __restrict__ parts, int n_parts,
                                     const int* __restrict__ part_plane_start,
                                     const float4* __restrict__ planes, const EdgeRec* __restrict__ recs,
                                     const uint2* __restrict__ recheck, const unsigned* __restrict__ recheck_count,
                                     unsigned recheck_cap, unsigned long long* __restrict__ score_q) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  unsigned n = *recheck_count;
  if (n > recheck_cap) n = recheck_cap;
  const double eps = (double)kSideEps;
  for (int64_t r = warp; r < n; r += nwarps) {
    const uint2 rec = recheck[r];
    int lo = 0, hi = n_parts - 1;
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (part_plane_start[mid] <= (int)rec.x) lo = mid; else hi = mid - 1;
    }
    const float4 pl = planes[rec.x];
    float nlo, nhi;
    plane_thresholds(pl, parts[lo].stats, nlo, nhi);
    const int64_t e0 = (int64_t)rec.y * kEdgeBlock;
    unsigned long long sum = 0;
    for (int64_t e = e0 + lane; e < e0 + kEdgeBlock; e += 32) {
      const EdgeRec er = recs[e];
      float v1 = fmaf(pl.x, er.x1, fmaf(pl.y, er.y1, fmaf(pl.z, er.z1, pl.w)));
      float v2 = fmaf(pl.x, er.x2, fmaf(pl.y, er.y2, fmaf(pl.z, er.z2, pl.w)));
      float sv = fmaxf(fminf(v1, v2), -fmaxf(v1, v2));
      if (sv < nhi) {
        sum += er.q;
      } else if (sv < nlo) {
        double w1 = side_value64(pl, er.x1, er.y1, er.z1);
        double w2 = side_value64(pl, er.x2, er.y2, er.z2);
        if ((w1 > eps && w2 < -eps) || (w1 < -eps && w2 > eps)) sum += er.q;
      }
    }
    for (int o = 16; o; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if (lane == 0 && sum) atomicAdd(&score_q[rec.x], sum);
  }
}

// Scores (float64) and per-part first argmax: one warp per part.
__global__ void batch_finish_kernel(const BatchPart* __restrict__ parts, int n_parts,
                                    const unsigned long long* __restrict__ score_q,
                                    double* __restrict__ scores, int* __restrict__ argmax) {
  const int lane = threadIdx.x & 31;
  const int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (p >= n_parts) return;
  const BatchPart& P = parts[p];
  const unsigned cmax = max(P.stats[0], max(P.stats[1], P.stats[2]));
  const int qexp = quantum_exp_from_cmax_bits(cmax);
  unsigned long long best = 0;
  int bi = P.P > 0 ? 0 : -1;
  for (int k = lane; k < P.P; k += 32) {
    const unsigned long long v = score_q[P.plane_begin + k];
    scores[P.plane_begin + k] = ldexp((double)v, qexp);
    if (v > best || (v == best && k < bi)) {
      best = v;
      bi = k;
    }
  }
  for (int o = 16; o; o >>= 1) {
    unsigned long long v2 = __shfl_xor_sync(0xffffffffu, best, o);
    int i2 = __shfl_xor_sync(0xffffffffu, bi, o);
    if (v2 > best || (v2 == best && i2 >= 0 && (bi < 0 || i2 < bi))) {
      best = v2;
      bi = i2;
    }
  }
  if (lane == 0) argmax[p] = bi;
}

}  // namespace vgpu

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
using namespace vgpu;

struct visacd_batch {
  int device = 0;
  int n_parts = 0;
  int64_t total_planes = 0;
  unsigned long long total_tiles = 0, total_words = 0, total_pairs = 0, edge_cap = 0, rec_cap = 0;
  unsigned recheck_cap = 0;
  int groups = 1, K = 1;
  std::vector<void*> allocs;
  BatchPart* d_parts = nullptr;
  BatchDyn* d_dyn = nullptr;
  unsigned long long *d_tile_start = nullptr, *d_word_start = nullptr;
  int* d_plane_start = nullptr;
  uint32_t* d_bits = nullptr;
  uint32_t* d_wcount = nullptr;
  uint64_t* d_woff = nullptr;
  uint32_t* d_edges = nullptr;
  EdgeRec* d_recs = nullptr;
  unsigned long long* d_score_q = nullptr;
  double* d_scores = nullptr;
  int* d_argmax = nullptr;
  uint2* d_recheck = nullptr;
  BatchCounters* d_cnt = nullptr;
  float4* d_planes = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<int> part_P;
};

static int balloc(visacd_batch* b, size_t bytes, void** p) {
  cudaError_t e = cudaMalloc(p, bytes < 256 ? 256 : bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_error("batch allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
    return VISACD_ERR_NO_MEMORY;
  }
  b->allocs.push_back(*p);
  return VISACD_OK;
}

// The run's kernel sequence (launched directly or captured into the graph).
static int batch_sequence(visacd_ctx* ctx, visacd_batch* b) {
  cudaStream_t st = ctx->stream;
  VCUDA(cudaMemsetAsync(b->d_cnt, 0, sizeof(BatchCounters), st));
  VCUDA(cudaMemsetAsync(b->d_bits, 0, (size_t)b->total_words * 4, st));
  VCUDA(cudaMemsetAsync(b->d_score_q, 0, (size_t)b->total_planes * 8, st));
  const unsigned gvis = (unsigned)(ctx->sm_count * 6);
  batch_visibility_kernel<8><<<gvis, kVisThreads, 0, st>>>(b->d_parts, b->n_parts, b->d_tile_start,
                                                           b->total_tiles, b->d_bits, b->d_cnt, ctx->d_status);
  VCUDA(cudaGetLastError());
  const unsigned gw = grid_for((int64_t)b->total_words, 256, 16LL * ctx->sm_count);
  batch_popc_kernel<<<gw, 256, 0, st>>>(b->d_bits, (int64_t)b->total_words, b->d_wcount);
  VCUDA(cudaGetLastError());
  VTRY(exclusive_scan_u32_to_u64(ctx, b->d_wcount, b->d_woff, (int64_t)b->total_words));
  batch_emit_kernel<<<gw, 256, 0, st>>>(b->d_parts, b->n_parts, b->d_word_start, b->d_bits,
                                        (int64_t)b->total_words, b->d_woff, b->d_edges, b->edge_cap,
                                        ctx->d_status);
  VCUDA(cudaGetLastError());
  batch_part_prep_kernel<<<1, 1024, 0, st>>>(b->d_parts, b->n_parts, b->d_woff, b->d_dyn);
  VCUDA(cudaGetLastError());
  const int ppb = 8;
  batch_pack_kernel<<<b->n_parts * ppb, 256, 0, st>>>(b->d_parts, b->d_dyn, b->d_edges, b->d_recs,
                                                      b->rec_cap, ppb);
  VCUDA(cudaGetLastError());
  const size_t smem = 2 * kEdgeBlock * sizeof(EdgeRec) + (size_t)b->K * kScoreThreads * 8;
  const unsigned gs = (unsigned)(b->n_parts * b->groups);
#define VISACD_BATCH_SCORE(KK)                                                                        \
  VCUDA(cudaFuncSetAttribute(batch_score_kernel<KK>, cudaFuncAttributeMaxDynamicSharedMemorySize,  \
                             (int)smem));                                                         \
  batch_score_kernel<KK><<<gs, kScoreThreads, smem, st>>>(b->d_parts, b->d_dyn, b->d_planes,       \
                                                          b->d_recs, b->d_score_q, b->d_recheck,  \
                                                          &b->d_cnt->recheck_count, b->recheck_cap, \
                                                          b->groups, ctx->d_status)
  switch (b->K) {
    case 8: VISACD_BATCH_SCORE(8); break;
    case 4: VISACD_BATCH_SCORE(4); break;
    case 2: VISACD_BATCH_SCORE(2); break;
    default: VISACD_BATCH_SCORE(1); break;
  }
#undef VISACD_BATCH_SCORE
  VCUDA(cudaGetLastError());
  batch_recheck_kernel<<<2 * ctx->sm_count, 256, 0, st>>>(b->d_parts, b->n_parts, b->d_plane_start,
                                                          b->d_planes, b->d_recs, b->d_recheck,
                                                          &b->d_cnt->recheck_count, b->recheck_cap,
                                                          b->d_score_q);
  VCUDA(cudaGetLastError());
  batch_finish_kernel<<<(b->n_parts * 32 + 255) / 256, 256, 0, st>>>(b->d_parts, b->n_parts, b->d_score_q,
                                                                     b->d_scores, b->d_argmax);
  VCUDA(cudaGetLastError());
  return VISACD_OK;
}

extern "C" int visacd_batch_destroy(visacd_batch* b) {
  if (!b) return VISACD_OK;
  cudaSetDevice(b->device);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  for (void* p : b->allocs) cudaFree(p);
  delete b;
  return VISACD_OK;
}

extern "C" int visacd_batch_create(visacd_ctx* ctx, int32_t n_parts, const float* const* pts,
                                   const int32_t* n_pts, const visacd_bvh* const* self_bvhs,
                                   const visacd_bvh* const* cage_bvhs, const float* const* planes,
                                   const int32_t* n_planes, int64_t edge_capacity, visacd_batch** out) {
  VCHECK(ctx && out && n_parts > 0 && pts && n_pts && self_bvhs && cage_bvhs && planes && n_planes,
         VISACD_ERR_INVALID_ARG, "batch_create: null argument");
  VCUDA(cudaSetDevice(ctx->device));
  *out = nullptr;
  visacd_batch* b = new visacd_batch();
  b->device = ctx->device;
  b->n_parts = n_parts;
  std::vector<BatchPart> hp(n_parts);
  std::vector<unsigned long long> tile_start(n_parts + 1), word_start(n_parts + 1);
  std::vector<int> plane_start(n_parts + 1);
  constexpr int TR = 8, TC = 4;
  int maxP = 0;
  auto fail = [&](int rc) {
    visacd_batch_destroy(b);
    return rc;
  };
  // Per-part device copies of points and Morton order.
  for (int p = 0; p < n_parts; ++p) {
    const int n = n_pts[p];
    if (n < 0 || (n > 0 && !pts[p]) || !self_bvhs[p] || !cage_bvhs[p] || n_planes[p] < 0 ||
        (n_planes[p] > 0 && !planes[p])) {
      set_error("batch_create: bad part %d", p);
      return fail(VISACD_ERR_INVALID_ARG);
    }
    if (self_bvhs[p]->depth > kStack || cage_bvhs[p]->depth > kStack ||
        (self_bvhs[p]->nt > 0 && self_bvhs[p]->nv != n)) {
      set_error("batch_create: part %d BVH does not match its points or is too deep", p);
      return fail(VISACD_ERR_INVALID_ARG);
    }
    BatchPart& P = hp[p];
    memset(&P, 0, sizeof(P));
    P.n = n;
    float* dpts = nullptr;
    int rc = balloc(b, (size_t)std::max(n, 1) * 12, (void**)&dpts);
    if (rc) return fail(rc);
    if (n) {
      cudaError_t e = cudaMemcpyAsync(dpts, pts[p], (size_t)n * 12, cudaMemcpyHostToDevice, ctx->stream);
      if (e != cudaSuccess) { set_error("batch_create: copy failed"); return fail(VISACD_ERR_CUDA); }
    }
    P.pts = dpts;
    // Morton order via the context's sort (same as the single-part path).
    uint32_t* perm = nullptr;
    rc = balloc(b, (size_t)std::max(n, 1) * 4, (void**)&perm);
    if (rc) return fail(rc);
    if (n > 1) {
      rc = vis_morton_order(ctx, dpts, n, perm);
      if (rc) return fail(rc);
    }
    P.perm = perm;
    P.ntr = (n + TR - 1) / TR;
    P.ntc = (n + TC - 1) / TC;
    std::vector<unsigned long long> rs(P.ntr + 1, 0);
    for (int r = 0; r < P.ntr; ++r) {
      long long c = (long long)P.ntc - ((long long)r * TR) / TC;
      rs[r + 1] = rs[r] + (unsigned long long)(c > 0 ? c : 0);
    }
    unsigned long long* drs = nullptr;
    rc = balloc(b, (size_t)(P.ntr + 1) * 8, (void**)&drs);
    if (rc) return fail(rc);
    cudaMemcpy(drs, rs.data(), (size_t)(P.ntr + 1) * 8, cudaMemcpyHostToDevice);
    P.row_start = drs;
    P.tile_begin = b->total_tiles;
    tile_start[p] = b->total_tiles;
    b->total_tiles += n > 1 ? rs[P.ntr] : 0;
    const unsigned long long np = (unsigned long long)n * (n > 0 ? n - 1 : 0) / 2;
    b->total_pairs += np;
    P.word_begin = b->total_words;
    word_start[p] = b->total_words;
    P.nwords = (np + 31) / 32;
    b->total_words += P.nwords;
    P.self_nodes = self_bvhs[p]->nodes;
    P.self_tris = self_bvhs[p]->tris;
    P.self_nt = self_bvhs[p]->nt;
    P.cage_nodes = cage_bvhs[p]->nodes;
    P.cage_tris = cage_bvhs[p]->tris;
    P.cage_nt = cage_bvhs[p]->nt;
    P.plane_begin = (int)b->total_planes;
    plane_start[p] = (int)b->total_planes;
    P.P = n_planes[p];
    b->part_P.push_back(n_planes[p]);
    b->total_planes += n_planes[p];
    maxP = std::max(maxP, n_planes[p]);
    // FP32 rounding statistics of the part's points (max |coordinate|).
    float mx[3] = {0, 0, 0};
    for (int i = 0; i < n; ++i)
      for (int a = 0; a < 3; ++a) {
        float x = pts[p][3 * (int64_t)i + a];
        if (std::isfinite(x)) mx[a] = std::max(mx[a], std::fabs(x));
      }
    for (int a = 0; a < 3; ++a) memcpy(&P.stats[a], &mx[a], 4);
  }
  tile_start[n_parts] = b->total_tiles;
  word_start[n_parts] = b->total_words;
  plane_start[n_parts] = (int)b->total_planes;
  b->K = maxP > 2 * kScoreThreads * 4 ? 4 : (maxP > kScoreThreads * 2 ? 2 : 1);
  b->groups = std::max(1, (maxP + kScoreThreads * b->K - 1) / (kScoreThreads * b->K));
  b->edge_cap = edge_capacity > 0 ? (unsigned long long)edge_capacity : std::max(1ull, b->total_pairs / 64 + 4096);
  b->rec_cap = b->edge_cap + 256ull * n_parts;
  const unsigned long long max_blocks = b->rec_cap / 256 + n_parts;
  unsigned long long rc_all = (unsigned long long)b->total_planes * max_blocks;
  b->recheck_cap = (unsigned)std::min<unsigned long long>(std::max<unsigned long long>(1ull << 20, rc_all / 128), 1ull << 30);
  int rc = VISACD_OK;
  rc = rc ? rc : balloc(b, (size_t)n_parts * sizeof(BatchPart), (void**)&b->d_parts);
  rc = rc ? rc : balloc(b, (size_t)n_parts * sizeof(BatchDyn), (void**)&b->d_dyn);
  rc = rc ? rc : balloc(b, (size_t)(n_parts + 1) * 8, (void**)&b->d_tile_start);
  rc = rc ? rc : balloc(b, (size_t)(n_parts + 1) * 8, (void**)&b->d_word_start);
  rc = rc ? rc : balloc(b, (size_t)(n_parts + 1) * 4, (void**)&b->d_plane_start);
  rc = rc ? rc : balloc(b, (size_t)b->total_words * 4, (void**)&b->d_bits);
  rc = rc ? rc : balloc(b, (size_t)b->total_words * 4, (void**)&b->d_wcount);
  rc = rc ? rc : balloc(b, (size_t)(b->total_words + 1) * 8, (void**)&b->d_woff);
  rc = rc ? rc : balloc(b, (size_t)b->edge_cap * 8, (void**)&b->d_edges);
  rc = rc ? rc : balloc(b, (size_t)b->rec_cap * sizeof(EdgeRec), (void**)&b->d_recs);
  rc = rc ? rc : balloc(b, (size_t)std::max<int64_t>(b->total_planes, 1) * 8, (void**)&b->d_score_q);
  rc = rc ? rc : balloc(b, (size_t)std::max<int64_t>(b->total_planes, 1) * 8, (void**)&b->d_scores);
  rc = rc ? rc : balloc(b, (size_t)n_parts * 4, (void**)&b->d_argmax);
  rc = rc ? rc : balloc(b, (size_t)b->recheck_cap * sizeof(uint2), (void**)&b->d_recheck);
  rc = rc ? rc : balloc(b, sizeof(BatchCounters), (void**)&b->d_cnt);
  rc = rc ? rc : balloc(b, (size_t)std::max<int64_t>(b->total_planes, 1) * 16, (void**)&b->d_planes);
  if (rc) return fail(rc);
  std::vector<float> allp((size_t)b->total_planes * 4);
  for (int p = 0; p < n_parts; ++p)
    memcpy(allp.data() + 4 * (size_t)plane_start[p], planes[p], (size_t)n_planes[p] * 16);
  cudaMemcpy(b->d_planes, allp.data(), allp.size() * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(b->d_parts, hp.data(), hp.size() * sizeof(BatchPart), cudaMemcpyHostToDevice);
  cudaMemcpy(b->d_tile_start, tile_start.data(), tile_start.size() * 8, cudaMemcpyHostToDevice);
  cudaMemcpy(b->d_word_start, word_start.data(), word_start.size() * 8, cudaMemcpyHostToDevice);
  cudaMemcpy(b->d_plane_start, plane_start.data(), plane_start.size() * 4, cudaMemcpyHostToDevice);
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    set_error("batch_create: %s", cudaGetErrorString(e));
    return fail(VISACD_ERR_CUDA);
  }
  *out = b;
  return VISACD_OK;
}

extern "C" int visacd_batch_run(visacd_ctx* ctx, visacd_batch* b, int use_graph) {
  VCHECK(ctx && b, VISACD_ERR_INVALID_ARG, "batch_run: null argument");
  VCUDA(cudaSetDevice(ctx->device));
  if (!use_graph) {
    VTRY(batch_sequence(ctx, b));
    ctx->launches += 10;
    return VISACD_OK;
  }
  if (!b->exec) {
    // The scan scratch must exist before capture (capture cannot allocate);
    // per-kernel timing events stay out of the graph.
    VTRY(ensure_slot(ctx, kSlotScanScratch, ((b->total_words + 2047) / 2048 + 2) * sizeof(uint64_t)));
    const bool timing = ctx->timing;
    ctx->timing = false;
    VCUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    int rc = batch_sequence(ctx, b);
    ctx->timing = timing;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    if (rc != VISACD_OK) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (e != cudaSuccess) {
      set_error("batch_run: graph capture failed: %s", cudaGetErrorString(e));
      return VISACD_ERR_CUDA;
    }
    b->graph = g;
    VCUDA(cudaGraphInstantiate(&b->exec, g, 0));
  }
  VCUDA(cudaGraphLaunch(b->exec, ctx->stream));
  ctx->launches += 10;
  return VISACD_OK;
}

extern "C" int visacd_batch_results(visacd_ctx* ctx, visacd_batch* b, int64_t* n_edges, double* scores,
                                    int32_t* argmax, uint32_t* edges, int64_t edge_capacity) {
  VCHECK(ctx && b, VISACD_ERR_INVALID_ARG, "batch_results: null argument");
  VCUDA(stream_wait(ctx));
  VTRY(check_status(ctx, "batch run"));
  std::vector<BatchDyn> dyn(b->n_parts);
  VCUDA(cudaMemcpy(dyn.data(), b->d_dyn, dyn.size() * sizeof(BatchDyn), cudaMemcpyDeviceToHost));
  BatchCounters c;
  VCUDA(cudaMemcpy(&c, b->d_cnt, sizeof(c), cudaMemcpyDeviceToHost));
  VCHECK(c.recheck_count <= b->recheck_cap, VISACD_ERR_CAPACITY,
         "batch: FP64 re-decision queue overflow (%u > %u)", c.recheck_count, b->recheck_cap);
  int64_t total = 0;
  for (int p = 0; p < b->n_parts; ++p) {
    if (n_edges) n_edges[p] = (int64_t)dyn[p].n_edges;
    total += (int64_t)dyn[p].n_edges;
  }
  VCHECK((unsigned long long)total <= b->edge_cap, VISACD_ERR_CAPACITY,
         "batch: %lld edges exceed the batch edge capacity %llu", (long long)total, b->edge_cap);
  if (scores && b->total_planes)
    VCUDA(cudaMemcpy(scores, b->d_scores, (size_t)b->total_planes * 8, cudaMemcpyDeviceToHost));
  if (argmax) VCUDA(cudaMemcpy(argmax, b->d_argmax, (size_t)b->n_parts * 4, cudaMemcpyDeviceToHost));
  if (edges) {
    VCHECK(edge_capacity >= total, VISACD_ERR_CAPACITY, "batch_results: edge buffer too small");
    if (total) VCUDA(cudaMemcpy(edges, b->d_edges, (size_t)total * 8, cudaMemcpyDeviceToHost));
  }
  return VISACD_OK;
}

extern "C" int visacd_batch_info(const visacd_batch* b, int64_t* total_pairs, int64_t* total_planes) {
  VCHECK(b, VISACD_ERR_INVALID_ARG, "batch_info: null batch");
  if (total_pairs) *total_pairs = (int64_t)b->total_pairs;
  if (total_planes) *total_planes = b->total_planes;
  return VISACD_OK;
}

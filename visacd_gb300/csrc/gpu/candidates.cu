// Candidate split planes and the split-plane search on the GPU.
//
// Reference: get_candidate_planes (lib/src/process.cpp:28-72) and the split
// search of decompose_iteration (lib/src/process.cpp:96-134). The host draws
// the edge indices from its engine (the draws are the random stream's and stay
// where the engine is); everything after the draw runs here:
//  0. A draw of an edge already drawn gives the same plane as its first draw,
//     which is always similar to it: the repeat is dropped whatever happened
//     to the first (kept, or dropped by a kept plane that is then similar to
//     the repeat as well). So only first draws are sent to the device, each
//     with its position in the draw sequence.
//  1. cand_planes_kernel: the perpendicular-bisector plane of each drawn edge
//     in FP64 with the host's operation order (explicit round-to-nearest
//     intrinsics, no contraction), so planes equal the host's bit for bit;
//     draws of edges shorter than 1e-6 are marked degenerate (the reference
//     skips them but still consumes the draw).
//  2. conflict_kernel (two passes: count, fill): for every pair j < k of valid
//     candidates, "k is similar to j" — |n_k . n_j| > cos 5 deg and
//     |d_k - d_j| < 1e-3, the reference's test in its FP64 order — over a
//     triangle of 256 x 256 tiles, with an FP32 offset pre-filter (a margin
//     far above the FP32 rounding of the offsets) in front of the FP64 test.
//     The similar earlier candidates of each k form a CSR list.
//  3. resolve_kernel (one CTA): the reference keeps candidate k when no kept
//     earlier candidate is similar to it. Kept / dropped are decided in rounds:
//     k is dropped as soon as one of its earlier neighbours is kept, kept once
//     all of them are dropped. The earliest undecided candidate always decides
//     (everything before it is decided), so at most D rounds; in practice a few.
//  4. compact_kernel (one CTA): ranks of the kept candidates in draw order;
//     the first num_planes are the result (the reference stops drawing once it
//     holds num_planes planes, so the draws used end at the num_planes-th).
// The split search then scores the kept planes and the flat-surface planes
// with the plane-scoring kernels (flat scores times flat_k) and takes the
// first maximum in the reference's order, all on the device; one small
// read-back returns the chosen plane.
#include "score_device.cuh"

namespace vgpu {

namespace {

constexpr int kCandTile = 256;

// A plane a x + b y + c z + d in FP64 (x, y, z, w = a, b, c, d).
struct __align__(32) Plane64 {
  double x, y, z, w;
};
enum : uint8_t { kUndecided = 0, kKept = 1, kDropped = 2, kInvalid = 3 };

// The perpendicular-bisector plane of edge idx (lib/src/process.cpp:45-53) in
// FP64 with the host's operation order; false for edges shorter than 1e-6.
__device__ __forceinline__ bool edge_bisector(const double* __restrict__ verts,
                                              const uint32_t* __restrict__ edges, int64_t idx,
                                              Plane64& pl) {
  const uint32_t i0 = edges[2 * idx], i1 = edges[2 * idx + 1];
  const double* p1 = verts + 3 * (int64_t)i0;
  const double* p2 = verts + 3 * (int64_t)i1;
  const double nx = __dsub_rn(p2[0], p1[0]), ny = __dsub_rn(p2[1], p1[1]), nz = __dsub_rn(p2[2], p1[2]);
  const double l =
      __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(nx, nx), __dmul_rn(ny, ny)), __dmul_rn(nz, nz)));
  if (l < 1e-6) return false;
  const double a = __ddiv_rn(nx, l), b = __ddiv_rn(ny, l), c = __ddiv_rn(nz, l);
  const double mx = __dmul_rn(__dadd_rn(p1[0], p2[0]), 0.5);
  const double my = __dmul_rn(__dadd_rn(p1[1], p2[1]), 0.5);
  const double mz = __dmul_rn(__dadd_rn(p1[2], p2[2]), 0.5);
  const double d = -__dadd_rn(__dadd_rn(__dmul_rn(a, mx), __dmul_rn(b, my)), __dmul_rn(c, mz));
  pl = Plane64{a, b, c, d};
  return true;
}

__global__ void cand_planes_kernel(const double* __restrict__ verts, int32_t n,
                                   const uint32_t* __restrict__ edges, int64_t E,
                                   const int32_t* __restrict__ draws, int32_t D,
                                   Plane64* __restrict__ planes, float* __restrict__ d32,
                                   uint8_t* __restrict__ state) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < D; k += gridDim.x * blockDim.x) {
    const int32_t idx = draws[k];
    uint8_t st = kInvalid;
    Plane64 pl = Plane64{0.0, 0.0, 0.0, 0.0};
    if (idx >= 0 && (int64_t)idx < E && edges[2 * (int64_t)idx] < (uint32_t)n &&
        edges[2 * (int64_t)idx + 1] < (uint32_t)n) {
      if (edge_bisector(verts, edges, idx, pl)) {
        st = kUndecided;
      } else {
        pl = Plane64{0.0, 0.0, 0.0, 0.0};
      }
    }
    planes[k] = pl;
    d32[k] = (float)pl.w;
    state[k] = st;
  }
}

// Tile x of the lower triangle (kt >= jt) of T x T tiles.
__device__ __forceinline__ void tri_tile(int x, int& kt, int& jt) {
  int r = (int)((sqrt(8.0 * x + 1.0) - 1.0) * 0.5);
  while ((r + 1) * (r + 2) / 2 <= x) ++r;
  while (r * (r + 1) / 2 > x) --r;
  kt = r;
  jt = x - r * (r + 1) / 2;
}

// Pass 0 counts, pass 1 fills the CSR lists of similar earlier candidates.
template <int PASS>
__global__ void __launch_bounds__(kCandTile) conflict_kernel(
    const Plane64* __restrict__ planes, const float* __restrict__ d32,
    const uint8_t* __restrict__ state, int32_t D, double normal_eps, uint32_t* __restrict__ count,
    const uint64_t* __restrict__ offset, uint32_t* __restrict__ fill, int32_t* __restrict__ list) {
  __shared__ Plane64 spl[kCandTile];
  __shared__ float sd[kCandTile];
  __shared__ uint8_t sst[kCandTile];
  int kt, jt;
  tri_tile(blockIdx.x, kt, jt);
  const int j0 = jt * kCandTile;
  const int j = j0 + threadIdx.x;
  if (j < D) {
    spl[threadIdx.x] = planes[j];
    sd[threadIdx.x] = d32[j];
    sst[threadIdx.x] = state[j];
  } else {
    sst[threadIdx.x] = kInvalid;
  }
  __syncthreads();
  const int k = kt * kCandTile + threadIdx.x;
  if (k >= D || state[k] == kInvalid) return;
  const Plane64 pk = planes[k];
  const float dk = d32[k];
  const int jend = min(kCandTile, k - j0);  // earlier candidates only
  uint32_t c = 0;
  for (int t = 0; t < jend; ++t) {
    if (sst[t] == kInvalid) continue;
    if (!(fabsf(dk - sd[t]) < 1.001e-3f)) continue;  // FP32 offsets differ by < 1e-6 from FP64
    const Plane64 pj = spl[t];
    const double dt =
        fabs(__dadd_rn(__dadd_rn(__dmul_rn(pk.x, pj.x), __dmul_rn(pk.y, pj.y)), __dmul_rn(pk.z, pj.z)));
    if (dt > normal_eps && fabs(__dsub_rn(pk.w, pj.w)) < 1e-3) {
      if (PASS == 0) {
        ++c;
      } else {
        const uint32_t pos = atomicAdd(&fill[k], 1u);
        list[offset[k] + pos] = j0 + t;
      }
    }
  }
  if (PASS == 0 && c) atomicAdd(&count[k], c);
}

// Greedy keep-first resolution in rounds (one CTA). status bit on overrun.
__global__ void resolve_kernel(const uint64_t* __restrict__ offset, const int32_t* __restrict__ list,
                               uint8_t* __restrict__ state, int32_t D, unsigned* __restrict__ status) {
  __shared__ int undecided;
  volatile uint8_t* st = state;
  bool done = false;
  for (int round = 0; round <= D + 1; ++round) {
    if (threadIdx.x == 0) undecided = 0;
    __syncthreads();
    for (int k = threadIdx.x; k < D; k += blockDim.x) {
      if (st[k] != kUndecided) continue;
      bool all_decided = true, any_kept = false;
      for (uint64_t q = offset[k]; q < offset[k + 1]; ++q) {
        const uint8_t s = st[list[q]];
        if (s == kKept) {
          any_kept = true;
          break;
        }
        if (s == kUndecided) all_decided = false;
      }
      if (any_kept) {
        st[k] = kDropped;
      } else if (all_decided) {
        st[k] = kKept;
      } else {
        undecided = 1;
      }
    }
    __syncthreads();
    if (!undecided) {
      done = true;
      break;
    }
    __syncthreads();
  }
  if (!done && threadIdx.x == 0) atomicOr(status, kStatusWorkOverrun);
}

// Ranks of kept candidates in draw order; the first num_planes are written
// out (FP64 and FP32). info[0] = planes out, info[1] = draws used (the
// position after the num_planes-th kept draw, or every draw).
__global__ void compact_kernel(const Plane64* __restrict__ planes, const uint8_t* __restrict__ state,
                               const int32_t* __restrict__ pos, int32_t D, int32_t all_draws,
                               int32_t num_planes, Plane64* __restrict__ out64,
                               float4* __restrict__ out32, int32_t* __restrict__ info) {
  __shared__ int warp_tot[32];
  __shared__ int carry_s;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int per = (D + blockDim.x - 1) / blockDim.x;
  const int k0 = tid * per, k1 = min(D, k0 + per);
  int mine = 0;
  for (int k = k0; k < k1; ++k) mine += state[k] == kKept;
  int incl = mine;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) warp_tot[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    int w = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0;
    int wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int v = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += v;
    }
    if (lane < 32) warp_tot[lane] = wi - w;  // exclusive prefix of warps
    if (lane == 31) carry_s = wi;             // total kept
  }
  __syncthreads();
  int rank = warp_tot[wid] + incl - mine;
  const int total = carry_s;
  for (int k = k0; k < k1; ++k) {
    if (state[k] != kKept) continue;
    if (rank < num_planes) {
      const Plane64 p = planes[k];
      out64[rank] = p;
      out32[rank] = make_float4((float)p.x, (float)p.y, (float)p.z, (float)p.w);
      if (rank == num_planes - 1) info[1] = pos[k] + 1;
    }
    ++rank;
  }
  if (tid == 0) {
    info[0] = min(total, num_planes);
    if (total < num_planes) info[1] = all_draws;
  }
}

__global__ void f64_to_f32_kernel(const double* __restrict__ in, float* __restrict__ out, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (float)in[i];
}

// Flat planes after the candidate slots, zero planes in the unused slots
// (score 0, never in the band, skipped by the arg-max).
__global__ void place_flat_kernel(const double* __restrict__ flat, int32_t F, int32_t cand_slots,
                                  const int32_t* __restrict__ info, Plane64* __restrict__ out64,
                                  float4* __restrict__ out32) {
  const int n_out = info[0];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cand_slots + F; i += gridDim.x * blockDim.x) {
    if (i < cand_slots) {
      if (i >= n_out) {
        out64[i] = Plane64{0.0, 0.0, 0.0, 0.0};
        out32[i] = make_float4(0.f, 0.f, 0.f, 0.f);
      }
    } else {
      const double* f = flat + 4 * (int64_t)(i - cand_slots);
      out64[i] = Plane64{f[0], f[1], f[2], f[3]};
      out32[i] = make_float4((float)f[0], (float)f[1], (float)f[2], (float)f[3]);
    }
  }
}

// First maximum over [kept candidates, flat planes x flat_k] in that order,
// compared as the reference compares them (lib/src/process.cpp:118-131): the
// scores are float, and a flat plane's score is multiplied by flat_k in double
// and stored back as float. Float rounding can make distinct exact sums equal,
// and then the first of them wins, as in the reference.
struct SplitOut {
  double plane[4];
  double score;
  int32_t index;      // in the reference's order (candidates, then flat planes); -1: none
  int32_t n_planes;   // kept candidates
  int32_t draws_used;
  uint32_t score_status;   // the scoring call's status bits
  uint32_t recheck_count;  // its FP64 queue demand
  uint32_t pad;
};

__global__ void split_argmax_kernel(const double* __restrict__ scores, const Plane64* __restrict__ planes,
                                    const int32_t* __restrict__ info, int32_t cand_slots, int32_t F,
                                    double flat_k, const unsigned* __restrict__ score_status,
                                    const unsigned* __restrict__ recheck_count,
                                    SplitOut* __restrict__ out) {
  const int n_out = info[0];
  const int total = n_out + F;
  float best = -1.0f;
  int best_i = 0x7fffffff;
  for (int r = threadIdx.x; r < total; r += blockDim.x) {
    const int slot = r < n_out ? r : cand_slots + (r - n_out);
    float s = __double2float_rn(scores[slot]);
    if (r >= n_out) s = __double2float_rn(__dmul_rn((double)s, flat_k));
    if (s > best || (s == best && r < best_i)) {
      best = s;
      best_i = r;
    }
  }
  __shared__ float sv[1024];
  __shared__ int si[1024];
  sv[threadIdx.x] = best;
  si[threadIdx.x] = best_i;
  __syncthreads();
  for (int o = blockDim.x / 2; o; o >>= 1) {
    if ((int)threadIdx.x < o) {
      const float v2 = sv[threadIdx.x + o];
      const int i2 = si[threadIdx.x + o];
      if (v2 > sv[threadIdx.x] || (v2 == sv[threadIdx.x] && i2 < si[threadIdx.x])) {
        sv[threadIdx.x] = v2;
        si[threadIdx.x] = i2;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const int r = si[0];
    out->n_planes = n_out;
    out->draws_used = info[1];
    out->score_status = score_status ? *score_status : 0u;
    out->recheck_count = recheck_count ? *recheck_count : 0u;
    if (total == 0 || r == 0x7fffffff) {
      out->index = -1;
      out->score = 0.0;
      for (int c = 0; c < 4; ++c) out->plane[c] = 0.0;
    } else {
      const int slot = r < n_out ? r : cand_slots + (r - n_out);
      const Plane64 p = planes[slot];
      out->index = r;
      out->score = (double)sv[0];
      out->plane[0] = p.x;
      out->plane[1] = p.y;
      out->plane[2] = p.z;
      out->plane[3] = p.w;
    }
  }
}

// ---- learned split search --------------------------------------------------
// Refinement of the proposer's planes: per proposal q, the kRefineK smallest
// (D, edge) pairs over the edges with a bisector plane b,
//   D = (2 - 2|c|) + dd^2,  c = n_q . n_b,  dd = (s d_q - d_b) / half,
//   s = +1 when c >= 0 else -1,
// in FP64 in this order. Each warp keeps a sorted list of 32 (key, edge)
// entries, lane l holding the l-th smallest; D maps to an unsigned key with the
// same order, so (key, edge) compares like (D, edge).
constexpr int kRefineK = 32;
constexpr int kRefineTile = 512;  // edges per block step; one warp per proposal
constexpr int kLearnedProps = 16;
constexpr int kRefineSlots = kLearnedProps * kRefineK;
constexpr int kProbeBase = kLearnedProps + kRefineSlots;  // first probe slot
constexpr unsigned long long kNoKey = ~0ull;
constexpr int32_t kNoEdge = 0x7fffffff;

struct __align__(16) RefineEntry {
  unsigned long long key;
  int32_t edge;
  int32_t pad;
};

__device__ __forceinline__ unsigned long long order_key(double v) {
  if (v != v) return kNoKey - 1;  // NaN after every number
  if (v == 0.0) v = 0.0;          // -0 with +0
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  return (b >> 63) ? ~b : (b | (1ull << 63));
}

__device__ __forceinline__ bool entry_less(unsigned long long ka, int32_t ia, unsigned long long kb,
                                           int32_t ib) {
  return ka < kb || (ka == kb && ia < ib);
}

// Offers one candidate per lane to the warp's sorted list (lk, li); all 32
// lanes call it. A candidate enters when it is below the list's last entry at
// its turn; the list stays sorted and holds distinct edges.
__device__ __forceinline__ void warp_offer(unsigned long long& lk, int32_t& li, unsigned long long ck,
                                           int32_t ci) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned long long tk = __shfl_sync(full, lk, 31);
  const int32_t ti = __shfl_sync(full, li, 31);
  unsigned want = __ballot_sync(full, entry_less(ck, ci, tk, ti));
  while (want) {
    const int src = __ffs(want) - 1;
    want &= want - 1;
    const unsigned long long xk = __shfl_sync(full, ck, src);
    const int32_t xi = __shfl_sync(full, ci, src);
    // Lanes whose entry lies after x: a suffix of the sorted list.
    const unsigned after = __ballot_sync(full, entry_less(xk, xi, lk, li));
    if (!after) continue;
    const int pos = __ffs(after) - 1;
    const unsigned long long uk = __shfl_up_sync(full, lk, 1);
    const int32_t ui = __shfl_up_sync(full, li, 1);
    if (lane == pos) {
      lk = xk;
      li = xi;
    } else if (lane > pos) {
      lk = uk;
      li = ui;
    }
  }
}

// Pass 1: block b scans edges [b chunk, (b + 1) chunk); warp q keeps
// proposal q's 32 nearest bisectors of the chunk and writes them to
// partial[b][q][0..32). The block computes each bisector once per tile.
__global__ void __launch_bounds__(kRefineTile) refine_partial_kernel(
    const double* __restrict__ verts, const uint32_t* __restrict__ edges, int64_t E,
    const double* __restrict__ props, double half, int64_t chunk, RefineEntry* __restrict__ partial) {
  __shared__ Plane64 tile[kRefineTile];
  __shared__ uint8_t valid[kRefineTile];
  const int q = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const double pa = props[4 * q], pb = props[4 * q + 1], pc = props[4 * q + 2], pd = props[4 * q + 3];
  unsigned long long lk = kNoKey;
  int32_t li = kNoEdge;
  const int64_t begin = (int64_t)blockIdx.x * chunk;
  const int64_t end = min(E, begin + chunk);
  for (int64_t base = begin; base < end; base += kRefineTile) {
    const int64_t i = base + threadIdx.x;
    Plane64 pl = Plane64{0.0, 0.0, 0.0, 0.0};
    valid[threadIdx.x] = (i < end) && edge_bisector(verts, edges, i, pl);
    tile[threadIdx.x] = pl;
    __syncthreads();
    for (int j = 0; j < kRefineTile; j += 32) {
      const int t = j + lane;
      unsigned long long ck = kNoKey;
      int32_t ci = kNoEdge;
      if (valid[t]) {
        const Plane64 b = tile[t];
        const double c = __dadd_rn(__dadd_rn(__dmul_rn(pa, b.x), __dmul_rn(pb, b.y)), __dmul_rn(pc, b.z));
        const double sg = c >= 0 ? 1.0 : -1.0;
        const double dd = __ddiv_rn(__dsub_rn(__dmul_rn(sg, pd), b.w), half);
        const double D = __dadd_rn(__dsub_rn(2.0, __dmul_rn(2.0, fabs(c))), __dmul_rn(dd, dd));
        ck = order_key(D);
        ci = (int32_t)(base + t);
      }
      warp_offer(lk, li, ck, ci);
    }
    __syncthreads();
  }
  partial[((int64_t)blockIdx.x * kLearnedProps + q) * kRefineK + lane] = RefineEntry{lk, li, 0};
}

// Pass 2 (one block of 16 warps): merges the blocks' lists per proposal,
// keeps the first `per` entries of each, and writes the union's bisector
// planes in edge order to out64/out32 [0, n) (zeros in [n, 512)); n to
// *n_refined.
__global__ void __launch_bounds__(kRefineTile) refine_merge_kernel(
    const RefineEntry* __restrict__ partial, int32_t blocks, int32_t per,
    const double* __restrict__ verts, const uint32_t* __restrict__ edges, Plane64* __restrict__ out64,
    float4* __restrict__ out32, int32_t* __restrict__ n_refined) {
  __shared__ int32_t sel[kRefineSlots];
  __shared__ int warp_base[kLearnedProps + 1];
  const int t = threadIdx.x, q = t >> 5, lane = t & 31;
  unsigned long long lk = kNoKey;
  int32_t li = kNoEdge;
  for (int b = 0; b < blocks; ++b) {
    const RefineEntry e = partial[((int64_t)b * kLearnedProps + q) * kRefineK + lane];
    warp_offer(lk, li, e.key, e.edge);
  }
  sel[t] = (lane < per) ? li : kNoEdge;
  __syncthreads();
  // Bitonic sort of the 512 edge indices, ascending.
  for (int k = 2; k <= kRefineSlots; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      const int x = t ^ j;
      if (x > t) {
        const int32_t a = sel[t], b = sel[x];
        if ((a > b) == ((t & k) == 0)) {
          sel[t] = b;
          sel[x] = a;
        }
      }
      __syncthreads();
    }
  }
  const int32_t v = sel[t];
  const bool keep = v != kNoEdge && (t == 0 || sel[t - 1] != v);
  const unsigned m = __ballot_sync(0xffffffffu, keep);
  if (lane == 0) warp_base[q + 1] = __popc(m);
  __syncthreads();
  if (t == 0) {
    warp_base[0] = 0;
    for (int w = 1; w <= kLearnedProps; ++w) warp_base[w] += warp_base[w - 1];
    *n_refined = warp_base[kLearnedProps];
  }
  __syncthreads();
  const int n = warp_base[kLearnedProps];
  if (keep) {
    const int pos = warp_base[q] + __popc(m & ((1u << lane) - 1u));
    Plane64 pl = Plane64{0.0, 0.0, 0.0, 0.0};
    edge_bisector(verts, edges, v, pl);
    out64[pos] = pl;
    out32[pos] = make_float4((float)pl.x, (float)pl.y, (float)pl.z, (float)pl.w);
  }
  if (t >= n) {
    out64[t] = Plane64{0.0, 0.0, 0.0, 0.0};
    out32[t] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

// The scored plane list of the learned search: [0, 16) proposals, [16, 528)
// refined (written by refine_merge_kernel), [528, 528 + probe_slots) the kept
// probe candidates (zeros after them), then the F flat planes.
__global__ void learned_assemble_kernel(const double* __restrict__ props, const Plane64* __restrict__ probe,
                                        const int32_t* __restrict__ cinfo, int32_t probe_slots,
                                        const double* __restrict__ flat, int32_t F,
                                        Plane64* __restrict__ out64, float4* __restrict__ out32) {
  const int n_probe = cinfo[0];
  const int total = kLearnedProps + probe_slots + F;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    Plane64 p = Plane64{0.0, 0.0, 0.0, 0.0};
    int slot;
    if (i < kLearnedProps) {
      p = Plane64{props[4 * i], props[4 * i + 1], props[4 * i + 2], props[4 * i + 3]};
      slot = i;
    } else if (i < kLearnedProps + probe_slots) {
      const int r = i - kLearnedProps;
      if (r < n_probe) p = probe[r];
      slot = kProbeBase + r;
    } else {
      const int r = i - kLearnedProps - probe_slots;
      p = Plane64{flat[4 * r], flat[4 * r + 1], flat[4 * r + 2], flat[4 * r + 3]};
      slot = kProbeBase + probe_slots + r;
    }
    out64[slot] = p;
    out32[slot] = make_float4((float)p.x, (float)p.y, (float)p.z, (float)p.w);
  }
}

struct LearnedOut {
  double plane[4];
  double score, best_prop, best_probe;
  int32_t index, n_refined, n_probe, draws_used, fallback;
  uint32_t score_status, recheck_count, pad;
};

// The decision over [proposals, refined, probe, flat x flat_k] (FP64 scores,
// as the host compares them): the best proposal or refined score, the best
// probe score (from 0), fallback when the former is below (1 - tol) x the
// latter, and the first maximum of all.
__global__ void learned_decide_kernel(const double* __restrict__ scores, const Plane64* __restrict__ planes,
                                      const int32_t* __restrict__ n_refined_p,
                                      const int32_t* __restrict__ cinfo, int32_t probe_slots, int32_t F,
                                      double flat_k, double tol, const unsigned* __restrict__ score_status,
                                      const unsigned* __restrict__ recheck_count,
                                      LearnedOut* __restrict__ out) {
  const int n_ref = *n_refined_p, n_probe = cinfo[0];
  const int n_prop = kLearnedProps + n_ref;
  const int total = n_prop + n_probe + F;
  double best = -1.0 / 0.0, bprop = -1.0 / 0.0, bprobe = 0.0;
  int best_r = 0x7fffffff;
  for (int r = threadIdx.x; r < total; r += blockDim.x) {
    int slot;
    double v;
    if (r < n_prop) {
      slot = r;
      v = scores[slot];
      bprop = fmax(bprop, v);
    } else if (r < n_prop + n_probe) {
      slot = kProbeBase + (r - n_prop);
      v = scores[slot];
      bprobe = fmax(bprobe, v);
    } else {
      slot = kProbeBase + probe_slots + (r - n_prop - n_probe);
      v = __dmul_rn(scores[slot], flat_k);
    }
    if (v > best || (v == best && r < best_r)) {
      best = v;
      best_r = r;
    }
  }
  __shared__ double sv[1024], sp[1024], sq[1024];
  __shared__ int si[1024];
  sv[threadIdx.x] = best;
  si[threadIdx.x] = best_r;
  sp[threadIdx.x] = bprop;
  sq[threadIdx.x] = bprobe;
  __syncthreads();
  for (int o = blockDim.x / 2; o; o >>= 1) {
    if ((int)threadIdx.x < o) {
      const int u = threadIdx.x + o;
      if (sv[u] > sv[threadIdx.x] || (sv[u] == sv[threadIdx.x] && si[u] < si[threadIdx.x])) {
        sv[threadIdx.x] = sv[u];
        si[threadIdx.x] = si[u];
      }
      sp[threadIdx.x] = fmax(sp[threadIdx.x], sp[u]);
      sq[threadIdx.x] = fmax(sq[threadIdx.x], sq[u]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const int r = si[0];
    out->n_refined = n_ref;
    out->n_probe = n_probe;
    out->draws_used = cinfo[1];
    out->best_prop = sp[0];
    out->best_probe = sq[0];
    out->fallback = sp[0] < __dmul_rn(__dsub_rn(1.0, tol), sq[0]) ? 1 : 0;
    out->score_status = score_status ? *score_status : 0u;
    out->recheck_count = recheck_count ? *recheck_count : 0u;
    const int slot = r < n_prop ? r
                     : (r < n_prop + n_probe ? kProbeBase + (r - n_prop)
                                             : kProbeBase + probe_slots + (r - n_prop - n_probe));
    const Plane64 p = planes[slot];
    out->index = r;
    out->score = sv[0];
    out->plane[0] = p.x;
    out->plane[1] = p.y;
    out->plane[2] = p.z;
    out->plane[3] = p.w;
  }
}

// Scratch of one candidate-plane generation, carved from the context's slot.
struct CandScratch {
  Plane64* planes;   // D
  float* d32;        // D
  uint8_t* state;    // D
  uint32_t* count;   // D
  uint32_t* fill;    // D
  uint64_t* offset;  // D + 1
  int32_t* info;     // 4
  int32_t* draws;    // D (first draws)
  int32_t* pos;      // D (their positions in the draw sequence)
  Plane64* out64;    // slots
  float4* out32;     // slots
  double* verts;     // 3 n
  uint32_t* edges;   // 2 E
  double* flat;      // 4 F
  SplitOut* split;   // 1
};

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// Uploads the inputs and runs steps 1-4; the kept planes land in s.out64 /
// s.out32 [0, info[0]), the draws used in info[1].
int generate(visacd_ctx* ctx, const double* verts, int32_t n, const uint32_t* edges, int64_t E,
             const int32_t* draws, int32_t D, int32_t num_planes, const double* flat, int32_t F,
             int32_t slots, CandScratch& s) {
  if (num_planes == 0) D = 0;  // the reference's loop does not draw at all
  // First draws of each edge and their positions.
  std::vector<int32_t> uniq, upos;
  {
    uniq.reserve(D);
    upos.reserve(D);
    if (E <= (1LL << 26)) {
      std::vector<uint8_t> seen((size_t)E, 0);
      for (int32_t k = 0; k < D; ++k)
        if (!seen[(size_t)draws[k]]) {
          seen[(size_t)draws[k]] = 1;
          uniq.push_back(draws[k]);
          upos.push_back(k);
        }
    } else {
      std::unordered_map<int32_t, char> seen;
      for (int32_t k = 0; k < D; ++k)
        if (seen.emplace(draws[k], 1).second) {
          uniq.push_back(draws[k]);
          upos.push_back(k);
        }
    }
  }
  const int32_t all_draws = D;
  D = (int32_t)uniq.size();
  const size_t b_planes = align256((size_t)D * sizeof(Plane64)), b_d32 = align256((size_t)D * 4),
               b_state = align256((size_t)D), b_cnt = align256((size_t)D * 4),
               b_off = align256((size_t)(D + 1) * 8), b_info = 256, b_draws = align256((size_t)D * 4),
               b_pos = align256((size_t)D * 4),
               b_o64 = align256((size_t)slots * sizeof(Plane64)),
               b_o32 = align256((size_t)slots * sizeof(float4)),
               b_verts = align256((size_t)n * 24), b_edges = align256((size_t)E * 8),
               b_flat = align256((size_t)F * 32), b_split = align256(sizeof(SplitOut));
  const size_t total = b_planes + b_d32 + b_state + 2 * b_cnt + b_off + b_info + b_draws + b_pos + b_o64 +
                       b_o32 + b_verts + b_edges + b_flat + b_split;
  VTRY(ensure_slot(ctx, kSlotCandidates, total));
  char* p = slot<char>(ctx, kSlotCandidates);
  auto take = [&](size_t b) {
    char* r = p;
    p += b;
    return r;
  };
  s.planes = reinterpret_cast<Plane64*>(take(b_planes));
  s.d32 = reinterpret_cast<float*>(take(b_d32));
  s.state = reinterpret_cast<uint8_t*>(take(b_state));
  s.count = reinterpret_cast<uint32_t*>(take(b_cnt));
  s.fill = reinterpret_cast<uint32_t*>(take(b_cnt));
  s.offset = reinterpret_cast<uint64_t*>(take(b_off));
  s.info = reinterpret_cast<int32_t*>(take(b_info));
  s.draws = reinterpret_cast<int32_t*>(take(b_draws));
  s.pos = reinterpret_cast<int32_t*>(take(b_pos));
  s.out64 = reinterpret_cast<Plane64*>(take(b_o64));
  s.out32 = reinterpret_cast<float4*>(take(b_o32));
  s.verts = reinterpret_cast<double*>(take(b_verts));
  s.edges = reinterpret_cast<uint32_t*>(take(b_edges));
  s.flat = reinterpret_cast<double*>(take(b_flat));
  s.split = reinterpret_cast<SplitOut*>(take(b_split));
  {
    Stager up(ctx);
    VTRY(up.reserve((size_t)n * 24 + (size_t)E * 8 + (size_t)D * 8 + (size_t)F * 32, 5));
    if (n) VTRY(up.put(s.verts, verts, (size_t)n * 24));
    if (E) VTRY(up.put(s.edges, edges, (size_t)E * 8));
    if (D) VTRY(up.put(s.draws, uniq.data(), (size_t)D * 4));
    if (D) VTRY(up.put(s.pos, upos.data(), (size_t)D * 4));
    if (F) VTRY(up.put(s.flat, flat, (size_t)F * 32));
  }
  VCUDA(cudaMemsetAsync(s.info, 0, b_info, ctx->stream));
  if (D == 0) {
    const int32_t none[2] = {0, all_draws};
    VCUDA(cudaMemcpyAsync(s.info, none, 8, cudaMemcpyHostToDevice, ctx->stream));
    VCUDA(stream_wait(ctx));
    return VISACD_OK;
  }
  VCUDA(cudaMemsetAsync(s.count, 0, 2 * b_cnt, ctx->stream));
  VLAUNCH(ctx, kKCandidates, grid_for(D, 256, 4LL * ctx->sm_count), 256, 0, cand_planes_kernel,
          s.verts, n, s.edges, E, s.draws, D, s.planes, s.d32, s.state);
  const int T = (D + kCandTile - 1) / kCandTile;
  const unsigned tiles = (unsigned)(T * (T + 1) / 2);
  const double normal_eps = std::cos(5.0 * M_PI / 180.0);
  VLAUNCH(ctx, kKCandidates, tiles, kCandTile, 0, conflict_kernel<0>, s.planes, s.d32, s.state, D,
          normal_eps, s.count, (const uint64_t*)nullptr, (uint32_t*)nullptr, (int32_t*)nullptr);
  VTRY(exclusive_scan_u32_to_u64(ctx, s.count, s.offset, D));
  // The lists' total size is only known on the device: read it back (one
  // 8-byte copy) to size the list buffer.
  uint64_t* h = nullptr;
  VTRY(pinned(ctx, sizeof(uint64_t), (void**)&h));
  VCUDA(cudaMemcpyAsync(h, s.offset + D, sizeof(uint64_t), cudaMemcpyDeviceToHost, ctx->stream));
  VCUDA(stream_wait(ctx));
  const uint64_t n_links = *h;
  VTRY(ensure_slot(ctx, kSlotCandLinks, (size_t)(n_links > 0 ? n_links : 1) * 4));
  int32_t* list = slot<int32_t>(ctx, kSlotCandLinks);
  if (n_links) {
    VLAUNCH(ctx, kKCandidates, tiles, kCandTile, 0, conflict_kernel<1>, s.planes, s.d32, s.state, D,
            normal_eps, (uint32_t*)nullptr, s.offset, s.fill, list);
  }
  VLAUNCH(ctx, kKCandidates, 1, 1024, 0, resolve_kernel, s.offset, list, s.state, D, ctx->d_status);
  VLAUNCH(ctx, kKCandidates, 1, 1024, 0, compact_kernel, s.planes, s.state, s.pos, D, all_draws,
          num_planes, s.out64, s.out32, s.info);
  return VISACD_OK;
}

int check_args(const double* verts, int32_t n, const uint32_t* edges, int64_t E, const int32_t* draws,
               int32_t D, int32_t num_planes) {
  VCHECK(n >= 0 && E >= 0 && D >= 0 && num_planes >= 0, VISACD_ERR_INVALID_ARG,
         "candidate_planes: negative size");
  VCHECK(n == 0 || verts, VISACD_ERR_INVALID_ARG, "candidate_planes: verts is NULL");
  VCHECK(E == 0 || edges, VISACD_ERR_INVALID_ARG, "candidate_planes: edges is NULL");
  VCHECK(D == 0 || draws, VISACD_ERR_INVALID_ARG, "candidate_planes: draws is NULL");
  VCHECK(E < (1LL << 31), VISACD_ERR_INVALID_ARG, "candidate_planes: too many edges");
  VCHECK(indices_in_range(draws, D, E), VISACD_ERR_INVALID_ARG,
         "candidate_planes: a draw is outside [0, E)");
  VCHECK(indices_in_range(reinterpret_cast<const int32_t*>(edges), 2 * E, n), VISACD_ERR_INVALID_ARG,
         "candidate_planes: an edge index is outside [0, n)");
  return VISACD_OK;
}

}  // namespace

}  // namespace vgpu

using namespace vgpu;

extern "C" int visacd_candidate_planes(visacd_ctx* ctx, const double* verts, int32_t n,
                                       const uint32_t* edges, int64_t E, const int32_t* draws,
                                       int32_t n_draws, int32_t num_planes, double* planes_out,
                                       int32_t* n_planes, int32_t* draws_used) {
  VCHECK(ctx, VISACD_ERR_INVALID_ARG, "candidate_planes: null context");
  VTRY(check_args(verts, n, edges, E, n_draws ? draws : draws, n_draws, num_planes));
  VCHECK(planes_out || num_planes == 0, VISACD_ERR_INVALID_ARG, "candidate_planes: planes_out is NULL");
  VCUDA(cudaSetDevice(ctx->device));
  const int32_t slots = std::max(1, std::min(num_planes, n_draws));
  CandScratch s;
  VTRY(generate(ctx, verts, n, edges, E, draws, n_draws, num_planes, nullptr, 0, slots, s));
  int32_t* h = nullptr;
  VTRY(pinned(ctx, 16, (void**)&h));
  VCUDA(cudaMemcpyAsync(h, s.info, 8, cudaMemcpyDeviceToHost, ctx->stream));
  VCUDA(stream_wait(ctx));
  const int32_t got = h[0], used = h[1];
  VTRY(check_status(ctx, "candidate_planes"));
  if (got) {
    VCUDA(cudaMemcpyAsync(planes_out, s.out64, (size_t)got * 32, cudaMemcpyDeviceToHost, ctx->stream));
    VCUDA(stream_wait(ctx));
  }
  if (n_planes) *n_planes = got;
  if (draws_used) *draws_used = used;
  return VISACD_OK;
}


extern "C" int visacd_split_search(visacd_ctx* ctx, const double* verts, int32_t n,
                                   const uint32_t* edges, int64_t E, const int32_t* draws,
                                   int32_t n_draws, int32_t num_planes, const double* flat_planes,
                                   int32_t n_flat, double flat_k, double* best_plane,
                                   visacd_split_info* info) {
  VCHECK(ctx, VISACD_ERR_INVALID_ARG, "split_search: null context");
  VTRY(check_args(verts, n, edges, E, draws, n_draws, num_planes));
  VCHECK(n_flat >= 0 && (n_flat == 0 || flat_planes), VISACD_ERR_INVALID_ARG,
         "split_search: flat_planes is NULL");
  VCHECK(best_plane, VISACD_ERR_INVALID_ARG, "split_search: best_plane is NULL");
  VCUDA(cudaSetDevice(ctx->device));
  const int32_t cand_slots = std::max(0, std::min(num_planes, n_draws));
  const int32_t slots = std::max(1, cand_slots + n_flat);
  CandScratch s;
  VTRY(generate(ctx, verts, n, edges, E, draws, n_draws, num_planes, flat_planes, n_flat, slots, s));
  VLAUNCH(ctx, kKCandidates, grid_for(cand_slots + n_flat, 256, 64), 256, 0, place_flat_kernel, s.flat,
          n_flat, cand_slots, s.info, s.out64, s.out32);
  const int32_t P = cand_slots + n_flat;
  VTRY(ensure_slot(ctx, kSlotPoints, (size_t)(n > 0 ? n : 1) * 12));
  float* pts32 = slot<float>(ctx, kSlotPoints);
  if (n) {
    VLAUNCH(ctx, kKCandidates, grid_for(3LL * n, 256, 4LL * ctx->sm_count), 256, 0, f64_to_f32_kernel,
            s.verts, pts32, 3LL * n);
  }
  VTRY(ensure_slot(ctx, kSlotScores, (size_t)(P > 0 ? P : 1) * 8));
  double* scores = slot<double>(ctx, kSlotScores);
  // Scoring as visacd_score_planes (device pointers); its status words are
  // copied into the read-back, and a full FP64 queue is rerun with room for
  // every queued block.
  unsigned rcap = score_recheck_capacity(P, E);
  SplitOut* h = nullptr;
  const size_t o_st = (sizeof(SplitOut) + 15) & ~size_t(15);
  VTRY(pinned(ctx, o_st + 16, (void**)&h));
  uint32_t* hst = reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(h) + o_st);
  for (int attempt = 0; attempt < 2; ++attempt) {
    const unsigned* st_status = nullptr;
    const unsigned* st_count = nullptr;
    VTRY(score_planes_device_async(ctx, reinterpret_cast<const float*>(s.out32), P, pts32, n, s.edges,
                                   E, scores, rcap, &st_status, &st_count));
    VLAUNCH(ctx, kKCandidates, 1, 1024, 0, split_argmax_kernel, scores, s.out64, s.info, cand_slots,
            n_flat, flat_k, st_status, st_count, s.split);
    VCUDA(cudaMemcpyAsync(h, s.split, sizeof(SplitOut), cudaMemcpyDeviceToHost, ctx->stream));
    VCUDA(cudaMemcpyAsync(hst, ctx->d_status, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
    VCUDA(stream_wait(ctx));
    VCHECK(!(h->score_status & kStatusMbarrierTimeout), VISACD_ERR_DEVICE,
           "split_search: a bulk-copy wait of the scoring kernel timed out");
    if (!(h->score_status & kStatusRecheckOverflow)) break;
    VCHECK(attempt == 0, VISACD_ERR_DEVICE, "split_search: FP64 queue overflow after a rerun");
    rcap = h->recheck_count;
  }
  const SplitOut r = *h;
  VTRY(status_result(ctx, *hst, "split_search"));
  for (int c = 0; c < 4; ++c) best_plane[c] = r.plane[c];
  if (info) {
    info->best_index = r.index;
    info->n_candidates = r.n_planes;
    info->draws_used = r.draws_used;
    info->best_score = r.score;
  }
  return VISACD_OK;
}

extern "C" int visacd_learned_split_search(visacd_lp* lp, const double* verts, int32_t n,
                                           const uint32_t* edges, int64_t E, const float* center,
                                           float scale, double half, int32_t refine_k,
                                           const int32_t* probe_draws, int32_t n_probe_draws,
                                           int32_t probe_planes, const double* flat_planes, int32_t n_flat,
                                           double flat_k, double tolerance, double* best_plane,
                                           visacd_learned_split_info* info) {
  VCHECK(lp, VISACD_ERR_INVALID_ARG, "learned_split_search: null proposer");
  visacd_ctx* ctx = lp_context(lp);
  VCHECK(ctx, VISACD_ERR_INVALID_ARG, "learned_split_search: the proposer's context was destroyed");
  VTRY(check_args(verts, n, edges, E, probe_draws, n_probe_draws, probe_planes));
  VCHECK(n > 0 && E > 0, VISACD_ERR_INVALID_ARG, "learned_split_search: a part without visibility edges");
  VCHECK(center && best_plane, VISACD_ERR_INVALID_ARG, "learned_split_search: center or best_plane is NULL");
  VCHECK(scale > 0.f && half > 0.0, VISACD_ERR_INVALID_ARG,
         "learned_split_search: scale and half must be positive");
  VCHECK(refine_k >= 0 && refine_k <= kRefineK, VISACD_ERR_INVALID_ARG,
         "learned_split_search: refine_k must be in [0, 32]");
  VCHECK(n_flat >= 0 && (n_flat == 0 || flat_planes), VISACD_ERR_INVALID_ARG,
         "learned_split_search: flat_planes is NULL");
  VCUDA(cudaSetDevice(ctx->device));
  const int32_t probe_slots = std::max(0, std::min(probe_planes, n_probe_draws));
  CandScratch s;
  VTRY(generate(ctx, verts, n, edges, E, probe_draws, n_probe_draws, probe_planes, flat_planes, n_flat,
                std::max(1, probe_slots), s));
  VTRY(ensure_slot(ctx, kSlotPoints, (size_t)n * 12));
  float* pts32 = slot<float>(ctx, kSlotPoints);
  VLAUNCH(ctx, kKCandidates, grid_for(3LL * n, 256, 4LL * ctx->sm_count), 256, 0, f64_to_f32_kernel, s.verts,
          pts32, 3LL * n);

  // Refinement blocks: up to two per SM, each a whole number of tiles.
  const int64_t tiles = (E + kRefineTile - 1) / kRefineTile;
  const int64_t want = std::min<int64_t>(tiles, 2LL * ctx->sm_count);
  const int64_t chunk = ((tiles + want - 1) / want) * kRefineTile;
  const int32_t blocks = (int32_t)((E + chunk - 1) / chunk);
  const int32_t P = kProbeBase + probe_slots + n_flat;
  const size_t b_props = 256 * 2, b_partial = align256((size_t)blocks * kRefineSlots * sizeof(RefineEntry)),
               b_o64 = align256((size_t)P * sizeof(Plane64)), b_o32 = align256((size_t)P * sizeof(float4)),
               b_nref = 256, b_out = align256(sizeof(LearnedOut));
  VTRY(ensure_slot(ctx, kSlotLearned, b_props + b_partial + b_o64 + b_o32 + b_nref + b_out));
  char* p = slot<char>(ctx, kSlotLearned);
  double* props = reinterpret_cast<double*>(p);
  RefineEntry* partial = reinterpret_cast<RefineEntry*>(p + b_props);
  Plane64* L64 = reinterpret_cast<Plane64*>(p + b_props + b_partial);
  float4* L32 = reinterpret_cast<float4*>(p + b_props + b_partial + b_o64);
  int32_t* nref = reinterpret_cast<int32_t*>(p + b_props + b_partial + b_o64 + b_o32);
  LearnedOut* dout = reinterpret_cast<LearnedOut*>(p + b_props + b_partial + b_o64 + b_o32 + b_nref);

  VTRY(lp_propose_device(lp, pts32, n, s.edges, E, center, scale, props));
  VLAUNCH(ctx, kKLpRefine, blocks, kRefineTile, 0, refine_partial_kernel, s.verts, s.edges, E, props, half,
          chunk, partial);
  VLAUNCH(ctx, kKLpRefine, 1, kRefineTile, 0, refine_merge_kernel, partial, blocks, refine_k, s.verts,
          s.edges, L64 + kLearnedProps, L32 + kLearnedProps, nref);
  VLAUNCH(ctx, kKLpSplit, grid_for(kLearnedProps + probe_slots + n_flat, 256, 64), 256, 0,
          learned_assemble_kernel, props, s.out64, s.info, probe_slots, s.flat, n_flat, L64, L32);

  VTRY(ensure_slot(ctx, kSlotScores, (size_t)P * 8));
  double* scores = slot<double>(ctx, kSlotScores);
  unsigned rcap = score_recheck_capacity(P, E);
  LearnedOut* h = nullptr;
  const size_t o_st = (sizeof(LearnedOut) + 15) & ~size_t(15);
  VTRY(pinned(ctx, o_st + 16, (void**)&h));
  uint32_t* hst = reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(h) + o_st);
  for (int attempt = 0; attempt < 2; ++attempt) {
    const unsigned* st_status = nullptr;
    const unsigned* st_count = nullptr;
    VTRY(score_planes_device_async(ctx, reinterpret_cast<const float*>(L32), P, pts32, n, s.edges, E, scores,
                                   rcap, &st_status, &st_count));
    VLAUNCH(ctx, kKLpSplit, 1, 1024, 0, learned_decide_kernel, scores, L64, nref, s.info, probe_slots,
            n_flat, flat_k, tolerance, st_status, st_count, dout);
    VCUDA(cudaMemcpyAsync(h, dout, sizeof(LearnedOut), cudaMemcpyDeviceToHost, ctx->stream));
    VCUDA(cudaMemcpyAsync(hst, ctx->d_status, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
    VCUDA(stream_wait(ctx));
    VCHECK(!(h->score_status & kStatusMbarrierTimeout), VISACD_ERR_DEVICE,
           "learned_split_search: a bulk-copy wait of the scoring kernel timed out");
    if (!(h->score_status & kStatusRecheckOverflow)) break;
    VCHECK(attempt == 0, VISACD_ERR_DEVICE, "learned_split_search: FP64 queue overflow after a rerun");
    rcap = h->recheck_count;
  }
  const LearnedOut r = *h;
  VTRY(status_result(ctx, *hst, "learned_split_search"));
  for (int c = 0; c < 4; ++c) best_plane[c] = r.plane[c];
  if (info) {
    info->best_index = r.index;
    info->n_refined = r.n_refined;
    info->n_probe = r.n_probe;
    info->draws_used = r.draws_used;
    info->fallback = r.fallback;
    info->reserved = 0;
    info->best_score = r.score;
    info->best_proposal_score = r.best_prop;
    info->best_probe_score = r.best_probe;
  }
  return VISACD_OK;
}

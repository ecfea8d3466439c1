// Visibility edges: for each vertex pair (i < j), trace the segment p_i -> p_j
// against the part itself and against its cage; the pair is an edge iff the
// segment leaves the cage and does not cross the part.
//
// Reference: lib/ptx/ray_segments.cu:49-125 (one OptiX ray per pair, origin
// p_i, tmin 0.001, tmax |p_j - p_i|, any-hit), lib/src/intersections.cpp:327-385
// (edge iff hits cage && !hits self; pairs whose endpoints are both old are
// skipped when is_new is given; edges in row-major (i, j) order).
//
// GB300 design:
//  * Vertices are Morton-sorted; a persistent warp takes an 8 x 4 tile of
//    (origin, target) positions from a global counter, so the 32 segments of a
//    warp start and end close together (coherent traversal, dynamic balance).
//  * Warp-packet any-hit traversal of a 64-byte-node LBVH (both child boxes per
//    node): the warp follows one path (ballot of per-lane box tests), node
//    records are broadcast loads, a per-warp stack lives in shared memory; the
//    cage test runs first and the self test only for lanes whose segment
//    leaves the cage (few: most vertex pairs of a part are interior chords,
//    which cross neither surface).
//  * Segment-triangle test: edge functions W = D.(B x C), ... relative to the
//    origin in FP32 with an a-priori rounding bound (8 roundings per term,
//    bounded by 17u |D|_1 L^2). Only tests whose signs fall inside the bound
//    are re-decided in FP64 (the same formula as the oracle).
//  * Self-test end-vertex policy: triangles incident to i or j are skipped.
//  * Results land in a bitset over the reference's linear pair index; a
//    popcount / scan / emit pass compacts it into the row-major edge list.
#include <math.h>

#include "traverse.cuh"

namespace vgpu {

// Pairs from which a call (or a part of a batched call) builds and uses the
// cage's free-space grid: below this the grid costs about what the walk saves.
constexpr int64_t kFreeGridMinPairs = 1 << 22;

struct VisParams {
  const float* pts;
  int32_t n;
  const uint32_t* rows;    // sorted positions -> original ids (rows of the tile space)
  const uint32_t* cols;    // same for columns
  int32_t nr, nc;
  int triangular;          // 1: rows == cols and pairs with row < col
  const uint8_t* is_new;   // masked mode
  const int32_t* newrank;  // masked mode: position of a new vertex in rows, else INT_MAX
  const float4* self_nodes;
  const float4* self_tris;
  int32_t self_nt;
  const float4* cage_nodes;
  const float4* cage_tris;
  int32_t cage_nt;
  uint32_t* bitset;
  VisCounters* cnt;
  unsigned* status;
  unsigned long long total_tiles;
  int64_t ntc;                          // tile columns
  int64_t ntr;                          // tile rows
  const unsigned long long* row_start;  // triangular mode: first tile of each tile row
  FreeGridView cage_free;               // the cage's free-space grid (lb null: none)
  // After a walk: the tiles with lanes left for the traversal, and per such
  // tile the lanes that are done (no pair, degenerate, or cleared).
  unsigned long long* pend_tiles;       // null: no walk, every tile is traversed
  uint32_t* pend_done;
};

// Work item w -> tile (tr, tc). Rectangle mode: row-major. Triangular mode:
// tile row tr holds tile columns [floor(TR tr / TC), ntc); row_start is the
// exclusive prefix of those counts (binary search).
__device__ __forceinline__ void tile_of(const VisParams& P, unsigned long long w, int64_t& tr,
                                        int64_t& tc, int TR, int TC) {
  if (!P.triangular) {
    tr = (int64_t)(w / (unsigned long long)P.ntc);
    tc = (int64_t)(w % (unsigned long long)P.ntc);
    return;
  }
  if (TR >= TC) {
    // r = TR / TC is an integer and row t holds ntc - r t tiles (never
    // negative: r (ntr - 1) <= ntc), so row t starts at
    // S(t) = t ntc - r t (t - 1) / 2. Solve S(t) <= w < S(t + 1) in FP64 and
    // settle the rounding with the exact integers.
    const int64_t r = TR / TC, ntc = P.ntc;
    auto S = [&](int64_t t) { return t * ntc - r * t * (t - 1) / 2; };
    const double b = (double)ntc + 0.5 * (double)r;
    const double disc = b * b - 2.0 * (double)r * (double)w;
    int64_t t = (int64_t)((b - sqrt(disc > 0.0 ? disc : 0.0)) / (double)r);
    t = t < 0 ? 0 : (t > P.ntr - 1 ? P.ntr - 1 : t);
    while (t > 0 && (unsigned long long)S(t) > w) --t;
    while (t < P.ntr - 1 && (unsigned long long)S(t + 1) <= w) ++t;
    tr = t;
    tc = t * r + (int64_t)(w - (unsigned long long)S(t));
    return;
  }
  int64_t lo = 0, hi = P.ntr - 1;
  while (lo < hi) {
    int64_t mid = (lo + hi + 1) >> 1;
    if (P.row_start[mid] <= w) lo = mid; else hi = mid - 1;
  }
  tr = lo;
  tc = (tr * TR) / TC + (int64_t)(w - P.row_start[tr]);
}

__global__ void tile_row_counts_kernel(int64_t ntr, int64_t ntc, int TR, int TC,
                                       uint32_t* __restrict__ counts) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < ntr;
       r += (int64_t)gridDim.x * blockDim.x) {
    int64_t c = ntc - (r * TR) / TC;
    counts[r] = (uint32_t)(c > 0 ? c : 0);
  }
}

// Per-lane counters of a visibility launch, reduced over the warp at the end.
struct VisLaneCounters {
  unsigned long long pairs = 0, edges = 0, self = 0, cage = 0, deg = 0;
  unsigned rechecks = 0, status_bits = 0, visits = 0, tri_tests = 0;
};

// The pair of `lane` in tile w of P's tile space (original vertex ids i < j),
// or valid = false. The walk and the traversal kernels share it, so a tile's
// lane means the same pair in both.
template <int TR>
__device__ __forceinline__ bool lane_pair(const VisParams& P, unsigned long long w, int lane, uint32_t& i,
                                          uint32_t& j) {
  constexpr int TC = 32 / TR;
  int64_t tr, tc;
  tile_of(P, w, tr, tc, TR, TC);
  const int64_t a = tr * TR + lane / TC;
  const int64_t b = tc * TC + lane % TC;
  bool valid;
  uint32_t oi = 0, oj = 0;
  if (P.triangular) {
    valid = a < b && b < P.nc;
    if (valid) {
      oi = P.rows[a];
      oj = P.cols[b];
    }
  } else {
    valid = a < P.nr && b < P.nc;
    if (valid) {
      oi = P.rows[a];
      oj = P.cols[b];
      valid = oi != oj && (!P.is_new[oj] || P.newrank[oj] > a);
    }
  }
  i = min(oi, oj);
  j = max(oi, oj);
  return valid;
}

// One tile (work item w of P's tile space) for the calling warp: the cage
// test, then the self test for lanes whose segment leaves the cage, and the
// edge bits. After a free-space walk (walked) the walk has taken the tile's
// pair and degenerate counts, and `done` marks the lanes it settled: they
// take no part.
template <int TR>
__device__ __forceinline__ void vis_tile(const VisParams& P, unsigned long long w, int lane,
                                         VisLaneCounters& c, bool walked, uint32_t done) {
  const int64_t n = P.n;
  uint32_t i, j;
  const bool mine = !((done >> lane) & 1u);
  const bool valid = lane_pair<TR>(P, w, lane, i, j) && mine;
  Seg s;
  float3 p = make_float3(0.f, 0.f, 0.f), q = make_float3(0.f, 0.f, 0.f);
  if (valid) {
    if (!walked) ++c.pairs;
    p = make_float3(P.pts[3 * (int64_t)i], P.pts[3 * (int64_t)i + 1], P.pts[3 * (int64_t)i + 2]);
    q = make_float3(P.pts[3 * (int64_t)j], P.pts[3 * (int64_t)j + 1], P.pts[3 * (int64_t)j + 2]);
  }
  make_seg(s, p, q, (int)i, (int)j);
  bool active = valid;
  if (valid && !(seg_len(s) > 0.f)) {  // coincident endpoints (or NaN): never an edge
    ++c.deg;
    active = false;
  }
  if (!__ballot_sync(0xffffffffu, active)) return;
  // The cage first: few segments leave it, so the self test runs for few.
  s.exclude = false;
  const bool cage_hit = packet_any_hit(P.cage_nodes, P.cage_tris, P.cage_nt, s, P.pts, active,
                                       c.rechecks, c.status_bits, c.visits, c.tri_tests);
  if (active && cage_hit) ++c.cage;
  active = active && cage_hit;
  s.exclude = true;
  const bool self_hit = packet_any_hit(P.self_nodes, P.self_tris, P.self_nt, s, P.pts, active,
                                       c.rechecks, c.status_bits, c.visits, c.tri_tests);
  if (active && self_hit) ++c.self;
  if (active && !self_hit) {
    ++c.edges;
    const int64_t k = row_start(i, n) + (int64_t)(j - i - 1);
    atomicOr(&P.bitset[k >> 5], 1u << (k & 31));
  }
}

__device__ __forceinline__ void vis_flush_counters(VisCounters* cnt, unsigned* status, int lane,
                                                   VisLaneCounters& c) {
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    c.pairs += __shfl_xor_sync(0xffffffffu, c.pairs, o);
    c.edges += __shfl_xor_sync(0xffffffffu, c.edges, o);
    c.self += __shfl_xor_sync(0xffffffffu, c.self, o);
    c.cage += __shfl_xor_sync(0xffffffffu, c.cage, o);
    c.deg += __shfl_xor_sync(0xffffffffu, c.deg, o);
    c.rechecks += __shfl_xor_sync(0xffffffffu, c.rechecks, o);
    c.tri_tests += __shfl_xor_sync(0xffffffffu, c.tri_tests, o);
    c.status_bits |= __shfl_xor_sync(0xffffffffu, c.status_bits, o);
  }
  if (lane == 0) {
    atomicAdd(&cnt->pairs, c.pairs);
    atomicAdd(&cnt->edges, c.edges);
    atomicAdd(&cnt->self_hits, c.self);
    atomicAdd(&cnt->cage_hits, c.cage);
    atomicAdd(&cnt->degenerate, c.deg);
    atomicAdd(&cnt->rechecks, (unsigned long long)c.rechecks);
    atomicAdd(&cnt->node_visits, (unsigned long long)c.visits);
    atomicAdd(&cnt->tri_tests, (unsigned long long)c.tri_tests);
    if (c.status_bits) atomicOr(status, c.status_bits);
  }
}

template <int TR, int MINB>
__global__ void __launch_bounds__(kVisThreads, MINB) visibility_kernel(VisParams P) {
  const int lane = threadIdx.x & 31;
  VisLaneCounters c;
  // After a walk only the tiles it left are traversed (their count is on the
  // device, written by the walk kernel before this launch).
  const unsigned long long items = P.pend_tiles ? P.cnt->pending : P.total_tiles;
  for (int guard = 0; guard < (1 << 30); ++guard) {
    unsigned long long w = 0;
    if (lane == 0) w = atomicAdd(&P.cnt->work, 1ull);
    w = __shfl_sync(0xffffffffu, w, 0);
    if (w >= items) break;
    if (P.pend_tiles)
      vis_tile<TR>(P, P.pend_tiles[w], lane, c, true, P.pend_done[w]);
    else
      vis_tile<TR>(P, w, lane, c, false, 0u);
  }
  vis_flush_counters(P.cnt, P.status, lane, c);
}

// The free-space walk over P's tile space, before the traversal kernel. It
// takes the pair and degenerate counts of every tile, and lists the tiles
// that keep a lane for the traversal (P.pend_tiles) with the lanes that are
// done (no pair, degenerate, or cleared: the segment cannot hit the cage;
// traverse.cuh, trace_free). Few registers, so many warps per SM hide the
// latency of the walk's dependent grid reads.
template <int TR>
__global__ void __launch_bounds__(kVisThreads, 16) visibility_walk_kernel(VisParams P) {
  const int lane = threadIdx.x & 31;
  unsigned long long pairs = 0, deg = 0, cleared = 0, steps = 0;
  for (int guard = 0; guard < (1 << 30); ++guard) {
    unsigned long long w = 0;
    if (lane == 0) w = atomicAdd(&P.cnt->walk_work, 1ull);
    w = __shfl_sync(0xffffffffu, w, 0);
    if (w >= P.total_tiles) break;
    uint32_t i, j;
    bool done = true;
    if (lane_pair<TR>(P, w, lane, i, j)) {
      ++pairs;
      const float px = P.pts[3 * (int64_t)i], py = P.pts[3 * (int64_t)i + 1], pz = P.pts[3 * (int64_t)i + 2];
      const float dx = __fsub_rn(P.pts[3 * (int64_t)j], px), dy = __fsub_rn(P.pts[3 * (int64_t)j + 1], py),
                  dz = __fsub_rn(P.pts[3 * (int64_t)j + 2], pz);
      const float len =
          __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
      if (!(len > 0.f)) {  // coincident endpoints (or NaN): never an edge (as in vis_tile)
        ++deg;
      } else if (trace_free(P.cage_free, px, py, pz, dx, dy, dz, len, steps)) {
        ++cleared;
      } else {
        done = false;
      }
    }
    const unsigned m = __ballot_sync(0xffffffffu, done);
    if (lane == 0 && m != 0xffffffffu) {
      const unsigned long long k = atomicAdd(&P.cnt->pending, 1ull);
      P.pend_tiles[k] = w;
      P.pend_done[k] = m;
    }
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    pairs += __shfl_xor_sync(0xffffffffu, pairs, o);
    deg += __shfl_xor_sync(0xffffffffu, deg, o);
    cleared += __shfl_xor_sync(0xffffffffu, cleared, o);
    steps += __shfl_xor_sync(0xffffffffu, steps, o);
  }
  if (lane == 0) {
    if (pairs) atomicAdd(&P.cnt->pairs, pairs);
    if (deg) atomicAdd(&P.cnt->degenerate, deg);
    if (cleared) atomicAdd(&P.cnt->certified, cleared);
    if (steps) atomicAdd(&P.cnt->trace_steps, steps);
  }
}

// Many parts in one persistent launch: the work items of all parts are
// numbered consecutively (part p owns [tile_start[p], tile_start[p + 1])),
// and each warp finds the part of its item by binary search. Every part keeps
// its own tile space, mask and bitset region; the counters are shared.
__device__ __forceinline__ int part_of(const unsigned long long* __restrict__ tile_start, int n_parts,
                                       unsigned long long w) {
  int lo = 0, hi = n_parts - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (tile_start[mid] <= w) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// With pend_tiles (after visibility_multi_walk_kernel) only the listed tiles
// are traversed, with the lanes the walk settled left out.
template <int TR, int MINB>
__global__ void __launch_bounds__(kVisThreads, MINB)
    visibility_multi_kernel(const VisParams* __restrict__ parts, int n_parts,
                            const unsigned long long* __restrict__ tile_start,
                            unsigned long long total_tiles, VisCounters* __restrict__ cnt,
                            unsigned* __restrict__ status, const unsigned long long* __restrict__ pend_tiles,
                            const uint32_t* __restrict__ pend_done) {
  const int lane = threadIdx.x & 31;
  VisLaneCounters c;
  const unsigned long long items = pend_tiles ? cnt->pending : total_tiles;
  for (int guard = 0; guard < (1 << 30); ++guard) {
    unsigned long long w = 0;
    if (lane == 0) w = atomicAdd(&cnt->work, 1ull);
    w = __shfl_sync(0xffffffffu, w, 0);
    if (w >= items) break;
    if (pend_tiles) {
      const unsigned long long g = pend_tiles[w];
      const int p = part_of(tile_start, n_parts, g);
      vis_tile<TR>(parts[p], g - tile_start[p], lane, c, true, pend_done[w]);
    } else {
      const int p = part_of(tile_start, n_parts, w);
      vis_tile<TR>(parts[p], w - tile_start[p], lane, c, false, 0u);
    }
  }
  vis_flush_counters(cnt, status, lane, c);
}

// The free-space walk over all parts' tiles (as visibility_walk_kernel; parts
// without a grid leave every pair to the traversal). Pending tiles are listed
// by their global number.
template <int TR>
__global__ void __launch_bounds__(kVisThreads, 16)
    visibility_multi_walk_kernel(const VisParams* __restrict__ parts, int n_parts,
                                 const unsigned long long* __restrict__ tile_start,
                                 unsigned long long total_tiles, VisCounters* __restrict__ cnt,
                                 unsigned long long* __restrict__ pend_tiles, uint32_t* __restrict__ pend_done) {
  const int lane = threadIdx.x & 31;
  unsigned long long pairs = 0, deg = 0, cleared = 0, steps = 0;
  for (int guard = 0; guard < (1 << 30); ++guard) {
    unsigned long long w = 0;
    if (lane == 0) w = atomicAdd(&cnt->walk_work, 1ull);
    w = __shfl_sync(0xffffffffu, w, 0);
    if (w >= total_tiles) break;
    const int pi = part_of(tile_start, n_parts, w);
    const VisParams& P = parts[pi];
    uint32_t i, j;
    bool done = true;
    if (lane_pair<TR>(P, w - tile_start[pi], lane, i, j)) {
      ++pairs;
      const float px = P.pts[3 * (int64_t)i], py = P.pts[3 * (int64_t)i + 1], pz = P.pts[3 * (int64_t)i + 2];
      const float dx = __fsub_rn(P.pts[3 * (int64_t)j], px), dy = __fsub_rn(P.pts[3 * (int64_t)j + 1], py),
                  dz = __fsub_rn(P.pts[3 * (int64_t)j + 2], pz);
      const float len =
          __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
      if (!(len > 0.f)) {
        ++deg;
      } else if (P.cage_free.lb != nullptr && trace_free(P.cage_free, px, py, pz, dx, dy, dz, len, steps)) {
        ++cleared;
      } else {
        done = false;
      }
    }
    const unsigned m = __ballot_sync(0xffffffffu, done);
    if (lane == 0 && m != 0xffffffffu) {
      const unsigned long long k = atomicAdd(&cnt->pending, 1ull);
      pend_tiles[k] = w;
      pend_done[k] = m;
    }
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    pairs += __shfl_xor_sync(0xffffffffu, pairs, o);
    deg += __shfl_xor_sync(0xffffffffu, deg, o);
    cleared += __shfl_xor_sync(0xffffffffu, cleared, o);
    steps += __shfl_xor_sync(0xffffffffu, steps, o);
  }
  if (lane == 0) {
    if (pairs) atomicAdd(&cnt->pairs, pairs);
    if (deg) atomicAdd(&cnt->degenerate, deg);
    if (cleared) atomicAdd(&cnt->certified, cleared);
    if (steps) atomicAdd(&cnt->trace_steps, steps);
  }
}

// ---- vertex ordering ------------------------------------------------------
__global__ void point_bounds_kernel(const float* __restrict__ pts, int32_t n,
                                    VisCounters* __restrict__ c) {
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      float x = pts[3 * i + a];
      if (fabsf(x) < INFINITY) {
        lo[a] = fminf(lo[a], x);
        hi[a] = fmaxf(hi[a], x);
      }
    }
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) {
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
      hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
    }
  }
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      if (lo[a] <= hi[a]) {
        atomicMin(&c->pmin[a], f2o_v(lo[a]));
        atomicMax(&c->pmax[a], f2o_v(hi[a]));
      }
    }
  }
}

__device__ __forceinline__ uint64_t spread21_v(uint64_t x) {
  x &= 0x1fffffull;
  x = (x | (x << 32)) & 0x1f00000000ffffull;
  x = (x | (x << 16)) & 0x1f0000ff0000ffull;
  x = (x | (x << 8)) & 0x100f00f00f00f00full;
  x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
  x = (x | (x << 2)) & 0x1249249249249249ull;
  return x;
}

__global__ void point_morton_kernel(const float* __restrict__ pts, int32_t n,
                                    const VisCounters* __restrict__ c, int bits, uint64_t* __restrict__ keys,
                                    uint32_t* __restrict__ vals) {
  float lo[3], sc[3];
  const float top = (float)((1u << bits) - 1u);
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    lo[a] = o2f_v(c->pmin[a]);
    float ext = o2f_v(c->pmax[a]) - lo[a];
    sc[a] = ext > 0.f ? top / ext : 0.f;
  }
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    uint64_t q[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      float x = (pts[3 * i + a] - lo[a]) * sc[a];
      x = fminf(fmaxf(x, 0.f), top);
      q[a] = (uint64_t)x;
    }
    keys[i] = (spread21_v(q[0]) << 2) | (spread21_v(q[1]) << 1) | spread21_v(q[2]);
    vals[i] = (uint32_t)i;
  }
}

__global__ void new_flags_kernel(const uint32_t* __restrict__ perm, const uint8_t* __restrict__ is_new,
                                 int32_t n, uint32_t* __restrict__ flags) {
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n;
       s += (int64_t)gridDim.x * blockDim.x)
    flags[s] = is_new[perm[s]] ? 1u : 0u;
}

__global__ void new_rows_kernel(const uint32_t* __restrict__ perm, const uint32_t* __restrict__ flags,
                                const uint64_t* __restrict__ off, int32_t n,
                                uint32_t* __restrict__ rows, int32_t* __restrict__ newrank) {
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n;
       s += (int64_t)gridDim.x * blockDim.x) {
    uint32_t v = perm[s];
    if (flags[s]) {
      rows[off[s]] = v;
      newrank[v] = (int32_t)off[s];
    } else {
      newrank[v] = 0x7fffffff;
    }
  }
}

// ---- bitset compaction ----------------------------------------------------
__global__ void bit_popc_kernel(const uint32_t* __restrict__ bits, int64_t nw,
                                uint32_t* __restrict__ counts) {
  for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < nw;
       w += (int64_t)gridDim.x * blockDim.x)
    counts[w] = __popc(bits[w]);
}

__global__ void bit_emit_kernel(const uint32_t* __restrict__ bits, int64_t nw,
                                const uint64_t* __restrict__ off, int64_t n,
                                uint32_t* __restrict__ edges) {
  for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < nw;
       w += (int64_t)gridDim.x * blockDim.x) {
    uint32_t m = bits[w];
    if (!m) continue;
    uint64_t o = off[w];
    const int64_t k0 = w * 32;
    // Row of k0: largest i with row_start(i) <= k0.
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
      edges[2 * o] = (uint32_t)i;
      edges[2 * o + 1] = (uint32_t)j;
      ++o;
    }
  }
}

// Launch shapes the autotuner chooses from: tile rows (tile = TR x 32/TR pairs
// per warp) and the minimum resident CTAs per SM (register budget).
struct VisVariant {
  int tr;
  int minb;
};
static const VisVariant kVisVariants[] = {{8, 6}, {8, 8}, {4, 6}, {16, 6}, {2, 6}, {1, 6}, {32, 6}};
constexpr int kNumVisVariants = sizeof(kVisVariants) / sizeof(kVisVariants[0]);
// Untuned calls: 8 x 4 tiles at 8 resident CTAs per SM, the autotuner's pick
// on the s5 blob and the fastest on clipped parts (masked) by 3-6 %.
constexpr int kDefaultVisVariant = 1;

static int launch_vis_variant(visacd_ctx* ctx, int v, const VisParams& P) {
  const unsigned grid = (unsigned)(ctx->sm_count * kVisVariants[v].minb);
  if (P.pend_tiles != nullptr) {
    const unsigned wg = (unsigned)(ctx->sm_count * 16);
    switch (kVisVariants[v].tr) {
      case 8: VLAUNCH(ctx, kKVisWalk, wg, kVisThreads, 0, visibility_walk_kernel<8>, P); break;
      case 4: VLAUNCH(ctx, kKVisWalk, wg, kVisThreads, 0, visibility_walk_kernel<4>, P); break;
      case 16: VLAUNCH(ctx, kKVisWalk, wg, kVisThreads, 0, visibility_walk_kernel<16>, P); break;
      case 2: VLAUNCH(ctx, kKVisWalk, wg, kVisThreads, 0, visibility_walk_kernel<2>, P); break;
      case 1: VLAUNCH(ctx, kKVisWalk, wg, kVisThreads, 0, visibility_walk_kernel<1>, P); break;
      default: VLAUNCH(ctx, kKVisWalk, wg, kVisThreads, 0, visibility_walk_kernel<32>, P); break;
    }
  }
  switch (v) {
    case 0: VLAUNCH(ctx, kKVisibility, grid, kVisThreads, 0, (visibility_kernel<8, 6>), P); break;
    case 1: VLAUNCH(ctx, kKVisibility, grid, kVisThreads, 0, (visibility_kernel<8, 8>), P); break;
    case 2: VLAUNCH(ctx, kKVisibility, grid, kVisThreads, 0, (visibility_kernel<4, 6>), P); break;
    case 3: VLAUNCH(ctx, kKVisibility, grid, kVisThreads, 0, (visibility_kernel<16, 6>), P); break;
    case 4: VLAUNCH(ctx, kKVisibility, grid, kVisThreads, 0, (visibility_kernel<2, 6>), P); break;
    case 5: VLAUNCH(ctx, kKVisibility, grid, kVisThreads, 0, (visibility_kernel<1, 6>), P); break;
    default: VLAUNCH(ctx, kKVisibility, grid, kVisThreads, 0, (visibility_kernel<32, 6>), P); break;
  }
  return VISACD_OK;
}

// Shape class of a visibility call: log2 buckets of n and triangle counts, and
// the masked flag. The autotuner caches its pick per class in the context.
static uint32_t vis_shape_class(int32_t n, bool masked, const visacd_bvh* a, const visacd_bvh* b) {
  auto lg = [](int64_t x) { int r = 0; while (x > 1) { x >>= 1; ++r; } return r; };
  return (uint32_t)lg(n) | ((uint32_t)lg(a->nt + 1) << 6) | ((uint32_t)lg(b->nt + 1) << 12) |
         ((uint32_t)masked << 18);
}

static int choose_vis_variant(visacd_ctx* ctx, int32_t n, bool masked, const visacd_bvh* a,
                              const visacd_bvh* b) {
  if (ctx->vis_variant_override >= 0 && ctx->vis_variant_override < kNumVisVariants)
    return ctx->vis_variant_override;
  auto it = ctx->vis_tuned.find(vis_shape_class(n, masked, a, b));
  if (it != ctx->vis_tuned.end()) return it->second;
  return kDefaultVisVariant;
}

// Morton order of n device points into perm (sorted position -> vertex).
int vis_morton_order(visacd_ctx* ctx, const float* d_pts, int32_t n, uint32_t* perm) {
  if (n <= 0) return VISACD_OK;
  VTRY(ensure_slot(ctx, kSlotCounters, sizeof(VisCounters)));
  VTRY(ensure_slot(ctx, kSlotVisKeys, (size_t)n * 8));
  VTRY(ensure_slot(ctx, kSlotVisKeysAlt, (size_t)n * 8));
  VTRY(ensure_slot(ctx, kSlotVisPermAlt, (size_t)n * 4));
  VisCounters* cnt = slot<VisCounters>(ctx, kSlotCounters);
  VisCounters* h = nullptr;
  VTRY(pinned(ctx, sizeof(VisCounters), (void**)&h));
  memset(h, 0, sizeof(VisCounters));
  for (int a = 0; a < 3; ++a) {
    h->pmin[a] = 0xffffffffu;
    h->pmax[a] = 0u;
  }
  VCUDA(cudaMemcpyAsync(cnt, h, sizeof(VisCounters), cudaMemcpyHostToDevice, ctx->stream));
  uint64_t* keys = slot<uint64_t>(ctx, kSlotVisKeys);
  const unsigned gp = grid_for(n, 256, 4LL * ctx->sm_count);
  VLAUNCH(ctx, kKVisPrep, gp, 256, 0, point_bounds_kernel, d_pts, n, cnt);
  VLAUNCH(ctx, kKVisPrep, gp, 256, 0, point_morton_kernel, d_pts, n, cnt, morton_bits(n), keys, perm);
  VTRY(radix_sort_u64(ctx, keys, perm, slot<uint64_t>(ctx, kSlotVisKeysAlt),
                      slot<uint32_t>(ctx, kSlotVisPermAlt), n, 3 * morton_bits(n)));
  VCUDA(stream_wait(ctx));
  return VISACD_OK;
}

static int vis_device(visacd_ctx* ctx, const float* d_pts, int32_t n, const uint8_t* d_new,
                      const visacd_bvh* self_bvh, const visacd_bvh* cage_bvh, int64_t* n_edges,
                      visacd_vis_stats* stats, int64_t pairs) {
  // The cage's free-space grid, for calls with many pairs (`pairs`: the
  // call's pair count, or a bound of it): built once per cage BVH, before this
  // call's counters take the shared scratch and staging buffers.
  const bool use_grid = ctx->vis_trace && n >= 2 && pairs >= kFreeGridMinPairs && cage_bvh->nt > 0;
  if (use_grid) VTRY(free_grid_build(ctx, const_cast<visacd_bvh*>(cage_bvh), pairs));
  VTRY(ensure_slot(ctx, kSlotCounters, sizeof(VisCounters)));
  VisCounters* cnt = slot<VisCounters>(ctx, kSlotCounters);
  VisCounters init;
  memset(&init, 0, sizeof(init));
  for (int a = 0; a < 3; ++a) {
    init.pmin[a] = 0xffffffffu;
    init.pmax[a] = 0u;
  }
  VisCounters* h = nullptr;
  VTRY(pinned(ctx, sizeof(VisCounters), (void**)&h));
  *h = init;
  VCUDA(cudaMemcpyAsync(cnt, h, sizeof(VisCounters), cudaMemcpyHostToDevice, ctx->stream));
  ctx->last_n_edges = 0;

  const int64_t np = (int64_t)n * (n - 1) / 2;
  const int64_t nw = (np + 31) / 32;
  if (n < 2) {
    if (n_edges) *n_edges = 0;
    if (stats) memset(stats, 0, sizeof(*stats));
    return VISACD_OK;
  }
  // Morton order of the points.
  VTRY(ensure_slot(ctx, kSlotVisKeys, (size_t)n * 8));
  VTRY(ensure_slot(ctx, kSlotVisKeysAlt, (size_t)n * 8));
  VTRY(ensure_slot(ctx, kSlotVisPerm, (size_t)n * 4));
  VTRY(ensure_slot(ctx, kSlotVisPermAlt, (size_t)n * 4));
  uint64_t* keys = slot<uint64_t>(ctx, kSlotVisKeys);
  uint32_t* perm = slot<uint32_t>(ctx, kSlotVisPerm);
  const unsigned gp = grid_for(n, 256, 4LL * ctx->sm_count);
  VLAUNCH(ctx, kKVisPrep, gp, 256, 0, point_bounds_kernel, d_pts, n, cnt);
  VLAUNCH(ctx, kKVisPrep, gp, 256, 0, point_morton_kernel, d_pts, n, cnt, morton_bits(n), keys, perm);
  VTRY(radix_sort_u64(ctx, keys, perm, slot<uint64_t>(ctx, kSlotVisKeysAlt),
                      slot<uint32_t>(ctx, kSlotVisPermAlt), n, 3 * morton_bits(n)));

  const int variant = choose_vis_variant(ctx, n, d_new != nullptr, self_bvh, cage_bvh);
  const int TR = kVisVariants[variant].tr, TC = 32 / TR;
  VisParams P;
  memset(&P, 0, sizeof(P));
  P.pts = d_pts;
  P.n = n;
  P.cols = perm;
  P.nc = n;
  P.ntc = (n + TC - 1) / TC;
  if (d_new) {
    // Rows: new vertices in Morton order (compaction by scan).
    VTRY(ensure_slot(ctx, kSlotWordCounts, (size_t)n * 4));
    VTRY(ensure_slot(ctx, kSlotWordOffsets, (size_t)(n + 1) * 8));
    VTRY(ensure_slot(ctx, kSlotVisRank, (size_t)n * 4 + (size_t)n * 4 + 256));
    uint32_t* flags = slot<uint32_t>(ctx, kSlotWordCounts);
    uint64_t* off = slot<uint64_t>(ctx, kSlotWordOffsets);
    uint32_t* rows = slot<uint32_t>(ctx, kSlotVisRank);
    int32_t* newrank = reinterpret_cast<int32_t*>(rows + ((n + 63) & ~63));
    VLAUNCH(ctx, kKVisPrep, gp, 256, 0, new_flags_kernel, perm, d_new, n, flags);
    VTRY(exclusive_scan_u32_to_u64(ctx, flags, off, n));
    VLAUNCH(ctx, kKVisPrep, gp, 256, 0, new_rows_kernel, perm, flags, off, n, rows, newrank);
    uint64_t* hn = nullptr;
    VTRY(pinned(ctx, 8, (void**)&hn));
    VCUDA(cudaMemcpyAsync(hn, off + n, 8, cudaMemcpyDeviceToHost, ctx->stream));
    VCUDA(stream_wait(ctx));
    P.rows = rows;
    P.nr = (int32_t)*hn;
    P.triangular = 0;
    P.is_new = d_new;
    P.newrank = newrank;
    P.ntr = (P.nr + TR - 1) / TR;
    P.total_tiles = (unsigned long long)P.ntr * (unsigned long long)P.ntc;
  } else {
    P.rows = perm;
    P.nr = n;
    P.triangular = 1;
    P.ntr = (n + TR - 1) / TR;
    VTRY(ensure_slot(ctx, kSlotVisRowTiles, (size_t)P.ntr * 4 + (size_t)(P.ntr + 1) * 8 + 256));
    uint32_t* rc = slot<uint32_t>(ctx, kSlotVisRowTiles);
    uint64_t* rs = reinterpret_cast<uint64_t*>(rc + ((P.ntr + 63) & ~63LL));
    VLAUNCH(ctx, kKVisPrep, grid_for(P.ntr, 256, 4LL * ctx->sm_count), 256, 0,
            tile_row_counts_kernel, P.ntr, P.ntc, TR, TC, rc);
    VTRY(exclusive_scan_u32_to_u64(ctx, rc, rs, P.ntr));
    P.row_start = reinterpret_cast<const unsigned long long*>(rs);
    // The same total as the device scan, counted here (no read-back).
    unsigned long long total = 0;
    for (int64_t r = 0; r < P.ntr; ++r) {
      const int64_t c = P.ntc - (r * TR) / TC;
      total += (unsigned long long)(c > 0 ? c : 0);
    }
    P.total_tiles = total;
  }
  P.self_nodes = self_bvh->nodes;
  P.self_tris = self_bvh->tris;
  P.self_nt = self_bvh->nt;
  P.cage_nodes = cage_bvh->nodes;
  P.cage_tris = cage_bvh->tris;
  P.cage_nt = cage_bvh->nt;
  // Large calls first clear what they can with the cage's free-space grid
  // (built at the top of this call): a walk kernel, then the traversal.
  if (use_grid && cage_bvh->free_lb && P.total_tiles > 0) {
    VTRY(ensure_slot(ctx, kSlotVisCleared, (size_t)P.total_tiles * 12 + 256));
    P.pend_tiles = slot<unsigned long long>(ctx, kSlotVisCleared);
    P.pend_done = reinterpret_cast<uint32_t*>(P.pend_tiles + P.total_tiles);
  }
  if (P.pend_tiles != nullptr) {
    const visacd_bvh* cb = cage_bvh;
    {
      P.cage_free.lb = cb->free_lb;
      P.cage_free.tex = cb->free_tex;
      P.cage_free.ox = cb->fg_ox;
      P.cage_free.oy = cb->fg_oy;
      P.cage_free.oz = cb->fg_oz;
      P.cage_free.h_up = cb->fg_h * 1.000001f;
      P.cage_free.inv_h = cb->fg_inv_h;
      P.cage_free.margin = cb->fg_margin;
      P.cage_free.nx = cb->fg_nx;
      P.cage_free.ny = cb->fg_ny;
      P.cage_free.nz = cb->fg_nz;
    }
  }
  VTRY(ensure_slot(ctx, kSlotBitset, (size_t)nw * 4));
  P.bitset = slot<uint32_t>(ctx, kSlotBitset);
  VCUDA(cudaMemsetAsync(P.bitset, 0, (size_t)nw * 4, ctx->stream));
  P.cnt = cnt;
  P.status = ctx->d_status;
  if (P.total_tiles > 0) VTRY(launch_vis_variant(ctx, variant, P));
  // Compaction: popcount, scan, emit in linear-pair order.
  VTRY(ensure_slot(ctx, kSlotWordCounts, (size_t)nw * 4));
  VTRY(ensure_slot(ctx, kSlotWordOffsets, (size_t)(nw + 1) * 8));
  uint32_t* wc = slot<uint32_t>(ctx, kSlotWordCounts);
  uint64_t* wo = slot<uint64_t>(ctx, kSlotWordOffsets);
  const unsigned gw = grid_for(nw, 256, 16LL * ctx->sm_count);
  VLAUNCH(ctx, kKBitPopc, gw, 256, 0, bit_popc_kernel, P.bitset, nw, wc);
  VTRY(exclusive_scan_u32_to_u64(ctx, wc, wo, nw));
  // Counters and the status word in one wait.
  uint32_t* hs = nullptr;
  VTRY(pinned(ctx, sizeof(VisCounters) + 64, (void**)&h));
  hs = reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(h) + ((sizeof(VisCounters) + 15) & ~size_t(15)));
  VCUDA(cudaMemcpyAsync(h, cnt, sizeof(VisCounters), cudaMemcpyDeviceToHost, ctx->stream));
  VCUDA(cudaMemcpyAsync(hs, ctx->d_status, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
  VCUDA(stream_wait(ctx));
  const VisCounters hc = *h;
  VTRY(status_result(ctx, *hs, "visibility"));
  const int64_t ne = (int64_t)hc.edges;
  VTRY(ensure_slot(ctx, kSlotEdgesOut, (size_t)(ne > 0 ? ne : 1) * 8));
  if (ne > 0) {
    VLAUNCH(ctx, kKBitEmit, gw, 256, 0, bit_emit_kernel, P.bitset, nw, wo, (int64_t)n,
            slot<uint32_t>(ctx, kSlotEdgesOut));
  }
  ctx->last_n_edges = ne;
  if (n_edges) *n_edges = ne;
  if (stats) {
    stats->pairs_tested = (int64_t)hc.pairs;
    stats->n_edges = ne;
    stats->self_hits = (int64_t)hc.self_hits;
    stats->cage_hits = (int64_t)hc.cage_hits;
    stats->fp64_rechecks = (int64_t)hc.rechecks;
    stats->degenerate = (int64_t)hc.degenerate;
    stats->node_visits = (int64_t)hc.node_visits;
    stats->tri_tests = (int64_t)hc.tri_tests;
  }
  ctx->last_vis_certified = (int64_t)hc.certified;
  ctx->last_vis_trace_steps = (int64_t)hc.trace_steps;
  return VISACD_OK;
}

// ---- several parts in one launch ------------------------------------------
// The edge list of all parts: word w of the concatenated bitset belongs to the
// part found by binary search over the parts' first words; its edges go to
// the global offset of the word (parts stay in order, each row-major).
__global__ void multi_emit_kernel(const VisParams* __restrict__ parts, int n_parts,
                                  const unsigned long long* __restrict__ word_start,
                                  const uint32_t* __restrict__ bits, int64_t nw,
                                  const uint64_t* __restrict__ off, uint32_t* __restrict__ edges) {
  for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < nw;
       w += (int64_t)gridDim.x * blockDim.x) {
    uint32_t m = bits[w];
    if (!m) continue;
    int lo = 0, hi = n_parts - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (word_start[mid] <= (unsigned long long)w) lo = mid; else hi = mid - 1;
    }
    const int64_t n = parts[lo].n;
    const int64_t k0 = (w - (int64_t)word_start[lo]) * 32;
    uint64_t o = off[w];
    double b2 = (double)(2 * n - 1);
    double disc = b2 * b2 - 8.0 * (double)k0;
    int64_t i = (int64_t)((b2 - sqrt(disc > 0 ? disc : 0.0)) * 0.5);
    if (i < 0) i = 0;
    if (i > n - 2) i = n - 2;
    while (i > 0 && row_start(i, n) > k0) --i;
    while (i + 1 <= n - 2 && row_start(i + 1, n) <= k0) ++i;
    while (m) {
      const int bpos = __ffs(m) - 1;
      m &= m - 1;
      const int64_t k = k0 + bpos;
      while (i + 1 <= n - 2 && row_start(i + 1, n) <= k) ++i;
      const int64_t j = k - row_start(i, n) + i + 1;
      edges[2 * o] = (uint32_t)i;
      edges[2 * o + 1] = (uint32_t)j;
      ++o;
    }
  }
}

// Edge offsets of the parts' first words (and the total) for the read-back.
__global__ void multi_part_offsets_kernel(const unsigned long long* __restrict__ word_start, int n_parts,
                                          const uint64_t* __restrict__ off, uint64_t* __restrict__ out) {
  for (int p = threadIdx.x; p <= n_parts; p += blockDim.x) out[p] = off[word_start[p]];
}

// Rows of a masked part (new vertices in Morton order) and their count.
__global__ void copy_count_kernel(const uint64_t* __restrict__ off, int32_t n, int32_t* __restrict__ out) {
  *out = (int32_t)off[n];
}

int visibility_multi_impl(visacd_ctx* ctx, int32_t n_parts, const float* const* pts, const int32_t* n_pts,
                          const uint8_t* const* is_new, const visacd_bvh* const* self_bvhs,
                          const visacd_bvh* const* cage_bvhs, int64_t* n_edges, visacd_vis_stats* stats) {
  VCHECK(ctx && n_parts > 0 && pts && n_pts && self_bvhs && cage_bvhs && n_edges, VISACD_ERR_INVALID_ARG,
         "visibility_batch: null argument");
  VCUDA(cudaSetDevice(ctx->device));
  constexpr int TR = 8, TC = 4;
  // Free-space grids of the large parts' cages (built once per cage BVH),
  // before this call takes the shared scratch and staging buffers.
  // A part's pairs: all of them, or (masked) those with a new endpoint.
  std::vector<int64_t> part_pairs(n_parts, 0);
  for (int p = 0; p < n_parts; ++p) {
    const int64_t n = std::max(n_pts[p], 0);
    int64_t pairs = n * (n > 0 ? n - 1 : 0) / 2;
    if (is_new && is_new[p] && pts[p]) {
      int64_t k = 0;
      for (int64_t v = 0; v < n; ++v) k += is_new[p][v] != 0;
      pairs -= (n - k) * (n - k - 1) / 2;
    }
    part_pairs[p] = pairs;
  }
  bool any_grid = false;
  if (ctx->vis_trace) {
    for (int p = 0; p < n_parts; ++p) {
      if (part_pairs[p] >= kFreeGridMinPairs && cage_bvhs[p] && cage_bvhs[p]->ctx && cage_bvhs[p]->nt > 0) {
        VTRY(free_grid_build(ctx, const_cast<visacd_bvh*>(cage_bvhs[p]), part_pairs[p]));
        any_grid = any_grid || cage_bvhs[p]->free_lb != nullptr;
      }
    }
  }
  // Layout of the per-part arrays in one buffer (256-byte aligned pieces).
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  std::vector<size_t> o_pts(n_parts), o_mask(n_parts), o_perm(n_parts), o_rows(n_parts),
      o_rank(n_parts), o_rs(n_parts);
  std::vector<int64_t> ntr_tri(n_parts, 0);
  size_t total = al(sizeof(int32_t) * (size_t)n_parts);  // masked row counts
  const size_t o_nr = 0;
  unsigned long long words = 0;
  std::vector<unsigned long long> word_start(n_parts + 1);
  for (int p = 0; p < n_parts; ++p) {
    const int32_t n = n_pts[p];
    const visacd_bvh* sb = self_bvhs[p];
    const visacd_bvh* cb = cage_bvhs[p];
    VCHECK(n >= 0 && (n == 0 || pts[p]) && sb && cb, VISACD_ERR_INVALID_ARG, "visibility_batch: bad part %d", p);
    VCHECK(n <= (1 << 24), VISACD_ERR_INVALID_ARG, "visibility_batch: part %d has n = %d above 2^24", p, n);
    VCHECK(sb->ctx && cb->ctx && sb->device == ctx->device && cb->device == ctx->device,
           VISACD_ERR_INVALID_ARG, "visibility_batch: part %d BVH is not on this context's device", p);
    VCHECK(sb->depth <= kStack && cb->depth <= kStack, VISACD_ERR_INVALID_ARG,
           "visibility_batch: part %d BVH depth %d/%d exceeds the traversal stack (%d)", p, sb->depth,
           cb->depth, kStack);
    VCHECK(sb->nt == 0 || sb->nv == n, VISACD_ERR_INVALID_ARG,
           "visibility_batch: part %d self BVH has %d vertices, points have %d", p, sb->nv, n);
    o_pts[p] = total;  total += al((size_t)std::max(n, 1) * 12);
    o_mask[p] = total; total += al((size_t)std::max(n, 1));
    o_perm[p] = total; total += al((size_t)std::max(n, 1) * 4);
    o_rows[p] = total; total += al((size_t)std::max(n, 1) * 4);
    o_rank[p] = total; total += al((size_t)std::max(n, 1) * 4);
    ntr_tri[p] = (n + TR - 1) / TR;
    o_rs[p] = total;   total += al((size_t)(ntr_tri[p] + 1) * 8);
    word_start[p] = words;
    const unsigned long long np = (unsigned long long)n * (unsigned long long)(n > 0 ? n - 1 : 0) / 2;
    words += (np + 31) / 32;
  }
  word_start[n_parts] = words;
  const size_t o_desc = total;
  total += al(sizeof(VisParams) * (size_t)n_parts);
  const size_t o_tiles = total;
  total += al(8 * (size_t)(n_parts + 1));
  const size_t o_words = total;
  total += al(8 * (size_t)(n_parts + 1));
  const size_t o_poff = total;
  total += al(8 * (size_t)(n_parts + 1));
  VTRY(ensure_slot(ctx, kSlotVisMulti, total));
  char* base = slot<char>(ctx, kSlotVisMulti);
  // Upload points, masks and the triangular tile-row starts.
  {
    size_t up_bytes = 0;
    for (int p = 0; p < n_parts; ++p) up_bytes += (size_t)n_pts[p] * 13 + (size_t)(ntr_tri[p] + 1) * 8;
    Stager up(ctx);
    VTRY(up.reserve(up_bytes + 8 * (size_t)(n_parts + 1), 3 * n_parts + 1));
    std::vector<uint64_t> rs;
    for (int p = 0; p < n_parts; ++p) {
      const int32_t n = n_pts[p];
      if (n) VTRY(up.put(base + o_pts[p], pts[p], (size_t)n * 12));
      if (n && is_new && is_new[p]) VTRY(up.put(base + o_mask[p], is_new[p], (size_t)n));
      const int64_t ntr = ntr_tri[p], ntc = (n + TC - 1) / TC;
      rs.assign((size_t)ntr + 1, 0);
      for (int64_t r = 0; r < ntr; ++r) {
        const int64_t c = ntc - (r * TR) / TC;
        rs[r + 1] = rs[r] + (uint64_t)(c > 0 ? c : 0);
      }
      VTRY(up.put(base + o_rs[p], rs.data(), rs.size() * 8));
    }
    VTRY(up.put(base + o_words, word_start.data(), 8 * (size_t)(n_parts + 1)));
  }
  // Morton order of each part; rows and ranks of the masked ones.
  int32_t* d_nr = reinterpret_cast<int32_t*>(base + o_nr);
  for (int p = 0; p < n_parts; ++p) {
    const int32_t n = n_pts[p];
    if (n < 2) continue;
    const float* dp = reinterpret_cast<const float*>(base + o_pts[p]);
    uint32_t* perm = reinterpret_cast<uint32_t*>(base + o_perm[p]);
    VTRY(ensure_slot(ctx, kSlotCounters, sizeof(VisCounters)));
    VTRY(ensure_slot(ctx, kSlotVisKeys, (size_t)n * 8));
    VTRY(ensure_slot(ctx, kSlotVisKeysAlt, (size_t)n * 8));
    VTRY(ensure_slot(ctx, kSlotVisPermAlt, (size_t)n * 4));
    VisCounters* cnt = slot<VisCounters>(ctx, kSlotCounters);
    VisCounters* h = nullptr;
    VTRY(pinned(ctx, sizeof(VisCounters), (void**)&h));
    memset(h, 0, sizeof(VisCounters));
    for (int a = 0; a < 3; ++a) {
      h->pmin[a] = 0xffffffffu;
      h->pmax[a] = 0u;
    }
    VCUDA(cudaMemcpyAsync(cnt, h, sizeof(VisCounters), cudaMemcpyHostToDevice, ctx->stream));
    uint64_t* keys = slot<uint64_t>(ctx, kSlotVisKeys);
    const unsigned gp = grid_for(n, 256, 4LL * ctx->sm_count);
    VLAUNCH(ctx, kKVisPrep, gp, 256, 0, point_bounds_kernel, dp, n, cnt);
    VLAUNCH(ctx, kKVisPrep, gp, 256, 0, point_morton_kernel, dp, n, cnt, morton_bits(n), keys, perm);
    VTRY(radix_sort_u64(ctx, keys, perm, slot<uint64_t>(ctx, kSlotVisKeysAlt),
                        slot<uint32_t>(ctx, kSlotVisPermAlt), n, 3 * morton_bits(n)));
    if (is_new && is_new[p]) {
      VTRY(ensure_slot(ctx, kSlotWordCounts, (size_t)n * 4));
      VTRY(ensure_slot(ctx, kSlotWordOffsets, (size_t)(n + 1) * 8));
      uint32_t* flags = slot<uint32_t>(ctx, kSlotWordCounts);
      uint64_t* off = slot<uint64_t>(ctx, kSlotWordOffsets);
      const uint8_t* dm = reinterpret_cast<const uint8_t*>(base + o_mask[p]);
      VLAUNCH(ctx, kKVisPrep, gp, 256, 0, new_flags_kernel, perm, dm, n, flags);
      VTRY(exclusive_scan_u32_to_u64(ctx, flags, off, n));
      VLAUNCH(ctx, kKVisPrep, gp, 256, 0, new_rows_kernel, perm, flags, off, n,
              reinterpret_cast<uint32_t*>(base + o_rows[p]), reinterpret_cast<int32_t*>(base + o_rank[p]));
      VLAUNCH(ctx, kKVisPrep, 1, 1, 0, copy_count_kernel, off, n, d_nr + p);
    }
  }
  std::vector<int32_t> nr(n_parts, 0);
  {
    int32_t* h = nullptr;
    VTRY(pinned(ctx, 4 * (size_t)n_parts, (void**)&h));
    VCUDA(cudaMemcpyAsync(h, d_nr, 4 * (size_t)n_parts, cudaMemcpyDeviceToHost, ctx->stream));
    VCUDA(stream_wait(ctx));
    memcpy(nr.data(), h, 4 * (size_t)n_parts);
  }
  // Part descriptors and the global work numbering.
  VTRY(ensure_slot(ctx, kSlotBitset, (size_t)std::max<unsigned long long>(words, 1) * 4));
  uint32_t* bits = slot<uint32_t>(ctx, kSlotBitset);
  VTRY(ensure_slot(ctx, kSlotCounters, sizeof(VisCounters)));
  VisCounters* cnt = slot<VisCounters>(ctx, kSlotCounters);
  std::vector<VisParams> desc(n_parts);
  std::vector<unsigned long long> tile_start(n_parts + 1, 0);
  unsigned long long tiles = 0;
  for (int p = 0; p < n_parts; ++p) {
    const int32_t n = n_pts[p];
    VisParams& P = desc[p];
    memset(&P, 0, sizeof(P));
    P.pts = reinterpret_cast<const float*>(base + o_pts[p]);
    P.n = n;
    P.cols = reinterpret_cast<const uint32_t*>(base + o_perm[p]);
    P.nc = n;
    P.ntc = (n + TC - 1) / TC;
    const bool masked = is_new && is_new[p];
    if (masked) {
      P.rows = reinterpret_cast<const uint32_t*>(base + o_rows[p]);
      P.nr = nr[p];
      P.triangular = 0;
      P.is_new = reinterpret_cast<const uint8_t*>(base + o_mask[p]);
      P.newrank = reinterpret_cast<const int32_t*>(base + o_rank[p]);
      P.ntr = (P.nr + TR - 1) / TR;
      P.total_tiles = n >= 2 ? (unsigned long long)P.ntr * (unsigned long long)P.ntc : 0ull;
    } else {
      P.rows = P.cols;
      P.nr = n;
      P.triangular = 1;
      P.ntr = ntr_tri[p];
      P.row_start = reinterpret_cast<const unsigned long long*>(base + o_rs[p]);
      unsigned long long t = 0;
      for (int64_t r = 0; r < P.ntr; ++r) {
        const int64_t c = P.ntc - (r * TR) / TC;
        t += (unsigned long long)(c > 0 ? c : 0);
      }
      P.total_tiles = n >= 2 ? t : 0ull;
    }
    P.self_nodes = self_bvhs[p]->nodes;
    P.self_tris = self_bvhs[p]->tris;
    P.self_nt = self_bvhs[p]->nt;
    P.cage_nodes = cage_bvhs[p]->nodes;
    P.cage_tris = cage_bvhs[p]->tris;
    P.cage_nt = cage_bvhs[p]->nt;
    const visacd_bvh* cb = cage_bvhs[p];
    if (any_grid && cb->free_lb && part_pairs[p] >= kFreeGridMinPairs) {
      P.cage_free.lb = cb->free_lb;
      P.cage_free.tex = cb->free_tex;
      P.cage_free.ox = cb->fg_ox;
      P.cage_free.oy = cb->fg_oy;
      P.cage_free.oz = cb->fg_oz;
      P.cage_free.h_up = cb->fg_h * 1.000001f;
      P.cage_free.inv_h = cb->fg_inv_h;
      P.cage_free.margin = cb->fg_margin;
      P.cage_free.nx = cb->fg_nx;
      P.cage_free.ny = cb->fg_ny;
      P.cage_free.nz = cb->fg_nz;
    }
    P.bitset = bits + word_start[p];
    P.cnt = cnt;
    P.status = ctx->d_status;
    tile_start[p] = tiles;
    tiles += P.total_tiles;
  }
  tile_start[n_parts] = tiles;
  {
    VisCounters init;
    memset(&init, 0, sizeof(init));
    Stager up(ctx);
    VTRY(up.reserve(sizeof(VisParams) * (size_t)n_parts + 8 * (size_t)(n_parts + 1) + sizeof(VisCounters), 3));
    VTRY(up.put(base + o_desc, desc.data(), sizeof(VisParams) * (size_t)n_parts));
    VTRY(up.put(base + o_tiles, tile_start.data(), 8 * (size_t)(n_parts + 1)));
    VTRY(up.put(cnt, &init, sizeof(VisCounters)));
  }
  if (words) VCUDA(cudaMemsetAsync(bits, 0, (size_t)words * 4, ctx->stream));
  const VisParams* d_desc = reinterpret_cast<const VisParams*>(base + o_desc);
  const unsigned long long* d_tiles = reinterpret_cast<const unsigned long long*>(base + o_tiles);
  const unsigned long long* d_words = reinterpret_cast<const unsigned long long*>(base + o_words);
  if (tiles) {
    unsigned long long* pend = nullptr;
    uint32_t* pend_done = nullptr;
    if (any_grid) {
      VTRY(ensure_slot(ctx, kSlotVisCleared, (size_t)tiles * 12 + 256));
      pend = slot<unsigned long long>(ctx, kSlotVisCleared);
      pend_done = reinterpret_cast<uint32_t*>(pend + tiles);
      VLAUNCH(ctx, kKVisWalk, (unsigned)(ctx->sm_count * 16), kVisThreads, 0, visibility_multi_walk_kernel<8>,
              d_desc, n_parts, d_tiles, tiles, cnt, pend, pend_done);
    }
    VLAUNCH(ctx, kKVisibility, (unsigned)(ctx->sm_count * 8), kVisThreads, 0, (visibility_multi_kernel<8, 8>),
            d_desc, n_parts, d_tiles, tiles, cnt, ctx->d_status, pend, pend_done);
  }
  // Compaction over the concatenated bitset.
  const int64_t nw = (int64_t)words;
  VTRY(ensure_slot(ctx, kSlotWordCounts, (size_t)std::max<int64_t>(nw, 1) * 4));
  VTRY(ensure_slot(ctx, kSlotWordOffsets, (size_t)(nw + 1) * 8));
  uint32_t* wc = slot<uint32_t>(ctx, kSlotWordCounts);
  uint64_t* wo = slot<uint64_t>(ctx, kSlotWordOffsets);
  const unsigned gw = grid_for(std::max<int64_t>(nw, 1), 256, 16LL * ctx->sm_count);
  if (nw) {
    VLAUNCH(ctx, kKBitPopc, gw, 256, 0, bit_popc_kernel, bits, nw, wc);
    VTRY(exclusive_scan_u32_to_u64(ctx, wc, wo, nw));
  } else {
    VCUDA(cudaMemsetAsync(wo, 0, 8, ctx->stream));
  }
  uint64_t* d_poff = reinterpret_cast<uint64_t*>(base + o_poff);
  VLAUNCH(ctx, kKVisPrep, 1, 256, 0, multi_part_offsets_kernel, d_words, n_parts, wo, d_poff);
  // Counters, part offsets and the status word in one wait.
  char* hb = nullptr;
  const size_t o_st = (sizeof(VisCounters) + 8 * (size_t)(n_parts + 1) + 15) & ~size_t(15);
  VTRY(pinned(ctx, o_st + 16, (void**)&hb));
  VCUDA(cudaMemcpyAsync(hb, cnt, sizeof(VisCounters), cudaMemcpyDeviceToHost, ctx->stream));
  VCUDA(cudaMemcpyAsync(hb + sizeof(VisCounters), d_poff, 8 * (size_t)(n_parts + 1), cudaMemcpyDeviceToHost,
                        ctx->stream));
  VCUDA(cudaMemcpyAsync(hb + o_st, ctx->d_status, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
  VCUDA(stream_wait(ctx));
  VisCounters hc;
  memcpy(&hc, hb, sizeof(hc));
  std::vector<uint64_t> poff(n_parts + 1);
  memcpy(poff.data(), hb + sizeof(VisCounters), 8 * (size_t)(n_parts + 1));
  uint32_t dev_status = 0;
  memcpy(&dev_status, hb + o_st, sizeof(uint32_t));
  VTRY(status_result(ctx, dev_status, "visibility_batch"));
  for (int p = 0; p < n_parts; ++p) n_edges[p] = (int64_t)(poff[p + 1] - poff[p]);
  const int64_t ne = (int64_t)poff[n_parts];
  VTRY(ensure_slot(ctx, kSlotEdgesOut, (size_t)(ne > 0 ? ne : 1) * 8));
  if (ne > 0) {
    VLAUNCH(ctx, kKBitEmit, gw, 256, 0, multi_emit_kernel, d_desc, n_parts, d_words, bits, nw, wo,
            slot<uint32_t>(ctx, kSlotEdgesOut));
  }
  ctx->last_n_edges = ne;
  if (stats) {
    stats->pairs_tested = (int64_t)hc.pairs;
    stats->n_edges = ne;
    stats->self_hits = (int64_t)hc.self_hits;
    stats->cage_hits = (int64_t)hc.cage_hits;
    stats->fp64_rechecks = (int64_t)hc.rechecks;
    stats->degenerate = (int64_t)hc.degenerate;
    stats->node_visits = (int64_t)hc.node_visits;
    stats->tri_tests = (int64_t)hc.tri_tests;
  }
  return VISACD_OK;
}

int visibility_impl(visacd_ctx* ctx, const float* pts, int32_t n, const uint8_t* is_new,
                    int device_ptrs, const visacd_bvh* self_bvh, const visacd_bvh* cage_bvh,
                    int64_t* n_edges, visacd_vis_stats* stats) {
  VCHECK(ctx && self_bvh && cage_bvh, VISACD_ERR_INVALID_ARG, "visibility: null argument");
  VCHECK(self_bvh->ctx && cage_bvh->ctx, VISACD_ERR_INVALID_ARG,
         "visibility: a BVH outlived the context it was built on");
  VCHECK(n >= 0 && (n == 0 || pts), VISACD_ERR_INVALID_ARG, "visibility: bad points");
  VCHECK(n <= (1 << 24), VISACD_ERR_INVALID_ARG, "visibility: n = %d above the 2^24 limit", n);
  VCHECK(self_bvh->device == ctx->device && cage_bvh->device == ctx->device,
         VISACD_ERR_INVALID_ARG, "visibility: BVH built on another device");
  VCHECK(self_bvh->depth <= kStack && cage_bvh->depth <= kStack, VISACD_ERR_INVALID_ARG,
         "visibility: BVH depth %d/%d exceeds the traversal stack (%d)", self_bvh->depth,
         cage_bvh->depth, kStack);
  VCHECK(self_bvh->nt == 0 || self_bvh->nv == n, VISACD_ERR_INVALID_ARG,
         "visibility: self BVH has %d vertices, points have %d", self_bvh->nv, n);
  VCUDA(cudaSetDevice(ctx->device));
  const float* d_pts = pts;
  const uint8_t* d_new = is_new;
  int64_t pairs = (int64_t)n * (n > 0 ? n - 1 : 0) / 2;
  if (is_new && !device_ptrs) {
    int64_t k = 0;
    for (int32_t v = 0; v < n; ++v) k += is_new[v] != 0;
    pairs -= ((int64_t)n - k) * ((int64_t)n - k - 1) / 2;
  }
  if (!device_ptrs && n > 0) {
    VTRY(ensure_slot(ctx, kSlotPoints, (size_t)n * 12));
    if (is_new) VTRY(ensure_slot(ctx, kSlotMask, (size_t)n));
    Stager up(ctx);
    VTRY(up.reserve((size_t)n * 13, 2));
    VTRY(up.put(ctx->buf[kSlotPoints].p, pts, (size_t)n * 12));
    d_pts = slot<float>(ctx, kSlotPoints);
    if (is_new) {
      VTRY(up.put(ctx->buf[kSlotMask].p, is_new, (size_t)n));
      d_new = slot<uint8_t>(ctx, kSlotMask);
    }
  }
  return vis_device(ctx, d_pts, n, d_new, self_bvh, cage_bvh, n_edges, stats, pairs);
}

}  // namespace vgpu

using namespace vgpu;

extern "C" int visacd_visibility(visacd_ctx* ctx, const float* pts, int32_t n,
                                 const uint8_t* is_new, int device_ptrs,
                                 const visacd_bvh* self_bvh, const visacd_bvh* cage_bvh,
                                 int64_t* n_edges, visacd_vis_stats* stats) {
  return visibility_impl(ctx, pts, n, is_new, device_ptrs, self_bvh, cage_bvh, n_edges, stats);
}

extern "C" int visacd_visibility_batch(visacd_ctx* ctx, int32_t n_parts, const float* const* pts,
                                       const int32_t* n_pts, const uint8_t* const* is_new,
                                       const visacd_bvh* const* self_bvhs,
                                       const visacd_bvh* const* cage_bvhs, int64_t* n_edges,
                                       visacd_vis_stats* stats) {
  return visibility_multi_impl(ctx, n_parts, pts, n_pts, is_new, self_bvhs, cage_bvhs, n_edges, stats);
}

extern "C" int visacd_visibility_edges(visacd_ctx* ctx, uint32_t* edges_out,
                                       int64_t capacity_edges) {
  VCHECK(ctx, VISACD_ERR_INVALID_ARG, "visibility_edges: null context");
  VCHECK(capacity_edges >= ctx->last_n_edges, VISACD_ERR_CAPACITY,
         "visibility_edges: capacity %lld < %lld edges", (long long)capacity_edges,
         (long long)ctx->last_n_edges);
  if (ctx->last_n_edges == 0) return VISACD_OK;
  VCHECK(edges_out, VISACD_ERR_INVALID_ARG, "visibility_edges: edges_out is NULL");
  VCUDA(cudaMemcpyAsync(edges_out, ctx->buf[kSlotEdgesOut].p, (size_t)ctx->last_n_edges * 8,
                        cudaMemcpyDeviceToHost, ctx->stream));
  VCUDA(stream_wait(ctx));
  return VISACD_OK;
}

extern "C" int visacd_visibility_edges_device(visacd_ctx* ctx, const uint32_t** d_edges,
                                              int64_t* n_edges) {
  VCHECK(ctx && d_edges && n_edges, VISACD_ERR_INVALID_ARG, "visibility_edges_device: null");
  *d_edges = slot<uint32_t>(ctx, kSlotEdgesOut);
  *n_edges = ctx->last_n_edges;
  return VISACD_OK;
}

extern "C" int visacd_compute_intersection_matrix(
    visacd_ctx* ctx, const float* verts, int32_t nv, const uint32_t* tris, int32_t nt,
    const uint8_t* is_new, const float* cage_verts, int32_t ncv, const uint32_t* cage_tris,
    int32_t nct, uint32_t* edges_out, int64_t capacity_edges, int64_t* n_edges,
    visacd_vis_stats* stats) {
  VCHECK(ctx && n_edges, VISACD_ERR_INVALID_ARG, "compute_intersection_matrix: null argument");
  visacd_bvh *sb = nullptr, *cb = nullptr;
  int rc = bvh_build(ctx, verts, nv, tris, nt, 0, &sb);
  if (rc == VISACD_OK) rc = bvh_build(ctx, cage_verts, ncv, cage_tris, nct, 0, &cb);
  if (rc == VISACD_OK) {
    // A BVH over a mesh with no triangles still needs the vertex count check.
    if (sb->nt == 0) sb->nv = nv;
    rc = visibility_impl(ctx, verts, nv, is_new, 0, sb, cb, n_edges, stats);
  }
  if (rc == VISACD_OK) {
    if (*n_edges > capacity_edges) {
      set_error("compute_intersection_matrix: %lld edges exceed capacity %lld",
                (long long)*n_edges, (long long)capacity_edges);
      rc = VISACD_ERR_CAPACITY;
    } else {
      rc = visacd_visibility_edges(ctx, edges_out, capacity_edges);
    }
  }
  visacd_bvh_destroy(sb);
  visacd_bvh_destroy(cb);
  return rc;
}

// ---------------------------------------------------------------------------
// Launch-shape control and the visibility autotuner.
// ---------------------------------------------------------------------------
extern "C" int visacd_vis_variant_count(void) { return kNumVisVariants; }

extern "C" int visacd_ctx_set_vis_variant(visacd_ctx* ctx, int variant) {
  VCHECK(ctx, VISACD_ERR_INVALID_ARG, "set_vis_variant: null context");
  VCHECK(variant >= -1 && variant < kNumVisVariants, VISACD_ERR_INVALID_ARG,
         "set_vis_variant: variant %d out of range", variant);
  ctx->vis_variant_override = variant;
  return VISACD_OK;
}

extern "C" int visacd_ctx_set_vis_trace(visacd_ctx* ctx, int enable) {
  VCHECK(ctx, VISACD_ERR_INVALID_ARG, "set_vis_trace: null context");
  ctx->vis_trace = enable != 0;
  return VISACD_OK;
}

extern "C" int visacd_ctx_vis_trace_counts(const visacd_ctx* ctx, int64_t* cleared, int64_t* grid_reads) {
  VCHECK(ctx, VISACD_ERR_INVALID_ARG, "vis_trace_counts: null context");
  if (cleared) *cleared = ctx->last_vis_certified;
  if (grid_reads) *grid_reads = ctx->last_vis_trace_steps;
  return VISACD_OK;
}

extern "C" int visacd_autotune_visibility(visacd_ctx* ctx, const float* pts, int32_t n,
                                          const uint8_t* is_new, int device_ptrs,
                                          const visacd_bvh* self_bvh, const visacd_bvh* cage_bvh,
                                          int* best_variant, double* ms_per_variant) {
  VCHECK(ctx && self_bvh && cage_bvh, VISACD_ERR_INVALID_ARG, "autotune: null argument");
  VCHECK(self_bvh->ctx && cage_bvh->ctx, VISACD_ERR_INVALID_ARG,
         "autotune: a BVH outlived the context it was built on");
  const int saved_override = ctx->vis_variant_override;
  const bool saved_timing = ctx->timing;
  int best = 0;
  double best_ms = 1e300;
  int rc = VISACD_OK;
  for (int v = 0; v < kNumVisVariants && rc == VISACD_OK; ++v) {
    ctx->vis_variant_override = v;
    double ms = 0.0;
    for (int rep = 0; rep < 2 && rc == VISACD_OK; ++rep) {
      ctx->timing = true;
      rc = visacd_ctx_reset_times(ctx);
      if (rc == VISACD_OK)
        rc = visibility_impl(ctx, pts, n, is_new, device_ptrs, self_bvh, cage_bvh, nullptr, nullptr);
      const char* names[64];
      double t[64];
      int64_t cnt[64];
      int nk = 0;
      if (rc == VISACD_OK) rc = visacd_ctx_kernel_times(ctx, names, t, cnt, 64, &nk);
      ms = 0.0;
      for (int k = 0; k < nk && k < 64; ++k)
        if (strcmp(names[k], kernel_name(kKVisibility)) == 0 || strcmp(names[k], kernel_name(kKVisWalk)) == 0)
          ms += t[k];
    }
    if (ms_per_variant) ms_per_variant[v] = ms;
    if (ms < best_ms) {
      best_ms = ms;
      best = v;
    }
  }
  ctx->vis_variant_override = saved_override;
  ctx->timing = saved_timing;
  visacd_ctx_reset_times(ctx);
  if (rc != VISACD_OK) return rc;
  ctx->vis_tuned[vis_shape_class(n, is_new != nullptr, self_bvh, cage_bvh)] = best;
  if (best_variant) *best_variant = best;
  return VISACD_OK;
}

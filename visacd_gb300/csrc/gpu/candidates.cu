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

__global__ void cand_planes_kernel(const double* __restrict__ verts, int32_t n,
                                   const uint32_t* __restrict__ edges, int64_t E,
                                   const int32_t* __restrict__ draws, int32_t D,
                                   Plane64* __restrict__ planes, float* __restrict__ d32,
                                   uint8_t* __restrict__ state) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < D; k += gridDim.x * blockDim.x) {
    const int32_t idx = draws[k];
    uint8_t st = kInvalid;
    Plane64 pl = Plane64{0.0, 0.0, 0.0, 0.0};
    if (idx >= 0 && (int64_t)idx < E) {
      const uint32_t i0 = edges[2 * (int64_t)idx], i1 = edges[2 * (int64_t)idx + 1];
      if (i0 < (uint32_t)n && i1 < (uint32_t)n) {
        const double* p1 = verts + 3 * (int64_t)i0;
        const double* p2 = verts + 3 * (int64_t)i1;
        const double nx = __dsub_rn(p2[0], p1[0]), ny = __dsub_rn(p2[1], p1[1]),
                     nz = __dsub_rn(p2[2], p1[2]);
        const double l = __dsqrt_rn(
            __dadd_rn(__dadd_rn(__dmul_rn(nx, nx), __dmul_rn(ny, ny)), __dmul_rn(nz, nz)));
        if (!(l < 1e-6)) {
          const double a = __ddiv_rn(nx, l), b = __ddiv_rn(ny, l), c = __ddiv_rn(nz, l);
          const double mx = __dmul_rn(__dadd_rn(p1[0], p2[0]), 0.5);
          const double my = __dmul_rn(__dadd_rn(p1[1], p2[1]), 0.5);
          const double mz = __dmul_rn(__dadd_rn(p1[2], p2[2]), 0.5);
          const double d =
              -__dadd_rn(__dadd_rn(__dmul_rn(a, mx), __dmul_rn(b, my)), __dmul_rn(c, mz));
          pl = Plane64{a, b, c, d};
          st = kUndecided;
        }
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
  VTRY(pinned(ctx, sizeof(SplitOut), (void**)&h));
  for (int attempt = 0; attempt < 2; ++attempt) {
    const unsigned* st_status = nullptr;
    const unsigned* st_count = nullptr;
    VTRY(score_planes_device_async(ctx, reinterpret_cast<const float*>(s.out32), P, pts32, n, s.edges,
                                   E, scores, rcap, &st_status, &st_count));
    VLAUNCH(ctx, kKCandidates, 1, 1024, 0, split_argmax_kernel, scores, s.out64, s.info, cand_slots,
            n_flat, flat_k, st_status, st_count, s.split);
    VCUDA(cudaMemcpyAsync(h, s.split, sizeof(SplitOut), cudaMemcpyDeviceToHost, ctx->stream));
    VCUDA(stream_wait(ctx));
    VCHECK(!(h->score_status & kStatusMbarrierTimeout), VISACD_ERR_DEVICE,
           "split_search: a bulk-copy wait of the scoring kernel timed out");
    if (!(h->score_status & kStatusRecheckOverflow)) break;
    VCHECK(attempt == 0, VISACD_ERR_DEVICE, "split_search: FP64 queue overflow after a rerun");
    rcap = h->recheck_count;
  }
  // The read-back shares the pinned staging area with the status check: copy
  // it out first.
  const SplitOut r = *h;
  VTRY(check_status(ctx, "split_search"));
  for (int c = 0; c < 4; ++c) best_plane[c] = r.plane[c];
  if (info) {
    info->best_index = r.index;
    info->n_candidates = r.n_planes;
    info->draws_used = r.draws_used;
    info->best_score = r.score;
  }
  return VISACD_OK;
}

// Per-part mesh clipping on the GPU (the cap triangulation stays on the host).
//
// Semantics of lib/src/clip.cpp:190-741, bit-exact with this project's host
// restatement (FP64 with explicit round-to-nearest intrinsics in the host's
// operation order):
//  1. clip_sides: side of every vertex (1e-6 test).
//  2. clip_classify: per triangle, the case. Triangles strictly on one side
//     (|sum of sides| = 3, including the all-on-plane case oriented by the face
//     normal) are "simple": they keep their vertices and emit themselves. All
//     others touch the plane and are compacted, in order, into a short list.
//  3. clip_resolve: one warp walks that list in triangle order — the only
//     order-dependent part: border points are deduplicated by vertex key, by
//     directed-edge key (with the reference's key overwrites) and by position
//     (1e-4 per coordinate, first match wins; the position scan runs across the
//     32 lanes). Emits each touching triangle's pieces, border edges (unique
//     unordered pairs, first occurrence) and the kept-vertex flags.
//  4. Order-preserving scans over per-triangle output counts and per-vertex
//     kept flags, then scatter + remap into part-local indices.
#include "common.cuh"

namespace vgpu {

constexpr int kClipResolveThreads = 32;

struct ClipCounters {
  unsigned n_touch;     // touching triangles
  unsigned n_border;    // border points
  unsigned n_bedges;    // unique border edges
  unsigned overflow;    // hash/table overflow (host retries on the CPU path)
  unsigned n_pos, n_neg;    // output triangles per side
  unsigned nv_pos, nv_neg;  // kept original vertices per side
};

struct PieceSlot {   // pieces of one touching triangle (<= 3 per side)
  int pos[3][3];
  int neg[3][3];
  int npos, nneg;
};

__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double ds(double a, double b) { return __dsub_rn(a, b); }

// ((p0 a + p1 b) + p2 c) + d, the host's order.
__device__ __forceinline__ int side_of(const double* p, const double* pl) {
  double r = da(da(da(dm(p[0], pl[0]), dm(p[1], pl[1])), dm(p[2], pl[2])), pl[3]);
  if (r > 1e-6) return 1;
  if (r < -1e-6) return -1;
  return 0;
}

// Orientation of a triangle lying in the plane (host face_normal + the sign
// rule of lib/include/core.hpp:169-176).
__device__ int coplanar_side(const double* p0, const double* p1, const double* p2, const double* pl) {
  double v0 = ds(p1[0], p0[0]), v1 = ds(p1[1], p0[1]), v2 = ds(p1[2], p0[2]);
  double w0 = ds(p2[0], p0[0]), w1 = ds(p2[1], p0[1]), w2 = ds(p2[2], p0[2]);
  double n0 = ds(dm(v1, w2), dm(v2, w1));
  double n1 = ds(dm(v2, w0), dm(v0, w2));
  double n2 = ds(dm(v0, w1), dm(v1, w0));
  double l = __dsqrt_rn(da(da(dm(n0, n0), dm(n1, n1)), dm(n2, n2)));
  double a0 = __ddiv_rn(n0, l), a1 = __ddiv_rn(n1, l), a2 = __ddiv_rn(n2, l);
  if (dm(a0, pl[0]) > 0 || dm(a1, pl[1]) > 0 || dm(a2, pl[2]) > 0) return -1;
  return 1;
}

// Plane-line intersection of p1-p2 in the host's formula order
// (lib/include/core.hpp:187-210 form), accepted inside the widened bbox.
__device__ bool intersect_segment(const double* pl, const double* p1, const double* p2, double* pi) {
  const double a = pl[0], b = pl[1], c = pl[2], d = pl[3], eps = 1e-6;
  double den = da(da(da(da(ds(dm(a, p2[0]), dm(a, p1[0])), dm(b, p2[1])), -dm(b, p1[1])), dm(c, p2[2])),
                  -dm(c, p1[2]));
  double n0 = ds(ds(ds(da(da(dm(dm(p1[0], b), p2[1]), dm(dm(p1[0], c), p2[2])), dm(p1[0], d)),
                        dm(dm(p2[0], b), p1[1])),
                     dm(dm(p2[0], c), p1[2])),
                  dm(p2[0], d));
  double n1 = ds(ds(ds(da(da(dm(dm(a, p2[0]), p1[1]), dm(dm(c, p1[1]), p2[2])), dm(p1[1], d)),
                        dm(dm(a, p1[0]), p2[1])),
                     dm(dm(c, p1[2]), p2[1])),
                  dm(p2[1], d));
  double n2 = ds(ds(ds(da(da(dm(dm(a, p2[0]), p1[2]), dm(dm(b, p2[1]), p1[2])), dm(p1[2], d)),
                        dm(dm(a, p1[0]), p2[2])),
                     dm(dm(b, p1[1]), p2[2])),
                  dm(p2[2], d));
  pi[0] = __ddiv_rn(n0, den);
  pi[1] = __ddiv_rn(n1, den);
  pi[2] = __ddiv_rn(n2, den);
  for (int k = 0; k < 3; ++k) {
    double lo = fmin(ds(p1[k], eps), ds(p2[k], eps)), hi = fmax(da(p1[k], eps), da(p2[k], eps));
    if (!(lo <= pi[k] && pi[k] <= hi)) return false;
  }
  return true;
}

__global__ void clip_sides_kernel(const double* __restrict__ v, int nv, const double* __restrict__ pl,
                                  signed char* __restrict__ side) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += gridDim.x * blockDim.x)
    side[i] = (signed char)side_of(v + 3 * (int64_t)i, pl);
}

// code: 0 simple pos, 1 simple neg, 2 touching. For simple triangles the kept
// flags of the three vertices are raised here.
__global__ void clip_classify_kernel(const double* __restrict__ v, const int* __restrict__ t, int nt,
                                     const double* __restrict__ pl, const signed char* __restrict__ side,
                                     unsigned char* __restrict__ code, uint32_t* __restrict__ touch_flag,
                                     unsigned char* __restrict__ keep_pos, unsigned char* __restrict__ keep_neg) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nt; i += gridDim.x * blockDim.x) {
    const int a = t[3 * i], b = t[3 * i + 1], c = t[3 * i + 2];
    int s0 = side[a], s1 = side[b], s2 = side[c];
    if (s0 == 0 && s1 == 0 && s2 == 0)
      s0 = s1 = s2 = coplanar_side(v + 3 * (int64_t)a, v + 3 * (int64_t)b, v + 3 * (int64_t)c, pl);
    const int sum = s0 + s1 + s2;
    if (sum == 3 || sum == -3) {
      code[i] = sum == 3 ? 0 : 1;
      touch_flag[i] = 0;
      unsigned char* k = sum == 3 ? keep_pos : keep_neg;
      k[a] = 1;
      k[b] = 1;
      k[c] = 1;
    } else {
      code[i] = 2;
      touch_flag[i] = 1;
    }
  }
}

__global__ void clip_compact_kernel(const uint32_t* __restrict__ flag, const uint64_t* __restrict__ off,
                                    int nt, int* __restrict__ list) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nt; i += gridDim.x * blockDim.x)
    if (flag[i]) list[off[i]] = i;
}

// ---- the ordered resolver (one CTA) ----------------------------------------
struct Resolver {
  const double* v;
  double* border;       // 3 doubles per border point
  int* vmap;            // mesh vertex -> border point (-1)
  int* ekeys;           // edge hash: key pairs (a, b), -1 empty
  int* evals;           // edge hash values
  int ecap;             // power of two
  int* bedge_a;         // unique border edges (1-based), in order
  int* bedge_b;
  int* bkeys;           // unordered-pair hash for edge dedup
  int bcap;
  int max_border;
  ClipCounters* cnt;
  unsigned* n_border;   // border point count (cnt->n_border, or a shared-memory copy)
  unsigned* n_bedges;   // border edge count (likewise)
};

// Shared-memory mode of the resolver: up to kSmemTouch touching triangles have
// at most 3 border points each, at most 6 directed-edge entries each and at
// most one border edge each, so tables of these capacities never fill.
constexpr int kSmemTouch = 1024;
constexpr int kSmemBorder = 3 * kSmemTouch + 16;
constexpr int kSmemEcap = 8192;
constexpr int kSmemBcap = 4096;
constexpr int kChunk = 32;
constexpr size_t kResolveSmem = (size_t)kSmemBorder * 24 + (size_t)kSmemEcap * 12 + (size_t)kSmemBcap * 8 +
                                (size_t)kChunk * 18 * 8 + (size_t)kChunk * 7 * 4 + 16;

// One warp resolves the touching triangles in order. Lane 0 owns every table
// update; the position scan runs across the 32 lanes (first match = smallest
// index with all three coordinates within 1e-4).
__device__ int find_near(Resolver& R, const double* p, int n) {
  int best = 0x7fffffff;
  for (int i = (int)(threadIdx.x & 31); i < n; i += 32) {
    const double* q = R.border + 3 * (int64_t)i;
    if (fabs(ds(q[0], p[0])) < 1e-4 && fabs(ds(q[1], p[1])) < 1e-4 && fabs(ds(q[2], p[2])) < 1e-4) {
      best = i;
      break;
    }
  }
  best = __reduce_min_sync(0xffffffffu, best);
  return best == 0x7fffffff ? -1 : best;
}

__device__ __forceinline__ unsigned hash2(int a, int b) {
  unsigned h = (unsigned)a * 0x9E3779B1u ^ ((unsigned)b + 0x7F4A7C15u) * 0x85EBCA77u;
  return h ^ (h >> 15);
}

// Directed edge table (thread 0 only).
__device__ int edge_get(Resolver& R, int a, int b) {
  unsigned m = (unsigned)R.ecap - 1u, h = hash2(a, b) & m;
  for (int probe = 0; probe < R.ecap; ++probe, h = (h + 1) & m) {
    if (R.ekeys[2 * h] == -1) return -1;
    if (R.ekeys[2 * h] == a && R.ekeys[2 * h + 1] == b) return R.evals[h];
  }
  return -1;
}
__device__ void edge_set(Resolver& R, int a, int b, int val) {
  unsigned m = (unsigned)R.ecap - 1u, h = hash2(a, b) & m;
  for (int probe = 0; probe < R.ecap; ++probe, h = (h + 1) & m) {
    if (R.ekeys[2 * h] == -1 || (R.ekeys[2 * h] == a && R.ekeys[2 * h + 1] == b)) {
      R.ekeys[2 * h] = a;
      R.ekeys[2 * h + 1] = b;
      R.evals[h] = val;
      return;
    }
  }
  R.cnt->overflow = 1;
}

__device__ __forceinline__ bool lane0() { return (threadIdx.x & 31) == 0; }

// Append a new border point (lane 0) or report overflow.
__device__ int append_border(Resolver& R, const double* p, int n) {
  if (n < R.max_border) {
    R.border[3 * n] = p[0];
    R.border[3 * n + 1] = p[1];
    R.border[3 * n + 2] = p[2];
    *R.n_border = n + 1;
    return n;
  }
  R.cnt->overflow = 1;
  return 0;
}

// Border point of a mesh vertex (whole warp calls; result broadcast).
__device__ int vertex_point(Resolver& R, int id) {
  int have = lane0() ? R.vmap[id] : 0;
  have = __shfl_sync(0xffffffffu, have, 0);
  if (have >= 0) return have;
  const int n = (int)*(volatile unsigned*)R.n_border;
  int f = find_near(R, R.v + 3 * (int64_t)id, n);
  if (lane0()) {
    if (f < 0) f = append_border(R, R.v + 3 * (int64_t)id, n);
    R.vmap[id] = f;
  }
  f = __shfl_sync(0xffffffffu, f, 0);
  __syncwarp();
  return f;
}

// Border point where edge (a, b) crosses the plane (whole warp).
__device__ int edge_point(Resolver& R, int a, int b, const double* p) {
  int have = 0;
  if (lane0()) {
    have = edge_get(R, a, b);
    if (have < 0) have = edge_get(R, b, a);
  }
  have = __shfl_sync(0xffffffffu, have, 0);
  if (have >= 0) return have;
  const int n = (int)*(volatile unsigned*)R.n_border;
  int f = find_near(R, p, n);
  if (lane0()) {
    if (f < 0) f = append_border(R, p, n);
    edge_set(R, a, b, f);
    edge_set(R, b, a, f);
  }
  f = __shfl_sync(0xffffffffu, f, 0);
  __syncwarp();
  return f;
}

// Unique unordered border edge, in first-occurrence order (thread 0 only).
__device__ void add_bedge(Resolver& R, int a, int b) {
  int lo = min(a, b), hi = max(a, b);
  unsigned m = (unsigned)R.bcap - 1u, h = hash2(lo, hi) & m;
  for (int probe = 0; probe < R.bcap; ++probe, h = (h + 1) & m) {
    if (R.bkeys[2 * h] == lo && R.bkeys[2 * h + 1] == hi) return;
    if (R.bkeys[2 * h] == -1) {
      R.bkeys[2 * h] = lo;
      R.bkeys[2 * h + 1] = hi;
      unsigned k = *R.n_bedges;
      R.bedge_a[k] = a;
      R.bedge_b[k] = b;
      *R.n_bedges = k + 1;
      return;
    }
  }
  R.cnt->overflow = 1;
}

__device__ __forceinline__ int bref(int b) { return -b - 1; }

// With at most kSmemTouch touching triangles the tables, the border points and
// the counters live in shared memory (copied out at the end); otherwise in
// the global buffers sized by the triangle count. Either way the triangles
// are staged 32 at a time, one lane each, together with everything about them
// that does not depend on the tables (sides with the coplanar rule, the three
// edge-plane intersections): the FP64 work runs once per triangle across the
// lanes, and the ordered walk reads the results from shared memory.
__global__ void __launch_bounds__(kClipResolveThreads) clip_resolve_kernel(
    const double* __restrict__ v, const int* __restrict__ t, const double* __restrict__ plp,
    const signed char* __restrict__ side, const int* __restrict__ list, Resolver R,
    PieceSlot* __restrict__ slots, unsigned char* __restrict__ keep_pos,
    unsigned char* __restrict__ keep_neg) {
  extern __shared__ __align__(16) unsigned char rsm[];
  double* sm_border = reinterpret_cast<double*>(rsm);
  int* sm_ekeys = reinterpret_cast<int*>(sm_border + 3 * kSmemBorder);
  int* sm_evals = sm_ekeys + 2 * kSmemEcap;
  int* sm_bkeys = sm_evals + kSmemEcap;
  double* ch_p = reinterpret_cast<double*>(sm_bkeys + 2 * kSmemBcap);  // kChunk x 9 vertex coordinates
  double* ch_pi = ch_p + kChunk * 9;                                   // kChunk x 9 edge intersections
  int* ch_id = reinterpret_cast<int*>(ch_pi + kChunk * 9);             // kChunk x 3
  int* ch_s = ch_id + kChunk * 3;                                      // kChunk x 3
  int* ch_f = ch_s + kChunk * 3;                                       // kChunk intersection flags
  unsigned* sm_cnt = reinterpret_cast<unsigned*>(ch_f + kChunk);       // n_border, n_bedges
  const int lane = threadIdx.x & 31;
  double pl[4] = {plp[0], plp[1], plp[2], plp[3]};
  const int ntouch = (int)R.cnt->n_touch;
  double* const global_border = R.border;
  const bool smem = ntouch <= kSmemTouch;
  if (smem) {
    for (int i = lane; i < 2 * kSmemEcap; i += 32) sm_ekeys[i] = -1;
    for (int i = lane; i < 2 * kSmemBcap; i += 32) sm_bkeys[i] = -1;
    if (lane == 0) sm_cnt[0] = sm_cnt[1] = 0;
    R.border = sm_border;
    R.ekeys = sm_ekeys;
    R.evals = sm_evals;
    R.ecap = kSmemEcap;
    R.bkeys = sm_bkeys;
    R.bcap = kSmemBcap;
    R.max_border = kSmemBorder;
    R.n_border = sm_cnt;
    R.n_bedges = sm_cnt + 1;
  } else {
    R.n_border = &R.cnt->n_border;
    R.n_bedges = &R.cnt->n_bedges;
  }
  __syncwarp();
  for (int li = 0; li < ntouch; ++li) {
    const int cc = li % kChunk;
    if (cc == 0) {
      __syncwarp();
      if (li + lane < ntouch) {
        const int tr = list[li + lane];
        int sl[3];
        for (int k = 0; k < 3; ++k) {
          const int vk = t[3 * tr + k];
          ch_id[3 * lane + k] = vk;
          sl[k] = side[vk];
          for (int a = 0; a < 3; ++a) ch_p[9 * lane + 3 * k + a] = v[3 * (int64_t)vk + a];
        }
        const double* q = ch_p + 9 * lane;
        if (sl[0] == 0 && sl[1] == 0 && sl[2] == 0) sl[0] = sl[1] = sl[2] = coplanar_side(q, q + 3, q + 6, pl);
        int fl = 0;
        for (int e = 0; e < 3; ++e)
          if (intersect_segment(pl, q + 3 * e, q + 3 * ((e + 1) % 3), ch_pi + 9 * lane + 3 * e)) fl |= 1 << e;
        for (int k = 0; k < 3; ++k) ch_s[3 * lane + k] = sl[k];
        ch_f[lane] = fl;
      }
      __syncwarp();
    }
    const int id[3] = {ch_id[3 * cc], ch_id[3 * cc + 1], ch_id[3 * cc + 2]};
    const double* p[3] = {ch_p + 9 * cc, ch_p + 9 * cc + 3, ch_p + 9 * cc + 6};
    const int s[3] = {ch_s[3 * cc], ch_s[3 * cc + 1], ch_s[3 * cc + 2]};
    const int sum = s[0] + s[1] + s[2];
    const int nzero = (s[0] == 0) + (s[1] == 0) + (s[2] == 0);
    PieceSlot out;
    out.npos = out.nneg = 0;
    auto emit = [&](bool pos, int x, int y, int z) {
      if (pos) {
        out.pos[out.npos][0] = x; out.pos[out.npos][1] = y; out.pos[out.npos][2] = z; ++out.npos;
      } else {
        out.neg[out.nneg][0] = x; out.neg[out.nneg][1] = y; out.neg[out.nneg][2] = z; ++out.nneg;
      }
    };
    auto keep = [&](bool pos, int vid) {
      if (lane0()) (pos ? keep_pos : keep_neg)[vid] = 1;
    };
    const bool one_pos = sum == 2 || (sum == 1 && nzero == 2);
    const bool one_neg = sum == -2 || (sum == -1 && nzero == 2);
    if (one_pos || one_neg) {
      const int sg = one_pos ? 1 : -1;
      if (sum == sg) {
        int k = s[0] != 0 ? 0 : (s[1] != 0 ? 1 : 2);
        int k1 = (k + 1) % 3, k2 = (k + 2) % 3;
        int b1, b2;
        if (sg > 0) {
          b1 = vertex_point(R, id[k1]);
          b2 = vertex_point(R, id[k2]);
        } else {
          b2 = vertex_point(R, id[k2]);
          b1 = vertex_point(R, id[k1]);
        }
        if (b1 != b2) {
          if (lane0()) {
            if (sg > 0) add_bedge(R, b1 + 1, b2 + 1);
            else add_bedge(R, b2 + 1, b1 + 1);
          }
          emit(sg > 0, id[k], bref(b1), bref(b2));
          keep(sg > 0, id[k]);
        }
      } else {
        int z = s[0] == 0 ? 0 : (s[1] == 0 ? 1 : 2);
        int bz = vertex_point(R, id[z]);
        if (z == 2) emit(sg > 0, id[0], id[1], bref(bz));
        else if (z == 0) emit(sg > 0, id[1], id[2], bref(bz));
        else emit(sg > 0, id[0], bref(bz), id[2]);
        for (int k = 0; k < 3; ++k)
          if (k != z) keep(sg > 0, id[k]);
      }
    } else {
      const double* pi[3] = {ch_pi + 9 * cc, ch_pi + 9 * cc + 3, ch_pi + 9 * cc + 6};
      const int fl = ch_f[cc];
      const bool f[3] = {(fl & 1) != 0, (fl & 2) != 0, (fl & 4) != 0};
      int e = -1;
      if (f[0] && f[1] && !f[2]) e = 0;
      else if (f[1] && f[2] && !f[0]) e = 1;
      else if (f[2] && f[0] && !f[1]) e = 2;
      if (e >= 0) {
        const int a = e, vv = (e + 1) % 3, c = (e + 2) % 3;
        edge_point(R, id[a], id[vv], pi[a]);
        edge_point(R, id[vv], id[c], pi[vv]);
        int fa = 0, fv = 0;
        if (lane0()) {
          fa = edge_get(R, id[a], id[vv]);
          fv = edge_get(R, id[vv], id[c]);
        }
        fa = __shfl_sync(0xffffffffu, fa, 0);
        fv = __shfl_sync(0xffffffffu, fv, 0);
        const bool apex_pos = s[vv] == 1;
        if (fv != fa) {
          if (lane0()) {
            if (apex_pos) add_bedge(R, fv + 1, fa + 1);
            else add_bedge(R, fa + 1, fv + 1);
          }
          keep(apex_pos, id[vv]);
          keep(!apex_pos, id[a]);
          keep(!apex_pos, id[c]);
          emit(apex_pos, id[vv], bref(fv), bref(fa));
          if (e == 0) {
            emit(!apex_pos, id[a], bref(fa), bref(fv));
            emit(!apex_pos, bref(fv), id[c], id[a]);
          } else {
            emit(!apex_pos, id[c], bref(fa), bref(fv));
            emit(!apex_pos, bref(fa), id[c], id[a]);
          }
        } else {
          keep(!apex_pos, id[a]);
          keep(!apex_pos, id[c]);
          emit(!apex_pos, e == 0 ? bref(fv) : bref(fa), id[c], id[a]);
        }
      } else if (f[0] && f[1] && f[2]) {
        const bool all_nz = s[0] != 0 && s[1] != 0 && s[2] != 0;
        auto same = [](const double* x, const double* y) {
          const double eps = (double)1e-5f;
          return fabs(ds(x[0], y[0])) < eps && fabs(ds(x[1], y[1])) < eps && fabs(ds(x[2], y[2])) < eps;
        };
        int k = -1;
        if (s[0] == 0 || (all_nz && same(pi[0], pi[2]))) k = 0;
        else if (s[1] == 0 || (all_nz && same(pi[0], pi[1]))) k = 1;
        else if (s[2] == 0 || (all_nz && same(pi[1], pi[2]))) k = 2;
        if (k >= 0) {
          const int k1 = (k + 1) % 3, k2 = (k + 2) % 3;
          const int bk = vertex_point(R, id[k]);
          if (lane0()) {
            edge_set(R, id[k], id[k1], bk);
            edge_set(R, id[k1], id[k], bk);
            edge_set(R, id[k2], id[k], bk);
            edge_set(R, id[k], id[k2], bk);
          }
          __syncwarp();
          edge_point(R, id[k1], id[k2], pi[k1]);
          int fo = lane0() ? edge_get(R, id[k1], id[k2]) : 0;
          fo = __shfl_sync(0xffffffffu, fo, 0);
          const int test = (k == 0) ? s[1] : s[0];
          const int u = (k == 1) ? k2 : k1;
          const int other = (k == 1) ? k1 : k2;
          int A, Bp;
          if (k == 1) { A = bk; Bp = fo; } else { A = fo; Bp = bk; }
          if (A != Bp) {
            if (lane0()) {
              if (test == 1) add_bedge(R, A + 1, Bp + 1);
              else add_bedge(R, Bp + 1, A + 1);
            }
            keep(test == 1, id[u]);
            keep(test != 1, id[other]);
            emit(test == 1, id[u], bref(A), bref(Bp));
            emit(test != 1, id[other], bref(Bp), bref(A));
          }
        }
      }
    }
    if (lane0()) slots[li] = out;
    __syncwarp();
  }
  if (smem) {
    const unsigned nb = sm_cnt[0];
    for (unsigned i = lane; i < 3 * nb; i += 32) global_border[i] = sm_border[i];
    if (lane == 0) {
      R.cnt->n_border = nb;
      R.cnt->n_bedges = sm_cnt[1];
    }
  }
}

// Per-triangle output counts (pos, neg) in triangle order.
__global__ void clip_counts_kernel(const unsigned char* __restrict__ code, const uint64_t* __restrict__ toff,
                                   const PieceSlot* __restrict__ slots, int nt, uint32_t* __restrict__ cpos,
                                   uint32_t* __restrict__ cneg) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nt; i += gridDim.x * blockDim.x) {
    unsigned char c = code[i];
    if (c == 0) { cpos[i] = 1; cneg[i] = 0; }
    else if (c == 1) { cpos[i] = 0; cneg[i] = 1; }
    else {
      const PieceSlot& s = slots[toff[i]];
      cpos[i] = (uint32_t)s.npos;
      cneg[i] = (uint32_t)s.nneg;
    }
  }
}

__global__ void keep_to_u32_kernel(const unsigned char* __restrict__ k, int n, uint32_t* __restrict__ o) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) o[i] = k[i];
}

// Scatter + remap: original vertex -> map - 1, border point b -> n_side + b.
__global__ void clip_scatter_kernel(const int* __restrict__ t, const unsigned char* __restrict__ code,
                                    const uint64_t* __restrict__ toff, const PieceSlot* __restrict__ slots,
                                    int nt, const uint64_t* __restrict__ opos, const uint64_t* __restrict__ oneg,
                                    const uint64_t* __restrict__ mpos, const uint64_t* __restrict__ mneg,
                                    const unsigned char* __restrict__ kpos, const unsigned char* __restrict__ kneg,
                                    int nv, int* __restrict__ out_pos, int* __restrict__ out_neg) {
  const unsigned npos_v = (unsigned)mpos[nv], nneg_v = (unsigned)mneg[nv];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nt; i += gridDim.x * blockDim.x) {
    auto rp = [&](int x) { return x >= 0 ? (int)mpos[x] : (int)npos_v + (-x - 1); };
    auto rn = [&](int x) { return x >= 0 ? (int)mneg[x] : (int)nneg_v + (-x - 1); };
    unsigned char c = code[i];
    if (c == 0) {
      int* o = out_pos + 3 * opos[i];
      o[0] = rp(t[3 * i]); o[1] = rp(t[3 * i + 1]); o[2] = rp(t[3 * i + 2]);
    } else if (c == 1) {
      int* o = out_neg + 3 * oneg[i];
      o[0] = rn(t[3 * i]); o[1] = rn(t[3 * i + 1]); o[2] = rn(t[3 * i + 2]);
    } else {
      const PieceSlot& s = slots[toff[i]];
      for (int k = 0; k < s.npos; ++k) {
        int* o = out_pos + 3 * (opos[i] + k);
        o[0] = rp(s.pos[k][0]); o[1] = rp(s.pos[k][1]); o[2] = rp(s.pos[k][2]);
      }
      for (int k = 0; k < s.nneg; ++k) {
        int* o = out_neg + 3 * (oneg[i] + k);
        o[0] = rn(s.neg[k][0]); o[1] = rn(s.neg[k][1]); o[2] = rn(s.neg[k][2]);
      }
    }
  }
  (void)kpos;
  (void)kneg;
}

// 1-based maps (0 = absent).
__global__ void clip_maps_kernel(const unsigned char* __restrict__ kpos, const unsigned char* __restrict__ kneg,
                                 const uint64_t* __restrict__ mpos, const uint64_t* __restrict__ mneg, int nv,
                                 int* __restrict__ map_pos, int* __restrict__ map_neg) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += gridDim.x * blockDim.x) {
    map_pos[i] = kpos[i] ? (int)mpos[i] + 1 : 0;
    map_neg[i] = kneg[i] ? (int)mneg[i] + 1 : 0;
  }
}

}  // namespace vgpu

using namespace vgpu;

static size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

extern "C" int visacd_clip(visacd_ctx* ctx, const double* verts, int32_t nv, const int32_t* tris,
                           int32_t nt, const double* plane, visacd_clip_result* res) {
  VCHECK(ctx && res && plane, VISACD_ERR_INVALID_ARG, "visacd_clip: null argument");
  VCHECK(nv >= 0 && nt >= 0 && (nv == 0 || verts) && (nt == 0 || tris), VISACD_ERR_INVALID_ARG,
         "visacd_clip: bad mesh");
  memset(res, 0, sizeof(*res));
  if (nt == 0 || nv == 0) return VISACD_OK;
  VCHECK(indices_in_range(tris, 3LL * nt, nv), VISACD_ERR_INVALID_ARG, "visacd_clip: triangle index out of range");
  VCUDA(cudaSetDevice(ctx->device));
  // Border points are bounded by the touching triangles (3 each).
  const int max_border = 3 * nt + 16;
  int ecap = 64;
  while (ecap < 8 * max_border) ecap <<= 1;
  int bcap = 64;
  while (bcap < 4 * max_border) bcap <<= 1;
  size_t off = 0;
  auto carve = [&](size_t b) { size_t o = off; off += align256(b); return o; };
  const size_t o_v = carve((size_t)nv * 24), o_t = carve((size_t)nt * 12), o_pl = carve(32),
               o_side = carve(nv), o_code = carve(nt), o_tf = carve((size_t)nt * 4),
               o_toff = carve((size_t)(nt + 1) * 8), o_list = carve((size_t)nt * 4),
               o_kp = carve(nv), o_kn = carve(nv), o_cnt = carve(sizeof(ClipCounters)),
               o_border = carve((size_t)max_border * 24), o_vmap = carve((size_t)nv * 4),
               o_ek = carve((size_t)ecap * 8), o_ev = carve((size_t)ecap * 4),
               o_ba = carve((size_t)max_border * 4 * 3), o_bb = carve((size_t)max_border * 4 * 3),
               o_bk = carve((size_t)bcap * 8), o_slots = carve((size_t)nt * sizeof(PieceSlot)),
               o_cp = carve((size_t)nt * 4), o_cn = carve((size_t)nt * 4),
               o_op = carve((size_t)(nt + 1) * 8), o_on = carve((size_t)(nt + 1) * 8),
               o_ku = carve((size_t)nv * 4), o_mp = carve((size_t)(nv + 1) * 8),
               o_mn = carve((size_t)(nv + 1) * 8), o_outp = carve((size_t)nt * 3 * 12),
               o_outn = carve((size_t)nt * 3 * 12), o_mapp = carve((size_t)nv * 4),
               o_mapn = carve((size_t)nv * 4);
  VTRY(ensure_slot(ctx, kSlotClip, off));
  char* B = slot<char>(ctx, kSlotClip);
  double* dv = (double*)(B + o_v);
  int* dt = (int*)(B + o_t);
  double* dpl = (double*)(B + o_pl);
  signed char* side = (signed char*)(B + o_side);
  unsigned char* code = (unsigned char*)(B + o_code);
  uint32_t* tf = (uint32_t*)(B + o_tf);
  uint64_t* toff = (uint64_t*)(B + o_toff);
  int* list = (int*)(B + o_list);
  unsigned char *kp = (unsigned char*)(B + o_kp), *kn = (unsigned char*)(B + o_kn);
  ClipCounters* cnt = (ClipCounters*)(B + o_cnt);
  Resolver R;
  R.v = dv;
  R.border = (double*)(B + o_border);
  R.vmap = (int*)(B + o_vmap);
  R.ekeys = (int*)(B + o_ek);
  R.evals = (int*)(B + o_ev);
  R.ecap = ecap;
  R.bedge_a = (int*)(B + o_ba);
  R.bedge_b = (int*)(B + o_bb);
  R.bkeys = (int*)(B + o_bk);
  R.bcap = bcap;
  R.max_border = max_border;
  R.cnt = cnt;
  PieceSlot* slots = (PieceSlot*)(B + o_slots);
  uint32_t *cp = (uint32_t*)(B + o_cp), *cn = (uint32_t*)(B + o_cn), *ku = (uint32_t*)(B + o_ku);
  uint64_t *op = (uint64_t*)(B + o_op), *on = (uint64_t*)(B + o_on), *mp = (uint64_t*)(B + o_mp),
           *mn = (uint64_t*)(B + o_mn);
  int *outp = (int*)(B + o_outp), *outn = (int*)(B + o_outn), *mapp = (int*)(B + o_mapp),
      *mapn = (int*)(B + o_mapn);
  cudaStream_t st = ctx->stream;
  Stager up(ctx);
  VTRY(up.reserve((size_t)nv * 24 + (size_t)nt * 12 + 32, 3));
  VTRY(up.put(dv, verts, (size_t)nv * 24));
  VTRY(up.put(dt, tris, (size_t)nt * 12));
  VTRY(up.put(dpl, plane, 32));
  VCUDA(cudaMemsetAsync(kp, 0, nv, st));
  VCUDA(cudaMemsetAsync(kn, 0, nv, st));
  VCUDA(cudaMemsetAsync(cnt, 0, sizeof(ClipCounters), st));
  VCUDA(cudaMemsetAsync(R.vmap, 0xff, (size_t)nv * 4, st));
  VCUDA(cudaMemsetAsync(R.ekeys, 0xff, (size_t)ecap * 8, st));
  VCUDA(cudaMemsetAsync(R.bkeys, 0xff, (size_t)bcap * 8, st));
  const unsigned gv = grid_for(nv, 256, 8LL * ctx->sm_count), gt = grid_for(nt, 256, 8LL * ctx->sm_count);
  VLAUNCH(ctx, kKClip, gv, 256, 0, clip_sides_kernel, dv, nv, dpl, side);
  VLAUNCH(ctx, kKClip, gt, 256, 0, clip_classify_kernel, dv, dt, nt, dpl, side, code, tf, kp, kn);
  VTRY(exclusive_scan_u32_to_u64(ctx, tf, toff, nt));
  VLAUNCH(ctx, kKClip, gt, 256, 0, clip_compact_kernel, tf, toff, nt, list);
  VCUDA(cudaMemcpyAsync(&cnt->n_touch, toff + nt, 4, cudaMemcpyDeviceToDevice, st));
  VCUDA(cudaFuncSetAttribute(clip_resolve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kResolveSmem));
  VLAUNCH(ctx, kKClipResolve, 1, kClipResolveThreads, kResolveSmem, clip_resolve_kernel, dv, dt, dpl, side,
          list, R, slots, kp, kn);
  VLAUNCH(ctx, kKClip, gt, 256, 0, clip_counts_kernel, code, toff, slots, nt, cp, cn);
  VTRY(exclusive_scan_u32_to_u64(ctx, cp, op, nt));
  VTRY(exclusive_scan_u32_to_u64(ctx, cn, on, nt));
  VLAUNCH(ctx, kKClip, gv, 256, 0, keep_to_u32_kernel, kp, nv, ku);
  VTRY(exclusive_scan_u32_to_u64(ctx, ku, mp, nv));
  VLAUNCH(ctx, kKClip, gv, 256, 0, keep_to_u32_kernel, kn, nv, ku);
  VTRY(exclusive_scan_u32_to_u64(ctx, ku, mn, nv));
  VLAUNCH(ctx, kKClip, gt, 256, 0, clip_scatter_kernel, dt, code, toff, slots, nt, op, on, mp, mn, kp,
          kn, nv, outp, outn);
  VLAUNCH(ctx, kKClip, gv, 256, 0, clip_maps_kernel, kp, kn, mp, mn, nv, mapp, mapn);
  // Counts back to the host.
  ClipCounters* h = nullptr;
  VTRY(pinned(ctx, 64 + 4 * sizeof(uint64_t), (void**)&h));
  uint64_t* h64 = reinterpret_cast<uint64_t*>(reinterpret_cast<char*>(h) + 64);
  VCUDA(cudaMemcpyAsync(h, cnt, sizeof(ClipCounters), cudaMemcpyDeviceToHost, st));
  VCUDA(cudaMemcpyAsync(h64 + 0, op + nt, 8, cudaMemcpyDeviceToHost, st));
  VCUDA(cudaMemcpyAsync(h64 + 1, on + nt, 8, cudaMemcpyDeviceToHost, st));
  VCUDA(cudaMemcpyAsync(h64 + 2, mp + nv, 8, cudaMemcpyDeviceToHost, st));
  VCUDA(cudaMemcpyAsync(h64 + 3, mn + nv, 8, cudaMemcpyDeviceToHost, st));
  VCUDA(stream_wait(ctx));
  VCHECK(!h->overflow, VISACD_ERR_CAPACITY, "visacd_clip: internal table overflow");
  ctx->clip_out.n_pos = (int32_t)h64[0];
  ctx->clip_out.n_neg = (int32_t)h64[1];
  ctx->clip_out.nv_pos = (int32_t)h64[2];
  ctx->clip_out.nv_neg = (int32_t)h64[3];
  ctx->clip_out.n_border = (int32_t)h->n_border;
  ctx->clip_out.n_border_edges = (int32_t)h->n_bedges;
  ctx->clip_out.n_touching = (int32_t)h->n_touch;
  ctx->clip_nv = nv;
  ctx->clip_ptrs[0] = outp;
  ctx->clip_ptrs[1] = outn;
  ctx->clip_ptrs[2] = mapp;
  ctx->clip_ptrs[3] = mapn;
  ctx->clip_ptrs[4] = R.border;
  ctx->clip_ptrs[5] = R.bedge_a;
  ctx->clip_ptrs[6] = R.bedge_b;
  *res = ctx->clip_out;
  return VISACD_OK;
}

extern "C" int visacd_clip_fetch(visacd_ctx* ctx, int32_t* pos_tris, int32_t* neg_tris,
                                 int32_t* pos_map, int32_t* neg_map, double* border,
                                 int32_t* border_edges) {
  VCHECK(ctx, VISACD_ERR_INVALID_ARG, "visacd_clip_fetch: null context");
  const visacd_clip_result& r = ctx->clip_out;
  cudaStream_t st = ctx->stream;
  if (pos_tris && r.n_pos) VCUDA(cudaMemcpyAsync(pos_tris, ctx->clip_ptrs[0], (size_t)r.n_pos * 12, cudaMemcpyDeviceToHost, st));
  if (neg_tris && r.n_neg) VCUDA(cudaMemcpyAsync(neg_tris, ctx->clip_ptrs[1], (size_t)r.n_neg * 12, cudaMemcpyDeviceToHost, st));
  if (pos_map) VCUDA(cudaMemcpyAsync(pos_map, ctx->clip_ptrs[2], (size_t)ctx->clip_nv * 4, cudaMemcpyDeviceToHost, st));
  if (neg_map) VCUDA(cudaMemcpyAsync(neg_map, ctx->clip_ptrs[3], (size_t)ctx->clip_nv * 4, cudaMemcpyDeviceToHost, st));
  if (border && r.n_border) VCUDA(cudaMemcpyAsync(border, ctx->clip_ptrs[4], (size_t)r.n_border * 24, cudaMemcpyDeviceToHost, st));
  if (border_edges && r.n_border_edges) {
    // Interleave (a, b) on the host side of the copy: fetch both columns.
    std::vector<int32_t> a(r.n_border_edges), b(r.n_border_edges);
    VCUDA(cudaMemcpyAsync(a.data(), ctx->clip_ptrs[5], (size_t)r.n_border_edges * 4, cudaMemcpyDeviceToHost, st));
    VCUDA(cudaMemcpyAsync(b.data(), ctx->clip_ptrs[6], (size_t)r.n_border_edges * 4, cudaMemcpyDeviceToHost, st));
    VCUDA(stream_wait(ctx));
    for (int32_t k = 0; k < r.n_border_edges; ++k) {
      border_edges[2 * k] = a[k];
      border_edges[2 * k + 1] = b[k];
    }
  }
  VCUDA(stream_wait(ctx));
  return VISACD_OK;
}

// Sampled face Hausdorff distance on the GPU (the hb term of the concavity
// metric, lib/include/hausdorff.hpp:214-298 / lib/src/cost.cpp:69-85).
//
// For every sample q of one surface: its 10 nearest samples on the other
// surface (exact k-NN, FP64 squared distances), then the smallest distance
// from q to the triangles those samples were drawn from (stopping below
// 1e-14); a minimum above 10 is replaced by the nearest-sample distance; the
// result is the largest minimum over both directions. Organised as a bounded
// max-min search with every shortcut exact:
//  * both sample sets are bucketed in uniform grids (counting sort) and both
//    meshes get FP32 triangle bounds (box, plane), in four launches plus a scan;
//  * a two-ring search gives each query an upper bound of its term (the
//    nearest sample's distance, rounded up); queries with no sample that
//    close are evaluated one warp each (hhead_kernel);
//  * the rest skip when their bound does not exceed the running maximum;
//  * k-NN candidates are ranked in FP32 with a proven rounding margin and the
//    exact 10 chosen in FP64; triangle distances whose FP32 lower bound cannot
//    lower the minimum are skipped.
//  * Point-triangle distance: closest point by Voronoi region (Ericson,
//    Real-Time Collision Detection 5.1.5) in FP64 with explicit round-to-
//    nearest intrinsics in the host's operation order, so values equal the
//    host implementation's.
#include <float.h>

#include "common.cuh"
#include "geom64.cuh"

namespace vgpu {

constexpr int kKnn = 10;

struct HGrid {
  double lo[3];
  double h;
  int dim[3];
  const int* start;   // cell -> first sorted point (size cells + 1)
  const int* order;   // sorted point ids
  const double* pts;  // 3 doubles per point
  const float4* spts; // points in cell order as float (x, y, z, id bits): the FP32 pre-filter
  int n;
  float eabs;         // bound of |FP32 distance - exact distance| for this grid's points and queries
};

__device__ __forceinline__ int cell_coord(double x, double lo, double h, int dim) {
  int c = (int)floor((x - lo) / h);
  return c < 0 ? 0 : (c >= dim ? dim - 1 : c);
}

// Exact k nearest samples of q by Chebyshev rings of grid cells around q's
// cell, until the k found are settled (the k-th is no farther than the ring
// radius) or every cell was seen.
__device__ __forceinline__ void knn_rings(const HGrid& G, const double (&q)[3], double (&bd)[kKnn],
                                          int (&bi)[kKnn], int& cnt) {
  const int cx = cell_coord(q[0], G.lo[0], G.h, G.dim[0]);
  const int cy = cell_coord(q[1], G.lo[1], G.h, G.dim[1]);
  const int cz = cell_coord(q[2], G.lo[2], G.h, G.dim[2]);
  const int rmax = max(G.dim[0], max(G.dim[1], G.dim[2]));
  const float qf[3] = {(float)q[0], (float)q[1], (float)q[2]};
  float thr = 3.4e38f;
  for (int r = 0; r <= rmax; ++r) {
    for (int dz = -r; dz <= r; ++dz) {
      const int z = cz + dz;
      if (z < 0 || z >= G.dim[2]) continue;
      for (int dy = -r; dy <= r; ++dy) {
        const int y = cy + dy;
        if (y < 0 || y >= G.dim[1]) continue;
        const bool face = abs(dz) == r || abs(dy) == r;
        for (int dx = -r; dx <= r; dx += (face ? 1 : 2 * r > 0 ? 2 * r : 1)) {
          const int x = cx + dx;
          if (x >= 0 && x < G.dim[0]) {
            const int c = (z * G.dim[1] + y) * G.dim[0] + x;
            for (int k = G.start[c]; k < G.start[c + 1]; ++k) {
              const float4 sp = G.spts[k];
              // FP32 pre-filter: a candidate whose FP32 distance exceeds the
              // current k-th distance by more than the rounding bound cannot
              // enter the list; the rest are decided in FP64.
              if (cnt == kKnn) {
                const float fx = sp.x - qf[0], fy = sp.y - qf[1], fz = sp.z - qf[2];
                if (fx * fx + fy * fy + fz * fz > thr) continue;
              }
              const int pi = __float_as_int(sp.w);
              const double* pp = G.pts + 3 * (int64_t)pi;
              const double ex = ds(pp[0], q[0]), ey = ds(pp[1], q[1]), ez = ds(pp[2], q[2]);
              const double d2 = da(da(dm(ex, ex), dm(ey, ey)), dm(ez, ez));
              if (cnt < kKnn || d2 < bd[cnt - 1]) {
                int j = cnt < kKnn ? cnt++ : kKnn - 1;
                while (j > 0 && bd[j - 1] > d2) {
                  bd[j] = bd[j - 1];
                  bi[j] = bi[j - 1];
                  --j;
                }
                bd[j] = d2;
                bi[j] = pi;
                if (cnt == kKnn) {
                  // (sqrt(kth) + eabs)^2 with every FP32 step rounded upwards
                  const float b = __fadd_ru(__fsqrt_ru(__double2float_ru(bd[kKnn - 1])), G.eabs);
                  thr = __fmul_ru(__fmul_ru(b, b), 1.0f + 1.0f / 65536.0f);
                }
              }
            }
          }
          if (dx == r) break;
        }
      }
    }
    const double rad = (double)r * G.h;
    if (cnt == kKnn && bd[kKnn - 1] <= rad * rad) return;
  }
}

// FP32 ranking variant of knn_rings: candidates are ranked by their FP32
// squared distance (kKnnF best kept), the rings stop once the 10th FP32
// distance plus the rounding bound lies inside the ring radius, and the exact
// 10 nearest are then chosen by FP64 among the kKnnF. Returns false when the
// FP32 list cannot prove it holds the exact 10 nearest (the 10th and the
// kKnnF-th FP32 distances closer than twice the bound), in which case the
// caller runs the exact FP64 walk.
constexpr int kKnnF = 16;
__device__ __forceinline__ bool knn_rings_f32(const HGrid& G, const double (&q)[3], double (&bd)[kKnn],
                                              int (&bi)[kKnn], int& cnt) {
  const int cx = cell_coord(q[0], G.lo[0], G.h, G.dim[0]);
  const int cy = cell_coord(q[1], G.lo[1], G.h, G.dim[1]);
  const int cz = cell_coord(q[2], G.lo[2], G.h, G.dim[2]);
  const int rmax = max(G.dim[0], max(G.dim[1], G.dim[2]));
  const float qf[3] = {(float)q[0], (float)q[1], (float)q[2]};
  const float hf = (float)G.h;
  float fd[kKnnF];
  int fi[kKnnF];
  int nf = 0;
  for (int r = 0; r <= rmax; ++r) {
    for (int dz = -r; dz <= r; ++dz) {
      const int z = cz + dz;
      if (z < 0 || z >= G.dim[2]) continue;
      for (int dy = -r; dy <= r; ++dy) {
        const int y = cy + dy;
        if (y < 0 || y >= G.dim[1]) continue;
        const bool face = abs(dz) == r || abs(dy) == r;
        for (int dx = -r; dx <= r; dx += (face ? 1 : 2 * r > 0 ? 2 * r : 1)) {
          const int x = cx + dx;
          if (x >= 0 && x < G.dim[0]) {
            const int c = (z * G.dim[1] + y) * G.dim[0] + x;
            for (int k = G.start[c]; k < G.start[c + 1]; ++k) {
              const float4 sp = G.spts[k];
              const float ex = sp.x - qf[0], ey = sp.y - qf[1], ez = sp.z - qf[2];
              const float d2 = ex * ex + ey * ey + ez * ez;
              if (nf < kKnnF || d2 < fd[nf - 1]) {
                int j = nf < kKnnF ? nf++ : kKnnF - 1;
                while (j > 0 && fd[j - 1] > d2) {
                  fd[j] = fd[j - 1];
                  fi[j] = fi[j - 1];
                  --j;
                }
                fd[j] = d2;
                fi[j] = __float_as_int(sp.w);
              }
            }
          }
          if (dx == r) break;
        }
      }
    }
    // Settled: 10 candidates whose exact distance is at most
    // sqrt(fd[9]) (1 + 2^-20) + eabs lie within the radius r h (less a
    // 1e-6 h allowance for the query's cell), so nothing unvisited is nearer.
    if (nf >= kKnn && __fadd_ru(__fmul_ru(__fsqrt_ru(fd[kKnn - 1]), 1.0f + 1.0f / 1048576.0f), G.eabs) <=
                          __fmul_rd((float)r, hf) * (1.0f - 1e-6f))
      break;
  }
  // The exact 10 nearest are among the kept ones when the kKnnF-th FP32
  // distance exceeds the 10th by more than twice the bound (or all were kept).
  if (nf == kKnnF &&
      !(__fsqrt_rd(fd[kKnnF - 1]) * (1.0f - 1.0f / 1048576.0f) >
        __fadd_ru(__fadd_ru(__fmul_ru(__fsqrt_ru(fd[kKnn - 1]), 1.0f + 1.0f / 1048576.0f), G.eabs), G.eabs)))
    return false;
  cnt = 0;
  for (int m = 0; m < nf; ++m) {
    const int pi = fi[m];
    const double* pp = G.pts + 3 * (int64_t)pi;
    const double ex = ds(pp[0], q[0]), ey = ds(pp[1], q[1]), ez = ds(pp[2], q[2]);
    const double d2 = da(da(dm(ex, ex), dm(ey, ey)), dm(ez, ez));
    if (cnt < kKnn || d2 < bd[cnt - 1]) {
      int j = cnt < kKnn ? cnt++ : kKnn - 1;
      while (j > 0 && bd[j - 1] > d2) {
        bd[j] = bd[j - 1];
        bi[j] = bi[j - 1];
        --j;
      }
      bd[j] = d2;
      bi[j] = pi;
    }
  }
  return true;
}

// One direction's data: queries Q against the other surface (grid G over its
// samples, the triangle each sample was drawn from, that mesh and its FP32
// triangle bounds).
struct HSide {
  const double* Q;
  int nq;
  HGrid G;
  const int* ids;
  const double* mv;
  const int* mt;
  const float4* tb;
};

// The query's term of the directed distance: the smallest FP64 distance to the
// triangles of its k nearest samples, in their order, stopping below 1e-14;
// the nearest-sample distance when that exceeds 10; DBL_MAX without samples.
// A triangle already seen, or whose FP32 lower bound (box gap or plane
// distance, minus the rounding margin) is not below the current minimum,
// cannot lower it and is not evaluated.
__device__ double query_term(const HSide& S, int qi, float tmargin) {
  const double q[3] = {S.Q[3 * (int64_t)qi], S.Q[3 * (int64_t)qi + 1], S.Q[3 * (int64_t)qi + 2]};
  double bd[kKnn];
  int bi[kKnn];
  int cnt = 0;
  if (!knn_rings_f32(S.G, q, bd, bi, cnt)) {
    cnt = 0;
    knn_rings(S.G, q, bd, bi, cnt);
  }
  double cmin = DBL_MAX;
  int seen[kKnn];
  const float qfx = (float)q[0], qfy = (float)q[1], qfz = (float)q[2];
  for (int j = 0; j < cnt; ++j) {
    const int tri = S.ids[bi[j]];
    bool dup = false;
    for (int u = 0; u < j; ++u) dup |= seen[u] == tri;
    seen[j] = tri;
    if (dup) continue;
    if (cmin < DBL_MAX) {
      const float4 lo = S.tb[3 * (int64_t)tri], hi = S.tb[3 * (int64_t)tri + 1], pl = S.tb[3 * (int64_t)tri + 2];
      const float gx = fmaxf(fmaxf(lo.x - qfx, qfx - hi.x), 0.f);
      const float gy = fmaxf(fmaxf(lo.y - qfy, qfy - hi.y), 0.f);
      const float gz = fmaxf(fmaxf(lo.z - qfz, qfz - hi.z), 0.f);
      const float lb = fmaxf(sqrtf(gx * gx + gy * gy + gz * gz), fabsf(pl.x * qfx + pl.y * qfy + pl.z * qfz + pl.w));
      if ((double)(lb - tmargin) >= cmin) continue;
    }
    const int* t = S.mt + 3 * (int64_t)tri;
    const double d = point_tri_dist(q, S.mv + 3 * (int64_t)t[0], S.mv + 3 * (int64_t)t[1], S.mv + 3 * (int64_t)t[2]);
    if (d < cmin) {
      cmin = d;
      if (cmin < 1e-14) break;
    }
  }
  if (cmin > 10 && cnt > 0) cmin = __dsqrt_rn(bd[0]);
  return cmin;
}

// The smallest not-yet-taken value across the warp's sorted per-lane lists
// (fd[ptr..]), taken: returns it and its id; ties go to the lower lane.
__device__ __forceinline__ float warp_take_min(const float (&fd)[kKnnF], const int (&fi)[kKnnF], int nf, int& ptr,
                                               int& id_out) {
  const int lane = threadIdx.x & 31;
  const float mine = ptr < nf ? fd[ptr] : 3.4e38f;
  float m = mine;
  for (int o = 16; o; o >>= 1) m = fminf(m, __shfl_xor_sync(0xffffffffu, m, o));
  const unsigned who = __ballot_sync(0xffffffffu, mine == m && ptr < nf);
  const int src = who ? __ffs(who) - 1 : 0;
  int id = ptr < nf ? fi[ptr] : -1;
  id = __shfl_sync(0xffffffffu, id, src);
  if (who && lane == src) ++ptr;
  id_out = who ? id : -1;
  return who ? m : 3.4e38f;
}

// query_term for one query by a whole warp (used for the few queries with the
// largest bounds, which are far from the other surface and walk many rings):
// the lanes split each ring's cells and each keeps its kKnnF smallest FP32
// distances, so the warp's kKnnF smallest are exact (a candidate a lane drops
// has kKnnF smaller ones in that lane alone); a warp tournament takes them in
// order. Same stop rule, same FP32-to-FP64 selection proof and the same term
// as query_term; returns false (on all lanes) when the proof fails, and the
// caller then uses query_term. Returns kTermSkipped (on all lanes) as soon as
// the nearest sample found bounds the term at or below *out_max, or strictly
// below `floor`: such a term cannot change the result.
constexpr int kTermOk = 0, kTermUnproven = 1, kTermSkipped = 2;
__device__ int query_term_warp(const HSide& S, int qi, double floor, const unsigned long long* out_max,
                               double& term) {
  const int lane = threadIdx.x & 31;
  const HGrid& G = S.G;
  const double q[3] = {S.Q[3 * (int64_t)qi], S.Q[3 * (int64_t)qi + 1], S.Q[3 * (int64_t)qi + 2]};
  const int cx = cell_coord(q[0], G.lo[0], G.h, G.dim[0]);
  const int cy = cell_coord(q[1], G.lo[1], G.h, G.dim[1]);
  const int cz = cell_coord(q[2], G.lo[2], G.h, G.dim[2]);
  const int rmax = max(G.dim[0], max(G.dim[1], G.dim[2]));
  const float qf[3] = {(float)q[0], (float)q[1], (float)q[2]};
  const float hf = (float)G.h;
  float fd[kKnnF];
  int fi[kKnnF];
  int nf = 0;
  int total = 0;  // candidates seen by the warp
  float g10 = 3.4e38f;
  for (int r = 0; r <= rmax; ++r) {
    const int side = 2 * r + 1;
    const int cube = side * side * side;
    int seen = 0;
    for (int t = lane; t < cube; t += 32) {
      const int dx = t % side - r, dy = (t / side) % side - r, dz = t / (side * side) - r;
      if (max(abs(dx), max(abs(dy), abs(dz))) != r) continue;
      const int x = cx + dx, y = cy + dy, z = cz + dz;
      if (x < 0 || x >= G.dim[0] || y < 0 || y >= G.dim[1] || z < 0 || z >= G.dim[2]) continue;
      const int c = (z * G.dim[1] + y) * G.dim[0] + x;
      for (int k = G.start[c]; k < G.start[c + 1]; ++k) {
        const float4 sp = G.spts[k];
        const float ex = sp.x - qf[0], ey = sp.y - qf[1], ez = sp.z - qf[2];
        const float d2 = ex * ex + ey * ey + ez * ez;
        ++seen;
        if (nf < kKnnF || d2 < fd[nf - 1]) {
          int j = nf < kKnnF ? nf++ : kKnnF - 1;
          while (j > 0 && fd[j - 1] > d2) {
            fd[j] = fd[j - 1];
            fi[j] = fi[j - 1];
            --j;
          }
          fd[j] = d2;
          fi[j] = __float_as_int(sp.w);
        }
      }
    }
    for (int o = 16; o; o >>= 1) seen += __shfl_xor_sync(0xffffffffu, seen, o);
    total += seen;
    if (seen > 0) {
      // The term is at most the nearest sample's distance, itself at most the
      // warp's smallest FP32 distance so far rounded upwards plus the bound.
      float m = nf > 0 ? fd[0] : 3.4e38f;
      for (int o = 16; o; o >>= 1) m = fminf(m, __shfl_xor_sync(0xffffffffu, m, o));
      const double ub = (double)__fadd_ru(__fmul_ru(__fsqrt_ru(m), 1.0f + 1.0f / 1048576.0f), G.eabs);
      const double cur = __longlong_as_double((long long)*(const volatile unsigned long long*)out_max);
      if (__shfl_sync(0xffffffffu, (ub <= cur || ub < floor) ? 1 : 0, 0)) return kTermSkipped;
    }
    if (total >= kKnn) {
      int ptr = 0, id;
      float v = 3.4e38f;
      for (int m = 0; m < kKnn; ++m) v = warp_take_min(fd, fi, nf, ptr, id);
      g10 = v;
      if (__fadd_ru(__fmul_ru(__fsqrt_ru(g10), 1.0f + 1.0f / 1048576.0f), G.eabs) <=
          __fmul_rd((float)r, hf) * (1.0f - 1e-6f))
        break;
    }
  }
  // The warp's kKnnF smallest (value, id) in order: lane m holds the m-th.
  float myv = 3.4e38f;
  int myid = -1;
  {
    int ptr = 0;
    for (int m = 0; m < kKnnF; ++m) {
      int id;
      const float v = warp_take_min(fd, fi, nf, ptr, id);
      if (lane == m) {
        myv = v;
        myid = id;
      }
    }
  }
  // The exact 10 nearest are among these when the kKnnF-th FP32 distance
  // exceeds the 10th by more than twice the bound (or all were kept).
  if (total > kKnnF) {
    const float v16 = __shfl_sync(0xffffffffu, myv, kKnnF - 1);
    const bool ok = __fsqrt_rd(v16) * (1.0f - 1.0f / 1048576.0f) >
                    __fadd_ru(__fadd_ru(__fmul_ru(__fsqrt_ru(g10), 1.0f + 1.0f / 1048576.0f), G.eabs), G.eabs);
    if (!ok) return kTermUnproven;
  }
  // Exact FP64 distances of the (up to) kKnnF candidates, the 10 nearest kept
  // in order (insertion in candidate order, as query_term).
  double d2 = DBL_MAX;
  if (myid >= 0) {
    const double* pp = G.pts + 3 * (int64_t)myid;
    const double ex = ds(pp[0], q[0]), ey = ds(pp[1], q[1]), ez = ds(pp[2], q[2]);
    d2 = da(da(dm(ex, ex), dm(ey, ey)), dm(ez, ez));
  }
  double bd[kKnn];
  int bi[kKnn];
  int cnt = 0;
  for (int m = 0; m < kKnnF; ++m) {
    const double v = __shfl_sync(0xffffffffu, d2, m);
    const int id = __shfl_sync(0xffffffffu, myid, m);
    if (id < 0) continue;
    if (cnt < kKnn || v < bd[cnt - 1]) {
      int j = cnt < kKnn ? cnt++ : kKnn - 1;
      while (j > 0 && bd[j - 1] > v) {
        bd[j] = bd[j - 1];
        bi[j] = bi[j - 1];
        --j;
      }
      bd[j] = v;
      bi[j] = id;
    }
  }
  // Point-triangle distances of the k nearest in parallel (lane j), then the
  // sequential minimum with the early stop below 1e-14, in order.
  double dj = DBL_MAX;
  int which = -1;
#pragma unroll
  for (int j = 0; j < kKnn; ++j)
    if (j == lane && j < cnt) which = bi[j];
  if (which >= 0) {
    const int tj = S.ids[which];
    const int* t = S.mt + 3 * (int64_t)tj;
    dj = point_tri_dist(q, S.mv + 3 * (int64_t)t[0], S.mv + 3 * (int64_t)t[1], S.mv + 3 * (int64_t)t[2]);
  }
  double cmin = DBL_MAX;
  for (int j = 0; j < cnt; ++j) {
    const double d = __shfl_sync(0xffffffffu, dj, j);
    if (d < cmin) {
      cmin = d;
      if (cmin < 1e-14) break;
    }
  }
  if (cmin > 10 && cnt > 0) cmin = __dsqrt_rn(bd[0]);
  term = cmin;
  return kTermOk;
}

// Upper bound of every query's term, one thread per query in its own grid's
// cell order: the distance to the nearest sample within two rings of cells
// around the query, in FP32 rounded upwards plus the coordinate rounding
// bound (the term is at most the distance to the nearest sample, itself at
// most this). A query with no sample that close gets no bound (+inf) and is
// appended to farlist (*far entries): those are evaluated one warp each.
// Entry e = base + position holds the bound and the query's id (bit 31:
// direction).
constexpr int kBoundRings = 2;
__global__ void __launch_bounds__(128) hbound_kernel(HSide S0, const int* __restrict__ qorder0, HSide S1,
                                                     const int* __restrict__ qorder1, float* __restrict__ ubs,
                                                     uint32_t* __restrict__ vals, unsigned* __restrict__ far,
                                                     int* __restrict__ farlist) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < S0.nq + S1.nq; e += gridDim.x * blockDim.x) {
    const int dir = e < S0.nq ? 0 : 1;
    const HSide& S = dir ? S1 : S0;
    const int qk = dir ? e - S0.nq : e;
    const int base = dir ? S0.nq : 0;
    const HGrid& G = S.G;
    const int qi = (dir ? qorder1 : qorder0)[qk];
    const double* qq = S.Q + 3 * (int64_t)qi;
    const double q[3] = {qq[0], qq[1], qq[2]};
    const int cx = cell_coord(q[0], G.lo[0], G.h, G.dim[0]);
    const int cy = cell_coord(q[1], G.lo[1], G.h, G.dim[1]);
    const int cz = cell_coord(q[2], G.lo[2], G.h, G.dim[2]);
    const float qf[3] = {(float)q[0], (float)q[1], (float)q[2]};
    float best = 3.4e38f;
    for (int r = 0; r <= kBoundRings; ++r) {
      for (int dz = -r; dz <= r; ++dz) {
        const int z = cz + dz;
        if (z < 0 || z >= G.dim[2]) continue;
        for (int dy = -r; dy <= r; ++dy) {
          const int y = cy + dy;
          if (y < 0 || y >= G.dim[1]) continue;
          const bool face = abs(dz) == r || abs(dy) == r;
          for (int dx = -r; dx <= r; dx += (face ? 1 : 2 * r > 0 ? 2 * r : 1)) {
            const int x = cx + dx;
            if (x >= 0 && x < G.dim[0]) {
              const int c = (z * G.dim[1] + y) * G.dim[0] + x;
              for (int k = G.start[c]; k < G.start[c + 1]; ++k) {
                const float4 sp = G.spts[k];
                const float ex = sp.x - qf[0], ey = sp.y - qf[1], ez = sp.z - qf[2];
                best = fminf(best, ex * ex + ey * ey + ez * ez);
              }
            }
            if (dx == r) break;
          }
        }
      }
      if (r >= 1 && best < 3.4e38f) break;
    }
    float ub = __int_as_float(0x7f800000);  // +inf: no bound
    if (best < 3.4e38f)
      ub = __fadd_ru(__fmul_ru(__fsqrt_ru(best), 1.0f + 1.0f / 1048576.0f), G.eabs);
    else
      farlist[atomicAdd(far, 1u)] = base + qk;
    ubs[base + qk] = ub;
    vals[base + qk] = (uint32_t)qi | ((uint32_t)dir << 31);
  }
}

// Terms of the queries without a bound (the farlist), one warp each: they are
// far from the other surface, walk many rings, and their exact terms start
// the running maximum that prunes the rest.
__global__ void __launch_bounds__(128) hhead_kernel(HSide A, HSide B, const uint32_t* __restrict__ vals,
                                                    const int* __restrict__ farlist,
                                                    const unsigned* __restrict__ far, float tmargin, double floor,
                                                    unsigned long long* __restrict__ out_max) {
  const int head = (int)*far;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < head; w += warps) {
    const uint32_t v = vals[farlist[w]];
    const int qi = (int)(v & 0x7FFFFFFFu);
    const HSide& S = (v >> 31) ? B : A;
    double term;
    const int status = query_term_warp(S, qi, floor, out_max, term);
    if (status == kTermSkipped) continue;
    if (status == kTermUnproven) term = query_term(S, qi, tmargin);
    if ((threadIdx.x & 31) == 0 && term < DBL_MAX)
      atomicMax(out_max, (unsigned long long)__double_as_longlong(term));
  }
}

// Terms of the queries with a bound (both directions, each in its own grid's
// cell order), maximum into out_max. A query whose bound does not exceed the
// maximum found so far cannot raise it and is skipped: the result is the same
// maximum. So is a query whose bound lies strictly below `floor`.
__global__ void __launch_bounds__(128) hquery_kernel(HSide A, HSide B, const float* __restrict__ ubs,
                                                     const uint32_t* __restrict__ vals, int end, float tmargin,
                                                     double floor, unsigned long long* __restrict__ out_max) {
  double local = 0.0;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < end; e += gridDim.x * blockDim.x) {
    const float ub = ubs[e];
    if (!(ub < __int_as_float(0x7f800000))) continue;  // no bound: evaluated by hhead_kernel
    const double cur = __longlong_as_double((long long)*(volatile unsigned long long*)out_max);
    if ((double)ub <= fmax(cur, local) || (double)ub < floor) continue;
    const uint32_t v = vals[e];
    const int qi = (int)(v & 0x7FFFFFFFu);
    const double cmin = (v >> 31) ? query_term(B, qi, tmargin) : query_term(A, qi, tmargin);
    if (cmin > local && DBL_MAX > cmin) local = cmin;
  }
  for (int o = 16; o; o >>= 1) local = fmax(local, __shfl_xor_sync(0xffffffffu, local, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out_max, (unsigned long long)__double_as_longlong(local));
}

}  // namespace vgpu

using namespace vgpu;

// Fused set-up of both sample sets and both meshes (one launch): the cell of
// every sample with per-cell counts (set B's cells follow set A's in one count
// array), and the FP32 triangle bounds of both meshes.
__global__ void hprep_kernel(HGrid ga, HGrid gb, int cells_a, int* __restrict__ cnt, int* __restrict__ cell_a,
                             int* __restrict__ cell_b, const double* __restrict__ mva, const int* __restrict__ mta,
                             int nta, float4* __restrict__ tba, const double* __restrict__ mvb,
                             const int* __restrict__ mtb, int ntb, float4* __restrict__ tbb) {
  const int64_t total = (int64_t)ga.n + gb.n + nta + ntb;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    if (i < ga.n || i < (int64_t)ga.n + gb.n) {
      const bool isa = i < ga.n;
      const HGrid& g = isa ? ga : gb;
      const int k = isa ? (int)i : (int)(i - ga.n);
      const double* p = g.pts + 3 * (int64_t)k;
      const int cx = cell_coord(p[0], g.lo[0], g.h, g.dim[0]);
      const int cy = cell_coord(p[1], g.lo[1], g.h, g.dim[1]);
      const int cz = cell_coord(p[2], g.lo[2], g.h, g.dim[2]);
      const int c = (cz * g.dim[1] + cy) * g.dim[0] + cx;
      (isa ? cell_a : cell_b)[k] = c;
      atomicAdd(&cnt[(isa ? 0 : cells_a) + c], 1);
    } else {
      const int64_t j = i - ga.n - gb.n;
      const bool isa = j < nta;
      const int t = isa ? (int)j : (int)(j - nta);
      const double* mv = isa ? mva : mvb;
      const int* mt = isa ? mta : mtb;
      float4* out = isa ? tba : tbb;
      const double* a = mv + 3 * (int64_t)mt[3 * (int64_t)t];
      const double* b = mv + 3 * (int64_t)mt[3 * (int64_t)t + 1];
      const double* c = mv + 3 * (int64_t)mt[3 * (int64_t)t + 2];
      float lo[3], hi[3];
      for (int q = 0; q < 3; ++q) {
        lo[q] = __double2float_rd(fmin(fmin(a[q], b[q]), c[q]));
        hi[q] = __double2float_ru(fmax(fmax(a[q], b[q]), c[q]));
      }
      const double ux = b[0] - a[0], uy = b[1] - a[1], uz = b[2] - a[2];
      const double vx = c[0] - a[0], vy = c[1] - a[1], vz = c[2] - a[2];
      double nx = uy * vz - uz * vy, ny = uz * vx - ux * vz, nz = ux * vy - uy * vx;
      const double nl = sqrt(nx * nx + ny * ny + nz * nz);
      float4 pl = make_float4(0.f, 0.f, 0.f, 0.f);
      if (nl > 1e-30) {
        nx /= nl;
        ny /= nl;
        nz /= nl;
        pl = make_float4((float)nx, (float)ny, (float)nz, (float)-(nx * a[0] + ny * a[1] + nz * a[2]));
      }
      out[3 * (int64_t)t] = make_float4(lo[0], lo[1], lo[2], 0.f);
      out[3 * (int64_t)t + 1] = make_float4(hi[0], hi[1], hi[2], 0.f);
      out[3 * (int64_t)t + 2] = pl;
    }
  }
}

// Counting-sort scatter of both sets (one launch) from the scanned counts.
__global__ void hscatter2_kernel(int na, int nb, int cells_a, const int* __restrict__ cell_a,
                                 const int* __restrict__ cell_b, const unsigned long long* __restrict__ off,
                                 int* __restrict__ fill, int* __restrict__ order_a, int* __restrict__ order_b) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < na + nb; i += gridDim.x * blockDim.x) {
    if (i < na) {
      const int c = cell_a[i];
      order_a[off[c] + atomicAdd(&fill[c], 1)] = i;
    } else {
      const int j = i - na, c = cells_a + cell_b[j];
      order_b[off[c] - off[cells_a] + atomicAdd(&fill[c], 1)] = j;
    }
  }
}

// Cell starts of both grids and the float copies of both sets in cell order.
__global__ void hfinish_kernel(int cells_a, int cells_b, const unsigned long long* __restrict__ off,
                               int* __restrict__ start_a, int* __restrict__ start_b, const double* __restrict__ pa,
                               const int* __restrict__ order_a, int na, float4* __restrict__ spa,
                               const double* __restrict__ pb, const int* __restrict__ order_b, int nb,
                               float4* __restrict__ spb) {
  const int64_t total = (int64_t)cells_a + 1 + cells_b + 1 + na + nb;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    if (i <= cells_a) {
      start_a[i] = (int)off[i];
    } else if (i <= (int64_t)cells_a + 1 + cells_b) {
      const int c = (int)(i - cells_a - 1);
      start_b[c] = (int)(off[cells_a + c] - off[cells_a]);
    } else {
      const int64_t k0 = i - cells_a - cells_b - 2;
      const bool isa = k0 < na;
      const int k = isa ? (int)k0 : (int)(k0 - na);
      const double* pts = isa ? pa : pb;
      const int q = (isa ? order_a : order_b)[k];
      (isa ? spa : spb)[k] = make_float4((float)pts[3 * (int64_t)q], (float)pts[3 * (int64_t)q + 1],
                                         (float)pts[3 * (int64_t)q + 2], __int_as_float(q));
    }
  }
}

namespace {
size_t al(size_t x) { return (x + 255) & ~size_t(255); }
}

extern "C" int visacd_face_hausdorff_floor(visacd_ctx* ctx, const double* va, int32_t nva, const int32_t* ta,
                                           int32_t nta, const double* xa, const int32_t* ida, int32_t na,
                                           const double* vb, int32_t nvb, const int32_t* tb, int32_t ntb,
                                           const double* xb, const int32_t* idb, int32_t nb, double floor,
                                           double* out) {
  VCHECK(ctx && out, VISACD_ERR_INVALID_ARG, "face_hausdorff: null argument");
  VCHECK(floor == floor, VISACD_ERR_INVALID_ARG, "face_hausdorff: floor is NaN");
  VCHECK(na > 0 && nb > 0 && nva > 0 && nvb > 0 && nta > 0 && ntb > 0, VISACD_ERR_INVALID_ARG,
         "face_hausdorff: empty input");
  VCUDA(cudaSetDevice(ctx->device));
  // Grid shape from the sample counts: about 2 samples per occupied cell on a
  // surface; at most 160 cells per axis.
  auto grid_for_points = [](const double* x, int n, HGrid& g) {
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int i = 0; i < n; ++i)
      for (int a = 0; a < 3; ++a) {
        lo[a] = std::min(lo[a], x[3 * (int64_t)i + a]);
        hi[a] = std::max(hi[a], x[3 * (int64_t)i + a]);
      }
    double ext = std::max(hi[0] - lo[0], std::max(hi[1] - lo[1], hi[2] - lo[2]));
    double area_like = 0;
    for (int a = 0; a < 3; ++a) area_like += (hi[a] - lo[a]) * (hi[(a + 1) % 3] - lo[(a + 1) % 3]);
    double h = std::sqrt(std::max(area_like, 1e-30) * 2.0 / std::max(n, 1));
    h = std::max(h, ext / 160.0);
    if (!(h > 0)) h = 1.0;
    for (int a = 0; a < 3; ++a) {
      g.lo[a] = lo[a];
      g.dim[a] = std::max(1, (int)std::ceil((hi[a] - lo[a]) / h) + 1);
    }
    g.h = h;
    g.n = n;
  };
  // One grid over each sample set (g[0] over A, g[1] over B).
  HGrid g[2];
  grid_for_points(xa, na, g[0]);
  grid_for_points(xb, nb, g[1]);
  // FP32 pre-filter bound: coordinates rounded to float differ by at most
  // 2^-24 |x| each, the difference and the squared sum add a few ulps; with
  // M the largest |coordinate| of both sets, |d_f32 - d| <= 8 M 2^-24.
  double M = 0;
  for (int k = 0; k < 2; ++k)
    for (int a = 0; a < 3; ++a)
      M = std::max(M, std::max(std::fabs(g[k].lo[a]), std::fabs(g[k].lo[a] + g[k].h * g[k].dim[a])));
  for (int k = 0; k < 2; ++k) g[k].eabs = (float)(M * std::ldexp(1.0, -21) + 1e-30);
  int cells[2];
  for (int k = 0; k < 2; ++k) cells[k] = g[k].dim[0] * g[k].dim[1] * g[k].dim[2];
  const int ncell = cells[0] + cells[1];
  size_t off = 0;
  auto carve = [&](size_t b) { size_t o = off; off += al(b); return o; };
  const size_t o_va = carve((size_t)nva * 24), o_ta = carve((size_t)nta * 12), o_xa = carve((size_t)na * 24),
               o_ia = carve((size_t)na * 4), o_vb = carve((size_t)nvb * 24), o_tb = carve((size_t)ntb * 12),
               o_xb = carve((size_t)nb * 24), o_ib = carve((size_t)nb * 4), o_tba = carve((size_t)nta * 48),
               o_tbb = carve((size_t)ntb * 48), o_ub = carve((size_t)(na + nb) * 4),
               o_vals = carve((size_t)(na + nb) * 4), o_far = carve((size_t)(na + nb) * 4);
  // Zeroed together: maximum + far count, per-cell counts and fills of both grids.
  const size_t zero_begin = off;
  const size_t o_mx = carve(64), o_cnt = carve((size_t)(ncell + 1) * 4), o_fill = carve((size_t)ncell * 4);
  const size_t zero_end = off;
  const size_t o_off = carve((size_t)(ncell + 1) * 8), o_sa = carve((size_t)(cells[0] + 1) * 4),
               o_sb = carve((size_t)(cells[1] + 1) * 4), o_oa = carve((size_t)na * 4), o_ob = carve((size_t)nb * 4),
               o_ca = carve((size_t)na * 4), o_cb = carve((size_t)nb * 4), o_pa = carve((size_t)na * 16),
               o_pb = carve((size_t)nb * 16);
  VTRY(ensure_slot(ctx, kSlotHausdorff, off));
  char* B = slot<char>(ctx, kSlotHausdorff);
  cudaStream_t st = ctx->stream;
  Stager up(ctx);
  VTRY(up.reserve((size_t)nva * 24 + (size_t)nta * 12 + (size_t)na * 28 + (size_t)nvb * 24 + (size_t)ntb * 12 +
                      (size_t)nb * 28,
                  8));
  VTRY(up.put(B + o_va, va, (size_t)nva * 24));
  VTRY(up.put(B + o_ta, ta, (size_t)nta * 12));
  VTRY(up.put(B + o_xa, xa, (size_t)na * 24));
  VTRY(up.put(B + o_ia, ida, (size_t)na * 4));
  VTRY(up.put(B + o_vb, vb, (size_t)nvb * 24));
  VTRY(up.put(B + o_tb, tb, (size_t)ntb * 12));
  VTRY(up.put(B + o_xb, xb, (size_t)nb * 24));
  VTRY(up.put(B + o_ib, idb, (size_t)nb * 4));
  VCUDA(cudaMemsetAsync(B + zero_begin, 0, zero_end - zero_begin, st));
  g[0].pts = (const double*)(B + o_xa);
  g[1].pts = (const double*)(B + o_xb);
  g[0].n = na;
  g[1].n = nb;
  const unsigned long long* offs = (const unsigned long long*)(B + o_off);
  // Both sets bucketed by counting sort (counts, one scan, scatter, starts)
  // and both meshes' triangle bounds: four launches plus the scan.
  VLAUNCH(ctx, kKHausdorff, grid_for((int64_t)na + nb + nta + ntb, 256, 8LL * ctx->sm_count), 256, 0, hprep_kernel,
          g[0], g[1], cells[0], (int*)(B + o_cnt), (int*)(B + o_ca), (int*)(B + o_cb), (const double*)(B + o_va),
          (const int*)(B + o_ta), nta, (float4*)(B + o_tba), (const double*)(B + o_vb), (const int*)(B + o_tb), ntb,
          (float4*)(B + o_tbb));
  VTRY(exclusive_scan_u32_to_u64(ctx, (const uint32_t*)(B + o_cnt), (uint64_t*)(B + o_off), ncell));
  VLAUNCH(ctx, kKHausdorff, grid_for((int64_t)na + nb, 256, 8LL * ctx->sm_count), 256, 0, hscatter2_kernel, na, nb,
          cells[0], (const int*)(B + o_ca), (const int*)(B + o_cb), offs, (int*)(B + o_fill), (int*)(B + o_oa),
          (int*)(B + o_ob));
  VLAUNCH(ctx, kKHausdorff, grid_for((int64_t)ncell + 2 + na + nb, 256, 8LL * ctx->sm_count), 256, 0,
          hfinish_kernel, cells[0], cells[1], offs, (int*)(B + o_sa), (int*)(B + o_sb), (const double*)(B + o_xa),
          (const int*)(B + o_oa), na, (float4*)(B + o_pa), (const double*)(B + o_xb), (const int*)(B + o_ob), nb,
          (float4*)(B + o_pb));
  g[0].start = (const int*)(B + o_sa);
  g[1].start = (const int*)(B + o_sb);
  g[0].order = (const int*)(B + o_oa);
  g[1].order = (const int*)(B + o_ob);
  g[0].spts = (const float4*)(B + o_pa);
  g[1].spts = (const float4*)(B + o_pb);
  unsigned long long* mx = (unsigned long long*)(B + o_mx);
  // Margin of the FP32 lower bounds: the plane evaluation's rounding (normal
  // and offset rounded to float, a few ulps of the largest coordinate), with
  // room to spare; the box gap is conservative by construction.
  const float tmargin = (float)(1e-9 + 256.0 * std::ldexp(1.0, -24) * (M + 4.0));
  // Direction 0: queries of B against A's samples / triangles; direction 1:
  // queries of A against B.
  HSide sd0{(const double*)(B + o_xb), nb, g[0], (const int*)(B + o_ia), (const double*)(B + o_va),
            (const int*)(B + o_ta), (const float4*)(B + o_tba)};
  HSide sd1{(const double*)(B + o_xa), na, g[1], (const int*)(B + o_ib), (const double*)(B + o_vb),
            (const int*)(B + o_tb), (const float4*)(B + o_tbb)};
  const int ntot = na + nb;
  uint32_t* vals = (uint32_t*)(B + o_vals);
  unsigned* far = (unsigned*)(B + o_mx + 8);  // zeroed with the maximum
  float* ubs = (float*)(B + o_ub);
  int* farlist = (int*)(B + o_far);
  VLAUNCH(ctx, kKHausdorffBound, grid_for(ntot, 128, 8LL * ctx->sm_count), 128, 0, hbound_kernel, sd0, g[1].order,
          sd1, g[0].order, ubs, vals, far, farlist);
  // The queries without a bound one warp each, then the rest with pruning.
  VLAUNCH(ctx, kKHausdorffHead, grid_for(32LL * ntot, 128, 8LL * ctx->sm_count), 128, 0, hhead_kernel, sd0, sd1,
          (const uint32_t*)vals, (const int*)farlist, (const unsigned*)far, tmargin, floor, mx);
  VLAUNCH(ctx, kKHausdorffQuery, grid_for(ntot, 128, 8LL * ctx->sm_count), 128, 0, hquery_kernel, sd0, sd1,
          (const float*)ubs, (const uint32_t*)vals, ntot, tmargin, floor, mx);
  unsigned long long* h = nullptr;
  VTRY(pinned(ctx, 8, (void**)&h));
  VCUDA(cudaMemcpyAsync(h, mx, 8, cudaMemcpyDeviceToHost, st));
  VCUDA(cudaStreamSynchronize(st));
  double r;
  memcpy(&r, h, 8);
  *out = r;
  return VISACD_OK;
}

extern "C" int visacd_face_hausdorff(visacd_ctx* ctx, const double* va, int32_t nva, const int32_t* ta,
                                     int32_t nta, const double* xa, const int32_t* ida, int32_t na,
                                     const double* vb, int32_t nvb, const int32_t* tb, int32_t ntb,
                                     const double* xb, const int32_t* idb, int32_t nb, double* out) {
  return visacd_face_hausdorff_floor(ctx, va, nva, ta, nta, xa, ida, na, vb, nvb, tb, ntb, xb, idb, nb, 0.0, out);
}

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
//  * Point-triangle distance: the reference's own formula (projection onto the
//    triangle's plane, barycentric test, else Pythagorean edge and vertex
//    distances; ref_point_tri_dist) in FP64 with explicit round-to-nearest
//    intrinsics in its operation order, so values equal the host's and the
//    reference's. On a degenerate triangle that formula can give NaN (the
//    triangle then never lowers a minimum) or a value below the true distance,
//    so every shortcut that relies on the true distance is applied only where
//    it holds for the formula:
//      - the FP32 lower-bound skip of a triangle only for regular triangles
//        (|cross product| >= 1e-6 of the longest edge squared, where the
//        formula is the true distance up to rounding far inside the margin);
//      - a query's upper bound is the formula's own value for the triangle of
//        a sample proven to be among its 10 nearest (the term is at most that,
//        or the nearest-sample distance when the rule for minima above 10
//        applies); queries without such a bound are evaluated in full.
#include <float.h>

#include "common.cuh"
#include "geom64.cuh"

namespace vgpu {

constexpr int kKnn = 10;
constexpr int kBoundRings = 2;  // rings of cells searched for each query's upper bound

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
    const float4 lo = S.tb[3 * (int64_t)tri];
    // Irregular triangles (lo.w == 0) are always evaluated: the bound holds
    // for the true distance, not for the formula there.
    if (cmin < DBL_MAX && lo.w != 0.f) {
      const float4 hi = S.tb[3 * (int64_t)tri + 1], pl = S.tb[3 * (int64_t)tri + 2];
      const float gx = fmaxf(fmaxf(lo.x - qfx, qfx - hi.x), 0.f);
      const float gy = fmaxf(fmaxf(lo.y - qfy, qfy - hi.y), 0.f);
      const float gz = fmaxf(fmaxf(lo.z - qfz, qfz - hi.z), 0.f);
      const float lb = fmaxf(sqrtf(gx * gx + gy * gy + gz * gz), fabsf(pl.x * qfx + pl.y * qfy + pl.z * qfz + pl.w));
      if ((double)(lb - tmargin) >= cmin) continue;
    }
    const int* t = S.mt + 3 * (int64_t)tri;
    const double d = ref_point_tri_dist(q, S.mv + 3 * (int64_t)t[0], S.mv + 3 * (int64_t)t[1], S.mv + 3 * (int64_t)t[2]);
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
// caller then uses query_term. (These queries are evaluated in full: the
// nearest sample's distance does not bound the reference formula's minimum
// when its triangle is degenerate, so it is not used to skip them.)
constexpr int kTermOk = 0, kTermUnproven = 1, kTermSkipped = 2;
// r0: the first ring to walk (0: every ring; the rings inside r0 must hold no
// sample of G).

template <class Prune>
__device__ int query_term_warp(const HSide& S, int qi, int r0, const Prune& prune, double& term) {
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
  for (int r = r0; r <= rmax; ++r) {
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
    dj = ref_point_tri_dist(q, S.mv + 3 * (int64_t)t[0], S.mv + 3 * (int64_t)t[1], S.mv + 3 * (int64_t)t[2]);
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

// ---- batched evaluation ----------------------------------------------------
// A batch holds J jobs; job j compares surface A_j (mesh 2j, sample set 2j)
// with surface B_j (mesh 2j + 1, sample set 2j + 1). Queries of set s are
// evaluated against the grid, samples and mesh of set s ^ 1 (sides[s]). All
// sets, meshes and grids are concatenated; a sample or a triangle finds its
// set / mesh by binary search in the offset tables.
struct HBatch {
  int nsets;                          // 2 J
  const long long* sample_off;        // nsets + 1
  const long long* tri_off;           // nsets + 1
  const long long* vert_off;          // nsets + 1
  const int* cell0;                   // nsets + 1: first cell of each set's grid
  const HGrid* grids;                 // nsets (start / order / spts filled in)
  const HSide* sides;                 // nsets
  const double* pts;                  // all samples
  const double* mv;                   // all vertices
  const int* mt;                      // all triangles (vertex indices local to their mesh)
  float4* tb;                         // FP32 bounds of all triangles (3 per triangle)
  const double* lower;                // per job: a known lower bound of the job's concavity (volume term)
  unsigned long long* job_max;        // per job: largest term found (double bits)
  unsigned long long* gmax;           // largest of the floor, the lower bounds and every term found
  const float* tmargin;               // per job
  int independent;                    // 1: no pruning across jobs
};

__device__ __forceinline__ int find_seg(const long long* __restrict__ off, int n, long long i) {
  int lo = 0, hi = n;  // off[lo] <= i < off[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (off[mid] <= i) lo = mid;
    else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ double load_max(const unsigned long long* p) {
  return __longlong_as_double((long long)*(const volatile unsigned long long*)p);
}

// Raise the job's maximum and the batch maximum with an exact term.
__device__ __forceinline__ void publish(const HBatch& H, int job, double term) {
  atomicMax(H.job_max + job, (unsigned long long)__double_as_longlong(term));
  if (!H.independent)
    atomicMax(H.gmax, (unsigned long long)__double_as_longlong(fmax(term, H.lower[job])));
}

// A term bounded by ub cannot change a result the caller uses when ub is at
// most the job's own maximum so far, or (pruning across jobs) strictly below
// the batch maximum: the jobs that attain the batch's largest concavity keep
// their exact values.
__device__ __forceinline__ bool prunable(const HBatch& H, int job, double ub) {
  if (ub <= load_max(H.job_max + job)) return true;
  return !H.independent && ub < load_max(H.gmax);
}

// Set-up (one launch): each sample's cell with per-cell counts, and the FP32
// bounds (box, plane) of every triangle.
__global__ void hprep_kernel(HBatch H, long long nsamp, long long ntri, int* __restrict__ cnt,
                             int* __restrict__ cell_of) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nsamp + ntri;
       i += (long long)gridDim.x * blockDim.x) {
    if (i < nsamp) {
      const int s = find_seg(H.sample_off, H.nsets, i);
      const HGrid& g = H.grids[s];
      const double* p = H.pts + 3 * i;
      const int cx = cell_coord(p[0], g.lo[0], g.h, g.dim[0]);
      const int cy = cell_coord(p[1], g.lo[1], g.h, g.dim[1]);
      const int cz = cell_coord(p[2], g.lo[2], g.h, g.dim[2]);
      const int c = (cz * g.dim[1] + cy) * g.dim[0] + cx;
      cell_of[i] = c;
      atomicAdd(&cnt[H.cell0[s] + c], 1);
    } else {
      const long long j = i - nsamp;
      const int m = find_seg(H.tri_off, H.nsets, j);
      const double* mv = H.mv + 3 * H.vert_off[m];
      const int* t = H.mt + 3 * j;
      const double* a = mv + 3 * (int64_t)t[0];
      const double* b = mv + 3 * (int64_t)t[1];
      const double* c = mv + 3 * (int64_t)t[2];
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
      // Regular: cross product at least 1e-6 of the longest edge squared.
      const double wx = c[0] - b[0], wy = c[1] - b[1], wz = c[2] - b[2];
      const double l2 = fmax(fmax(ux * ux + uy * uy + uz * uz, vx * vx + vy * vy + vz * vz),
                             wx * wx + wy * wy + wz * wz);
      const float regular = (nl >= 1e-6 * l2 && l2 > 0.0) ? 1.f : 0.f;
      if (nl > 1e-30) {
        nx /= nl;
        ny /= nl;
        nz /= nl;
        pl = make_float4((float)nx, (float)ny, (float)nz, (float)-(nx * a[0] + ny * a[1] + nz * a[2]));
      }
      H.tb[3 * j] = make_float4(lo[0], lo[1], lo[2], regular);
      H.tb[3 * j + 1] = make_float4(hi[0], hi[1], hi[2], 0.f);
      H.tb[3 * j + 2] = pl;
    }
  }
}

// Counting-sort scatter of every set from the scanned counts: order holds,
// per set, its local sample indices in cell order.
__global__ void hscatter_kernel(HBatch H, long long nsamp, const int* __restrict__ cell_of,
                                const unsigned long long* __restrict__ off, int* __restrict__ fill,
                                int* __restrict__ order) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nsamp;
       i += (long long)gridDim.x * blockDim.x) {
    const int s = find_seg(H.sample_off, H.nsets, i);
    const int c = H.cell0[s] + cell_of[i];
    const long long s0 = H.sample_off[s];
    order[s0 + (long long)(off[c] - off[H.cell0[s]]) + atomicAdd(&fill[c], 1)] = (int)(i - s0);
  }
}

// Cell starts of every grid (set s's at start[cell0[s] + s ...], cells + 1
// entries) and the float copies of every set in cell order (w = local index).
__global__ void hfinish_kernel(HBatch H, long long nsamp, int ncells, const unsigned long long* __restrict__ off,
                               const int* __restrict__ order, int* __restrict__ start, float4* __restrict__ spts) {
  const long long nstart = (long long)ncells + H.nsets;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nstart + nsamp;
       i += (long long)gridDim.x * blockDim.x) {
    if (i < nstart) {
      // entry i belongs to the set s with cell0[s] + s <= i < cell0[s + 1] + s + 1
      int lo = 0, hi = H.nsets;
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if ((long long)H.cell0[mid] + mid <= i) lo = mid;
        else hi = mid;
      }
      const int c = (int)(i - H.cell0[lo] - lo);
      start[i] = (int)(off[H.cell0[lo] + c] - off[H.cell0[lo]]);
    } else {
      const long long k = i - nstart;
      const int s = find_seg(H.sample_off, H.nsets, k);
      const long long s0 = H.sample_off[s];
      const int q = order[k];
      const double* p = H.pts + 3 * (s0 + q);
      spts[k] = make_float4((float)p[0], (float)p[1], (float)p[2], __int_as_float(q));
    }
  }
}

// Samples of G within ring r of cell (cx, cy, cz) whose FP32 squared distance
// to qf is at most lim: count and the smallest one (value, local id).
__device__ __forceinline__ void ring_scan(const HGrid& G, int cx, int cy, int cz, int r, const float (&qf)[3],
                                          float lim, float& best, int& best_id, int& count) {
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
            if (d2 < best) {
              best = d2;
              best_id = __float_as_int(sp.w);
            }
            count += d2 <= lim;
          }
        }
        if (dx == r) break;
      }
    }
  }
}

// Upper bound of every query's term, one thread per query (all sets, each in
// its own grid's cell order). The nearest sample s within up to
// kBoundRings + 1 rings (FP32) is proven to be among the exact 10 nearest
// when at most 10 samples lie within its distance plus twice the rounding
// bound and that distance lies inside the rings searched. The term is then at
// most the formula's distance r_s from the query to s's triangle (a minimum
// over the 10 nearest includes it, or an earlier evaluated value, or a
// skipped one provably not smaller) or, under the rule for minima above 10,
// the nearest-sample distance: the bound is the larger of the two, rounded
// upwards plus the coordinate rounding bound. Queries without a proof, or
// with r_s NaN or DBL_MAX (a degenerate triangle), get no bound (+inf) and
// are appended to farlist (*far entries): those are evaluated one warp each.
// qref[e] = (set, local query index).
__global__ void __launch_bounds__(128) hbound_kernel(HBatch H, long long nsamp, const int* __restrict__ order,
                                                     float* __restrict__ ubs, int2* __restrict__ qref,
                                                     unsigned* __restrict__ far, long long* __restrict__ farlist) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < nsamp;
       e += (long long)gridDim.x * blockDim.x) {
    const int s = find_seg(H.sample_off, H.nsets, e);
    const int qi = order[e];
    const HSide& S = H.sides[s];
    const HGrid& G = S.G;
    const double* qq = S.Q + 3 * (int64_t)qi;
    const double q[3] = {qq[0], qq[1], qq[2]};
    const int cx = cell_coord(q[0], G.lo[0], G.h, G.dim[0]);
    const int cy = cell_coord(q[1], G.lo[1], G.h, G.dim[1]);
    const int cz = cell_coord(q[2], G.lo[2], G.h, G.dim[2]);
    const float qf[3] = {(float)q[0], (float)q[1], (float)q[2]};
    const float hf = (float)G.h;
    float best = 3.4e38f;
    int best_id = -1, unused = 0;
    int r_end = -1;
    float dist_up = 0.f, reach = 0.f;
    for (int r = 0; r <= kBoundRings + 1; ++r) {
      ring_scan(G, cx, cy, cz, r, qf, -1.f, best, best_id, unused);
      r_end = r;
      if (best < 3.4e38f) {
        dist_up = __fmul_ru(__fsqrt_ru(best), 1.0f + 1.0f / 1048576.0f);
        reach = __fadd_ru(dist_up, __fmul_ru(2.0f, G.eabs));
        if (reach <= __fmul_rd((float)r, hf) * (1.0f - 1e-6f)) break;
      }
    }
    float ub = __int_as_float(0x7f800000);  // +inf: no bound
    bool proven = best < 3.4e38f && reach <= __fmul_rd((float)r_end, hf) * (1.0f - 1e-6f);
    if (proven) {
      // Samples whose exact distance can be at most s's: FP32 distance at
      // most reach (squared, rounded up).
      const float lim = __fmul_ru(__fmul_ru(reach, reach), 1.0f + 1.0f / 262144.0f);
      float b2 = 3.4e38f;
      int id2 = -1, count = 0;
      for (int r = 0; r <= r_end; ++r) ring_scan(G, cx, cy, cz, r, qf, lim, b2, id2, count);
      proven = count <= kKnn;
    }
    if (proven) {
      const int* t = S.mt + 3 * (int64_t)S.ids[best_id];
      const double rs =
          ref_point_tri_dist(q, S.mv + 3 * (int64_t)t[0], S.mv + 3 * (int64_t)t[1], S.mv + 3 * (int64_t)t[2]);
      if (rs < DBL_MAX) {
        const float rsf = __fadd_ru(__fmul_ru(__double2float_ru(rs), 1.0f + 1.0f / 1048576.0f), G.eabs);
        ub = fmaxf(__fadd_ru(dist_up, G.eabs), rsf);
      } else {
        proven = false;
      }
    }
    if (!proven) farlist[atomicAdd(far, 1u)] = e;
    ubs[e] = ub;
    qref[e] = make_int2(s, qi);
  }
}

// Terms of the queries without a bound (the farlist), one warp each: mostly
// queries far from the other surface, which walk many rings (and a few near a
// degenerate triangle); their exact terms raise the maxima that prune the rest.
__global__ void __launch_bounds__(128) hhead_kernel(HBatch H, const int2* __restrict__ qref,
                                                    const long long* __restrict__ farlist,
                                                    const unsigned* __restrict__ far) {
  const int head = (int)*far;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < head; w += warps) {
    const int2 r = qref[farlist[w]];
    const int job = r.x >> 1;
    const HSide& S = H.sides[r.x];
    double term;
    const int status =
        query_term_warp(S, r.y, 0, [&](double ub) { return prunable(H, job, ub); }, term);
    if (status == kTermSkipped) continue;
    if (status == kTermUnproven) term = query_term(S, r.y, H.tmargin[job]);
    if ((threadIdx.x & 31) == 0 && term < DBL_MAX) publish(H, job, term);
  }
}

// Terms of the queries with a bound; a query whose bound cannot change a used
// result (prunable) is skipped.
__global__ void __launch_bounds__(128) hquery_kernel(HBatch H, const float* __restrict__ ubs,
                                                     const int2* __restrict__ qref, long long nsamp) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < nsamp;
       e += (long long)gridDim.x * blockDim.x) {
    const float ub = ubs[e];
    if (!(ub < __int_as_float(0x7f800000))) continue;  // no bound: evaluated by hhead_kernel
    const int2 r = qref[e];
    const int job = r.x >> 1;
    if (prunable(H, job, (double)ub)) continue;
    const double cmin = query_term(H.sides[r.x], r.y, H.tmargin[job]);
    if (DBL_MAX > cmin) publish(H, job, cmin);
  }
}

}  // namespace vgpu

using namespace vgpu;

namespace {
size_t al(size_t x) { return (x + 255) & ~size_t(255); }

// Grid over a sample set: about 2 samples per occupied cell on a surface, at
// most 160 cells per axis.
void grid_for_points(const double* x, long long n, HGrid& g) {
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (long long i = 0; i < n; ++i)
    for (int a = 0; a < 3; ++a) {
      lo[a] = std::min(lo[a], x[3 * i + a]);
      hi[a] = std::max(hi[a], x[3 * i + a]);
    }
  double ext = std::max(hi[0] - lo[0], std::max(hi[1] - lo[1], hi[2] - lo[2]));
  double area_like = 0;
  for (int a = 0; a < 3; ++a) area_like += (hi[a] - lo[a]) * (hi[(a + 1) % 3] - lo[(a + 1) % 3]);
  double h = std::sqrt(std::max(area_like, 1e-30) * 2.0 / (double)std::max(n, 1LL));
  h = std::max(h, ext / 160.0);
  if (!(h > 0)) h = 1.0;
  for (int a = 0; a < 3; ++a) {
    g.lo[a] = lo[a];
    g.dim[a] = std::max(1, (int)std::ceil((hi[a] - lo[a]) / h) + 1);
  }
  g.h = h;
  g.n = (int)n;
}
}  // namespace

extern "C" int visacd_face_hausdorff_batch(visacd_ctx* ctx, int32_t njobs, const double* verts,
                                           const int64_t* vert_off, const int32_t* tris, const int64_t* tri_off,
                                           const double* samples, const int32_t* sample_tri,
                                           const int64_t* sample_off, const double* lower, double floor,
                                           int32_t independent, double* out) {
  VCHECK(ctx && out && vert_off && tri_off && sample_off, VISACD_ERR_INVALID_ARG,
         "face_hausdorff_batch: null argument");
  VCHECK(njobs >= 0, VISACD_ERR_INVALID_ARG, "face_hausdorff_batch: negative job count");
  VCHECK(floor == floor, VISACD_ERR_INVALID_ARG, "face_hausdorff_batch: floor is NaN");
  if (njobs == 0) return VISACD_OK;
  const int S = 2 * njobs;
  VCHECK(vert_off[0] == 0 && tri_off[0] == 0 && sample_off[0] == 0, VISACD_ERR_INVALID_ARG,
         "face_hausdorff_batch: offsets must start at 0");
  VCHECK(verts && tris && samples && sample_tri, VISACD_ERR_INVALID_ARG, "face_hausdorff_batch: null array");
  for (int s = 0; s < S; ++s) {
    const int64_t nv = vert_off[s + 1] - vert_off[s], nt = tri_off[s + 1] - tri_off[s],
                  ns = sample_off[s + 1] - sample_off[s];
    VCHECK(nv > 0 && nt > 0 && ns > 0, VISACD_ERR_INVALID_ARG, "face_hausdorff_batch: empty surface %d", s);
    VCHECK(indices_in_range(tris + 3 * tri_off[s], 3 * nt, nv), VISACD_ERR_INVALID_ARG,
           "face_hausdorff_batch: vertex index out of range (surface %d)", s);
    VCHECK(indices_in_range(sample_tri + sample_off[s], ns, nt), VISACD_ERR_INVALID_ARG,
           "face_hausdorff_batch: sample triangle out of range (surface %d)", s);
  }
  if (lower)
    for (int j = 0; j < njobs; ++j)
      VCHECK(lower[j] == lower[j], VISACD_ERR_INVALID_ARG, "face_hausdorff_batch: lower bound is NaN");
  VCUDA(cudaSetDevice(ctx->device));
  const long long NV = vert_off[S], NT = tri_off[S], NS = sample_off[S];
  // Grids and rounding bounds per job (both sets of a job share M).
  std::vector<HGrid> grids(S);
  std::vector<float> tmargin(njobs);
  std::vector<int> cell0(S + 1, 0);
  for (int s = 0; s < S; ++s) grid_for_points(samples + 3 * sample_off[s], sample_off[s + 1] - sample_off[s], grids[s]);
  for (int j = 0; j < njobs; ++j) {
    // FP32 pre-filter bound: coordinates rounded to float differ by at most
    // 2^-24 |x| each, the difference and the squared sum add a few ulps; with
    // M the largest |coordinate| of both sets, |d_f32 - d| <= 8 M 2^-24.
    double M = 0;
    for (int k = 2 * j; k < 2 * j + 2; ++k)
      for (int a = 0; a < 3; ++a)
        M = std::max(M, std::max(std::fabs(grids[k].lo[a]), std::fabs(grids[k].lo[a] + grids[k].h * grids[k].dim[a])));
    for (int k = 2 * j; k < 2 * j + 2; ++k) grids[k].eabs = (float)(M * std::ldexp(1.0, -21) + 1e-30);
    // Margin of the FP32 triangle lower bounds: the plane evaluation's rounding
    // (normal and offset rounded to float, a few ulps of the largest
    // coordinate), with room to spare; the box gap is conservative.
    tmargin[j] = (float)(1e-9 + 256.0 * std::ldexp(1.0, -24) * (M + 4.0));
  }
  for (int s = 0; s < S; ++s) cell0[s + 1] = cell0[s] + grids[s].dim[0] * grids[s].dim[1] * grids[s].dim[2];
  const int ncell = cell0[S];
  double gmax0 = std::max(floor, 0.0);
  std::vector<double> low(njobs, 0.0);
  if (lower)
    for (int j = 0; j < njobs; ++j) {
      low[j] = std::max(lower[j], 0.0);
      gmax0 = std::max(gmax0, low[j]);
    }
  // Device layout: the uploaded block first (one copy), then the scratch.
  size_t off = 0;
  auto carve = [&](size_t b) { size_t o = off; off += al(b); return o; };
  const size_t o_v = carve((size_t)NV * 24), o_t = carve((size_t)NT * 12), o_x = carve((size_t)NS * 24),
               o_id = carve((size_t)NS * 4), o_soff = carve((size_t)(S + 1) * 8), o_toff = carve((size_t)(S + 1) * 8),
               o_voff = carve((size_t)(S + 1) * 8), o_c0 = carve((size_t)(S + 1) * 4),
               o_low = carve((size_t)njobs * 8), o_tm = carve((size_t)njobs * 4), o_gm = carve(8),
               o_grids = carve(sizeof(HGrid) * S), o_sides = carve(sizeof(HSide) * S);
  const size_t upload = off;
  // Zeroed together: job maxima, far count, per-cell counts and fills.
  const size_t zero_begin = off;
  const size_t o_jm = carve((size_t)njobs * 8), o_far = carve(8), o_cnt = carve((size_t)(ncell + 1) * 4),
               o_fill = carve((size_t)ncell * 4);
  const size_t zero_end = off;
  const size_t o_off = carve((size_t)(ncell + 1) * 8), o_cell = carve((size_t)NS * 4),
               o_order = carve((size_t)NS * 4), o_start = carve((size_t)(ncell + S) * 4),
               o_spts = carve((size_t)NS * 16), o_tb = carve((size_t)NT * 48), o_ub = carve((size_t)NS * 4),
               o_qref = carve((size_t)NS * 8), o_farl = carve((size_t)NS * 8);
  VTRY(ensure_slot(ctx, kSlotHausdorff, off));
  char* D = slot<char>(ctx, kSlotHausdorff);
  cudaStream_t st = ctx->stream;
  // Device pointers of every grid and side.
  for (int s = 0; s < S; ++s) {
    HGrid& g = grids[s];
    g.start = (const int*)(D + o_start) + cell0[s] + s;
    g.order = (const int*)(D + o_order) + sample_off[s];
    g.pts = (const double*)(D + o_x) + 3 * sample_off[s];
    g.spts = (const float4*)(D + o_spts) + sample_off[s];
  }
  std::vector<HSide> sides(S);
  for (int s = 0; s < S; ++s) {
    const int o = s ^ 1;
    HSide& d = sides[s];
    d.Q = (const double*)(D + o_x) + 3 * sample_off[s];
    d.nq = (int)(sample_off[s + 1] - sample_off[s]);
    d.G = grids[o];
    d.ids = (const int*)(D + o_id) + sample_off[o];
    d.mv = (const double*)(D + o_v) + 3 * vert_off[o];
    d.mt = (const int*)(D + o_t) + 3 * tri_off[o];
    d.tb = (const float4*)(D + o_tb) + 3 * tri_off[o];
  }
  Stager up(ctx);
  VTRY(up.reserve(upload, 1));
  char* h = up.host();
  auto put = [&](size_t o, const void* src, size_t bytes) {
    if (bytes) std::memcpy(h + o, src, bytes);
  };
  put(o_v, verts, (size_t)NV * 24);
  put(o_t, tris, (size_t)NT * 12);
  put(o_x, samples, (size_t)NS * 24);
  put(o_id, sample_tri, (size_t)NS * 4);
  put(o_soff, sample_off, (size_t)(S + 1) * 8);
  put(o_toff, tri_off, (size_t)(S + 1) * 8);
  put(o_voff, vert_off, (size_t)(S + 1) * 8);
  put(o_c0, cell0.data(), (size_t)(S + 1) * 4);
  put(o_low, low.data(), (size_t)njobs * 8);
  put(o_tm, tmargin.data(), (size_t)njobs * 4);
  put(o_gm, &gmax0, 8);
  put(o_grids, grids.data(), sizeof(HGrid) * S);
  put(o_sides, sides.data(), sizeof(HSide) * S);
  VTRY(up.copy(D, upload));
  VCUDA(cudaMemsetAsync(D + zero_begin, 0, zero_end - zero_begin, st));
  HBatch H;
  H.nsets = S;
  H.sample_off = (const long long*)(D + o_soff);
  H.tri_off = (const long long*)(D + o_toff);
  H.vert_off = (const long long*)(D + o_voff);
  H.cell0 = (const int*)(D + o_c0);
  H.grids = (const HGrid*)(D + o_grids);
  H.sides = (const HSide*)(D + o_sides);
  H.pts = (const double*)(D + o_x);
  H.mv = (const double*)(D + o_v);
  H.mt = (const int*)(D + o_t);
  H.tb = (float4*)(D + o_tb);
  H.lower = (const double*)(D + o_low);
  H.job_max = (unsigned long long*)(D + o_jm);
  H.gmax = (unsigned long long*)(D + o_gm);
  H.tmargin = (const float*)(D + o_tm);
  H.independent = independent ? 1 : 0;
  int* cnt = (int*)(D + o_cnt);
  unsigned long long* offs = (unsigned long long*)(D + o_off);
  const unsigned gp = grid_for(NS + NT, 256, 8LL * ctx->sm_count), gs = grid_for(NS, 256, 8LL * ctx->sm_count);
  VLAUNCH(ctx, kKHausdorff, gp, 256, 0, hprep_kernel, H, NS, NT, cnt, (int*)(D + o_cell));
  VTRY(exclusive_scan_u32_to_u64(ctx, (const uint32_t*)cnt, (uint64_t*)offs, ncell));
  VLAUNCH(ctx, kKHausdorff, gs, 256, 0, hscatter_kernel, H, NS, (const int*)(D + o_cell),
          (const unsigned long long*)offs, (int*)(D + o_fill), (int*)(D + o_order));
  VLAUNCH(ctx, kKHausdorff, grid_for(NS + ncell + S, 256, 8LL * ctx->sm_count), 256, 0, hfinish_kernel, H, NS,
          ncell, (const unsigned long long*)offs, (const int*)(D + o_order), (int*)(D + o_start),
          (float4*)(D + o_spts));
  unsigned* far = (unsigned*)(D + o_far);
  VLAUNCH(ctx, kKHausdorffBound, grid_for(NS, 128, 8LL * ctx->sm_count), 128, 0, hbound_kernel, H, NS,
          (const int*)(D + o_order), (float*)(D + o_ub), (int2*)(D + o_qref), far, (long long*)(D + o_farl));
  // The queries without a bound one warp each, then the rest with pruning.
  VLAUNCH(ctx, kKHausdorffHead, grid_for(32LL * NS, 128, 8LL * ctx->sm_count), 128, 0, hhead_kernel, H,
          (const int2*)(D + o_qref), (const long long*)(D + o_farl), (const unsigned*)far);
  VLAUNCH(ctx, kKHausdorffQuery, grid_for(NS, 128, 8LL * ctx->sm_count), 128, 0, hquery_kernel, H,
          (const float*)(D + o_ub), (const int2*)(D + o_qref), NS);
  double* hres = nullptr;
  VTRY(pinned(ctx, (size_t)njobs * 8, (void**)&hres));
  VCUDA(cudaMemcpyAsync(hres, D + o_jm, (size_t)njobs * 8, cudaMemcpyDeviceToHost, st));
  VCUDA(stream_wait(ctx));
  std::memcpy(out, hres, (size_t)njobs * 8);
  return VISACD_OK;
}

extern "C" int visacd_face_hausdorff_floor(visacd_ctx* ctx, const double* va, int32_t nva, const int32_t* ta,
                                           int32_t nta, const double* xa, const int32_t* ida, int32_t na,
                                           const double* vb, int32_t nvb, const int32_t* tb, int32_t ntb,
                                           const double* xb, const int32_t* idb, int32_t nb, double floor,
                                           double* out) {
  VCHECK(ctx && out, VISACD_ERR_INVALID_ARG, "face_hausdorff: null argument");
  VCHECK(na > 0 && nb > 0 && nva > 0 && nvb > 0 && nta > 0 && ntb > 0, VISACD_ERR_INVALID_ARG,
         "face_hausdorff: empty input");
  VCHECK(va && ta && xa && ida && vb && tb && xb && idb, VISACD_ERR_INVALID_ARG, "face_hausdorff: null array");
  // One job: the two surfaces' arrays side by side.
  std::vector<double> v((size_t)(nva + nvb) * 3), x((size_t)(na + nb) * 3);
  std::vector<int32_t> t((size_t)(nta + ntb) * 3), id((size_t)(na + nb));
  std::memcpy(v.data(), va, (size_t)nva * 24);
  std::memcpy(v.data() + 3 * (size_t)nva, vb, (size_t)nvb * 24);
  std::memcpy(t.data(), ta, (size_t)nta * 12);
  std::memcpy(t.data() + 3 * (size_t)nta, tb, (size_t)ntb * 12);
  std::memcpy(x.data(), xa, (size_t)na * 24);
  std::memcpy(x.data() + 3 * (size_t)na, xb, (size_t)nb * 24);
  std::memcpy(id.data(), ida, (size_t)na * 4);
  std::memcpy(id.data() + na, idb, (size_t)nb * 4);
  const int64_t voff[3] = {0, nva, (int64_t)nva + nvb}, toff[3] = {0, nta, (int64_t)nta + ntb},
                soff[3] = {0, na, (int64_t)na + nb};
  return visacd_face_hausdorff_batch(ctx, 1, v.data(), voff, t.data(), toff, x.data(), id.data(), soff, nullptr,
                                     floor, 0, out);
}

extern "C" int visacd_face_hausdorff(visacd_ctx* ctx, const double* va, int32_t nva, const int32_t* ta,
                                     int32_t nta, const double* xa, const int32_t* ida, int32_t na,
                                     const double* vb, int32_t nvb, const int32_t* tb, int32_t ntb,
                                     const double* xb, const int32_t* idb, int32_t nb, double* out) {
  return visacd_face_hausdorff_floor(ctx, va, nva, ta, nta, xa, ida, na, vb, nvb, tb, ntb, xb, idb, nb, 0.0, out);
}

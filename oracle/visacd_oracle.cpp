// visacd_oracle.cpp — CPU restatement of VisACD's visibility-edge hot path.
//
// TEST INFRASTRUCTURE ONLY. This library is the checker for the GPU kernels:
// only the tests, the smoke check and the CPU-baseline leg of the benchmark
// load it. The product path never calls into it.
//
// Every function states the reference code it restates (paths are inside the
// VisACD source tree). Arithmetic is IEEE double unless stated, built with
// -ffp-contract=off so that the order of operations written here is the order
// executed.
//
// Parity pins:
//  * plane scoring: against outputs of the reference CUDA kernel
//    (lib/cuda/plane_intersections.cu) run on a GB300, stored as fixtures.
//  * candidate planes: the same std::mt19937 + std::uniform_int_distribution
//    (libstdc++) calls in the same order as lib/src/process.cpp:28-72.
//  * visibility: the reference's OptiX path cannot run here (SDK absent), so the
//    end-vertex policy is this project's own and visibility parity is unpinned
//    against OptiX; the oracle defines it.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <random>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {

int oracle_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void oracle_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

// ---------------------------------------------------------------------------
// Plane scoring — lib/cuda/plane_intersections.cu:7-67.
// side(x) = +1 if v > eps, -1 if v < -eps, else 0, eps = 1e-6f (:15, :46-47);
// an edge contributes iff both sides are non-zero and differ (:50-57).
// v is evaluated in double from the float inputs as ((a x + b y) + c z) + d.
// scores_fp64[p]: sum of the double length of crossing edges.
// q_scores[p]:    sum of the FP32 length (IEEE ops, fixed order) quantized to
//                 2^qexp, qexp = e - 22 with max|coord| < 2^e — the exact
//                 integer the GPU kernel produces.
// Edges with an index >= N are skipped (:34-36); edges with a non-finite
// endpoint are skipped too.
// ---------------------------------------------------------------------------
static inline double side_value(const float* pl, const float* x) {
  double ax = (double)pl[0] * (double)x[0];
  double by = (double)pl[1] * (double)x[1];
  double cz = (double)pl[2] * (double)x[2];
  return ((ax + by) + cz) + (double)pl[3];
}

static inline float edge_len32(const float* a, const float* b) {
  float dx = b[0] - a[0], dy = b[1] - a[1], dz = b[2] - a[2];
  float s = (dx * dx + dy * dy) + dz * dz;
  return sqrtf(s);
}

static int quantum_exp(const float* pts, int32_t N) {
  float m = 0.f;
  for (int64_t i = 0; i < 3LL * N; i += 3) {
    if (!(std::isfinite(pts[i]) && std::isfinite(pts[i + 1]) && std::isfinite(pts[i + 2])))
      continue;
    for (int a = 0; a < 3; ++a) m = std::max(m, fabsf(pts[i + a]));
  }
  uint32_t bits;
  memcpy(&bits, &m, 4);
  int eb = (int)((bits >> 23) & 0xffu);
  int e = eb >= 1 ? eb - 126 : -126;
  return e - 22;
}

int oracle_score_planes(const float* planes, int32_t P, const float* pts, int32_t N,
                        const uint32_t* edges, int64_t E, double* scores_fp64,
                        uint64_t* q_scores, int32_t* qexp_out, int64_t* skipped_out) {
  const double eps = (double)1e-6f;
  const int qexp = quantum_exp(pts, N);
  std::vector<uint32_t> q((size_t)E);
  std::vector<double> len64((size_t)E);
  std::vector<uint8_t> ok((size_t)E);
  int64_t skipped = 0;
  for (int64_t e = 0; e < E; ++e) {
    uint32_t i = edges[2 * e], j = edges[2 * e + 1];
    bool good = i < (uint32_t)N && j < (uint32_t)N;
    if (good) {
      const float *a = pts + 3 * (int64_t)i, *b = pts + 3 * (int64_t)j;
      for (int k = 0; k < 3; ++k) good = good && std::isfinite(a[k]) && std::isfinite(b[k]);
    }
    ok[e] = good;
    if (!good) {
      ++skipped;
      q[e] = 0;
      len64[e] = 0;
      continue;
    }
    const float *a = pts + 3 * (int64_t)i, *b = pts + 3 * (int64_t)j;
    float l32 = edge_len32(a, b);
    q[e] = (uint32_t)nearbyintf(ldexpf(l32, -qexp));
    double dx = (double)b[0] - (double)a[0], dy = (double)b[1] - (double)a[1],
           dz = (double)b[2] - (double)a[2];
    len64[e] = sqrt((dx * dx + dy * dy) + dz * dz);
  }
#pragma omp parallel for schedule(dynamic, 4)
  for (int32_t p = 0; p < P; ++p) {
    const float* pl = planes + 4 * (int64_t)p;
    double s = 0.0;
    uint64_t qs = 0;
    for (int64_t e = 0; e < E; ++e) {
      if (!ok[e]) continue;
      const float* a = pts + 3 * (int64_t)edges[2 * e];
      const float* b = pts + 3 * (int64_t)edges[2 * e + 1];
      double v1 = side_value(pl, a), v2 = side_value(pl, b);
      int s1 = (v1 > eps) - (v1 < -eps), s2 = (v2 > eps) - (v2 < -eps);
      if (s1 != 0 && s2 != 0 && s1 != s2) {
        s += len64[e];
        qs += q[e];
      }
    }
    if (scores_fp64) scores_fp64[p] = s;
    if (q_scores) q_scores[p] = qs;
  }
  if (qexp_out) *qexp_out = qexp;
  if (skipped_out) *skipped_out = skipped;
  return 0;
}

// The reference kernel's FP32 arithmetic, restated on the CPU for comparison
// with the GPU reference outputs: v = a*x + b*y + c*z + d in float with the
// products and sums in source order (no contraction), sides against 1e-6f,
// float length sqrtf(dx*dx + dy*dy + dz*dz), float accumulation in edge order.
int oracle_score_planes_ref32(const float* planes, int32_t P, const float* pts, int32_t N,
                              const uint32_t* edges, int64_t E, float* scores) {
  const float eps = 1e-6f;
#pragma omp parallel for schedule(dynamic, 4)
  for (int32_t p = 0; p < P; ++p) {
    const float* pl = planes + 4 * (int64_t)p;
    float s = 0.f;
    for (int64_t e = 0; e < E; ++e) {
      uint32_t i = edges[2 * e], j = edges[2 * e + 1];
      if (i >= (uint32_t)N || j >= (uint32_t)N) continue;
      const float *a = pts + 3 * (int64_t)i, *b = pts + 3 * (int64_t)j;
      float v1 = pl[0] * a[0] + pl[1] * a[1] + pl[2] * a[2] + pl[3];
      float v2 = pl[0] * b[0] + pl[1] * b[1] + pl[2] * b[2] + pl[3];
      int s1 = (v1 > eps) - (v1 < -eps), s2 = (v2 > eps) - (v2 < -eps);
      if (s1 != 0 && s1 == s2) continue;
      if (s1 == 0 || s2 == 0) continue;
      float dx = b[0] - a[0], dy = b[1] - a[1], dz = b[2] - a[2];
      s += sqrtf(dx * dx + dy * dy + dz * dz);
    }
    scores[p] = s;
  }
  return 0;
}

// ---------------------------------------------------------------------------
// Segment-triangle test — lib/ptx/ray_segments.cu:49-111 with OptiX's
// any-hit triangle test replaced by an explicit formula.
// Segment p -> q, parameter t in [tmin/|q-p|, 1], tmin = 0.001f (:99-100).
// Edge functions relative to p: W_a = D.(B x C), W_b = D.(C x A),
// W_c = D.(A x B) with A = a - p etc.; the line meets the closed triangle iff
// all three have one sign; det = W_a + W_b + W_c, t = A.(B x C) / det.
// Grazing: the decision could flip if each W moved by 1e-6 (|W_a|+|W_b|+|W_c|),
// |det| by 1e-6 |D| |n|, or t by 1e-6.
// ---------------------------------------------------------------------------
struct TriDecision {
  bool hit;
  bool certain;  // false: within the grazing band
};

static inline TriDecision seg_tri64(const float* p, const float* q, const float* a,
                                    const float* b, const float* c) {
  const double Ax = (double)a[0] - (double)p[0], Ay = (double)a[1] - (double)p[1],
               Az = (double)a[2] - (double)p[2];
  const double Bx = (double)b[0] - (double)p[0], By = (double)b[1] - (double)p[1],
               Bz = (double)b[2] - (double)p[2];
  const double Cx = (double)c[0] - (double)p[0], Cy = (double)c[1] - (double)p[1],
               Cz = (double)c[2] - (double)p[2];
  const double Dx = (double)q[0] - (double)p[0], Dy = (double)q[1] - (double)p[1],
               Dz = (double)q[2] - (double)p[2];
  const double BCx = By * Cz - Bz * Cy, BCy = Bz * Cx - Bx * Cz, BCz = Bx * Cy - By * Cx;
  const double CAx = Cy * Az - Cz * Ay, CAy = Cz * Ax - Cx * Az, CAz = Cx * Ay - Cy * Ax;
  const double ABx = Ay * Bz - Az * By, ABy = Az * Bx - Ax * Bz, ABz = Ax * By - Ay * Bx;
  const double Wa = (Dx * BCx + Dy * BCy) + Dz * BCz;
  const double Wb = (Dx * CAx + Dy * CAy) + Dz * CAz;
  const double Wc = (Dx * ABx + Dy * ABy) + Dz * ABz;
  const double det = (Wa + Wb) + Wc;
  const double vol = (Ax * BCx + Ay * BCy) + Az * BCz;
  const double len = sqrt((Dx * Dx + Dy * Dy) + Dz * Dz);
  const double tmin = (double)0.001f;
  // Decision (identical to the GPU FP64 path).
  bool hit = false;
  if (det != 0.0) {
    bool inside = (Wa >= 0.0 && Wb >= 0.0 && Wc >= 0.0) || (Wa <= 0.0 && Wb <= 0.0 && Wc <= 0.0);
    if (inside) {
      double lhs = vol * len, rhs = tmin * det;
      hit = det > 0.0 ? (lhs >= rhs && vol <= det) : (lhs <= rhs && vol >= det);
    }
  }
  // Grazing band.
  const double tau = 1e-6;
  const double S = fabs(Wa) + fabs(Wb) + fabs(Wc);
  const double dl = tau * S;
  bool in_possible = (Wa >= -dl && Wb >= -dl && Wc >= -dl) || (Wa <= dl && Wb <= dl && Wc <= dl);
  bool in_certain = (Wa > dl && Wb > dl && Wc > dl) || (Wa < -dl && Wb < -dl && Wc < -dl);
  const double nx = ABx + BCx + CAx, ny = ABy + BCy + CAy, nz = ABz + BCz + CAz;
  const double nlen = sqrt(nx * nx + ny * ny + nz * nz);
  bool det_ok = fabs(det) > tau * len * nlen;
  bool certain;
  if (!in_possible) {
    certain = true;
  } else if (det_ok) {
    double t = vol / det, tm = tmin / len;
    bool t_in = t > tm + tau && t < 1.0 - tau;
    bool t_out = t < tm - tau || t > 1.0 + tau;
    certain = t_out || (in_certain && t_in);
  } else {
    certain = false;
  }
  return {hit, certain};
}

// Result of one segment against one mesh: hit, and whether any grazing
// triangle could change it.
struct MeshDecision {
  bool hit;
  bool robust;
};

static MeshDecision seg_mesh_brute(const float* p, const float* q, int64_t vi, int64_t vj,
                                   const float* verts, const uint32_t* tris, int32_t nt,
                                   bool exclude) {
  bool hit = false, certain_hit = false, graze = false;
  for (int32_t t = 0; t < nt; ++t) {
    uint32_t i0 = tris[3 * t], i1 = tris[3 * t + 1], i2 = tris[3 * t + 2];
    if (exclude && (i0 == vi || i1 == vi || i2 == vi || i0 == vj || i1 == vj || i2 == vj))
      continue;
    TriDecision d = seg_tri64(p, q, verts + 3 * (int64_t)i0, verts + 3 * (int64_t)i1,
                              verts + 3 * (int64_t)i2);
    hit = hit || d.hit;
    if (d.certain) {
      if (d.hit) certain_hit = true;
    } else {
      graze = true;
    }
    if (certain_hit) break;
  }
  return {hit, certain_hit || !graze};
}

// ---------------------------------------------------------------------------
// CPU BVH (median split, FP64 boxes widened by a relative 1e-9) for the larger
// oracle runs and the CPU baseline. Traversal visits every box the segment can
// touch and applies seg_tri64 to each candidate triangle, so its decisions
// equal the brute-force ones.
// ---------------------------------------------------------------------------
struct CpuNode {
  double lo[3], hi[3];
  int32_t left, right;  // children, or -1
  int32_t first, count; // leaf range into the triangle order
};

struct CpuBvh {
  std::vector<CpuNode> nodes;
  std::vector<int32_t> order;
};

static void build_cpu_bvh(const float* v, const uint32_t* t, int32_t nt, CpuBvh& bvh) {
  bvh.nodes.clear();
  bvh.order.resize(nt);
  std::vector<double> cen(3 * (size_t)nt);
  for (int32_t k = 0; k < nt; ++k) {
    bvh.order[k] = k;
    for (int a = 0; a < 3; ++a)
      cen[3 * k + a] = ((double)v[3 * t[3 * k] + a] + v[3 * t[3 * k + 1] + a] + v[3 * t[3 * k + 2] + a]) / 3.0;
  }
  struct Item { int32_t node, first, count; };
  std::vector<Item> stack;
  bvh.nodes.push_back(CpuNode());
  stack.push_back({0, 0, nt});
  while (!stack.empty()) {
    Item it = stack.back();
    stack.pop_back();
    CpuNode nd;
    for (int a = 0; a < 3; ++a) { nd.lo[a] = INFINITY; nd.hi[a] = -INFINITY; }
    for (int32_t k = it.first; k < it.first + it.count; ++k) {
      int32_t tr = bvh.order[k];
      for (int c = 0; c < 3; ++c)
        for (int a = 0; a < 3; ++a) {
          double x = v[3 * t[3 * tr + c] + a];
          nd.lo[a] = std::min(nd.lo[a], x);
          nd.hi[a] = std::max(nd.hi[a], x);
        }
    }
    for (int a = 0; a < 3; ++a) {
      double pad = 1e-9 * std::max(1.0, std::max(fabs(nd.lo[a]), fabs(nd.hi[a])));
      nd.lo[a] -= pad;
      nd.hi[a] += pad;
    }
    nd.left = nd.right = -1;
    nd.first = it.first;
    nd.count = it.count;
    if (it.count > 4) {
      int ax = 0;
      double ext = -1;
      for (int a = 0; a < 3; ++a)
        if (nd.hi[a] - nd.lo[a] > ext) { ext = nd.hi[a] - nd.lo[a]; ax = a; }
      int32_t mid = it.first + it.count / 2;
      std::nth_element(bvh.order.begin() + it.first, bvh.order.begin() + mid,
                       bvh.order.begin() + it.first + it.count,
                       [&](int32_t x, int32_t y) { return cen[3 * x + ax] < cen[3 * y + ax]; });
      int32_t l = (int32_t)bvh.nodes.size();
      bvh.nodes.push_back(CpuNode());
      int32_t r = (int32_t)bvh.nodes.size();
      bvh.nodes.push_back(CpuNode());
      nd.left = l;
      nd.right = r;
      stack.push_back({l, it.first, mid - it.first});
      stack.push_back({r, mid, it.first + it.count - mid});
    }
    bvh.nodes[it.node] = nd;
  }
}

static inline bool seg_box(const double* o, const double* d, const CpuNode& nd) {
  double tn = 0.0, tf = 1.0;
  for (int a = 0; a < 3; ++a) {
    if (fabs(d[a]) < 1e-300) {
      if (o[a] < nd.lo[a] || o[a] > nd.hi[a]) return false;
      continue;
    }
    double inv = 1.0 / d[a];
    double t0 = (nd.lo[a] - o[a]) * inv, t1 = (nd.hi[a] - o[a]) * inv;
    if (t0 > t1) std::swap(t0, t1);
    tn = std::max(tn, t0);
    tf = std::min(tf, t1);
  }
  return tn <= tf * (1.0 + 1e-12) + 1e-15;
}

static MeshDecision seg_mesh_bvh(const float* p, const float* q, int64_t vi, int64_t vj,
                                 const float* verts, const uint32_t* tris, const CpuBvh& bvh,
                                 bool exclude) {
  if (bvh.order.empty()) return {false, true};
  double o[3] = {p[0], p[1], p[2]};
  double d[3] = {(double)q[0] - p[0], (double)q[1] - p[1], (double)q[2] - p[2]};
  int32_t stk[128];
  int sp = 0;
  stk[sp++] = 0;
  bool hit = false, graze = false;
  while (sp) {
    const CpuNode& nd = bvh.nodes[stk[--sp]];
    if (!seg_box(o, d, nd)) continue;
    if (nd.left < 0) {
      for (int32_t k = nd.first; k < nd.first + nd.count; ++k) {
        int32_t t = bvh.order[k];
        uint32_t i0 = tris[3 * t], i1 = tris[3 * t + 1], i2 = tris[3 * t + 2];
        if (exclude && (i0 == vi || i1 == vi || i2 == vi || i0 == vj || i1 == vj || i2 == vj))
          continue;
        TriDecision td = seg_tri64(p, q, verts + 3 * (int64_t)i0, verts + 3 * (int64_t)i1,
                                   verts + 3 * (int64_t)i2);
        hit = hit || td.hit;
        if (td.certain) {
          if (td.hit) return {true, true};
        } else {
          graze = true;
        }
      }
    } else {
      if (sp + 2 > 128) return {true, false};
      stk[sp++] = nd.right;
      stk[sp++] = nd.left;
    }
  }
  return {hit, !graze};
}

static inline int64_t row_start(int64_t i, int64_t n) { return i * (2 * n - i - 1) / 2; }

// ---------------------------------------------------------------------------
// Visibility — lib/src/intersections.cpp:327-385 and ray_segments.cu:49-111.
// For each pair i < j (only pairs with an is_new endpoint when is_new != NULL,
// :62-68), edge iff the segment hits the cage and does not hit the part, where
// the part's triangles incident to i or j are skipped (end-vertex policy).
// Pairs with coincident endpoints are never edges (:88-93).
// out_bits: one byte per linear pair index (row-major, i < j):
//   0 = not an edge, 1 = edge; bit 1 (value 2) marks a grazing pair.
// A pair is grazing when its edge decision rests on a test within the 1e-6
// band: the cage test is decided first; a robust cage miss decides "no edge"
// whatever the part test gives, and a robust part hit decides "no edge"
// whatever the cage test gives; otherwise the pair is grazing if either test
// is within the band.
// Returns the number of edges; *n_grazing gets the number of grazing pairs.
// use_bvh selects the BVH traversal (same decisions) over brute force.
// row_begin/row_end restrict the rows computed (for bounded CPU samples);
// pass 0, n for all.
// ---------------------------------------------------------------------------
static int64_t visibility_rows(const float* pts, int32_t n, const uint8_t* is_new,
                               const uint32_t* tris, int32_t nt, const float* cage_v,
                               const uint32_t* cage_t, int32_t nct, int use_bvh,
                               const int32_t* rows, int32_t n_rows, uint8_t* out_bits,
                               int64_t* n_grazing, int64_t* n_pairs) {
  CpuBvh sb, cb;
  if (use_bvh) {
    build_cpu_bvh(pts, tris, nt, sb);
    build_cpu_bvh(cage_v, cage_t, nct, cb);
  }
  int64_t edges = 0, grazing = 0, pairs = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : edges, grazing, pairs)
  for (int32_t r = 0; r < n_rows; ++r) {
    const int32_t i = rows[r];
    if (i < 0 || i >= n) continue;
    for (int32_t j = i + 1; j < n; ++j) {
      int64_t k = row_start(i, n) + (j - i - 1);
      uint8_t r = 0;
      if (is_new && !is_new[i] && !is_new[j]) {
        if (out_bits) out_bits[k] = 0;
        continue;
      }
      ++pairs;
      const float *p = pts + 3 * (int64_t)i, *q = pts + 3 * (int64_t)j;
      if (p[0] == q[0] && p[1] == q[1] && p[2] == q[2]) {
        if (out_bits) out_bits[k] = 0;
        continue;
      }
      MeshDecision c = use_bvh ? seg_mesh_bvh(p, q, -1, -1, cage_v, cage_t, cb, false)
                               : seg_mesh_brute(p, q, -1, -1, cage_v, cage_t, nct, false);
      bool edge = false, graze = false;
      if (!c.hit && c.robust) {
        edge = false;
      } else {
        MeshDecision s = use_bvh ? seg_mesh_bvh(p, q, i, j, pts, tris, sb, true)
                                 : seg_mesh_brute(p, q, i, j, pts, tris, nt, true);
        if (s.hit && s.robust) {
          edge = false;
        } else {
          edge = !s.hit && c.hit;
          graze = !s.robust || !c.robust;
        }
      }
      if (edge) {
        r |= 1;
        ++edges;
      }
      if (graze) {
        r |= 2;
        ++grazing;
      }
      if (out_bits) out_bits[k] = r;
    }
  }
  if (n_grazing) *n_grazing = grazing;
  if (n_pairs) *n_pairs = pairs;
  return edges;
}

int64_t oracle_visibility(const float* pts, int32_t n, const uint8_t* is_new,
                          const uint32_t* tris, int32_t nt, const float* cage_v, int32_t ncv,
                          const uint32_t* cage_t, int32_t nct, int use_bvh, int32_t row_begin,
                          int32_t row_end, uint8_t* out_bits, int64_t* n_grazing,
                          int64_t* n_pairs) {
  (void)ncv;
  if (row_end > n) row_end = n;
  if (row_begin < 0) row_begin = 0;
  std::vector<int32_t> rows;
  for (int32_t i = row_begin; i < row_end; ++i) rows.push_back(i);
  return visibility_rows(pts, n, is_new, tris, nt, cage_v, cage_t, nct, use_bvh, rows.data(),
                         (int32_t)rows.size(), out_bits, n_grazing, n_pairs);
}

// The same for an explicit list of pair rows i (each row: the pairs (i, j),
// j > i); out_bits is still indexed by the linear pair index of all n(n-1)/2
// pairs and only the listed rows are written.
int64_t oracle_visibility_rows(const float* pts, int32_t n, const uint8_t* is_new,
                               const uint32_t* tris, int32_t nt, const float* cage_v,
                               const uint32_t* cage_t, int32_t nct, const int32_t* rows,
                               int32_t n_rows, uint8_t* out_bits, int64_t* n_grazing,
                               int64_t* n_pairs) {
  return visibility_rows(pts, n, is_new, tris, nt, cage_v, cage_t, nct, 1, rows, n_rows, out_bits,
                         n_grazing, n_pairs);
}

// ---------------------------------------------------------------------------
// Candidate planes — lib/src/process.cpp:28-72. Perpendicular-bisector planes
// of randomly drawn edges: up to num_planes planes from at most 5 * num_planes
// draws of std::uniform_int_distribution<int>(0, E - 1) on std::mt19937(seed);
// degenerate edges (|p2 - p1| < 1e-6) are skipped; a plane is dropped when an
// accepted one has |n.n'| > cos(5 deg) and |d - d'| < 1e-3.
// out: num_planes x 4 doubles (a, b, c, d). Returns the number of planes.
// ---------------------------------------------------------------------------
int32_t oracle_candidate_planes(const double* verts, const uint32_t* edges, int64_t E,
                                int32_t num_planes, uint32_t seed, double* out,
                                int32_t* draws_used) {
  if (draws_used) *draws_used = 0;
  if (E == 0) return 0;
  std::mt19937 eng(seed);
  std::uniform_int_distribution<> dis(0, (int)(E - 1));
  const double normal_eps = cos(5.0 * M_PI / 180.0);
  const double dist_eps = 1e-3;
  int32_t np = 0;
  for (int i = 0; i < num_planes * 5 && np < num_planes; ++i) {
    if (draws_used) *draws_used = i + 1;
    int idx = dis(eng);
    const double* p1 = verts + 3 * (int64_t)edges[2 * (int64_t)idx];
    const double* p2 = verts + 3 * (int64_t)edges[2 * (int64_t)idx + 1];
    double n[3] = {p2[0] - p1[0], p2[1] - p1[1], p2[2] - p1[2]};
    double len = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    if (len < 1e-6) continue;
    n[0] = n[0] / len;
    n[1] = n[1] / len;
    n[2] = n[2] / len;
    double m[3] = {(p1[0] + p2[0]) * 0.5, (p1[1] + p2[1]) * 0.5, (p1[2] + p2[2]) * 0.5};
    double d = -(n[0] * m[0] + n[1] * m[1] + n[2] * m[2]);
    bool similar = false;
    for (int32_t k = 0; k < np; ++k) {
      const double* pk = out + 4 * (int64_t)k;
      double dot = fabs(n[0] * pk[0] + n[1] * pk[1] + n[2] * pk[2]);
      if (dot > normal_eps && fabs(d - pk[3]) < dist_eps) {
        similar = true;
        break;
      }
    }
    if (!similar) {
      double* o = out + 4 * (int64_t)np;
      o[0] = n[0];
      o[1] = n[1];
      o[2] = n[2];
      o[3] = d;
      ++np;
    }
  }
  return np;
}

// The first n edge draws of the loop above: uniform_int_distribution<int>(0,
// E - 1) on std::mt19937(seed), in order.
void oracle_edge_draws(int64_t E, int32_t n, uint32_t seed, int32_t* out) {
  if (E <= 0) return;
  std::mt19937 eng(seed);
  std::uniform_int_distribution<> dis(0, (int)(E - 1));
  for (int32_t k = 0; k < n; ++k) out[k] = dis(eng);
}

// Independent segment-triangle decisions (the precision sweep): seg is S x 6
// (p, q), tri is S x 9 (a, b, c), float32. out[k]: bit 0 = hit, bit 1 = the
// decision lies in the grazing band. Returns the number of hits.
int64_t oracle_seg_tri_batch(const float* seg, const float* tri, int64_t S, uint8_t* out) {
  int64_t hits = 0;
#pragma omp parallel for schedule(static) reduction(+ : hits)
  for (int64_t k = 0; k < S; ++k) {
    const float* sp = seg + 6 * k;
    const float* t = tri + 9 * k;
    TriDecision d = seg_tri64(sp, sp + 3, t, t + 3, t + 6);
    out[k] = (uint8_t)((d.hit ? 1 : 0) | (d.certain ? 0 : 2));
    hits += d.hit ? 1 : 0;
  }
  return hits;
}

// ---------------------------------------------------------------------------
// Surface samples — Mesh::extract_point_set, lib/src/core.cpp:144-232, with
// base 1 and one_per_tri: triangle areas (the reference's triangle_area
// expression, lib/include/core.hpp:119-130), resolution max(1000, res * area),
// triangles drawn by std::discrete_distribution<size_t> over the areas, each
// sample at (1 - sqrt(a)) p0 + sqrt(a)(1 - b) p1 + b sqrt(a) p2 with a, b from
// std::uniform_real_distribution<double>(0, 1), all on std::mt19937(seed), one
// at a time; then one sample on every triangle not drawn, in index order.
// out_xyz / out_ids hold up to cap samples; next4 = the engine's next four
// outputs afterwards. Returns the sample count (or -1 when cap is too small).
// ---------------------------------------------------------------------------
int64_t oracle_sample_points(const double* verts, const int32_t* tris, int32_t nt, int32_t res, uint32_t seed,
                             double* out_xyz, int32_t* out_ids, int64_t cap, uint32_t* next4) {
  if (nt <= 0) return 0;
  std::vector<double> areas(nt);
  double total = 0;
  for (int32_t i = 0; i < nt; ++i) {
    const double* p0 = verts + 3 * (int64_t)tris[3 * i];
    const double* p1 = verts + 3 * (int64_t)tris[3 * i + 1];
    const double* p2 = verts + 3 * (int64_t)tris[3 * i + 2];
    double a = p1[0] * p0[1] - p2[0] * p0[1] - p0[0] * p1[1] + p2[0] * p1[1] + p0[0] * p2[1] - p1[0] * p2[1];
    double b = p1[0] * p0[2] - p2[0] * p0[2] - p0[0] * p1[2] + p2[0] * p1[2] + p0[0] * p2[2] - p1[0] * p2[2];
    double c = p1[1] * p0[2] - p2[1] * p0[2] - p0[1] * p1[2] + p2[1] * p1[2] + p0[1] * p2[2] - p1[1] * p2[2];
    areas[i] = 0.5 * sqrt(pow(a, 2) + pow(b, 2) + pow(c, 2));
    total += areas[i];
  }
  const size_t resolution = (size_t)std::max(1000, (int)(res * (total / 1.0)));
  std::mt19937 eng(seed);
  std::discrete_distribution<size_t> pick(areas.begin(), areas.end());
  std::uniform_real_distribution<double> uni(0.0, 1.0);
  std::vector<char> drawn(nt, 0);
  int64_t n = 0;
  auto emit = [&](size_t ti) {
    double a = uni(eng);
    double b = uni(eng);
    const double* p0 = verts + 3 * (int64_t)tris[3 * ti];
    const double* p1 = verts + 3 * (int64_t)tris[3 * ti + 1];
    const double* p2 = verts + 3 * (int64_t)tris[3 * ti + 2];
    if (n < cap) {
      for (int k = 0; k < 3; ++k)
        out_xyz[3 * n + k] = (1 - sqrt(a)) * p0[k] + (sqrt(a) * (1 - b)) * p1[k] + b * sqrt(a) * p2[k];
      out_ids[n] = (int32_t)ti;
    }
    ++n;
  };
  for (size_t s = 0; s < resolution; ++s) {
    const size_t ti = pick(eng);
    emit(ti);
    drawn[ti] = 1;
  }
  for (int32_t i = 0; i < nt; ++i)
    if (!drawn[i]) emit((size_t)i);
  for (int k = 0; k < 4; ++k) next4[k] = (uint32_t)eng();
  return n <= cap ? n : -1;
}

}  // extern "C"

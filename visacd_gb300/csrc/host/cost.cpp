// Concavity metric: h = max(k * rv, hb) with rv the radius of the sphere whose
// volume is the part/hull volume difference and hb a sampled symmetric
// Hausdorff distance between the two surfaces.
//
// Semantics of lib/src/cost.cpp:45-123 and lib/include/hausdorff.hpp:214-298,
// sampling of lib/src/core.cpp:144-232 (area-weighted triangle choice by
// std::discrete_distribution, two std::uniform_real_distribution draws per
// sample, one extra sample per untouched triangle, all from the process-wide
// engine, the std::mt19937 sequence, in the reference's order; the draws are
// made in bulk with the same values, see extract_point_set). The host
// nearest-sample search is this
// project's kd-tree (the reference uses nanoflann); distances to the sampled
// triangles are the reference's own formula (ref_point_triangle_distance).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <limits>
#include <numeric>
#include <queue>
#include <random>
#include <vector>

#include "geometry.hpp"
#include "gpu_bridge.hpp"

namespace visacd {

constexpr double kPi = 3.14159265;  // the reference's constant (lib/include/cost.hpp:6)

namespace {

// The draws of std::discrete_distribution<size_t> over the same weights (two
// or more), made faster: its result is the first index of the cumulative
// probabilities not below a canonical uniform p, found here through a guide
// table (bucket floor(p n) -> first index whose cumulative value reaches the
// bucket's start) and a short forward scan; every result is checked to be that
// first index, falling back to a binary search, so it equals the
// distribution's draw for the same p.
class DiscreteSampler {
 public:
  explicit DiscreteSampler(const std::discrete_distribution<size_t>& d) {
    const auto prob = d.probabilities();
    cp_.resize(prob.size());
    std::partial_sum(prob.begin(), prob.end(), cp_.begin());
    if (!cp_.empty()) cp_.back() = 1.0;
    const size_t n = cp_.size();
    scale_ = (double)n;
    guide_.resize(n + 1);
    size_t i = 0;
    for (size_t j = 0; j <= n; ++j) {
      const double lo = (double)j / scale_;
      while (i < n && cp_[i] < lo) ++i;
      guide_[j] = i;
    }
  }
  size_t find(double p) const {
    size_t j = (size_t)(p * scale_);
    if (j >= guide_.size()) j = guide_.size() - 1;
    size_t i = guide_[j];
    if (i > 0 && cp_[i - 1] >= p) return std::lower_bound(cp_.begin(), cp_.end(), p) - cp_.begin();
    while (i < cp_.size() && cp_[i] < p) ++i;
    return i;
  }

 private:
  std::vector<double> cp_;
  std::vector<size_t> guide_;
  double scale_ = 0;
};

// A sample of triangle ti at barycentric draws a, b (lib/src/core.cpp:176-191).
inline Vec3 tri_sample(const Mesh& m, size_t ti, double a, double b) {
  const auto& t = m.triangles[ti];
  const Vec3 &v0 = m.vertices[t[0]], &v1 = m.vertices[t[1]], &v2 = m.vertices[t[2]];
  const double sa = std::sqrt(a);  // correctly rounded: one evaluation serves all six uses
  Vec3 v;
  for (int k = 0; k < 3; ++k) v[k] = (1 - sa) * v0[k] + (sa * (1 - b)) * v1[k] + b * sa * v2[k];
  return v;
}

}  // namespace

// Engine outputs are taken in bulk: a draw of the triangle distribution takes
// two outputs (one canonical double; none when there is a single triangle,
// which std::discrete_distribution returns without drawing), each of the two
// uniform doubles two, so sample j of the first loop reads a fixed window of
// the output stream and the samples are computed independently (in parallel
// for large counts); the untouched triangles then take four outputs each, in
// index order. Same values as drawing one by one.
void extract_point_set(const Mesh& m, std::vector<Vec3>& samples, std::vector<int>& tri_ids,
                       size_t resolution, double base, bool one_per_tri) {
  if (m.triangles.empty() || m.vertices.empty()) return;
  const size_t T = m.triangles.size();
  std::vector<double> areas(T);
  double total = 0;
  for (size_t i = 0; i < T; ++i) {
    const auto& t = m.triangles[i];
    areas[i] = triangle_area(m.vertices[t[0]], m.vertices[t[1]], m.vertices[t[2]]);
    total += areas[i];
  }
  if (base != 0) resolution = size_t(std::max(1000, int(resolution * (total / base))));
  std::discrete_distribution<size_t> pick(areas.begin(), areas.end());
  Mt19937& eng = random_engine();
  // Triangles drawn at least once (a bitmap: only membership matters, the
  // untouched ones are visited in index order below).
  std::vector<char> touched(T, 0);
  const size_t b0 = samples.size();
  if ((total > 0 && std::isfinite(total)) || T == 1) {
    const int per = T == 1 ? 4 : 6;
    std::vector<uint32_t> w((size_t)per * resolution);
    eng.fill(w.data(), w.size());
    samples.resize(b0 + resolution);
    tri_ids.resize(b0 + resolution);
    const DiscreteSampler fast(pick);
#pragma omp parallel for schedule(static) if (resolution >= 2048)
    for (long j = 0; j < (long)resolution; ++j) {
      const uint32_t* q = w.data() + (size_t)per * j;
      size_t ti = 0;
      if (T > 1) {
        ti = fast.find(canonical53(q[0], q[1]));
        q += 2;
      }
      samples[b0 + j] = tri_sample(m, ti, canonical53(q[0], q[1]), canonical53(q[2], q[3]));
      tri_ids[b0 + j] = (int)ti;
    }
    for (size_t j = 0; j < resolution; ++j) touched[tri_ids[b0 + j]] = 1;
  } else {
    // Degenerate weights (zero or non-finite total): the distribution itself.
    std::uniform_real_distribution<double> uni(0.0, 1.0);
    for (size_t done = 0; done < resolution; ++done) {
      const size_t ti = pick(eng);
      const double a = uni(eng);
      const double b = uni(eng);
      samples.push_back(tri_sample(m, ti, a, b));
      tri_ids.push_back((int)ti);
      touched[ti] = 1;
    }
  }
  if (!one_per_tri) return;
  std::vector<int> rest;
  for (size_t i = 0; i < T; ++i)
    if (!touched[i]) rest.push_back((int)i);
  std::vector<uint32_t> w(4 * rest.size());
  eng.fill(w.data(), w.size());
  const size_t b1 = samples.size();
  samples.resize(b1 + rest.size());
  tri_ids.resize(b1 + rest.size());
#pragma omp parallel for schedule(static) if (rest.size() >= 2048)
  for (long k = 0; k < (long)rest.size(); ++k) {
    const uint32_t* q = w.data() + 4 * k;
    samples[b1 + k] = tri_sample(m, (size_t)rest[k], canonical53(q[0], q[1]), canonical53(q[2], q[3]));
    tri_ids[b1 + k] = rest[k];
  }
}

namespace {

// Static 3D kd-tree over a point set for k-nearest queries.
class KdTree {
 public:
  explicit KdTree(const std::vector<Vec3>& pts) : P(pts) {
    idx.resize(pts.size());
    for (size_t i = 0; i < idx.size(); ++i) idx[i] = (int)i;
    if (!idx.empty()) build(0, (int)idx.size(), 0);
  }
  // k nearest (ascending squared distance).
  void knn(const Vec3& q, int k, std::vector<std::pair<double, int>>& out) const {
    out.clear();
    if (idx.empty()) return;
    std::priority_queue<std::pair<double, int>> heap;
    search(0, q, k, heap);
    out.resize(heap.size());
    for (int i = (int)heap.size() - 1; i >= 0; --i) {
      out[i] = heap.top();
      heap.pop();
    }
  }

 private:
  struct Node {
    int lo, hi, left, right, axis;
    double split;
  };
  const std::vector<Vec3>& P;
  std::vector<int> idx;
  std::vector<Node> nodes;

  int build(int lo, int hi, int depth) {
    int id = (int)nodes.size();
    nodes.push_back({lo, hi, -1, -1, 0, 0.0});
    if (hi - lo <= 10) return id;
    double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
    for (int i = lo; i < hi; ++i)
      for (int a = 0; a < 3; ++a) {
        mn[a] = std::min(mn[a], P[idx[i]][a]);
        mx[a] = std::max(mx[a], P[idx[i]][a]);
      }
    int ax = 0;
    for (int a = 1; a < 3; ++a)
      if (mx[a] - mn[a] > mx[ax] - mn[ax]) ax = a;
    int mid = (lo + hi) / 2;
    std::nth_element(idx.begin() + lo, idx.begin() + mid, idx.begin() + hi,
                     [&](int x, int y) { return P[x][ax] < P[y][ax]; });
    nodes[id].axis = ax;
    nodes[id].split = P[idx[mid]][ax];
    int l = build(lo, mid, depth + 1);
    int r = build(mid, hi, depth + 1);
    nodes[id].left = l;
    nodes[id].right = r;
    return id;
  }

  void search(int n, const Vec3& q, int k, std::priority_queue<std::pair<double, int>>& heap) const {
    const Node& nd = nodes[n];
    if (nd.left < 0) {
      for (int i = nd.lo; i < nd.hi; ++i) {
        const Vec3& p = P[idx[i]];
        double d = (p[0] - q[0]) * (p[0] - q[0]) + (p[1] - q[1]) * (p[1] - q[1]) + (p[2] - q[2]) * (p[2] - q[2]);
        if ((int)heap.size() < k) heap.push({d, idx[i]});
        else if (d < heap.top().first) {
          heap.pop();
          heap.push({d, idx[i]});
        }
      }
      return;
    }
    double diff = q[nd.axis] - nd.split;
    int first = diff < 0 ? nd.left : nd.right, second = diff < 0 ? nd.right : nd.left;
    search(first, q, k, heap);
    if ((int)heap.size() < k || diff * diff < heap.top().first) search(second, q, k, heap);
  }
};

// The reference's point-triangle distance (lib/include/hausdorff.hpp:97-212),
// restated with its arithmetic in its order: the plane distance when the
// point's projection passes the barycentric test, else the smallest of the
// three edge distances (Pythagoras on the projection along the edge; +max
// double when the projection falls outside the edge) and the three vertex
// distances, combined by std::min (a NaN operand drops out when it is the
// second one). On proper triangles this is the exact distance up to rounding;
// on degenerate ones (zero area, repeated vertices) the NaNs of the plane
// normal and of 0/0 projections make it differ, and those values decide which
// part the reference splits next, so they are kept as they are.
constexpr double kRefInf = std::numeric_limits<double>::max();
inline double sq(double x) { return x * x; }
inline double ref_min(double a, double b) { return (b < a) ? b : a; }

double ref_point_point(const Vec3& p, const Vec3& q) {
  return std::sqrt(sq(p[0] - q[0]) + sq(p[1] - q[1]) + sq(p[2] - q[2]));
}

double ref_point_segment(const Vec3& p, const Vec3& s0, const Vec3& s1) {
  const double BA0 = p[0] - s1[0], BA1 = p[1] - s1[1], BA2 = p[2] - s1[2];
  const double BC0 = s0[0] - s1[0], BC1 = s0[1] - s1[1], BC2 = s0[2] - s1[2];
  const double proj = (BA0 * BC0 + BA1 * BC1 + BA2 * BC2) / std::sqrt(sq(BC0) + sq(BC1) + sq(BC2));
  const double ab = std::sqrt(sq(BA0) + sq(BA1) + sq(BA2));
  const double bc = std::sqrt(sq(BC0) + sq(BC1) + sq(BC2));
  if (proj < 0 || proj > bc) return kRefInf;
  return std::sqrt(sq(ab) - sq(proj));
}

bool ref_in_triangle(const Vec3& p, const Vec3& t0, const Vec3& t1, const Vec3& t2) {
  const Vec3 v0 = t2 - t0, v1 = t1 - t0, v2 = p - t0;
  const double d00 = v0[0] * v0[0] + v0[1] * v0[1] + v0[2] * v0[2];
  const double d01 = v0[0] * v1[0] + v0[1] * v1[1] + v0[2] * v1[2];
  const double d02 = v0[0] * v2[0] + v0[1] * v2[1] + v0[2] * v2[2];
  const double d11 = v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2];
  const double d12 = v1[0] * v2[0] + v1[1] * v2[1] + v1[2] * v2[2];
  const double inv = 1.0 / (d00 * d11 - d01 * d01);
  const double u = (d11 * d02 - d01 * d12) * inv;
  const double v = (d00 * d12 - d01 * d02) * inv;
  return (u >= 0) && (v >= 0) && (u + v <= 1);
}

}  // namespace

double ref_point_triangle_distance(const Vec3& pt, const Vec3& t0, const Vec3& t1, const Vec3& t2) {
  const double A = (t1[1] - t0[1]) * (t2[2] - t0[2]) - (t1[2] - t0[2]) * (t2[1] - t0[1]);
  const double B = (t1[2] - t0[2]) * (t2[0] - t0[0]) - (t1[0] - t0[0]) * (t2[2] - t0[2]);
  const double C = (t1[0] - t0[0]) * (t2[1] - t0[1]) - (t1[1] - t0[1]) * (t2[0] - t0[0]);
  const double a = A / std::sqrt(sq(A) + sq(B) + sq(C));
  const double b = B / std::sqrt(sq(A) + sq(B) + sq(C));
  const double c = C / std::sqrt(sq(A) + sq(B) + sq(C));
  const double d = 0 - (a * t0[0] + b * t0[1] + c * t0[2]);
  const double dist = std::fabs(a * pt[0] + b * pt[1] + c * pt[2] + d) / std::sqrt(sq(a) + sq(b) + sq(c));
  const double r = pt[0] * a + pt[1] * b + pt[2] * c + d;  // Plane::side(pt, 1e-8)
  Vec3 proj = pt;
  if (r > 1e-8) {
    proj = {pt[0] - a * dist, pt[1] - b * dist, pt[2] - c * dist};
  } else if (r < -1 * 1e-8) {
    proj = {pt[0] + a * dist, pt[1] + b * dist, pt[2] + c * dist};
  }
  if (ref_in_triangle(proj, t0, t1, t2)) return dist;
  const double ab = ref_point_segment(pt, t0, t1), bc = ref_point_segment(pt, t1, t2),
               ca = ref_point_segment(pt, t2, t0);
  const double pa = ref_point_point(pt, t0), pb = ref_point_point(pt, t1), pc = ref_point_point(pt, t2);
  return ref_min(ref_min(ref_min(ab, bc), ca), ref_min(ref_min(pa, pb), pc));
}

namespace {

// One direction of the face Hausdorff distance: for each query sample, the
// smallest distance to the triangles of its 10 nearest samples on the other
// side (lib/include/hausdorff.hpp:236-263).
double directed(const std::vector<Vec3>& Q, const KdTree& tree, const Mesh& other,
                const std::vector<int>& other_ids) {
  double cmax = 0;
#pragma omp parallel
  {
    std::vector<std::pair<double, int>> nn;
    double local = 0;
#pragma omp for schedule(static)
    for (int64_t i = 0; i < (int64_t)Q.size(); ++i) {
      tree.knn(Q[i], 10, nn);
      double cmin = kInf;
      for (const auto& r : nn) {
        const auto& t = other.triangles[other_ids[r.second]];
        double d = ref_point_triangle_distance(Q[i], other.vertices[t[0]], other.vertices[t[1]],
                                               other.vertices[t[2]]);
        if (d < cmin) {
          cmin = d;
          if (cmin < 1e-14) break;
        }
      }
      if (cmin > 10 && !nn.empty()) cmin = std::sqrt(nn[0].first);
      if (cmin > local && kInf > cmin) local = cmin;
    }
#pragma omp critical
    cmax = std::max(cmax, local);
  }
  return cmax;
}

double face_hausdorff(const Mesh& A, const std::vector<Vec3>& XA, const std::vector<int>& idA,
                      const Mesh& B, const std::vector<Vec3>& XB, const std::vector<int>& idB) {
  KdTree ta(XA), tb(XB);
  return std::max(directed(XB, ta, A, idA), directed(XA, tb, B, idB));
}

}  // namespace

double compute_rv(const Mesh& a, const Mesh& b) {
  double v1 = mesh_volume(a), v2 = mesh_volume(b);
  return std::pow(3 * std::fabs(v1 - v2) / (4 * kPi), 1.0 / 3);
}

double compute_rv3(const Mesh& c1, const Mesh& c2, const Mesh& ch) {
  double v1 = mesh_volume(c1), v2 = mesh_volume(c2), v3 = mesh_volume(ch);
  return std::pow(3 * std::fabs(v1 + v2 - v3) / (4 * kPi), 1.0 / 3);
}

void sample_hb(const Mesh& a, const Mesh& b, unsigned int resolution, HbSamples& s) {
  auto& tm = concavity_times();
  const auto t0 = std::chrono::steady_clock::now();
  extract_point_set(a, s.s1, s.i1, resolution, 1, true);
  extract_point_set(b, s.s2, s.i2, resolution, 1, true);
  tm.sample_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  tm.samples += (long long)(s.s1.size() + s.s2.size());
}

double eval_hb(const Mesh& a, const Mesh& b, const HbSamples& s, double floor) {
  if (s.s1.empty() || s.s2.empty()) return kInf;
  auto& tm = concavity_times();
  const auto t0 = std::chrono::steady_clock::now();
  const double h = !checker_hooks().host_concavity ? gpu::face_hausdorff(a, s.s1, s.i1, b, s.s2, s.i2, floor)
                                          : face_hausdorff(a, s.s1, s.i1, b, s.s2, s.i2);
  tm.hausdorff_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  tm.calls++;
  return h;
}

std::vector<double> eval_hb_batch(const std::vector<const Mesh*>& a, const std::vector<const Mesh*>& b,
                                  const std::vector<const HbSamples*>& s, const std::vector<double>& lower,
                                  double floor, bool independent) {
  const size_t J = a.size();
  std::vector<double> out(J, kInf);
  if (checker_hooks().host_concavity) {
    for (size_t j = 0; j < J; ++j) out[j] = eval_hb(*a[j], *b[j], *s[j]);
    return out;
  }
  auto& tm = concavity_times();
  const auto t0 = std::chrono::steady_clock::now();
  // Jobs without samples are kInf (as eval_hb); the rest go in one call, with
  // the floor raised to the kInf concavities when pruning across jobs.
  std::vector<const Mesh*> ga, gb;
  std::vector<const HbSamples*> gs;
  std::vector<double> gl;
  std::vector<size_t> where;
  for (size_t j = 0; j < J; ++j) {
    if (s[j]->s1.empty() || s[j]->s2.empty()) {
      floor = std::max(floor, kInf);
      continue;
    }
    ga.push_back(a[j]);
    gb.push_back(b[j]);
    gs.push_back(s[j]);
    if (!lower.empty()) gl.push_back(lower[j]);
    where.push_back(j);
  }
  if (!where.empty()) {
    const std::vector<double> r = gpu::face_hausdorff_batch(ga, gb, gs, gl, independent ? 0.0 : floor, independent);
    for (size_t k = 0; k < where.size(); ++k) out[where[k]] = r[k];
  }
  tm.hausdorff_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  tm.calls += (long long)where.size();
  return out;
}

double compute_hb(const Mesh& a, const Mesh& b, unsigned int resolution) {
  HbSamples s;
  sample_hb(a, b, resolution, s);
  return eval_hb(a, b, s);
}

ConcavityTimes& concavity_times() {
  static thread_local ConcavityTimes t;
  return t;
}

// Merge cost between two hulls and their joint hull (lib/src/cost.cpp:87-105).
// The reference's hulls keep every input point as a vertex, so the joint hull
// always has as many vertices as the two inputs together and the sampled term
// is zero; the same holds here because convex_hull keeps all input points.
double compute_hb3(const Mesh& c1, const Mesh& c2, const Mesh& ch, unsigned int resolution) {
  if (c1.vertices.size() + c2.vertices.size() == ch.vertices.size()) return 0.0;
  Mesh both = c1;
  const int off = (int)c1.vertices.size();
  both.vertices.insert(both.vertices.end(), c2.vertices.begin(), c2.vertices.end());
  for (auto t : c2.triangles) both.triangles.push_back({t[0] + off, t[1] + off, t[2] + off});
  return compute_hb(both, ch, resolution);
}

double compute_h(const Mesh& a, const Mesh& b, double k, unsigned int resolution) {
  double h1 = compute_rv(a, b);
  double h2 = compute_hb(a, b, resolution);
  return std::max(h1 * k, h2);
}

double compute_h3(const Mesh& c1, const Mesh& c2, const Mesh& ch, double k, unsigned int resolution) {
  double h1 = compute_rv3(c1, c2, ch);
  double h2 = compute_hb3(c1, c2, ch, resolution + 2000);
  return std::max(h1 * k, h2);
}

double mesh_dist(const Mesh& a, const Mesh& b) {
  if (a.vertices.empty() || b.vertices.empty()) return kInf;
  KdTree tb(b.vertices);
  double best = kInf;
  std::vector<std::pair<double, int>> nn;
  for (const auto& v : a.vertices) {
    tb.knn(v, 1, nn);
    best = std::min(best, std::sqrt(nn[0].first));
  }
  return best;
}

}  // namespace visacd

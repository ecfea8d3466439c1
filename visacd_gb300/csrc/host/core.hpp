// Host data model of the decomposition driver.
//
// Mirrors the reference's data types (lib/include/core.hpp:18-64,
// lib/include/config.hpp:7-30): a triangle mesh with float64 vertices and
// int32 triangles, per-vertex "new" flags set by clipping, and the part's
// visibility edges (i < j); planes a x + b y + c z + d = 0 with the 1e-6 side
// test; a process-wide configuration and random engine.
#pragma once

#include <array>
#include <cmath>
#include <cstdint>
#include <limits>
#include <random>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace visacd {

using Vec3 = std::array<double, 3>;
using Tri = std::array<int, 3>;
using Edge = std::pair<unsigned int, unsigned int>;

constexpr double kInf = std::numeric_limits<double>::max();

inline Vec3 operator+(const Vec3& a, const Vec3& b) { return {a[0] + b[0], a[1] + b[1], a[2] + b[2]}; }
inline Vec3 operator-(const Vec3& a, const Vec3& b) { return {a[0] - b[0], a[1] - b[1], a[2] - b[2]}; }
inline Vec3 operator*(const Vec3& a, double s) { return {a[0] * s, a[1] * s, a[2] * s}; }
inline Vec3 operator/(const Vec3& a, double s) {
  if (s == 0) throw std::runtime_error("division of a vector by zero");
  return {a[0] / s, a[1] / s, a[2] / s};
}
inline double dot(const Vec3& a, const Vec3& b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
inline Vec3 cross(const Vec3& a, const Vec3& b) {
  return {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
}
inline double norm(const Vec3& a) { return std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); }
inline Vec3 normalized(const Vec3& a) {
  double l = norm(a);
  if (l == 0) throw std::runtime_error("cannot normalise a zero-length vector");
  return {a[0] / l, a[1] / l, a[2] / l};
}

// Unit normal of a triangle (lib/include/core.hpp:148-167 formula order).
Vec3 face_normal(const Vec3& p1, const Vec3& p2, const Vec3& p3);
// Triangle area (lib/include/core.hpp:124-137 formula order).
double triangle_area(const Vec3& p0, const Vec3& p1, const Vec3& p2);

struct Plane {
  double a = 0, b = 0, c = 0, d = 0;
  Plane() = default;
  Plane(double a_, double b_, double c_, double d_) : a(a_), b(b_), c(c_), d(d_) {}
  double eval(const Vec3& p) const { return p[0] * a + p[1] * b + p[2] * c + d; }
  // +1 / -1 beyond eps, else 0 (lib/include/core.hpp:178-185).
  int side(const Vec3& p, double eps = 1e-6) const {
    double r = eval(p);
    if (r > eps) return 1;
    if (r < -eps) return -1;
    return 0;
  }
};

struct Mesh {
  std::vector<Vec3> vertices;
  std::vector<Tri> triangles;
  std::vector<bool> is_new;
  std::vector<Edge> intersecting_edges;

  void clear() {
    vertices.clear();
    triangles.clear();
  }
  // Geometry only (lib/src/core.cpp:247-254 copies vertices and triangles).
  Mesh copy_geometry() const {
    Mesh m;
    m.vertices = vertices;
    m.triangles = triangles;
    return m;
  }
};
using MeshList = std::vector<Mesh>;

struct Config {
  bool return_parts = false;
  std::string score_mode = "concavity";  // or "edge"
  double flat_surface_min_area = 0.1;
  bool use_flat_surfaces = true;
  double flat_surface_k = 2.0;
  bool use_merging = false;
  // Additions of this implementation (not in the reference's Config).
  bool verbose = true;   // the "[visacd] ..." progress lines
  // Split-plane search: "exhaustive" (the reference's random candidate draw)
  // or "learned" (16 planes from the learned proposer plus a probe of
  // `proposer_probe_planes` random candidates; when the best proposal scores
  // more than `proposer_tolerance` below the probe's best, the split falls back
  // to the full candidate draw).
  std::string plane_proposer = "exhaustive";
  std::string proposer_weights;  // float32 parameter file of the proposer
  int proposer_probe_planes = 64;
  int proposer_refine = 32;  // bisector planes kept per proposal in the refinement (0..32)
  double proposer_tolerance = 0.01;
};

Config& config();

// Test hooks, not part of the user-visible configuration: each routes one
// stage through the host restatement that its GPU kernels are checked
// against (the tests compare the two, and run host-only checks on machines
// without a GPU). Off by default; the product path is the GPU kernels.
struct CheckerHooks {
  bool host_clip = false;        // host clip instead of the GPU clip kernels
  bool host_concavity = false;   // host Hausdorff term of the concavity metric
  bool host_remesh = false;      // host SDF remesh (manifold and cages)
  bool host_merge = false;       // host hull-pair distances in hull merging
  bool host_hull = false;        // host QuickHull instead of visacd_convex_hulls
  bool record_visibility = false;  // keep every visibility call and split search
};
CheckerHooks& checker_hooks();

// Visibility calls recorded while checker_hooks().record_visibility is on.
struct VisibilityRecord {
  Mesh part, cage;  // part with is_new and the edges found for it
};
std::vector<VisibilityRecord>& recorded_visibility();
// Split searches recorded alongside: (planes scored, points, edges, index of
// the chosen plane, its float score).
std::vector<std::array<double, 5>>& recorded_splits();

// The 32-bit Mersenne Twister MT19937 (Matsumoto and Nishimura, 1998) with the
// parameters and seeding std::mt19937 is defined with, so the same seed gives
// the same output sequence (the engine of lib/src/core.cpp:27). A class of its
// own so that many outputs can be taken in one call (fill), which the sampling
// loops use; it meets the uniform random bit generator requirements, so the
// standard distributions draw from it exactly as from std::mt19937.
class Mt19937 {
 public:
  using result_type = uint32_t;
  static constexpr result_type min() { return 0u; }
  static constexpr result_type max() { return 0xffffffffu; }
  explicit Mt19937(result_type s = 5489u) { seed(s); }
  void seed(result_type s);
  result_type operator()() {
    if (pos_ >= kN) twist();
    return out_[pos_++];
  }
  // The next n outputs, in order.
  void fill(uint32_t* out, size_t n);

 private:
  static constexpr int kN = 624, kM = 397;
  static uint32_t temper(uint32_t y) {
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    return y ^ (y >> 18);
  }
  void twist();
  uint32_t x_[kN];
  uint32_t out_[kN];  // the current block's outputs (tempered state)
  int pos_ = kN;
};

// std::generate_canonical<double, 53> of two successive outputs (lo, hi) of a
// 32-bit engine: (lo + hi 2^32) / 2^64 with the sum rounded to double, and the
// largest double below 1 in place of 1.
inline double canonical53(uint32_t lo, uint32_t hi) {
  const double r = ((double)lo + (double)hi * 0x1p32) * 0x1p-64;
  return r < 1.0 ? r : 0x1.fffffffffffffp-1;
}

// Surface samples of a pair of meshes for the concavity metric (points and the
// triangle each was drawn from).
struct HbSamples {
  std::vector<Vec3> s1, s2;
  std::vector<int> i1, i2;
};

// The process-wide engine, or the calling thread's own one while a
// process_batch worker has installed it (set_thread_engine(nullptr) clears).
Mt19937& random_engine();
void set_thread_engine(Mt19937* eng);
void set_seed(unsigned int seed);

// Bounding box (xmin, xmax, ymin, ymax, zmin, zmax).
std::array<double, 6> bbox(const Mesh& m);
// Map to [-1, 1] along the longest axis; returns the original bbox
// (lib/src/core.cpp:262-291).
std::array<double, 6> normalize(Mesh& m);
void unnormalize(Mesh& m, const std::array<double, 6>& box);  // core.cpp:293-307

// Signed volume (lib/src/cost.cpp:24-43 term order).
double mesh_volume(const Mesh& m);

}  // namespace visacd

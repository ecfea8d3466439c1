// Product-side half of the reference harness (compiled with this project's
// host include path): the stand-in implementations the reference's sources
// call for their absent third-party libraries, in plain arrays so the
// reference-side half (ref_shim.cpp) needs none of this project's headers.
// TEST INFRASTRUCTURE ONLY (built into oracle/_ref).
#include <array>
#include <vector>

#include "geometry.hpp"

namespace visacd {

// qhull stand-in: facets of this project's hull (orientation is fixed later by
// the reference's own cvx_fix_normals).
std::vector<std::array<int, 3>> hull_facets_for_ref(const std::vector<double>& coords) {
  std::vector<Vec3> pts(coords.size() / 3);
  for (size_t i = 0; i < pts.size(); ++i) pts[i] = {coords[3 * i], coords[3 * i + 1], coords[3 * i + 2]};
  Mesh h = convex_hull(pts, false);
  return std::vector<std::array<int, 3>>(h.triangles.begin(), h.triangles.end());
}

// OpenVDB stand-in: this project's SDF remesh (host restatement; the GPU
// kernels produce the same mesh).
void remesh_for_ref(const std::vector<double>& v, const std::vector<int>& t, double scale,
                    double level, std::vector<double>& ov, std::vector<int>& ot) {
  Mesh m;
  m.vertices.resize(v.size() / 3);
  for (size_t i = 0; i < m.vertices.size(); ++i) m.vertices[i] = {v[3 * i], v[3 * i + 1], v[3 * i + 2]};
  m.triangles.resize(t.size() / 3);
  for (size_t i = 0; i < m.triangles.size(); ++i) m.triangles[i] = {t[3 * i], t[3 * i + 1], t[3 * i + 2]};
  manifold_preprocess_host(m, scale, level);
  ov.clear();
  ot.clear();
  for (auto& p : m.vertices) ov.insert(ov.end(), p.begin(), p.end());
  for (auto& q : m.triangles) ot.insert(ot.end(), q.begin(), q.end());
}

}  // namespace visacd

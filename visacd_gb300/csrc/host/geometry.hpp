// Host geometry of the decomposition driver (CPU, C++): the parts of VisACD's
// pipeline around the GPU hot path.
#pragma once

#include <vector>

#include "core.hpp"

namespace visacd {

// ---- remesh.cpp: SDF remeshing (replaces lib/src/preprocess.cpp:18-67) ----
void manifold_preprocess(Mesh& m, double scale, double level);
// The host restatement, which manifold_preprocess runs only under the test hook
// checker_hooks().host_remesh (the GPU path, visacd_sdf_remesh, produces the
// same mesh bit for bit).
void manifold_preprocess_host(Mesh& m, double scale, double level);
Vec3 closest_point_on_triangle(const Vec3& p, const Vec3& a, const Vec3& b, const Vec3& c);
double point_triangle_distance(const Vec3& p, const Vec3& a, const Vec3& b, const Vec3& c);
// The reference's distance of the concavity metric (hausdorff.hpp:156-212):
// equal to point_triangle_distance up to rounding on proper triangles, not on
// degenerate ones (see cost.cpp).
double ref_point_triangle_distance(const Vec3& pt, const Vec3& t0, const Vec3& t1, const Vec3& t2);

// ---- hull.cpp: convex hull (replaces qhull "Qt Pp", lib/src/core.cpp:59-111).
// As with qhull, the hull mesh keeps every input point as a vertex (interior
// ones unreferenced) and triangulates the hull facets. fix_normals orients
// every facet away from the vertex centroid (lib/src/core.cpp:33-57).
Mesh convex_hull(const std::vector<Vec3>& pts, bool fix_normals = true);

// ---- clip.cpp: split a mesh by a plane (lib/src/clip.cpp:190-741).
// Returns {pos, neg} (or {mesh} when a side is empty); pos_map/neg_map give,
// for every input vertex, its 1-based index in pos/neg (0 = absent). Border
// vertices are appended to both parts and flagged is_new.
MeshList clip(const Mesh& mesh, const Plane& plane, std::vector<int>& pos_map,
              std::vector<int>& neg_map);

// Same parts from the GPU clip's outputs (part-local triangles without the
// cap, 1-based maps, border points, 1-based border edges); the cap is
// triangulated here.
MeshList assemble_clip(const Mesh& mesh, const Plane& plane, const std::vector<Tri>& pos_tris,
                       const std::vector<Tri>& neg_tris, const std::vector<int>& pos_map,
                       const std::vector<int>& neg_map, const std::vector<Vec3>& border,
                       const std::vector<std::pair<int, int>>& bedges);

// ---- cap2d.cpp: triangulation of the region a planar border graph encloses
// (stand-in for CDT's insertVertices/insertEdges/eraseOuterTrianglesAndHoles).
// xy: 2 doubles per point; edges 0-based; triangles CCW. False if nothing closed.
bool triangulate_border_2d(const std::vector<double>& xy, const std::vector<std::pair<int, int>>& edges,
                           std::vector<Tri>& tris);

// ---- cost.cpp: concavity metric (lib/src/cost.cpp, lib/include/hausdorff.hpp).
void extract_point_set(const Mesh& m, std::vector<Vec3>& samples, std::vector<int>& tri_ids,
                       size_t resolution, double base, bool one_per_tri);
double compute_rv(const Mesh& a, const Mesh& b);
double compute_rv3(const Mesh& c1, const Mesh& c2, const Mesh& ch);
double compute_hb(const Mesh& a, const Mesh& b, unsigned int resolution);
// compute_hb in two steps: the samples of both surfaces (the random draws, in
// the reference's order), then the value. With floor > 0 the value is exact
// when it is >= floor and some value below floor otherwise (the GPU skips the
// sample terms that cannot reach floor); the host metric is always exact.
void sample_hb(const Mesh& a, const Mesh& b, unsigned int resolution, HbSamples& s);
double eval_hb(const Mesh& a, const Mesh& b, const HbSamples& s, double floor = 0.0);
// eval_hb of many pairs in one GPU call: job j is (a[j], b[j], s[j]). With
// `independent` every value is exact; otherwise, with lower[j] a known lower
// bound of job j's concavity and M the largest of floor and every
// max(lower[j], value[j]), the jobs whose value equals M get it exactly and the
// others some value not above theirs (the host metric is always exact).
std::vector<double> eval_hb_batch(const std::vector<const Mesh*>& a, const std::vector<const Mesh*>& b,
                                  const std::vector<const HbSamples*>& s, const std::vector<double>& lower,
                                  double floor, bool independent);
double compute_hb3(const Mesh& c1, const Mesh& c2, const Mesh& ch, unsigned int resolution);
double compute_h(const Mesh& a, const Mesh& b, double k, unsigned int resolution);
double compute_h3(const Mesh& c1, const Mesh& c2, const Mesh& ch, double k, unsigned int resolution);
double mesh_dist(const Mesh& a, const Mesh& b);

// Per-thread time split of the concavity metric (ms) for benchmarks.
struct ConcavityTimes {
  double sample_ms = 0, hausdorff_ms = 0, hull_ms = 0;
  long long samples = 0, calls = 0;
};
ConcavityTimes& concavity_times();

// ---- surfaces.cpp: flat-surface planes (lib/src/support_surface.cpp:14-183).
struct Surface {
  std::vector<int> triangle_ids;
  double area = 0.0;
  Plane plane;
};
std::vector<Surface> extract_surfaces(const Mesh& mesh, double min_area);

// ---- postprocess.cpp (lib/src/postprocess.cpp) ----
void separate_disjoint(MeshList& parts);
void multimerge_ch(MeshList& meshes, MeshList& hulls, double current_concavity, double threshold);

}  // namespace visacd

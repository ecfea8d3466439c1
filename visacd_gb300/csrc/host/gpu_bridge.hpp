// The host driver's calls into the sm_103a kernels (C ABI, include/visacd_gpu.h).
// Any non-zero status becomes std::runtime_error (RuntimeError in Python).
#pragma once

#include <vector>

#include "core.hpp"

struct visacd_ctx;

namespace visacd {
namespace gpu {

// Process-wide context on device VISACD_DEVICE (default 0), created on first use.
visacd_ctx* context();

// compute_intersection_matrix(mesh, cage) of lib/src/intersections.cpp:327-385:
// pairs with a new endpoint when mesh.is_new is non-empty, else all pairs.
std::vector<Edge> visibility_edges(const Mesh& mesh, const Mesh& cage);

// Plane scores (float64, exact crossing classification) and the first argmax.
std::vector<double> score_planes(const std::vector<Plane>& planes, const std::vector<Vec3>& pts,
                                 const std::vector<Edge>& edges);

// Per-part clipping on the GPU (visacd_clip) + host cap: same parts and maps
// as clip() in clip.cpp.
MeshList clip(const Mesh& mesh, const Plane& plane, std::vector<int>& pos_map,
              std::vector<int>& neg_map);

// Sampled face Hausdorff distance on the GPU (visacd_face_hausdorff).
double face_hausdorff(const Mesh& A, const std::vector<Vec3>& XA, const std::vector<int>& idA,
                      const Mesh& B, const std::vector<Vec3>& XB, const std::vector<int>& idB);

struct Counters {
  long long vis_calls = 0, vis_pairs = 0, vis_edges = 0, score_calls = 0, plane_edge_pairs = 0;
  double vis_ms = 0, score_ms = 0;
};
Counters& counters();

}  // namespace gpu
}  // namespace visacd

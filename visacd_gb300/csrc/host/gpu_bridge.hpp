// The host driver's calls into the sm_103a kernels (C ABI, include/visacd_gpu.h).
// Any non-zero status becomes std::runtime_error (RuntimeError in Python).
#pragma once

#include <vector>

#include "core.hpp"

struct visacd_ctx;

namespace visacd {
namespace gpu {

// The calling thread's context: a ThreadContext installed on this thread, else
// the process-wide context on device VISACD_DEVICE (default 0), created on
// first use.
visacd_ctx* context();
int default_device();

// A context (own stream and buffers) for the lifetime of the object, used by
// context() on the creating thread; process_batch workers hold one each.
class ThreadContext {
 public:
  // blocking_wait: the context's waits sleep instead of spinning (many
  // workers sharing the host cores).
  explicit ThreadContext(int device, bool blocking_wait = false);
  ~ThreadContext();
  ThreadContext(const ThreadContext&) = delete;
  ThreadContext& operator=(const ThreadContext&) = delete;

 private:
  visacd_ctx* ctx_ = nullptr;
  visacd_ctx* prev_ = nullptr;
};

// The learned proposer's 16 planes for a part with visibility edges, in the
// part's own coordinates (network inputs are taken in the part's bounding-box
// frame; parameters from config().proposer_weights).
std::vector<Plane> propose_planes(const Mesh& mesh);

// The learned split search in one GPU call (visacd_learned_split_search): the
// proposer's planes, their refinement by nearby bisector planes
// (config().proposer_refine per proposal), a probe of
// config().proposer_probe_planes candidates drawn from the process engine, and
// the flat planes (scores times flat_k), scored together. fallback is set when
// the proposals score more than config().proposer_tolerance below the probe's
// best: the caller then runs the full search. Returns true with the first
// maximum otherwise.
bool learned_split_search(const Mesh& mesh, const std::vector<Plane>& flat_planes, double flat_k, Plane& out,
                          bool& fallback);

// compute_intersection_matrix(mesh, cage) of lib/src/intersections.cpp:327-385:
// pairs with a new endpoint when mesh.is_new is non-empty, else all pairs.
std::vector<Edge> visibility_edges(const Mesh& mesh, const Mesh& cage);

// visibility_edges of several parts in one GPU call (visacd_visibility_batch:
// per-part preparation, one persistent visibility launch over all parts, one
// compaction). Part k is traced against cages[k]; same edges as one
// visibility_edges call per part.
std::vector<std::vector<Edge>> visibility_edges_batch(const std::vector<const Mesh*>& parts,
                                                      const std::vector<const Mesh*>& cages);

// Plane scores (float64, exact crossing classification) and the first argmax.
std::vector<double> score_planes(const std::vector<Plane>& planes, const std::vector<Vec3>& pts,
                                 const std::vector<Edge>& edges);

// get_candidate_planes (lib/src/process.cpp:28-72) with the planes and their
// near-duplicate filter on the GPU (visacd_candidate_planes): the edge draws
// come from the process engine, which ends where the reference's loop leaves
// it. Same planes, in the same order, as the host restatement.
std::vector<Plane> candidate_planes(const std::vector<Vec3>& vertices, const std::vector<Edge>& edges,
                                    int num_planes);

// The split search of lib/src/process.cpp:96-134 on the GPU
// (visacd_split_search): num_planes candidate planes, then the flat planes
// with scores times flat_k; the first maximum. False when nothing is scored.
bool split_search(const Mesh& mesh, const std::vector<Plane>& flat_planes, double flat_k,
                  int num_planes, Plane& out);

// Per-part clipping on the GPU (visacd_clip) + host cap: same parts and maps
// as clip() in clip.cpp.
MeshList clip(const Mesh& mesh, const Plane& plane, std::vector<int>& pos_map,
              std::vector<int>& neg_map);

// SDF remesh on the GPU (visacd_sdf_remesh): replaces m by the iso-surface at
// `level` outside it, on voxels of size 1/scale; same mesh as the host's
// manifold_preprocess_host.
void sdf_remesh(Mesh& m, double scale, double level);

// Convex hulls of many point sets in one launch (visacd_convex_hulls): the
// same meshes as convex_hull(*sets[k], fix_normals), every input point a vertex.
MeshList convex_hulls(const std::vector<const std::vector<Vec3>*>& sets, bool fix_normals);

// mesh_dist of hull pairs on the GPU (visacd_hull_distances); DBL_MAX where the
// bounding boxes are farther apart than cutoff.
std::vector<double> hull_distances(const MeshList& hulls, const std::vector<std::pair<int, int>>& pairs,
                                   double cutoff);

// Sampled face Hausdorff distance on the GPU (visacd_face_hausdorff_floor):
// exact when it is >= floor, otherwise some value below floor.
double face_hausdorff(const Mesh& A, const std::vector<Vec3>& XA, const std::vector<int>& idA,
                      const Mesh& B, const std::vector<Vec3>& XB, const std::vector<int>& idB,
                      double floor = 0.0);

// Face Hausdorff distances of many surface pairs in one call
// (visacd_face_hausdorff_batch): job j compares *a[j] (samples s[j]->s1 / i1)
// with *b[j] (s[j]->s2 / i2); lower, floor and independent as there.
std::vector<double> face_hausdorff_batch(const std::vector<const Mesh*>& a, const std::vector<const Mesh*>& b,
                                         const std::vector<const HbSamples*>& s, const std::vector<double>& lower,
                                         double floor, bool independent);

// Per-thread call counters.
struct Counters {
  long long vis_calls = 0, vis_pairs = 0, vis_edges = 0, score_calls = 0, plane_edge_pairs = 0;
  long long lp_calls = 0, lp_fallbacks = 0;
  double vis_ms = 0, score_ms = 0, lp_ms = 0;
};
Counters& counters();

}  // namespace gpu
}  // namespace visacd

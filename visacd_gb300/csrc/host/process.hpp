// Decomposition driver: visacd.process(mesh, concavity, num_parts).
#pragma once

#include <vector>

#include "core.hpp"
#include "geometry.hpp"

namespace visacd {

struct ProcessResult {
  MeshList parts;
  double concavity = 0;
  int num_parts = 0;
};

// lib/src/process.cpp:28-72.
std::vector<Plane> get_candidate_planes(const std::vector<Vec3>& vertices,
                                        const std::vector<Edge>& edges, int num_planes);

// lib/src/process.cpp:82-181: one split of `mesh`; returns true when there is
// nothing left to cut (no candidate planes or no visibility edges).
bool decompose_iteration(Mesh& mesh, MeshList& parts, Mesh& cage,
                         const std::vector<Plane>& flat_planes);

// The learned search's refinement on the host: for each proposal, the
// perpendicular-bisector planes of the `per` visibility edges nearest to it
// under the proposer's training distance, in edge order, each edge once. The
// split search runs it on the GPU (visacd_learned_split_search); this
// statement is what tests check that against.
std::vector<Plane> refine_proposals(const Mesh& mesh, const std::vector<Plane>& prop, int per);

double compute_part_score(const Mesh& part);
int get_part_with_highest_score(const MeshList& parts);
// Convex hulls of the parts kept from one iteration to the next (a hull
// depends on the part's vertices alone and draws no random numbers): entry i
// belongs to parts[i] while valid[i]; process() erases the entry of the part
// it splits, and entries past the end are built when needed.
struct HullCache {
  MeshList hulls;
  std::vector<char> valid;
  void erase(size_t i) {
    if (i < hulls.size()) {
      hulls.erase(hulls.begin() + (long)i);
      valid.erase(valid.begin() + (long)i);
    }
  }
  // Hulls of all parts: cached ones kept, missing ones built in parallel.
  const MeshList& update(const MeshList& parts);
};

int get_part_with_highest_concavity(const MeshList& parts, double& max_concavity, HullCache* cache = nullptr);
double compute_final_concavity(const MeshList& parts, const MeshList& hulls);

// lib/src/process.cpp:238-347.
ProcessResult process(Mesh mesh, double concavity, int num_parts);

// Many meshes decomposed concurrently (no counterpart in the reference, whose
// process() takes one mesh): `threads` workers (0 = all hardware threads), each
// with its own GPU context and stream, pull meshes from a shared counter. Mesh i
// runs with its own engine (the std::mt19937 sequence) seeded with seeds[i], so its result equals
// set_seed(seeds[i]); process(meshes[i], concavity, num_parts) whatever the
// thread count or order. Worker threads do not log.
std::vector<ProcessResult> process_batch(const MeshList& meshes, double concavity, int num_parts,
                                         const std::vector<unsigned int>& seeds, int threads);

// Per-stage wall time of the last process() call (ms), for benchmarks; after
// process_batch, the sums over all its meshes (thread-seconds, not wall time).
struct StageTimes {
  double preprocess = 0, visibility = 0, scoring = 0, clip = 0, concavity = 0, cages = 0,
         hulls = 0, total = 0;
  int iterations = 0;
};
const StageTimes& last_stage_times();

}  // namespace visacd

// Reference-side half of the reference harness (oracle/_ref): the VisACD host
// sources compiled in place (lib/src/{clip,core,cost,postprocess,process,
// support_surface}.cpp), linked to
//  * compute_intersection_matrix  -> the FP64 oracle visibility (same
//    semantics and end-vertex policy as the GPU kernel), replacing OptiX;
//  * classify_and_rate_planes     -> the oracle's exact scoring, as float;
//  * manifold_preprocess          -> this project's SDF remesh (OpenVDB absent);
//  * CDT / qhull                  -> this project's cap triangulation / hull.
// Everything else — clipping, border dedup, flat surfaces, components, the
// concavity metric with its sampling and kd-tree, candidate planes, the
// decomposition loop and its use of the random engine — is the reference's
// own code. C entry points for the tests. TEST INFRASTRUCTURE ONLY.
#include <clip.hpp>
#include <config.hpp>
#include <core.hpp>
#include <cost.hpp>
#include <intersections.hpp>
#include <postprocess.hpp>
#include <preprocess.hpp>
#include <process.hpp>
#include <support_surface.hpp>

#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

extern "C" {
int64_t oracle_visibility(const float* pts, int32_t n, const uint8_t* is_new, const uint32_t* tris,
                          int32_t nt, const float* cage_v, int32_t ncv, const uint32_t* cage_t,
                          int32_t nct, int use_bvh, int32_t row_begin, int32_t row_end,
                          uint8_t* out_bits, int64_t* n_grazing, int64_t* n_pairs);
int oracle_score_planes(const float* planes, int32_t P, const float* pts, int32_t N,
                        const uint32_t* edges, int64_t E, double* scores_fp64, uint64_t* q_scores,
                        int32_t* qexp_out, int64_t* skipped_out);
}

namespace visacd {
void remesh_for_ref(const std::vector<double>& v, const std::vector<int>& t, double scale,
                    double level, std::vector<double>& ov, std::vector<int>& ot);
}

namespace neural_acd {

std::vector<std::pair<unsigned int, unsigned int>> compute_intersection_matrix(
    Mesh& mesh, Mesh& cage, OptixDeviceContext&) {
  const int n = (int)mesh.vertices.size();
  std::vector<float> v(3 * n), cv(3 * cage.vertices.size());
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) v[3 * i + k] = (float)mesh.vertices[i][k];
  for (size_t i = 0; i < cage.vertices.size(); ++i)
    for (int k = 0; k < 3; ++k) cv[3 * i + k] = (float)cage.vertices[i][k];
  std::vector<uint8_t> mask;
  if (!mesh.is_new.empty()) {
    mask.assign(n, 0);
    for (int i = 0; i < n && i < (int)mesh.is_new.size(); ++i) mask[i] = mesh.is_new[i];
  }
  const int64_t np = (int64_t)n * (n - 1) / 2;
  std::vector<uint8_t> bits((size_t)std::max<int64_t>(np, 1));
  int64_t ng = 0, npr = 0;
  oracle_visibility(v.data(), n, mask.empty() ? nullptr : mask.data(),
                    reinterpret_cast<const uint32_t*>(mesh.triangles.data()), (int32_t)mesh.triangles.size(),
                    cv.data(), (int32_t)cage.vertices.size(),
                    reinterpret_cast<const uint32_t*>(cage.triangles.data()), (int32_t)cage.triangles.size(),
                    1, 0, n, bits.data(), &ng, &npr);
  std::vector<std::pair<unsigned int, unsigned int>> out;
  int64_t k = 0;
  for (int i = 0; i < n; ++i)
    for (int j = i + 1; j < n; ++j, ++k)
      if (bits[k] & 1) out.push_back({(unsigned)i, (unsigned)j});
  return out;
}

void manifold_preprocess(Mesh& m, double scale, double level_set) {
  std::vector<double> v, ov;
  std::vector<int> t, ot;
  for (auto& p : m.vertices) v.insert(v.end(), p.begin(), p.end());
  for (auto& q : m.triangles) t.insert(t.end(), q.begin(), q.end());
  visacd::remesh_for_ref(v, t, scale, level_set, ov, ot);
  m.clear();
  for (size_t i = 0; i + 2 < ov.size(); i += 3) m.vertices.push_back({ov[i], ov[i + 1], ov[i + 2]});
  for (size_t i = 0; i + 2 < ot.size(); i += 3) m.triangles.push_back({ot[i], ot[i + 1], ot[i + 2]});
}

std::vector<Plane> get_candidate_planes(std::vector<Vec3D>& vertices,
                                        std::vector<std::pair<unsigned int, unsigned int>>& edges,
                                        int num_planes);
}  // namespace neural_acd

static std::vector<std::array<double, 5>> g_score_trace;

extern "C" void classify_and_rate_planes(const float* planes, const float* points,
                                         const unsigned int* edges, float* scores, int numPlanes,
                                         int numPoints, int numEdges) {
  std::vector<uint64_t> q(numPlanes > 0 ? numPlanes : 1);
  int32_t qexp = 0;
  int64_t sk = 0;
  oracle_score_planes(planes, numPlanes, points, numPoints, edges, numEdges, nullptr, q.data(), &qexp, &sk);
  for (int p = 0; p < numPlanes; ++p) scores[p] = (float)std::ldexp((double)q[p], qexp);
  // Trace of the split searches (size and first float maximum), for tests.
  int best = 0;
  for (int p = 1; p < numPlanes; ++p)
    if (scores[p] > scores[best]) best = p;
  g_score_trace.push_back({(double)numPlanes, (double)numPoints, (double)numEdges, (double)best,
                           numPlanes > 0 ? (double)scores[best] : 0.0});
}

// ---- C entry points for the tests -----------------------------------------
using neural_acd::Mesh;
static std::vector<Mesh> g_parts;
static std::vector<int> g_map1, g_map2;

static Mesh make_mesh(const double* v, int nv, const int* t, int nt) {
  Mesh m;
  for (int i = 0; i < nv; ++i) m.vertices.push_back({v[3 * i], v[3 * i + 1], v[3 * i + 2]});
  for (int i = 0; i < nt; ++i) m.triangles.push_back({t[3 * i], t[3 * i + 1], t[3 * i + 2]});
  return m;
}

extern "C" {

int ref_part_count(void) { return (int)g_parts.size(); }

// The split searches since the last call: rows of (planes, points, edges,
// first maximum, its float score); returns the count and clears the trace.
int ref_score_trace(double* out, int cap) {
  const int n = (int)g_score_trace.size();
  for (int i = 0; i < n && i < cap; ++i)
    for (int k = 0; k < 5; ++k) out[5 * i + k] = g_score_trace[i][k];
  g_score_trace.clear();
  return n;
}
int ref_part_sizes(int i, int* nv, int* nt, int* nedges) {
  if (i < 0 || i >= (int)g_parts.size()) return -1;
  *nv = (int)g_parts[i].vertices.size();
  *nt = (int)g_parts[i].triangles.size();
  *nedges = (int)g_parts[i].intersecting_edges.size();
  return 0;
}
int ref_get_part(int i, double* v, int* t, uint8_t* is_new, uint32_t* edges) {
  if (i < 0 || i >= (int)g_parts.size()) return -1;
  const Mesh& m = g_parts[i];
  for (size_t k = 0; k < m.vertices.size(); ++k)
    for (int a = 0; a < 3; ++a) v[3 * k + a] = m.vertices[k][a];
  for (size_t k = 0; k < m.triangles.size(); ++k)
    for (int a = 0; a < 3; ++a) t[3 * k + a] = m.triangles[k][a];
  if (is_new)
    for (size_t k = 0; k < m.vertices.size(); ++k) is_new[k] = k < m.is_new.size() ? m.is_new[k] : 0;
  if (edges)
    for (size_t k = 0; k < m.intersecting_edges.size(); ++k) {
      edges[2 * k] = m.intersecting_edges[k].first;
      edges[2 * k + 1] = m.intersecting_edges[k].second;
    }
  return 0;
}
void ref_get_maps(int* m1, int* m2) {
  std::memcpy(m1, g_map1.data(), g_map1.size() * sizeof(int));
  std::memcpy(m2, g_map2.data(), g_map2.size() * sizeof(int));
}

void ref_set_seed(unsigned int seed) { neural_acd::set_seed(seed); }

// lib/src/clip.cpp:190 clip(mesh, plane) -> parts + 1-based maps.
int ref_clip(const double* v, int nv, const int* t, int nt, const double* plane) {
  Mesh m = make_mesh(v, nv, t, nt);
  neural_acd::Plane pl(plane[0], plane[1], plane[2], plane[3]);
  int *m1 = nullptr, *m2 = nullptr;
  g_parts = neural_acd::clip(m, pl, m1, m2);
  g_map1.assign(m1, m1 + nv);
  g_map2.assign(m2, m2 + nv);
  delete[] m1;
  delete[] m2;
  return (int)g_parts.size();
}

int ref_separate_disjoint(const double* v, int nv, const int* t, int nt) {
  g_parts.clear();
  g_parts.push_back(make_mesh(v, nv, t, nt));
  neural_acd::separate_disjoint(g_parts);
  return (int)g_parts.size();
}

int ref_extract_surfaces(const double* v, int nv, const int* t, int nt, double min_area,
                         double* planes, double* areas, int cap) {
  Mesh m = make_mesh(v, nv, t, nt);
  auto s = neural_acd::extract_surfaces(m, min_area);
  for (int i = 0; i < (int)s.size() && i < cap; ++i) {
    planes[4 * i] = s[i].plane.a;
    planes[4 * i + 1] = s[i].plane.b;
    planes[4 * i + 2] = s[i].plane.c;
    planes[4 * i + 3] = s[i].plane.d;
    areas[i] = s[i].area;
  }
  return (int)s.size();
}

int ref_candidate_planes(const double* v, int nv, const uint32_t* e, int ne, int num,
                         double* out) {
  std::vector<neural_acd::Vec3D> verts;
  for (int i = 0; i < nv; ++i) verts.push_back({v[3 * i], v[3 * i + 1], v[3 * i + 2]});
  std::vector<std::pair<unsigned int, unsigned int>> edges;
  for (int i = 0; i < ne; ++i) edges.push_back({e[2 * i], e[2 * i + 1]});
  auto p = neural_acd::get_candidate_planes(verts, edges, num);
  for (size_t i = 0; i < p.size(); ++i) {
    out[4 * i] = p[i].a;
    out[4 * i + 1] = p[i].b;
    out[4 * i + 2] = p[i].c;
    out[4 * i + 3] = p[i].d;
  }
  return (int)p.size();
}

// compute_ch(fix_normals) then compute_h(mesh, hull, k, resolution, 42)
// (lib/src/process.cpp:208-226 per part).
double ref_compute_h(const double* v, int nv, const int* t, int nt, double k, unsigned res) {
  Mesh m = make_mesh(v, nv, t, nt);
  Mesh h;
  m.compute_ch(h, true);
  return neural_acd::compute_h(m, h, k, res, 42);
}

double ref_hull_volume(const double* v, int nv, int* ntris) {
  Mesh m = make_mesh(v, nv, nullptr, 0);
  Mesh h;
  m.compute_ch(h, true);
  *ntris = (int)h.triangles.size();
  return neural_acd::get_mesh_volume(h);
}

// The reference's btConvexHullComputer path (Mesh::compute_vch,
// lib/src/core.cpp:113-142, with the outward-normal fix): hull vertices
// (out_v, cap_v x 3) and fan-triangulated faces (out_t, cap_t x 3). Returns
// the triangle count, or -1 if a buffer is too small; *nv_out gets the
// vertex count.
int ref_hull_bt(const double* v, int nv, double* out_v, int cap_v, int* out_t, int cap_t,
                int* nv_out) {
  Mesh m = make_mesh(v, nv, nullptr, 0);
  Mesh h;
  m.compute_vch(h, true);
  *nv_out = (int)h.vertices.size();
  if ((int)h.vertices.size() > cap_v || (int)h.triangles.size() > cap_t) return -1;
  for (size_t i = 0; i < h.vertices.size(); ++i)
    for (int k = 0; k < 3; ++k) out_v[3 * i + k] = h.vertices[i][k];
  for (size_t i = 0; i < h.triangles.size(); ++i)
    for (int k = 0; k < 3; ++k) out_t[3 * i + k] = h.triangles[i][k];
  return (int)h.triangles.size();
}

// multimerge_ch (lib/src/postprocess.cpp:64-200) on the given parts
// (concatenated: part k has nv[k] vertices and nt[k] triangles), with their
// hulls from compute_ch and the engine seeded with `seed` first. The merged
// hulls land in the part store; returns their count.
int ref_multimerge(const double* v, const int* nv, const int* t, const int* nt, int nparts,
                   double current_concavity, double threshold, unsigned seed) {
  neural_acd::MeshList parts, hulls;
  for (int k = 0; k < nparts; ++k) {
    parts.push_back(make_mesh(v, nv[k], t, nt[k]));
    v += 3 * (size_t)nv[k];
    t += 3 * (size_t)nt[k];
  }
  for (auto& p : parts) {
    Mesh h;
    p.compute_ch(h, true);
    hulls.push_back(h);
  }
  neural_acd::set_seed(seed);
  neural_acd::multimerge_ch(parts, hulls, current_concavity, threshold);
  g_parts = hulls;
  return (int)hulls.size();
}

// lib/src/process.cpp:238 process(mesh, concavity, num_parts); parts land in
// the part store.
int ref_process(const double* v, int nv, const int* t, int nt, double concavity, int num_parts,
                int score_mode_edge, int return_parts, int use_merging, double* out_concavity) {
  neural_acd::config.score_mode = score_mode_edge ? "edge" : "concavity";
  neural_acd::config.return_parts = return_parts != 0;
  neural_acd::config.use_merging = use_merging != 0;
  Mesh m = make_mesh(v, nv, t, nt);
  neural_acd::ProcessResult r = neural_acd::process(m, concavity, num_parts);
  g_parts = r.parts;
  *out_concavity = r.concavity;
  neural_acd::config.score_mode = "concavity";
  neural_acd::config.return_parts = false;
  neural_acd::config.use_merging = false;
  return r.num_parts;
}

}  // extern "C"

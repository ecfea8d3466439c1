// The decomposition loop (lib/src/process.cpp:28-347): remesh, cage, flat
// planes, initial visibility, then repeatedly split the worst part by the
// candidate plane that cuts the most visibility-edge length; finally hulls,
// final concavity and (optionally) hull merging. Visibility and plane scoring
// run on the GPU through the C ABI; the rest is host C++.
#include "process.hpp"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <iostream>
#include <sstream>
#include <string>

#include "gpu_bridge.hpp"

namespace visacd {

namespace {
StageTimes g_times;
double now_ms() {
  return std::chrono::duration<double, std::milli>(
             std::chrono::steady_clock::now().time_since_epoch())
      .count();
}
void log(const std::string& msg) {
  if (!config().verbose) return;
  std::cout << "[visacd] " << msg << "\n";
  std::cout.flush();
}
}  // namespace

const StageTimes& last_stage_times() { return g_times; }

std::vector<Plane> get_candidate_planes(const std::vector<Vec3>& vertices,
                                        const std::vector<Edge>& edges, int num_planes) {
  std::vector<Plane> planes;
  if (edges.empty()) return planes;
  std::uniform_int_distribution<> dis(0, (int)edges.size() - 1);
  const double normal_eps = std::cos(5.0 * M_PI / 180.0);
  const double dist_eps = 1e-3;
  std::mt19937& eng = random_engine();
  for (int i = 0; i < num_planes * 5 && (int)planes.size() < num_planes; ++i) {
    int idx = dis(eng);
    const Vec3 p1 = vertices[edges[idx].first];
    const Vec3 p2 = vertices[edges[idx].second];
    Vec3 n = p2 - p1;
    if (norm(n) < 1e-6) continue;
    n = normalized(n);
    Vec3 m = (p1 + p2) * 0.5;
    double d = -(n[0] * m[0] + n[1] * m[1] + n[2] * m[2]);
    bool similar = false;
    for (const auto& p : planes) {
      double dt = std::fabs(n[0] * p.a + n[1] * p.b + n[2] * p.c);
      if (dt > normal_eps && std::fabs(d - p.d) < dist_eps) {
        similar = true;
        break;
      }
    }
    if (!similar) planes.emplace_back(n[0], n[1], n[2], d);
  }
  return planes;
}

bool decompose_iteration(Mesh& mesh, MeshList& parts, Mesh& cage,
                         const std::vector<Plane>& flat_planes) {
  double t0 = now_ms();
  std::vector<Plane> planes = get_candidate_planes(mesh.vertices, mesh.intersecting_edges, 2500);
  const size_t flat_offset = planes.size();
  planes.insert(planes.end(), flat_planes.begin(), flat_planes.end());
  if (planes.empty() || mesh.intersecting_edges.empty()) {
    parts.push_back(mesh);
    return true;
  }
  std::vector<double> scores = gpu::score_planes(planes, mesh.vertices, mesh.intersecting_edges);
  for (size_t i = flat_offset; i < planes.size(); ++i) scores[i] *= config().flat_surface_k;
  const size_t best = std::max_element(scores.begin(), scores.end()) - scores.begin();
  const Plane plane = planes[best];
  double t1 = now_ms();
  g_times.scoring += t1 - t0;

  std::vector<int> map1, map2;
  MeshList halves = config().gpu_clip ? gpu::clip(mesh, plane, map1, map2)
                                      : clip(mesh, plane, map1, map2);
  double t2 = now_ms();
  g_times.clip += t2 - t1;
  if (halves.size() < 2) {
    parts.push_back(mesh);
    return false;
  }
  for (const auto& e : mesh.intersecting_edges) {
    const int a = (int)e.first, b = (int)e.second;
    if (map1[a] && map1[b]) halves[0].intersecting_edges.push_back({(unsigned)(map1[a] - 1), (unsigned)(map1[b] - 1)});
    if (map2[a] && map2[b]) halves[1].intersecting_edges.push_back({(unsigned)(map2[a] - 1), (unsigned)(map2[b] - 1)});
  }
  separate_disjoint(halves);
  for (auto& part : halves) {
    if (part.vertices.size() < 10) continue;
    double c0 = now_ms();
    cage = part.copy_geometry();
    manifold_preprocess(cage, 40, 0.02);
    double c1 = now_ms();
    g_times.cages += c1 - c0;
    std::vector<Edge> fresh = gpu::visibility_edges(part, cage);
    g_times.visibility += now_ms() - c1;
    part.intersecting_edges.insert(part.intersecting_edges.end(), fresh.begin(), fresh.end());
    parts.push_back(part);
  }
  return false;
}

double compute_part_score(const Mesh& part) {
  double s = 0;
  for (const auto& e : part.intersecting_edges) s += norm(part.vertices[e.second] - part.vertices[e.first]);
  return s;
}

int get_part_with_highest_score(const MeshList& parts) {
  double best = -1.0;
  int idx = -1;
  for (int i = 0; i < (int)parts.size(); ++i) {
    double s = compute_part_score(parts[i]);
    if (s > best) {
      best = s;
      idx = i;
    }
  }
  return idx;
}

int get_part_with_highest_concavity(const MeshList& parts, double& max_concavity) {
  MeshList hulls;
  hulls.reserve(parts.size());
  for (const auto& p : parts) hulls.push_back(convex_hull(p.vertices, true));
  int idx = -1;
  for (int i = 0; i < (int)parts.size(); ++i) {
    double c = compute_h(parts[i], hulls[i], 0.3, 3000);
    if (c > max_concavity) {
      max_concavity = c;
      idx = i;
    }
  }
  return idx;
}

double compute_final_concavity(const MeshList& parts, const MeshList& hulls) {
  double h = 0;
  for (size_t i = 0; i < parts.size(); ++i) {
    double c = compute_hb(parts[i], hulls[i], 10000);
    if (c > h) h = c;
  }
  return h;
}

ProcessResult process(Mesh mesh, double concavity, int num_parts) {
  g_times = StageTimes();
  const double t_start = now_ms();
  gpu::context();
  auto box = normalize(mesh);
  log("Preprocessing mesh (" + std::to_string(mesh.vertices.size()) + " verts)...");
  Mesh original = mesh.copy_geometry();
  manifold_preprocess(mesh, 30, 0.55 / 30);
  if (mesh.vertices.size() > 15000) {
    mesh = original.copy_geometry();
    manifold_preprocess(mesh, 20, 0.55 / 20);
  }
  log("Remeshed to " + std::to_string(mesh.vertices.size()) + " verts.");
  Mesh cage = mesh.copy_geometry();
  manifold_preprocess(cage, 40, 0.03);
  std::vector<Plane> flat_planes;
  MeshList parts;
  if (config().use_flat_surfaces) {
    auto surfaces = extract_surfaces(mesh, config().flat_surface_min_area);
    log("Detected " + std::to_string(surfaces.size()) + " flat surface(s).");
    for (auto& s : surfaces) flat_planes.push_back(s.plane);
  }
  parts.push_back(mesh);
  separate_disjoint(parts);
  g_times.preprocess = now_ms() - t_start;
  {
    double t0 = now_ms();
    for (auto& part : parts) {
      auto e = gpu::visibility_edges(part, cage);
      part.intersecting_edges.insert(part.intersecting_edges.end(), e.begin(), e.end());
    }
    g_times.visibility += now_ms() - t0;
  }
  log("Starting decomposition (max parts=" + std::to_string(num_parts) + ", concavity threshold=" +
      std::to_string(concavity) + ", mode=" + config().score_mode + ").");
  for (int i = 0; i < num_parts - 1; ++i) {
    int idx = -1;
    if (config().score_mode == "edge") {
      idx = get_part_with_highest_score(parts);
    } else if (config().score_mode == "concavity") {
      double t0 = now_ms();
      double mc = -1;
      idx = get_part_with_highest_concavity(parts, mc);
      g_times.concavity += now_ms() - t0;
      if (mc < concavity) {
        log("Step " + std::to_string(i + 1) + ": concavity " + std::to_string(mc).substr(0, 6) +
            " < threshold, stopping.");
        break;
      }
    }
    if (idx == -1) break;
    log("Step " + std::to_string(i + 1) + "/" + std::to_string(num_parts - 1) + ": splitting part " +
        std::to_string(idx) + " (" + std::to_string(parts.size()) + " parts total).");
    Mesh part = parts[idx];
    parts.erase(parts.begin() + idx);
    g_times.iterations++;
    if (decompose_iteration(part, parts, cage, flat_planes)) {
      log("No more intersecting edges, stopping early.");
      break;
    }
  }
  log("Computing convex hulls for " + std::to_string(parts.size()) + " parts...");
  double th = now_ms();
  MeshList hulls;
  for (const auto& p : parts) hulls.push_back(convex_hull(p.vertices, true));
  double final_c = compute_final_concavity(parts, hulls);
  if (config().use_merging) {
    log("Merging parts...");
    multimerge_ch(parts, hulls, final_c, concavity);
  }
  g_times.hulls = now_ms() - th;
  for (auto& h : hulls) unnormalize(h, box);
  for (auto& p : parts) unnormalize(p, box);
  MeshList& out = config().return_parts ? parts : hulls;
  const int n = (int)out.size();
  char buf[128];
  std::snprintf(buf, sizeof(buf), "Done. parts=%d  concavity=%.4f", n, final_c);
  log(buf);
  g_times.total = now_ms() - t_start;
  return {out, final_c, n};
}

}  // namespace visacd

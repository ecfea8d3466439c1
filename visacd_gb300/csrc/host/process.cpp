// The decomposition loop (lib/src/process.cpp:28-347): remesh, cage, flat
// planes, initial visibility, then repeatedly split the worst part by the
// candidate plane that cuts the most visibility-edge length; finally hulls,
// final concavity and (optionally) hull merging. Visibility and plane scoring
// run on the GPU through the C ABI; the rest is host C++.
#include "process.hpp"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <iostream>
#include <numeric>
#include <sstream>
#include <string>
#include <thread>
#include <unordered_map>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "gpu_bridge.hpp"

namespace visacd {

namespace {
thread_local StageTimes g_times;
thread_local bool tl_quiet = false;  // process_batch workers do not log
double now_ms() {
  return std::chrono::duration<double, std::milli>(
             std::chrono::steady_clock::now().time_since_epoch())
      .count();
}
void log(const std::string& msg) {
  if (!config().verbose || tl_quiet) return;
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
  Mt19937& eng = random_engine();
  // A candidate is dropped when any kept plane has |d - d'| < dist_eps and a
  // normal within 5 degrees; only whether one exists matters, so the kept
  // planes are bucketed by floor(d / dist_eps) and a candidate is compared
  // with the planes of the buckets within two of its own (every plane with
  // |d - d'| < dist_eps lies there), with the same two tests.
  std::unordered_map<long long, std::vector<int>> by_d;
  auto bucket = [&](double d) { return (long long)std::floor(d / dist_eps); };
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
    const long long key = bucket(d);
    for (long long k = key - 2; k <= key + 2 && !similar; ++k) {
      auto it = by_d.find(k);
      if (it == by_d.end()) continue;
      for (int j : it->second) {
        const Plane& p = planes[j];
        double dt = std::fabs(n[0] * p.a + n[1] * p.b + n[2] * p.c);
        if (dt > normal_eps && std::fabs(d - p.d) < dist_eps) {
          similar = true;
          break;
        }
      }
    }
    if (!similar) {
      by_d[key].push_back((int)planes.size());
      planes.emplace_back(n[0], n[1], n[2], d);
    }
  }
  return planes;
}

namespace {

// The reference's split-plane search (lib/src/process.cpp:96-134): 2500 random
// candidates plus the flat-surface planes (scores x flat_surface_k), first
// maximum, all on the GPU after the edge draws. Returns false when there is
// nothing to score.
bool exhaustive_plane(const Mesh& mesh, const std::vector<Plane>& flat_planes, Plane& out) {
  return gpu::split_search(mesh, flat_planes, config().flat_surface_k, 2500, out);
}

}  // namespace

// Refinement of the proposals: for each proposal, the perpendicular-bisector
// planes (the reference's candidate form, lib/src/process.cpp:45-53) of the
// `per` visibility edges whose bisectors are nearest to it, under the distance
// the proposer is trained with: 2 - 2|n_q . n_e| + ((s d_q - d_e) / half)^2,
// s = sign(n_q . n_e). Returned in edge order, each edge once. The host
// statement of the GPU refinement (refine_partial_kernel, refine_merge_kernel),
// for tests.
std::vector<Plane> refine_proposals(const Mesh& mesh, const std::vector<Plane>& prop, int per) {
  const auto& V = mesh.vertices;
  const auto& E = mesh.intersecting_edges;
  auto b = bbox(mesh);
  double half = 0.5 * std::max(b[1] - b[0], std::max(b[3] - b[2], b[5] - b[4]));
  if (!(half > 0)) half = 1.0;
  std::vector<Plane> bis;
  bis.reserve(E.size());
  for (const auto& e : E) {
    Vec3 n = V[e.second] - V[e.first];
    const double ln = norm(n);
    if (ln < 1e-6) continue;
    n = n / ln;
    const Vec3 m = (V[e.first] + V[e.second]) * 0.5;
    bis.emplace_back(n[0], n[1], n[2], -dot(n, m));
  }
  const int k = std::min<int>(per, (int)bis.size());
  std::vector<char> keep(bis.size(), 0);
  if (k > 0) {
    // The k smallest (distance, index) pairs per proposal (a unique set: the
    // pairs are distinct), in one pass over the bisectors with a bounded
    // max-heap per proposal.
    using Item = std::pair<double, int>;
    std::vector<std::vector<Item>> heaps(prop.size());
    for (auto& h : heaps) h.reserve(k + 1);
    for (size_t i = 0; i < bis.size(); ++i) {
      for (size_t q = 0; q < prop.size(); ++q) {
        const Plane& p = prop[q];
        const double c = p.a * bis[i].a + p.b * bis[i].b + p.c * bis[i].c;
        const double s = c >= 0 ? 1.0 : -1.0;
        const double dd = (s * p.d - bis[i].d) / half;
        const Item it{2.0 - 2.0 * std::fabs(c) + dd * dd, (int)i};
        auto& h = heaps[q];
        if ((int)h.size() < k) {
          h.push_back(it);
          std::push_heap(h.begin(), h.end());
        } else if (it < h.front()) {
          std::pop_heap(h.begin(), h.end());
          h.back() = it;
          std::push_heap(h.begin(), h.end());
        }
      }
    }
    for (const auto& h : heaps)
      for (const auto& it : h) keep[it.second] = 1;
  }
  std::vector<Plane> out;
  for (size_t i = 0; i < bis.size(); ++i)
    if (keep[i]) out.push_back(bis[i]);
  return out;
}

namespace {

// Learned search: the proposer's 16 planes refined by nearby bisector planes,
// a probe of proposer_probe_planes random candidates (the reference's draw,
// smaller) and the flat planes, scored together by the exact kernel, all in
// one GPU call. If the best learned plane scores more than proposer_tolerance
// below the probe's best, the proposals are not trusted for this split and the
// exhaustive search runs instead, with the draws after the probe's.
bool learned_plane(const Mesh& mesh, const std::vector<Plane>& flat_planes, Plane& out) {
  bool fallback = false;
  if (gpu::learned_split_search(mesh, flat_planes, config().flat_surface_k, out, fallback)) return true;
  if (!fallback) return false;
  gpu::counters().lp_fallbacks++;
  return exhaustive_plane(mesh, flat_planes, out);
}

}  // namespace

bool decompose_iteration(Mesh& mesh, MeshList& parts, Mesh& cage,
                         const std::vector<Plane>& flat_planes) {
  double t0 = now_ms();
  Plane plane;
  const bool ok = config().plane_proposer == "learned" ? learned_plane(mesh, flat_planes, plane)
                                                       : exhaustive_plane(mesh, flat_planes, plane);
  if (!ok) {
    parts.push_back(mesh);
    return true;
  }
  double t1 = now_ms();
  g_times.scoring += t1 - t0;

  std::vector<int> map1, map2;
  MeshList halves = !checker_hooks().host_clip ? gpu::clip(mesh, plane, map1, map2)
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
  // Every new sub-part gets its cage, then all of them are traced in one
  // batched visibility call (the reference traces them one by one,
  // lib/src/process.cpp:165-178; neither step draws random numbers, so the
  // order does not change results).
  std::vector<Mesh> cages;
  std::vector<const Mesh*> todo, todo_cages;
  std::vector<size_t> which;
  cages.reserve(halves.size());
  for (size_t k = 0; k < halves.size(); ++k) {
    if (halves[k].vertices.size() < 10) continue;
    double c0 = now_ms();
    cages.push_back(halves[k].copy_geometry());
    manifold_preprocess(cages.back(), 40, 0.02);
    g_times.cages += now_ms() - c0;
    which.push_back(k);
  }
  for (size_t k = 0; k < which.size(); ++k) {
    todo.push_back(&halves[which[k]]);
    todo_cages.push_back(&cages[k]);
  }
  if (!todo.empty()) {
    double c1 = now_ms();
    std::vector<std::vector<Edge>> fresh = gpu::visibility_edges_batch(todo, todo_cages);
    g_times.visibility += now_ms() - c1;
    for (size_t k = 0; k < which.size(); ++k) {
      Mesh& part = halves[which[k]];
      part.intersecting_edges.insert(part.intersecting_edges.end(), fresh[k].begin(), fresh[k].end());
    }
    cage = cages.back();
  }
  for (size_t k : which) parts.push_back(halves[k]);
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

const MeshList& HullCache::update(const MeshList& parts) {
  const size_t n = parts.size();
  hulls.resize(n);
  valid.resize(n, 0);
  std::vector<int> todo;
  for (size_t i = 0; i < n; ++i)
    if (!valid[i]) todo.push_back((int)i);
  // Hulls draw no random numbers: built in parallel (same result in any order).
#pragma omp parallel for schedule(dynamic, 1) if (todo.size() > 1)
  for (int k = 0; k < (int)todo.size(); ++k) hulls[todo[k]] = convex_hull(parts[todo[k]].vertices, true);
  for (int i : todo) valid[i] = 1;
  return hulls;
}

int get_part_with_highest_concavity(const MeshList& parts, double& max_concavity, HullCache* cache) {
  const auto t0 = std::chrono::steady_clock::now();
  HullCache local;
  const MeshList& hulls = (cache ? *cache : local).update(parts);
  concavity_times().hull_ms +=
      std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  // compute_h(part, hull, 0.3, 3000) of every part, of which only the first
  // maximum and its value are used. The samples are drawn in the reference's
  // order (part i, then its hull, for i = 0, 1, ...); the sampled terms of all
  // parts are then evaluated in one batch that skips sample terms unable to
  // reach the batch's running maximum (seeded with the volume terms), so the
  // parts attaining the largest concavity get their exact values and every
  // other part a value below it.
  const int n = (int)parts.size();
  std::vector<HbSamples> smp(n);
  std::vector<double> c(n);
  for (int i = 0; i < n; ++i) {
    c[i] = compute_rv(parts[i], hulls[i]) * 0.3;
    sample_hb(parts[i], hulls[i], 3000, smp[i]);
  }
  std::vector<const Mesh*> pa(n), pb(n);
  std::vector<const HbSamples*> ps(n);
  for (int i = 0; i < n; ++i) {
    pa[i] = &parts[i];
    pb[i] = &hulls[i];
    ps[i] = &smp[i];
  }
  const std::vector<double> hb = eval_hb_batch(pa, pb, ps, c, std::max(max_concavity, 0.0), false);
  for (int i = 0; i < n; ++i) c[i] = std::max(c[i], hb[i]);
  int idx = -1;
  for (int i = 0; i < n; ++i) {
    if (c[i] > max_concavity) {
      max_concavity = c[i];
      idx = i;
    }
  }
  return idx;
}

double compute_final_concavity(const MeshList& parts, const MeshList& hulls) {
  // The largest compute_hb(part, hull, 10000): samples drawn in order, values
  // evaluated in one batch pruned against its running maximum, as in
  // get_part_with_highest_concavity.
  const size_t n = parts.size();
  std::vector<HbSamples> smp(n);
  for (size_t i = 0; i < n; ++i) sample_hb(parts[i], hulls[i], 10000, smp[i]);
  std::vector<const Mesh*> pa(n), pb(n);
  std::vector<const HbSamples*> ps(n);
  for (size_t i = 0; i < n; ++i) {
    pa[i] = &parts[i];
    pb[i] = &hulls[i];
    ps[i] = &smp[i];
  }
  const std::vector<double> hb = eval_hb_batch(pa, pb, ps, {}, 0.0, false);
  double h = 0;
  for (size_t i = 0; i < n; ++i)
    if (hb[i] > h) h = hb[i];
  return h;
}

ProcessResult process(Mesh mesh, double concavity, int num_parts) {
  if (config().plane_proposer != "exhaustive" && config().plane_proposer != "learned")
    throw std::runtime_error("config.plane_proposer must be 'exhaustive' or 'learned'");
  if (config().proposer_refine < 0 || config().proposer_refine > 32)
    throw std::runtime_error("config.proposer_refine must be in [0, 32]");
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
    std::vector<const Mesh*> ps, cs;
    for (auto& part : parts) {
      ps.push_back(&part);
      cs.push_back(&cage);
    }
    std::vector<std::vector<Edge>> e = gpu::visibility_edges_batch(ps, cs);
    for (size_t k = 0; k < parts.size(); ++k)
      parts[k].intersecting_edges.insert(parts[k].intersecting_edges.end(), e[k].begin(), e[k].end());
    g_times.visibility += now_ms() - t0;
  }
  HullCache hull_cache;
  log("Starting decomposition (max parts=" + std::to_string(num_parts) + ", concavity threshold=" +
      std::to_string(concavity) + ", mode=" + config().score_mode + ").");
  for (int i = 0; i < num_parts - 1; ++i) {
    int idx = -1;
    if (config().score_mode == "edge") {
      idx = get_part_with_highest_score(parts);
    } else if (config().score_mode == "concavity") {
      double t0 = now_ms();
      double mc = -1;
      idx = get_part_with_highest_concavity(parts, mc, &hull_cache);
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
    hull_cache.erase((size_t)idx);
    g_times.iterations++;
    if (decompose_iteration(part, parts, cage, flat_planes)) {
      log("No more intersecting edges, stopping early.");
      break;
    }
  }
  log("Computing convex hulls for " + std::to_string(parts.size()) + " parts...");
  double th = now_ms();
  MeshList hulls = hull_cache.update(parts);
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

std::vector<ProcessResult> process_batch(const MeshList& meshes, double concavity, int num_parts,
                                         const std::vector<unsigned int>& seeds, int threads) {
  if (seeds.size() != meshes.size())
    throw std::runtime_error("process_batch: one seed per mesh is required");
  const int n = (int)meshes.size();
  std::vector<ProcessResult> results(n);
  if (n == 0) return results;
  if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
  threads = std::min(threads, n);
  std::atomic<int> next{0};
  std::vector<std::string> errors(n);
  std::vector<StageTimes> times(threads);
  std::vector<gpu::Counters> counts(threads);
  std::vector<ConcavityTimes> ctimes(threads);
  auto worker = [&](int w) {
    try {
      gpu::ThreadContext tctx(gpu::default_device(), threads > 1);
      tl_quiet = true;
#ifdef _OPENMP
      omp_set_num_threads(1);  // the batch is the parallelism; no nested teams
#endif
      Mt19937 eng;
      set_thread_engine(&eng);
      gpu::counters() = gpu::Counters();
      concavity_times() = ConcavityTimes();
      for (int i = next++; i < n; i = next++) {
        eng.seed(seeds[i]);
        try {
          results[i] = process(meshes[i], concavity, num_parts);
        } catch (const std::exception& e) {
          errors[i] = e.what();
        }
        const StageTimes& t = g_times;
        StageTimes& acc = times[w];
        acc.preprocess += t.preprocess;
        acc.visibility += t.visibility;
        acc.scoring += t.scoring;
        acc.clip += t.clip;
        acc.concavity += t.concavity;
        acc.cages += t.cages;
        acc.hulls += t.hulls;
        acc.total += t.total;
        acc.iterations += t.iterations;
      }
      set_thread_engine(nullptr);
      tl_quiet = false;
      counts[w] = gpu::counters();
      ctimes[w] = concavity_times();
    } catch (const std::exception& e) {
      for (int i = next++; i < n; i = next++) errors[i] = e.what();
    }
  };
  std::vector<std::thread> pool;
  for (int w = 0; w < threads; ++w) pool.emplace_back(worker, w);
  for (auto& t : pool) t.join();
  StageTimes sum;
  for (const auto& t : times) {
    sum.preprocess += t.preprocess;
    sum.visibility += t.visibility;
    sum.scoring += t.scoring;
    sum.clip += t.clip;
    sum.concavity += t.concavity;
    sum.cages += t.cages;
    sum.hulls += t.hulls;
    sum.total += t.total;
    sum.iterations += t.iterations;
  }
  g_times = sum;
  // Counters of the workers (zeroed per thread) are added to the caller's.
  auto& c = gpu::counters();
  auto& ct = concavity_times();
  for (int w = 0; w < threads; ++w) {
    const auto& k = counts[w];
    c.vis_calls += k.vis_calls;
    c.vis_pairs += k.vis_pairs;
    c.vis_edges += k.vis_edges;
    c.score_calls += k.score_calls;
    c.plane_edge_pairs += k.plane_edge_pairs;
    c.lp_calls += k.lp_calls;
    c.lp_fallbacks += k.lp_fallbacks;
    c.vis_ms += k.vis_ms;
    c.score_ms += k.score_ms;
    c.lp_ms += k.lp_ms;
    ct.sample_ms += ctimes[w].sample_ms;
    ct.hausdorff_ms += ctimes[w].hausdorff_ms;
    ct.hull_ms += ctimes[w].hull_ms;
    ct.samples += ctimes[w].samples;
    ct.calls += ctimes[w].calls;
  }
  for (int i = 0; i < n; ++i)
    if (!errors[i].empty())
      throw std::runtime_error("process_batch: mesh " + std::to_string(i) + ": " + errors[i]);
  return results;
}

}  // namespace visacd

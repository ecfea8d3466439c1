// Connected components of parts and greedy hull merging.
//
// separate_disjoint: lib/src/postprocess.cpp:202-326 — split each part into
// edge-connected triangle components (numbered by their lowest triangle),
// vertices renumbered in first-use order, is_new carried over, each visibility
// edge given to the first component holding both endpoints; components with
// |volume| < 1e-6 are dropped.
// multimerge_ch: lib/src/postprocess.cpp:64-200 — the reference's packed
// lower-triangular cost matrix, its update order and its indexing are kept
// as they are (they decide which hulls merge).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <map>
#include <numeric>
#include <unordered_map>
#include <vector>

#include "geometry.hpp"
#include "gpu_bridge.hpp"

namespace visacd {

namespace {

int find_root(std::vector<int>& p, int x) {
  while (p[x] != x) {
    p[x] = p[p[x]];
    x = p[x];
  }
  return x;
}

// Edge-connected components with flat structures: an open-addressing table
// from undirected edge to the first triangle holding it (the union of every
// triangle with that one gives the components whatever the order), then each
// component's triangles in index order with its vertices numbered on first use
// (a stamp per vertex marks the component being built).
MeshList separate_step(const Mesh& part) {
  const int T = (int)part.triangles.size();
  if (T == 0) return {};
  std::vector<int> uf(T);
  std::iota(uf.begin(), uf.end(), 0);
  size_t cap = 64;
  while (cap < 6 * (size_t)T) cap <<= 1;
  std::vector<uint64_t> keys(cap, ~0ull);
  std::vector<int> first(cap);
  const uint64_t mask = cap - 1;
  for (int i = 0; i < T; ++i) {
    const auto& t = part.triangles[i];
    const std::pair<int, int> e[3] = {std::minmax(t[0], t[1]), std::minmax(t[1], t[2]),
                                      std::minmax(t[0], t[2])};
    for (const auto& k : e) {
      const uint64_t key = ((uint64_t)(uint32_t)k.first << 32) | (uint32_t)k.second;
      uint64_t h = (key * 0x9E3779B97F4A7C15ull) >> 20;
      for (;; ++h) {
        const uint64_t slot = h & mask;
        if (keys[slot] == ~0ull) {
          keys[slot] = key;
          first[slot] = i;
          break;
        }
        if (keys[slot] == key) {
          int a = find_root(uf, first[slot]), b = find_root(uf, i);
          if (a != b) uf[std::max(a, b)] = std::min(a, b);
          break;
        }
      }
    }
  }
  // Component ids in order of their lowest triangle.
  std::vector<int> comp(T), comp_of_root(T, -1);
  int nparts = 0;
  for (int i = 0; i < T; ++i) {
    int r = find_root(uf, i);
    if (comp_of_root[r] < 0) comp_of_root[r] = nparts++;
    comp[i] = comp_of_root[r];
  }
  // Triangles grouped by component, in index order within each.
  std::vector<int> start(nparts + 1, 0), order(T);
  for (int i = 0; i < T; ++i) ++start[comp[i] + 1];
  for (int p = 0; p < nparts; ++p) start[p + 1] += start[p];
  {
    std::vector<int> fill(start.begin(), start.end() - 1);
    for (int i = 0; i < T; ++i) order[fill[comp[i]]++] = i;
  }
  MeshList out(nparts);
  const bool has_new = !part.is_new.empty();
  const size_t NV = part.vertices.size();
  std::vector<int> stamp(NV, -1), local(NV);
  std::vector<char> taken(part.intersecting_edges.size(), 0);
  for (int p = 0; p < nparts; ++p) {
    Mesh& m = out[p];
    m.triangles.reserve(start[p + 1] - start[p]);
    for (int k0 = start[p]; k0 < start[p + 1]; ++k0) {
      const int i = order[k0];
      Tri nt;
      for (int k = 0; k < 3; ++k) {
        const int g = part.triangles[i][k];
        if (stamp[g] != p) {
          stamp[g] = p;
          local[g] = (int)m.vertices.size();
          m.vertices.push_back(part.vertices[g]);
          if (has_new) m.is_new.push_back(part.is_new[g]);
        }
        nt[k] = local[g];
      }
      m.triangles.push_back(nt);
    }
    // Each visibility edge goes to the first component holding both endpoints.
    for (size_t k = 0; k < part.intersecting_edges.size(); ++k) {
      if (taken[k]) continue;
      const auto& e = part.intersecting_edges[k];
      if (stamp[e.first] == p && stamp[e.second] == p) {
        m.intersecting_edges.push_back({(unsigned)local[e.first], (unsigned)local[e.second]});
        taken[k] = 1;
      }
    }
  }
  return out;
}

// mesh_dist of each listed hull pair, compared by the caller with `threshold`
// only: the GPU kernel (visacd_hull_distances) returns the same value, or
// DBL_MAX for pairs whose bounding boxes are already farther apart than
// threshold.
std::vector<double> pair_distances(const MeshList& cvxs, const std::vector<std::pair<int, int>>& pairs,
                                   double threshold) {
  if (!checker_hooks().host_merge) return gpu::hull_distances(cvxs, pairs, threshold);
  std::vector<double> d(pairs.size());
  for (size_t k = 0; k < pairs.size(); ++k) d[k] = mesh_dist(cvxs[pairs[k].first], cvxs[pairs[k].second]);
  return d;
}

// Hulls of the unions of hull pairs (the reference's merge_ch,
// lib/src/postprocess.cpp:30-43: the hull of both vertex lists, the pair's
// first hull first), many in one launch of visacd_convex_hulls (the host
// QuickHull under the test hook host_hull; both give the same meshes). Hulls
// draw no random numbers, so building the ones a cost pass needs before that
// pass changes nothing.
MeshList union_hulls(const MeshList& cvxs, const std::vector<std::pair<int, int>>& pairs) {
  std::vector<std::vector<Vec3>> pts(pairs.size());
  std::vector<const std::vector<Vec3>*> sets(pairs.size());
  for (size_t k = 0; k < pairs.size(); ++k) {
    const Mesh &a = cvxs[pairs[k].first], &b = cvxs[pairs[k].second];
    pts[k] = a.vertices;
    pts[k].insert(pts[k].end(), b.vertices.begin(), b.vertices.end());
    sets[k] = &pts[k];
  }
  if (!checker_hooks().host_hull) return gpu::convex_hulls(sets, true);
  MeshList h(pairs.size());
#pragma omp parallel for schedule(dynamic, 1) if (pairs.size() > 1)
  for (long k = 0; k < (long)pairs.size(); ++k) h[k] = convex_hull(pts[k], true);
  return h;
}

// The pairs of `pairs` closer than threshold, with their union hulls.
MeshList close_union_hulls(const MeshList& cvxs, const std::vector<std::pair<int, int>>& pairs,
                           const std::vector<double>& dist, double threshold) {
  std::vector<std::pair<int, int>> close;
  for (size_t k = 0; k < pairs.size(); ++k)
    if (dist[k] < threshold) close.push_back(pairs[k]);
  return union_hulls(cvxs, close);
}

}  // namespace

void separate_disjoint(MeshList& parts) {
  MeshList out;
  for (const auto& p : parts)
    for (auto& c : separate_step(p))
      if (std::fabs(mesh_volume(c)) >= 1e-6) out.push_back(std::move(c));
  parts.swap(out);
}

void multimerge_ch(MeshList& meshes, MeshList& cvxs, double current_concavity, double threshold) {
  const size_t n = cvxs.size();
  if (n <= 1) return;
  const size_t bound = ((n - 1) * n) >> 1;
  std::vector<double> cost(bound), precost(bound);
  std::vector<std::pair<int, int>> all_pairs(bound);
  for (size_t idx = 0; idx < bound; ++idx) {
    size_t p1 = (size_t)(std::sqrt(8.0 * idx + 1) - 1) >> 1;
    size_t sum = (p1 * (p1 + 1)) >> 1;
    all_pairs[idx] = {(int)(p1 + 1), (int)(idx - sum)};
  }
  const std::vector<double> all_dist = pair_distances(cvxs, all_pairs, threshold);
  const MeshList all_ch = close_union_hulls(cvxs, all_pairs, all_dist, threshold);
  size_t next_ch = 0;
  for (size_t idx = 0; idx < bound; ++idx) {
    const size_t p1 = (size_t)all_pairs[idx].first, p2 = (size_t)all_pairs[idx].second;
    double dist = all_dist[idx];
    if (dist < threshold) {
      const Mesh& ch = all_ch[next_ch++];
      cost[idx] = compute_h3(cvxs[p1], cvxs[p2], ch, 0.3, 10000);
      precost[idx] = std::max(compute_h(meshes[p1], cvxs[p1], 0.3, 10000),
                              compute_h(meshes[p2], cvxs[p2], 0.3, 10000));
    } else {
      cost[idx] = kInf;
    }
  }
  // precost is indexed the way the reference indexes it; reads past its end
  // (possible for tiny matrices) count as 0.
  auto pre = [&](size_t i) { return i < precost.size() ? precost[i] : 0.0; };
  size_t cost_size = n;
  for (size_t guard = 0; guard < 4 * bound + 16; ++guard) {
    // First minimum of the packed matrix.
    int addr = -1;
    double best = kInf;
    for (size_t i = 0; i < cost.size(); ++i)
      if (cost[i] < best) {
        best = cost[i];
        addr = (int)i;
      }
    if (addr < 0) break;
    if (best > threshold) break;
    if (best + pre((size_t)addr) > current_concavity) {
      cost[addr] = kInf;
      continue;
    }
    const size_t addrI = ((size_t)(int)std::sqrt(1 + (8.0 * addr)) - 1) >> 1;
    const size_t p1 = addrI + 1;
    const size_t p2 = addr - ((addrI * (addrI + 1)) >> 1);
    MeshList cch = union_hulls(cvxs, {{(int)p1, (int)p2}});
    cvxs[p2] = std::move(cch[0]);
    std::swap(cvxs[p1], cvxs[cvxs.size() - 1]);
    cvxs.pop_back();
    cost_size -= 1;
    // Costs against the merged hull (row p2, then column p2).
    std::vector<std::pair<int, int>> row_pairs;
    for (size_t i = 0; i < cost_size; ++i)
      if (i != p2) row_pairs.push_back({(int)p2, (int)i});
    const std::vector<double> row_dist = pair_distances(cvxs, row_pairs, threshold);
    const MeshList row_ch = close_union_hulls(cvxs, row_pairs, row_dist, threshold);
    next_ch = 0;
    size_t row = ((p2 - 1) * p2) >> 1;
    for (size_t i = 0; i < p2; ++i) {
      double dist = row_dist[i];
      if (dist < threshold) {
        const Mesh& ch = row_ch[next_ch++];
        cost[row] = compute_h3(cvxs[p2], cvxs[i], ch, 0.3, 10000);
        precost[row++] = std::max(pre(p2) + best, pre(i));
      } else {
        cost[row++] = kInf;
      }
    }
    row += p2;
    for (size_t i = p2 + 1; i < cost_size; ++i) {
      double dist = row_dist[i - 1];
      if (dist < threshold) {
        const Mesh& ch = row_ch[next_ch++];
        cost[row] = compute_h3(cvxs[p2], cvxs[i], ch, 0.3, 10000);
        precost[row] = std::max(pre(p2) + best, pre(i));
      } else {
        cost[row] = kInf;
      }
      row += i;
    }
    // Move the last row/column into p1's place.
    const size_t erase_idx = ((cost_size - 1) * cost_size) >> 1;
    if (p1 < cost_size) {
      row = (addrI * p1) >> 1;
      size_t top = erase_idx;
      for (size_t i = 0; i < p1; ++i) {
        if (i != p2) {
          cost[row] = cost[top];
          precost[row] = precost[top];
        }
        ++row;
        ++top;
      }
      ++top;
      row += p1;
      for (size_t i = p1 + 1; i < cost_size; ++i) {
        cost[row] = cost[top];
        precost[row] = precost[top++];
        row += i;
      }
    }
    cost.resize(erase_idx);
    precost.resize(erase_idx);
  }
}

}  // namespace visacd

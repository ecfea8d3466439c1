// Flat-surface planes: grow regions of edge-adjacent triangles whose normals
// stay within cos > 0.999 of the region's running mean, keep regions with area
// above min_area (at most the 40 largest), put a plane 0.02 outside each along
// its mean normal, and drop near-duplicate planes.
//
// Semantics of lib/src/support_surface.cpp:14-183. The adjacency is gathered
// through the same hash-map type with the same insertion sequence so the
// growth order (which decides region membership) is the reference's.
#include <algorithm>
#include <cmath>
#include <queue>
#include <unordered_map>
#include <vector>

#include "geometry.hpp"

namespace visacd {

std::vector<Surface> extract_surfaces(const Mesh& mesh, double min_area) {
  const auto& tris = mesh.triangles;
  const auto& V = mesh.vertices;
  const int T = (int)tris.size();
  std::vector<Vec3> nrm(T);
  for (int i = 0; i < T; ++i) nrm[i] = face_normal(V[tris[i][0]], V[tris[i][1]], V[tris[i][2]]);

  std::unordered_map<long long, std::vector<int>> by_edge;
  by_edge.reserve((size_t)T * 3);
  auto key = [](int a, int b) {
    if (a > b) std::swap(a, b);
    return ((long long)a << 32) | (unsigned long long)b;
  };
  for (int i = 0; i < T; ++i) {
    const auto& t = tris[i];
    by_edge[key(t[0], t[1])].push_back(i);
    by_edge[key(t[1], t[2])].push_back(i);
    by_edge[key(t[2], t[0])].push_back(i);
  }
  std::vector<std::vector<int>> adj(T);
  for (const auto& kv : by_edge) {
    const auto& l = kv.second;
    if (l.size() < 2) continue;
    for (int a : l)
      for (int b : l)
        if (a != b) adj[a].push_back(b);
  }
  auto cos_sim = [](const Vec3& a, const Vec3& b) {
    return dot(a, b) / (std::sqrt(dot(a, a)) * std::sqrt(dot(b, b)));
  };
  std::vector<char> used(T, 0);
  std::vector<Surface> regions;
  for (int s = 0; s < T; ++s) {
    if (used[s]) continue;
    Surface surf;
    surf.triangle_ids.push_back(s);
    used[s] = 1;
    Vec3 mean = nrm[s];
    std::queue<int> q;
    q.push(s);
    while (!q.empty()) {
      int t = q.front();
      q.pop();
      for (int nb : adj[t]) {
        if (used[nb]) continue;
        if (cos_sim(mean, nrm[nb]) > 0.999) {
          used[nb] = 1;
          surf.triangle_ids.push_back(nb);
          mean = (mean * (double)(surf.triangle_ids.size() - 1) + nrm[nb]) /
                 (double)surf.triangle_ids.size();
          q.push(nb);
        }
      }
    }
    regions.push_back(std::move(surf));
  }
  std::vector<Surface> kept;
  for (auto& S : regions) {
    double A = 0;
    for (int t : S.triangle_ids) A += triangle_area(V[tris[t][0]], V[tris[t][1]], V[tris[t][2]]);
    S.area = A;
    if (A > min_area) kept.push_back(S);
  }
  if (kept.size() > 40) {
    std::sort(kept.begin(), kept.end(), [](const Surface& a, const Surface& b) { return a.area > b.area; });
    kept.resize(40);
  }
  for (auto& S : kept) {
    Vec3 n = {0, 0, 0}, pt = {0, 0, 0};
    for (int t : S.triangle_ids) {
      const auto& tr = tris[t];
      n = n + face_normal(V[tr[0]], V[tr[1]], V[tr[2]]);
      pt = pt + (V[tr[0]] + V[tr[1]] + V[tr[2]]) / 3.0;
    }
    n = normalized(n);
    pt = pt / (double)S.triangle_ids.size();
    pt = pt + n * 2e-2;
    S.plane = Plane(n[0], n[1], n[2], -dot(n, pt));
  }
  std::vector<Surface> uniq;
  for (const auto& S : kept) {
    bool dup = false;
    for (const auto& U : uniq) {
      const Plane &p1 = S.plane, &p2 = U.plane;
      double d = p1.a * p2.a + p1.b * p2.b + p1.c * p2.c + p1.d * p2.d;
      double m1 = std::sqrt(p1.a * p1.a + p1.b * p1.b + p1.c * p1.c + p1.d * p1.d);
      double m2 = std::sqrt(p2.a * p2.a + p2.b * p2.b + p2.c * p2.c + p2.d * p2.d);
      if (m1 > 1e-9 && m2 > 1e-9 && std::fabs(d) / (m1 * m2) > 1.0 - 1e-4) {
        dup = true;
        break;
      }
    }
    if (!dup) uniq.push_back(S);
  }
  return uniq;
}

}  // namespace visacd

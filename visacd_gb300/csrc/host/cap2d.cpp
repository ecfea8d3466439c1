// Triangulation of the region a planar border graph encloses (the clip cap).
//
// Stands in for the CDT library call of lib/src/clip.cpp:153-163
// (insertVertices, insertEdges, eraseOuterTrianglesAndHoles), which is absent
// here. The faces of the planar graph are traced with angle-sorted half-edges;
// a face is filled when a point just inside it has odd crossing parity against
// all border edges (the even-odd rule of eraseOuterTrianglesAndHoles); islands
// inside a filled face are bridged in as holes; each face is ear-clipped. Output
// triangles index the input points and are counter-clockwise.
#include <algorithm>
#include <cmath>
#include <set>
#include <vector>

#include "geometry.hpp"

namespace visacd {

namespace {

struct P2 {
  double x, y;
};

double area2(const std::vector<P2>& q, const std::vector<int>& loop) {
  double s = 0;
  for (size_t i = 0; i < loop.size(); ++i) {
    const P2 &a = q[loop[i]], &b = q[loop[(i + 1) % loop.size()]];
    s += a.x * b.y - b.x * a.y;
  }
  return s;
}

bool point_in_loop(const std::vector<P2>& q, const std::vector<int>& loop, P2 p) {
  bool in = false;
  for (size_t i = 0, j = loop.size() - 1; i < loop.size(); j = i++) {
    const P2 &a = q[loop[i]], &b = q[loop[j]];
    if ((a.y > p.y) != (b.y > p.y) && p.x < (b.x - a.x) * (p.y - a.y) / (b.y - a.y) + a.x) in = !in;
  }
  return in;
}

double orient(const P2& a, const P2& b, const P2& c) {
  return (b.x - a.x) * (c.y - a.y) - (b.y - a.y) * (c.x - a.x);
}

bool in_triangle(const P2& a, const P2& b, const P2& c, const P2& p) {
  return orient(a, b, p) >= 0 && orient(b, c, p) >= 0 && orient(c, a, p) >= 0;
}

// Ear clipping of a CCW simple polygon (indices may repeat at bridges). Only
// reflex vertices can lie inside an ear. When rounding leaves no valid ear
// (runs of nearly collinear border points), the most convex vertex is clipped
// anyway: the sliver keeps every border edge covered, so the part stays closed.
void ear_clip(const std::vector<P2>& q, std::vector<int> poly, std::vector<Tri>& out) {
  size_t guard = 0;
  while (poly.size() > 3 && guard++ < 4 * poly.size() * poly.size() + 16) {
    const size_t n = poly.size();
    std::vector<char> reflex(n);
    for (size_t i = 0; i < n; ++i)
      reflex[i] = orient(q[poly[(i + n - 1) % n]], q[poly[i]], q[poly[(i + 1) % n]]) <= 0;
    bool clipped = false;
    for (size_t i = 0; i < n; ++i) {
      if (reflex[i]) continue;
      int ia = poly[(i + n - 1) % n], ib = poly[i], ic = poly[(i + 1) % n];
      const P2 &a = q[ia], &b = q[ib], &c = q[ic];
      bool ok = true;
      for (size_t k = 0; k < n && ok; ++k) {
        if (!reflex[k]) continue;
        int ik = poly[k];
        if (ik == ia || ik == ib || ik == ic) continue;
        if (in_triangle(a, b, c, q[ik])) ok = false;
      }
      if (!ok) continue;
      out.push_back({ia, ib, ic});
      poly.erase(poly.begin() + i);
      clipped = true;
      break;
    }
    if (!clipped) {
      size_t best = 0;
      double bo = -1e300;
      for (size_t i = 0; i < n; ++i) {
        double o = orient(q[poly[(i + n - 1) % n]], q[poly[i]], q[poly[(i + 1) % n]]);
        if (o > bo) { bo = o; best = i; }
      }
      int ia = poly[(best + n - 1) % n], ib = poly[best], ic = poly[(best + 1) % n];
      if (ia != ib && ib != ic && ia != ic) out.push_back({ia, ib, ic});
      poly.erase(poly.begin() + best);
    }
  }
  if (poly.size() == 3 && poly[0] != poly[1] && poly[1] != poly[2] && poly[0] != poly[2])
    out.push_back({poly[0], poly[1], poly[2]});
}

// Splice a CW hole into a CCW outer polygon through a mutually visible pair.
void bridge_hole(const std::vector<P2>& q, std::vector<int>& outer, const std::vector<int>& hole) {
  size_t hm = 0;
  for (size_t i = 1; i < hole.size(); ++i)
    if (q[hole[i]].x > q[hole[hm]].x) hm = i;
  const P2 M = q[hole[hm]];
  // Closest outer vertex to M that is visible (no outer edge crosses M-V).
  size_t best = 0;
  double bd = 1e300;
  for (size_t i = 0; i < outer.size(); ++i) {
    const P2& V = q[outer[i]];
    double d = (V.x - M.x) * (V.x - M.x) + (V.y - M.y) * (V.y - M.y);
    if (d >= bd) continue;
    bool vis = true;
    for (size_t k = 0; k < outer.size() && vis; ++k) {
      int a = outer[k], b = outer[(k + 1) % outer.size()];
      if (a == outer[i] || b == outer[i]) continue;
      const P2 &A = q[a], &B = q[b];
      double o1 = orient(M, V, A), o2 = orient(M, V, B), o3 = orient(A, B, M), o4 = orient(A, B, V);
      if (((o1 > 0) != (o2 > 0)) && ((o3 > 0) != (o4 > 0))) vis = false;
    }
    if (vis) {
      bd = d;
      best = i;
    }
  }
  std::vector<int> merged(outer.begin(), outer.begin() + best + 1);
  for (size_t k = 0; k <= hole.size(); ++k) merged.push_back(hole[(hm + k) % hole.size()]);
  merged.push_back(outer[best]);
  merged.insert(merged.end(), outer.begin() + best + 1, outer.end());
  outer.swap(merged);
}

}  // namespace

bool triangulate_border_2d(const std::vector<double>& xy, const std::vector<std::pair<int, int>>& bedges0,
                           std::vector<Tri>& tris) {
  const int nb = (int)(xy.size() / 2);
  std::vector<P2> q(nb);
  for (int i = 0; i < nb; ++i) q[i] = {xy[2 * i], xy[2 * i + 1]};
  std::vector<std::pair<int, int>> bedges;
  for (auto& e : bedges0) bedges.push_back({e.first + 1, e.second + 1});
  // Faces of the planar border graph: unique undirected edges, neighbours
  // sorted by angle, half-edges walked with the face on the left.
  std::vector<std::vector<int>> adj(nb);
  {
    std::set<std::pair<int, int>> seen;
    for (auto& e : bedges) {
      int a = e.first - 1, b = e.second - 1;
      if (a < 0 || b < 0 || a >= nb || b >= nb || a == b) continue;
      if (!seen.insert(std::minmax(a, b)).second) continue;
      adj[a].push_back(b);
      adj[b].push_back(a);
    }
  }
  for (int v = 0; v < nb; ++v)
    std::sort(adj[v].begin(), adj[v].end(), [&](int x, int y) {
      return std::atan2(q[x].y - q[v].y, q[x].x - q[v].x) < std::atan2(q[y].y - q[v].y, q[y].x - q[v].x);
    });
  std::vector<std::vector<char>> used(nb);
  for (int v = 0; v < nb; ++v) used[v].assign(adj[v].size(), 0);
  auto slot_of = [&](int v, int w) {
    for (size_t k = 0; k < adj[v].size(); ++k)
      if (adj[v][k] == w) return (int)k;
    return -1;
  };
  std::vector<std::vector<int>> cycles;
  for (int u0 = 0; u0 < nb; ++u0)
    for (size_t k0 = 0; k0 < adj[u0].size(); ++k0) {
      if (used[u0][k0]) continue;
      std::vector<int> cyc;
      int u = u0, k = (int)k0;
      bool ok = false;
      for (int guard = 0; guard < 4 * nb + 8; ++guard) {
        used[u][k] = 1;
        cyc.push_back(u);
        int v = adj[u][k];
        int pos = slot_of(v, u);
        if (pos < 0) break;
        int deg = (int)adj[v].size();
        int nk = (pos - 1 + deg) % deg;  // next neighbour clockwise from u
        u = v;
        k = nk;
        if (u == u0 && k == (int)k0) {
          ok = true;
          break;
        }
        if (used[u][k]) break;
      }
      if (ok && cyc.size() >= 3) cycles.push_back(cyc);
    }
  if (cycles.empty()) return false;
  // Even-odd test against every border edge.
  auto parity = [&](P2 p) {
    bool in = false;
    for (int a = 0; a < nb; ++a)
      for (int b : adj[a]) {
        if (b < a) continue;
        const P2 &A = q[a], &B = q[b];
        if ((A.y > p.y) != (B.y > p.y) && p.x < (B.x - A.x) * (p.y - A.y) / (B.y - A.y) + A.x) in = !in;
      }
    return in;
  };
  const size_t nc = cycles.size();
  std::vector<double> ar(nc);
  for (size_t i = 0; i < nc; ++i) ar[i] = area2(q, cycles[i]);
  std::vector<char> solid(nc, 0);
  for (size_t i = 0; i < nc; ++i) {
    if (ar[i] <= 0) continue;
    // A point just left of the longest boundary edge lies inside this face.
    const auto& c = cycles[i];
    size_t best = 0;
    double bl = -1;
    for (size_t k = 0; k < c.size(); ++k) {
      const P2 &A = q[c[k]], &B = q[c[(k + 1) % c.size()]];
      double l = std::hypot(B.x - A.x, B.y - A.y);
      if (l > bl) { bl = l; best = k; }
    }
    const P2 &A = q[c[best]], &B = q[c[(best + 1) % c.size()]];
    P2 m = {(A.x + B.x) / 2 - (B.y - A.y) * 1e-4, (A.y + B.y) / 2 + (B.x - A.x) * 1e-4};
    solid[i] = parity(m);
  }
  for (size_t i = 0; i < nc; ++i) {
    if (ar[i] <= 0 || !solid[i]) continue;
    std::vector<int> outer = cycles[i];
    // Holes: clockwise cycles whose smallest enclosing face is this one.
    std::vector<std::vector<int>> holes;
    for (size_t j = 0; j < nc; ++j) {
      if (ar[j] >= 0) continue;
      const P2 probe = q[cycles[j][0]];
      int owner = -1;
      for (size_t f = 0; f < nc; ++f) {
        if (ar[f] <= 0) continue;
        bool shares = false;
        for (int v : cycles[f])
          if (v == cycles[j][0]) { shares = true; break; }
        if (shares || !point_in_loop(q, cycles[f], probe)) continue;
        if (owner < 0 || ar[f] < ar[owner]) owner = (int)f;
      }
      if (owner == (int)i) holes.push_back(cycles[j]);
    }
    std::sort(holes.begin(), holes.end(), [&](const std::vector<int>& a, const std::vector<int>& b) {
      double ma = -1e300, mb = -1e300;
      for (int v : a) ma = std::max(ma, q[v].x);
      for (int v : b) mb = std::max(mb, q[v].x);
      return ma > mb;
    });
    for (auto& h : holes) bridge_hole(q, outer, h);
    ear_clip(q, outer, tris);
  }
  return true;
}

}  // namespace visacd

// Convex hull of a point set (3D QuickHull, Barber et al. 1996) with a flat
// fallback for coplanar input.
//
// Stands in for qhull "Qt Pp" (lib/src/core.cpp:59-111): like that call the
// returned mesh keeps every input point as a vertex and lists triangulated hull
// facets; with fix_normals the facets are oriented away from the vertex
// centroid (lib/src/core.cpp:33-57).
#include <algorithm>
#include <cmath>
#include <vector>

#include "geometry.hpp"

namespace visacd {

namespace {

// A face; its outside set is the segment [out, out + nout) of the hull's
// append-only pool (each face's set is written once, when the face is made).
struct Face {
  int v[3];
  int nb[3];  // neighbour across edge (v[e], v[(e+1)%3])
  Vec3 n;
  double off;
  int out = 0, nout = 0;
  bool alive = true;
  int visit = -1;
};

struct Hull {
  const std::vector<Vec3>& P;
  std::vector<Face> F;
  std::vector<int> pool;
  double eps;
  explicit Hull(const std::vector<Vec3>& p) : P(p) {}

  int add_face(int a, int b, int c) {
    Face f;
    f.v[0] = a;
    f.v[1] = b;
    f.v[2] = c;
    f.nb[0] = f.nb[1] = f.nb[2] = -1;
    Vec3 n = cross(P[b] - P[a], P[c] - P[a]);
    double l = norm(n);
    f.n = l > 0 ? n / l : Vec3{0, 0, 0};
    f.off = dot(f.n, P[a]);
    F.push_back(f);
    return (int)F.size() - 1;
  }
  double dist(int f, int p) const { return dot(F[f].n, P[p]) - F[f].off; }
  // Each of pts goes to the first of the faces f0..f0+L-1 with the largest
  // distance above eps (or nowhere); every face's set is then appended to the
  // pool in point order. best is scratch.
  void assign(const int* pts, int m, int f0, int L, std::vector<int>& best) {
    best.resize(m);
    for (int q = 0; q < L; ++q) F[f0 + q].nout = 0;
    for (int k = 0; k < m; ++k) {
      int bf = -1;
      double bd = eps;
      for (int q = 0; q < L; ++q) {
        const double d = dist(f0 + q, pts[k]);
        if (d > bd) {
          bd = d;
          bf = q;
        }
      }
      best[k] = bf;
      if (bf >= 0) ++F[f0 + bf].nout;
    }
    int top = (int)pool.size();
    for (int q = 0; q < L; ++q) {
      F[f0 + q].out = top;
      top += F[f0 + q].nout;
      F[f0 + q].nout = 0;
    }
    pool.resize(top);
    for (int k = 0; k < m; ++k)
      if (best[k] >= 0) {
        Face& f = F[f0 + best[k]];
        pool[f.out + f.nout++] = pts[k];
      }
  }
};

void link(std::vector<Face>& F, int f, int a, int b, int g) {
  for (int e = 0; e < 3; ++e)
    if (F[f].v[e] == a && F[f].v[(e + 1) % 3] == b) {
      F[f].nb[e] = g;
      return;
    }
}

Mesh flat_hull(const std::vector<Vec3>& pts, bool fix_normals);

}  // namespace

Mesh convex_hull(const std::vector<Vec3>& pts, bool fix_normals) {
  Mesh out;
  out.vertices = pts;
  const int n = (int)pts.size();
  if (n < 3) return out;
  // Scale-aware tolerance.
  double ext = 0;
  for (const auto& p : pts)
    for (int a = 0; a < 3; ++a) ext = std::max(ext, std::fabs(p[a]));
  const double eps = std::max(ext, 1e-300) * 1e-11;
  // Initial simplex: extreme pair, farthest from the line, farthest from the plane.
  int ex[6] = {0, 0, 0, 0, 0, 0};
  for (int i = 0; i < n; ++i)
    for (int a = 0; a < 3; ++a) {
      if (pts[i][a] < pts[ex[2 * a]][a]) ex[2 * a] = i;
      if (pts[i][a] > pts[ex[2 * a + 1]][a]) ex[2 * a + 1] = i;
    }
  int i0 = ex[0], i1 = ex[1];
  double best = -1;
  for (int a = 0; a < 6; ++a)
    for (int b = a + 1; b < 6; ++b) {
      double d = norm(pts[ex[a]] - pts[ex[b]]);
      if (d > best) {
        best = d;
        i0 = ex[a];
        i1 = ex[b];
      }
    }
  if (best <= eps) return out;
  Vec3 dir = (pts[i1] - pts[i0]) / best;
  int i2 = -1;
  best = eps;
  for (int i = 0; i < n; ++i) {
    Vec3 w = pts[i] - pts[i0];
    double d = norm(w - dir * dot(w, dir));
    if (d > best) {
      best = d;
      i2 = i;
    }
  }
  if (i2 < 0) return out;  // collinear
  Vec3 nrm = normalized(cross(pts[i1] - pts[i0], pts[i2] - pts[i0]));
  int i3 = -1;
  best = eps;
  for (int i = 0; i < n; ++i) {
    double d = std::fabs(dot(nrm, pts[i] - pts[i0]));
    if (d > best) {
      best = d;
      i3 = i;
    }
  }
  if (i3 < 0) return flat_hull(pts, fix_normals);

  Hull H(pts);
  H.eps = eps;
  // Orient the tetrahedron's faces outward.
  if (dot(nrm, pts[i3] - pts[i0]) > 0) std::swap(i1, i2);
  int f0 = H.add_face(i0, i1, i2);
  int f1 = H.add_face(i0, i3, i1);
  int f2 = H.add_face(i1, i3, i2);
  int f3 = H.add_face(i2, i3, i0);
  auto& F = H.F;
  // Neighbour links by shared (reversed) edges.
  for (int a = 0; a < 4; ++a)
    for (int e = 0; e < 3; ++e) {
      int u = F[a].v[e], w = F[a].v[(e + 1) % 3];
      for (int b = 0; b < 4; ++b) {
        if (a == b) continue;
        for (int e2 = 0; e2 < 3; ++e2)
          if (F[b].v[e2] == w && F[b].v[(e2 + 1) % 3] == u) F[a].nb[e] = b;
      }
    }
  (void)f0;
  (void)f1;
  (void)f2;
  (void)f3;
  H.F.reserve((size_t)8 * n + 64);
  H.pool.reserve((size_t)4 * n + 64);
  std::vector<int> choice, orphans, stack, visible, nf;
  {
    std::vector<int> rest;
    rest.reserve(n);
    for (int i = 0; i < n; ++i)
      if (i != i0 && i != i1 && i != i2 && i != i3) rest.push_back(i);
    H.assign(rest.data(), (int)rest.size(), 0, 4, choice);
  }
  std::vector<std::pair<int, int>> horizon, loop;  // (face, edge) on the visible side
  std::vector<char> used;
  int iter = 0;
  for (size_t cur = 0; cur < F.size(); ++cur) {
    if (!F[cur].alive || F[cur].nout == 0) continue;
    if (++iter > 4 * n + 64) break;
    // Farthest outside point of this face.
    int apex = -1;
    double bd = -1;
    for (int k = 0; k < F[cur].nout; ++k) {
      const int p = H.pool[F[cur].out + k];
      double d = H.dist((int)cur, p);
      if (d > bd) {
        bd = d;
        apex = p;
      }
    }
    // Visible set by flood fill from cur.
    visible.clear();
    horizon.clear();
    stack.assign(1, (int)cur);
    F[cur].visit = iter;
    while (!stack.empty()) {
      int f = stack.back();
      stack.pop_back();
      visible.push_back(f);
      for (int e = 0; e < 3; ++e) {
        int g = F[f].nb[e];
        if (g < 0 || F[g].visit == iter) continue;
        if (H.dist(g, apex) > eps) {
          F[g].visit = iter;
          stack.push_back(g);
        } else {
          horizon.push_back({f, e});
        }
      }
    }
    // Order the horizon as a loop: edge (u, w) of face f seen from outside.
    loop.clear();
    {
      used.assign(horizon.size(), 0);
      loop.push_back(horizon[0]);
      used[0] = 1;
      for (size_t k = 1; k < horizon.size(); ++k) {
        int w = F[loop.back().first].v[(loop.back().second + 1) % 3];
        bool found = false;
        for (size_t h = 0; h < horizon.size(); ++h) {
          if (used[h]) continue;
          if (F[horizon[h].first].v[horizon[h].second] == w) {
            loop.push_back(horizon[h]);
            used[h] = 1;
            found = true;
            break;
          }
        }
        if (!found) break;
      }
      if (loop.size() != horizon.size()) {  // numerically inconsistent horizon
        F[cur].nout = 0;
        continue;
      }
    }
    // Collect orphaned outside points.
    orphans.clear();
    for (int f : visible) {
      F[f].alive = false;
      for (int k = 0; k < F[f].nout; ++k) {
        const int p = H.pool[F[f].out + k];
        if (p != apex) orphans.push_back(p);
      }
      F[f].nout = 0;
    }
    // New faces (u, w, apex) for each horizon edge.
    nf.resize(loop.size());
    const int first = (int)F.size();
    for (size_t k = 0; k < loop.size(); ++k) {
      int f = loop[k].first, e = loop[k].second;
      int u = F[f].v[e], w = F[f].v[(e + 1) % 3];
      int g = F[f].nb[e];
      int nfi = H.add_face(u, w, apex);
      nf[k] = nfi;
      F[nfi].nb[0] = g;
      link(F, g, w, u, nfi);
    }
    for (size_t k = 0; k < loop.size(); ++k) {
      int a = nf[k], b = nf[(k + 1) % loop.size()];
      F[a].nb[1] = b;  // edge (w, apex) shared with the next face's (apex, u')
      F[b].nb[2] = a;
    }
    H.assign(orphans.data(), (int)orphans.size(), first, (int)loop.size(), choice);
  }
  for (const auto& f : F)
    if (f.alive) out.triangles.push_back({f.v[0], f.v[1], f.v[2]});
  if (fix_normals) {
    Vec3 c = {0, 0, 0};
    for (const auto& v : out.vertices) c = c + v;
    c = c / (double)out.vertices.size();
    for (auto& t : out.triangles) {
      Vec3 nn = cross(out.vertices[t[1]] - out.vertices[t[0]], out.vertices[t[2]] - out.vertices[t[0]]);
      if (dot(nn, c - out.vertices[t[0]]) > 0) std::swap(t[1], t[2]);
    }
  }
  return out;
}

namespace {

// Coplanar input: 2D hull in the plane, closed as two opposite fans.
Mesh flat_hull(const std::vector<Vec3>& pts, bool fix_normals) {
  (void)fix_normals;
  Mesh out;
  out.vertices = pts;
  const int n = (int)pts.size();
  Vec3 o = pts[0];
  int ia = 0;
  double bd = -1;
  for (int i = 0; i < n; ++i) {
    double d = norm(pts[i] - o);
    if (d > bd) { bd = d; ia = i; }
  }
  Vec3 u = normalized(pts[ia] - o);
  Vec3 nrm = {0, 0, 0};
  bd = -1;
  for (int i = 0; i < n; ++i) {
    Vec3 c = cross(u, pts[i] - o);
    if (norm(c) > bd) { bd = norm(c); nrm = c; }
  }
  if (bd <= 0) return out;
  nrm = normalized(nrm);
  Vec3 v = cross(nrm, u);
  std::vector<std::pair<std::pair<double, double>, int>> q(n);
  for (int i = 0; i < n; ++i) q[i] = {{dot(pts[i] - o, u), dot(pts[i] - o, v)}, i};
  std::sort(q.begin(), q.end());
  auto crs = [&](int a, int b, int c) {
    return (q[b].first.first - q[a].first.first) * (q[c].first.second - q[a].first.second) -
           (q[b].first.second - q[a].first.second) * (q[c].first.first - q[a].first.first);
  };
  std::vector<int> h;
  for (int pass = 0; pass < 2; ++pass) {
    size_t start = h.size();
    for (int k = 0; k < n; ++k) {
      int i = pass == 0 ? k : n - 1 - k;
      while (h.size() >= start + 2 && crs(h[h.size() - 2], h.back(), i) <= 0) h.pop_back();
      h.push_back(i);
    }
    h.pop_back();
  }
  if (h.size() < 3) return out;
  for (size_t k = 1; k + 1 < h.size(); ++k) {
    int a = q[h[0]].second, b = q[h[k]].second, c = q[h[k + 1]].second;
    out.triangles.push_back({a, b, c});
    out.triangles.push_back({a, c, b});
  }
  return out;
}

}  // namespace

}  // namespace visacd

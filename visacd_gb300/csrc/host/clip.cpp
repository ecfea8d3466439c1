// Split a triangle mesh by a plane into its positive and negative parts and
// close both with a cap in the plane.
//
// Semantics of lib/src/clip.cpp:190-741 (itself derived from CoACD): vertices
// are classified with the 1e-6 side test; triangles wholly on one side (zero
// vertices allowed) go to that side with their on-plane vertices replaced by
// border points; crossing triangles are split at the plane through the
// segment intersections (with the reference's per-case vertex orders, because
// triangle order and winding feed the seeded sampling downstream). Border
// points are deduplicated by vertex / edge key and by position (1e-4 per
// coordinate, first match wins). The cap is a constrained triangulation of the
// border edges in the plane frame of lib/src/clip.cpp:19-120; the CDT library
// the reference uses is absent here, so the cap is this project's own: the
// faces of the planar border graph are traced (angle-sorted half-edges), a face
// is filled when an interior point has odd crossing parity against all border
// edges (the even-odd rule of CDT's eraseOuterTrianglesAndHoles), islands
// inside a filled face are bridged in as holes, and the result is ear-clipped.
#include <algorithm>
#include <cmath>
#include <map>
#include <set>
#include <vector>

#include "geometry.hpp"

namespace visacd {

namespace {

struct Border {
  std::vector<Vec3> pts;
  std::map<int, int> vmap;                  // mesh vertex -> border point
  std::map<std::pair<int, int>, int> emap;  // directed mesh edge -> border point

  int find_near(const Vec3& p) const {
    for (int i = 0; i < (int)pts.size(); ++i)
      if (std::fabs(pts[i][0] - p[0]) < 1e-4 && std::fabs(pts[i][1] - p[1]) < 1e-4 &&
          std::fabs(pts[i][2] - p[2]) < 1e-4)
        return i;
    return -1;
  }
  // Border point of a mesh vertex lying on the plane.
  int vertex_point(int id, const Vec3& p) {
    auto it = vmap.find(id);
    if (it != vmap.end()) return it->second;
    int f = find_near(p);
    if (f < 0) {
      f = (int)pts.size();
      pts.push_back(p);
    }
    vmap[id] = f;
    return f;
  }
  // Border point where mesh edge (a, b) crosses the plane.
  int edge_point(int a, int b, const Vec3& p) {
    auto it = emap.find({a, b});
    if (it != emap.end()) return it->second;
    it = emap.find({b, a});
    if (it != emap.end()) return it->second;
    int f = find_near(p);
    if (f < 0) {
      f = (int)pts.size();
      pts.push_back(p);
    }
    emap[{a, b}] = f;
    emap[{b, a}] = f;
    return f;
  }
  void force_edge(int a, int b, int v) {
    emap[{a, b}] = v;
    emap[{b, a}] = v;
  }
  int edge(int a, int b) { return emap[{a, b}]; }
};

// Plane-line intersection of segment p1-p2, accepted when it lies in the
// segment's bounding box widened by eps (lib/include/core.hpp:187-210 form).
bool intersect_segment(const Plane& pl, const Vec3& p1, const Vec3& p2, Vec3& pi,
                       double eps = 1e-6) {
  const double a = pl.a, b = pl.b, c = pl.c, d = pl.d;
  const double den = a * p2[0] - a * p1[0] + b * p2[1] - b * p1[1] + c * p2[2] - c * p1[2];
  pi[0] = (p1[0] * b * p2[1] + p1[0] * c * p2[2] + p1[0] * d - p2[0] * b * p1[1] -
           p2[0] * c * p1[2] - p2[0] * d) / den;
  pi[1] = (a * p2[0] * p1[1] + c * p1[1] * p2[2] + p1[1] * d - a * p1[0] * p2[1] -
           c * p1[2] * p2[1] - p2[1] * d) / den;
  pi[2] = (a * p2[0] * p1[2] + b * p2[1] * p1[2] + p1[2] * d - a * p1[0] * p2[2] -
           b * p1[1] * p2[2] - p2[2] * d) / den;
  for (int k = 0; k < 3; ++k)
    if (!(std::min(p1[k] - eps, p2[k] - eps) <= pi[k] && pi[k] <= std::max(p1[k] + eps, p2[k] + eps)))
      return false;
  return true;
}

bool same_point(const Vec3& p, const Vec3& q) {
  const double eps = (double)1e-5f;
  return std::fabs(p[0] - q[0]) < eps && std::fabs(p[1] - q[1]) < eps && std::fabs(p[2] - q[2]) < eps;
}

// Orientation used when all three vertices lie on the plane
// (lib/include/core.hpp:169-176).
int coplanar_side(const Vec3& p0, const Vec3& p1, const Vec3& p2, const Plane& pl) {
  Vec3 n = face_normal(p0, p1, p2);
  if (n[0] * pl.a > 0 || n[1] * pl.b > 0 || n[2] * pl.c > 0) return -1;
  return 1;
}

// ---- cap triangulation (planar part in cap2d.cpp) ---------------------------
struct P2 {
  double x, y;
};

// Triangulate the region bounded by the border edges (1-based pairs) in the
// plane frame; triangles are CCW in that frame (like CDT output).
bool triangulate_cap(const std::vector<Vec3>& border, const std::vector<std::pair<int, int>>& bedges,
                     const Plane& plane, std::vector<Tri>& tris) {
  const int nb = (int)border.size();
  // Plane frame (lib/src/clip.cpp:19-120): idx1 = first point farther than
  // 0.01 from point 0, idx2 = first later point not collinear.
  int i1 = -1;
  for (int i = 1; i < nb; ++i)
    if (norm(border[0] - border[i]) > 0.01) { i1 = i; break; }
  if (i1 < 0) return false;
  int i2 = -1;
  for (int i = 2; i < nb; ++i) {
    if (i == i1) continue;
    Vec3 ab = border[i1] - border[0], bc = border[i] - border[i1];
    double r = dot(ab, bc) / (norm(ab) * norm(bc));
    if (std::fabs(std::fabs(r) - 1) > 1e-6 && std::fabs(r) < kInf) { i2 = i; break; }
  }
  if (i2 < 0) return false;
  Vec3 p0 = border[0], p1 = border[i1], p2 = border[i2];
  Vec3 nrm = face_normal(p0, p1, p2);
  if (nrm[0] * plane.a + nrm[1] * plane.b + nrm[2] * plane.c > 0) std::swap(p0, p2);
  Vec3 R0 = normalized(p0 - p1);
  Vec3 R2 = normalized(cross(R0, p2 - p0));
  Vec3 R1 = normalized(cross(R0, R2));
  std::vector<P2> q(nb);
  for (int i = 0; i < nb; ++i) {
    Vec3 w = border[i] - p0;
    q[i] = {dot(R0, w), dot(R1, w)};
  }
  std::vector<std::pair<int, int>> e0;
  e0.reserve(bedges.size());
  for (auto& e : bedges) e0.push_back({e.first - 1, e.second - 1});
  std::vector<double> xy(2 * (size_t)nb);
  for (int i = 0; i < nb; ++i) {
    xy[2 * i] = q[i].x;
    xy[2 * i + 1] = q[i].y;
  }
  return triangulate_border_2d(xy, e0, tris);
}

}  // namespace

// Parts from the GPU clip outputs: kept vertices in input order, border
// points appended to both, cap triangulated here (same tail as clip()).
MeshList assemble_clip(const Mesh& mesh, const Plane& plane, const std::vector<Tri>& pos_tris,
                       const std::vector<Tri>& neg_tris, const std::vector<int>& pos_map,
                       const std::vector<int>& neg_map, const std::vector<Vec3>& border,
                       const std::vector<std::pair<int, int>>& bedges) {
  const int N = (int)mesh.vertices.size();
  Mesh pos, neg;
  int np = 0, nn = 0;
  for (int i = 0; i < N; ++i) {
    if (pos_map[i]) {
      pos.vertices.push_back(mesh.vertices[i]);
      ++np;
    }
    if (neg_map[i]) {
      neg.vertices.push_back(mesh.vertices[i]);
      ++nn;
    }
  }
  if (np == 0 || nn == 0) return MeshList{mesh};
  std::vector<Tri> cap;
  if (border.size() > 2) triangulate_cap(border, bedges, plane, cap);
  const int nbp = (int)border.size();
  pos.is_new.assign(np + nbp, false);
  neg.is_new.assign(nn + nbp, false);
  for (int i = 0; i < nbp; ++i) {
    pos.vertices.push_back(border[i]);
    neg.vertices.push_back(border[i]);
    pos.is_new[np + i] = true;
    neg.is_new[nn + i] = true;
  }
  pos.triangles = pos_tris;
  neg.triangles = neg_tris;
  for (const auto& t : cap) {
    pos.triangles.push_back({np + t[0], np + t[1], np + t[2]});
    neg.triangles.push_back({nn + t[2], nn + t[1], nn + t[0]});
  }
  return MeshList{pos, neg};
}

MeshList clip(const Mesh& mesh, const Plane& plane, std::vector<int>& pos_map,
              std::vector<int>& neg_map) {
  const int N = (int)mesh.vertices.size();
  Mesh pos, neg;
  std::vector<char> in_pos(N, 0), in_neg(N, 0);
  std::vector<std::pair<int, int>> bedges;
  Border B;
  auto ref = [](int b) { return -b - 1; };  // border point reference in a triangle

  for (const auto& t : mesh.triangles) {
    const int id[3] = {t[0], t[1], t[2]};
    const Vec3 p[3] = {mesh.vertices[id[0]], mesh.vertices[id[1]], mesh.vertices[id[2]]};
    int s[3] = {plane.side(p[0]), plane.side(p[1]), plane.side(p[2])};
    if (s[0] == 0 && s[1] == 0 && s[2] == 0) s[0] = s[1] = s[2] = coplanar_side(p[0], p[1], p[2], plane);
    const int sum = s[0] + s[1] + s[2];
    const int nzero = (s[0] == 0) + (s[1] == 0) + (s[2] == 0);
    const bool one_side_pos = sum == 3 || sum == 2 || (sum == 1 && nzero == 2);
    const bool one_side_neg = sum == -3 || sum == -2 || (sum == -1 && nzero == 2);
    if (one_side_pos || one_side_neg) {
      const int sg = one_side_pos ? 1 : -1;
      Mesh& dst = one_side_pos ? pos : neg;
      std::vector<char>& keep = one_side_pos ? in_pos : in_neg;
      if (sum == sg) {  // one vertex off the plane, two on it
        int k = s[0] != 0 ? 0 : (s[1] != 0 ? 1 : 2);
        int k1 = (k + 1) % 3, k2 = (k + 2) % 3;
        // The positive side registers k+1 then k+2, the negative side the reverse.
        int b1, b2;
        if (sg > 0) {
          b1 = B.vertex_point(id[k1], p[k1]);
          b2 = B.vertex_point(id[k2], p[k2]);
        } else {
          b2 = B.vertex_point(id[k2], p[k2]);
          b1 = B.vertex_point(id[k1], p[k1]);
        }
        if (b1 != b2) {
          if (sg > 0) bedges.push_back({b1 + 1, b2 + 1});
          else bedges.push_back({b2 + 1, b1 + 1});
          dst.triangles.push_back({id[k], ref(b1), ref(b2)});
          keep[id[k]] = 1;
        }
      } else if (sum == 2 * sg) {  // two vertices off the plane, one on it
        int z = s[0] == 0 ? 0 : (s[1] == 0 ? 1 : 2);
        int bz = B.vertex_point(id[z], p[z]);
        if (z == 2) dst.triangles.push_back({id[0], id[1], ref(bz)});
        else if (z == 0) dst.triangles.push_back({id[1], id[2], ref(bz)});
        else dst.triangles.push_back({id[0], ref(bz), id[2]});
        for (int k = 0; k < 3; ++k)
          if (k != z) keep[id[k]] = 1;
      } else {  // wholly on one side
        dst.triangles.push_back(t);
        keep[id[0]] = keep[id[1]] = keep[id[2]] = 1;
      }
      continue;
    }
    // Crossing triangle.
    Vec3 pi[3];
    bool f[3];
    for (int e = 0; e < 3; ++e) f[e] = intersect_segment(plane, p[e], p[(e + 1) % 3], pi[e]);
    // Two crossed edges e and e+1 sharing vertex v = e+1 (the apex); the third
    // edge is uncrossed.
    int e = -1;
    if (f[0] && f[1] && !f[2]) e = 0;
    else if (f[1] && f[2] && !f[0]) e = 1;
    else if (f[2] && f[0] && !f[1]) e = 2;
    if (e >= 0) {
      const int a = e, v = (e + 1) % 3, c = (e + 2) % 3;  // edges (a,v) and (v,c)
      B.edge_point(id[a], id[v], pi[a]);
      B.edge_point(id[v], id[c], pi[v]);
      const int fa = B.edge(id[a], id[v]), fv = B.edge(id[v], id[c]);
      const bool apex_pos = s[v] == 1;
      Mesh& apex_dst = apex_pos ? pos : neg;
      Mesh& base_dst = apex_pos ? neg : pos;
      std::vector<char>& apex_keep = apex_pos ? in_pos : in_neg;
      std::vector<char>& base_keep = apex_pos ? in_neg : in_pos;
      // The base quad (c, a, fa, fv) is split along a-fv when the crossed
      // edges are (0,1),(1,2), and along c-fa otherwise (the reference's
      // per-case choice).
      if (fv != fa) {
        if (apex_pos) bedges.push_back({fv + 1, fa + 1});
        else bedges.push_back({fa + 1, fv + 1});
        apex_keep[id[v]] = 1;
        base_keep[id[a]] = base_keep[id[c]] = 1;
        apex_dst.triangles.push_back({id[v], ref(fv), ref(fa)});
        if (e == 0) {
          base_dst.triangles.push_back({id[a], ref(fa), ref(fv)});
          base_dst.triangles.push_back({ref(fv), id[c], id[a]});
        } else {
          base_dst.triangles.push_back({id[c], ref(fa), ref(fv)});
          base_dst.triangles.push_back({ref(fa), id[c], id[a]});
        }
      } else {
        base_keep[id[a]] = base_keep[id[c]] = 1;
        base_dst.triangles.push_back({e == 0 ? ref(fv) : ref(fa), id[c], id[a]});
      }
      continue;
    }
    if (!(f[0] && f[1] && f[2])) continue;
    const bool all_nz = s[0] != 0 && s[1] != 0 && s[2] != 0;
    // The plane passes through vertex k: the crossing is the opposite edge.
    int k = -1;
    if (s[0] == 0 || (all_nz && same_point(pi[0], pi[2]))) k = 0;
    else if (s[1] == 0 || (all_nz && same_point(pi[0], pi[1]))) k = 1;
    else if (s[2] == 0 || (all_nz && same_point(pi[1], pi[2]))) k = 2;
    if (k < 0) continue;
    const int k1 = (k + 1) % 3, k2 = (k + 2) % 3;
    const int bk = B.vertex_point(id[k], p[k]);
    B.force_edge(id[k], id[k1], bk);
    B.force_edge(id[k2], id[k], bk);
    B.edge_point(id[k1], id[k2], pi[k1]);
    const int fo = B.edge(id[k1], id[k2]);
    // Which of the two other vertices is positive decides the split.
    // k == 0 tests s[1]; k == 1 and k == 2 test s[0].
    const int test = (k == 0) ? s[1] : s[0];
    // u: vertex whose side is tested; `other`: the remaining off-plane vertex.
    const int u = (k == 1) ? k2 : k1;
    // Border point order of the triangles per case (lib/src/clip.cpp:477-599).
    int A, Bp;  // (first, second) border refs of the triangle at u
    if (k == 0) { A = fo; Bp = bk; }
    else if (k == 1) { A = bk; Bp = fo; }
    else { A = fo; Bp = bk; }
    const int other = (k == 1) ? k1 : k2;
    if (test == 1) {
      if (A != Bp) {
        bedges.push_back({A + 1, Bp + 1});
        in_pos[id[u]] = 1;
        in_neg[id[other]] = 1;
        pos.triangles.push_back({id[u], ref(A), ref(Bp)});
        neg.triangles.push_back({id[other], ref(Bp), ref(A)});
      }
    } else {
      if (Bp != A) {
        bedges.push_back({Bp + 1, A + 1});
        in_neg[id[u]] = 1;
        in_pos[id[other]] = 1;
        neg.triangles.push_back({id[u], ref(A), ref(Bp)});
        pos.triangles.push_back({id[other], ref(Bp), ref(A)});
      }
    }
  }

  // Unique border edges (first occurrence of each unordered pair).
  {
    std::set<std::pair<int, int>> seen;
    std::vector<std::pair<int, int>> uniq;
    for (auto& e : bedges)
      if (seen.insert(std::minmax(e.first, e.second)).second) uniq.push_back(e);
    bedges.swap(uniq);
  }
  std::vector<Tri> cap;
  if (B.pts.size() > 2) triangulate_cap(B.pts, bedges, plane, cap);

  pos_map.assign(N, 0);
  neg_map.assign(N, 0);
  int np = 0, nn = 0;
  for (int i = 0; i < N; ++i) {
    if (in_pos[i]) {
      pos.vertices.push_back(mesh.vertices[i]);
      pos_map[i] = ++np;
    }
    if (in_neg[i]) {
      neg.vertices.push_back(mesh.vertices[i]);
      neg_map[i] = ++nn;
    }
  }
  if (np == 0 || nn == 0) return MeshList{mesh};
  const int nbp = (int)B.pts.size();
  pos.is_new.assign(np + nbp, false);
  neg.is_new.assign(nn + nbp, false);
  for (int i = 0; i < nbp; ++i) {
    pos.vertices.push_back(B.pts[i]);
    neg.vertices.push_back(B.pts[i]);
    pos.is_new[np + i] = true;
    neg.is_new[nn + i] = true;
  }
  auto remap = [](Mesh& m, const std::vector<int>& proj, int base) {
    for (auto& t : m.triangles)
      for (int k = 0; k < 3; ++k) t[k] = t[k] >= 0 ? proj[t[k]] - 1 : -t[k] + base - 1;
  };
  remap(pos, pos_map, np);
  remap(neg, neg_map, nn);
  for (const auto& t : cap) {
    pos.triangles.push_back({np + t[0], np + t[1], np + t[2]});
    neg.triangles.push_back({nn + t[2], nn + t[1], nn + t[0]});
  }
  return MeshList{pos, neg};
}

}  // namespace visacd

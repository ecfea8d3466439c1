// Stand-in for the CDT library API used by lib/src/clip.cpp:153-187: collects
// vertices and constraint edges and fills `triangles` with this project's
// planar-graph cap triangulation (even-odd fill, like eraseOuterTrianglesAndHoles).
#pragma once
#include <array>
#include <utility>
#include <vector>

namespace visacd {
using Tri = std::array<int, 3>;
bool triangulate_border_2d(const std::vector<double>& xy, const std::vector<std::pair<int, int>>& edges,
                           std::vector<Tri>& tris);
}  // namespace visacd

namespace CDT {
enum class VertexInsertionOrder { AsProvided, Auto };
template <typename T> struct V2d { T x, y; };
struct Triangle { std::array<unsigned int, 3> vertices; };

template <typename T> class Triangulation {
 public:
  std::vector<V2d<T>> vertices;
  std::vector<Triangle> triangles;
  explicit Triangulation(VertexInsertionOrder) {}
  template <class It, class GX, class GY> void insertVertices(It b, It e, GX gx, GY gy) {
    for (; b != e; ++b) vertices.push_back({gx(*b), gy(*b)});
  }
  template <class It, class GS, class GE> void insertEdges(It b, It e, GS gs, GE ge) {
    for (; b != e; ++b) edges_.push_back({(int)gs(*b), (int)ge(*b)});
  }
  void eraseOuterTrianglesAndHoles() {
    std::vector<double> xy;
    for (auto& v : vertices) { xy.push_back(v.x); xy.push_back(v.y); }
    std::vector<visacd::Tri> t;
    visacd::triangulate_border_2d(xy, edges_, t);
    for (auto& x : t) triangles.push_back({{(unsigned)x[0], (unsigned)x[1], (unsigned)x[2]}});
  }
 private:
  std::vector<std::pair<int, int>> edges_;
};
}  // namespace CDT

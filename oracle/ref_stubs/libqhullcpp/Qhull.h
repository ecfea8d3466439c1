// Stand-in for the qhull C++ API used by lib/src/core.cpp:59-97: runQhull
// computes this project's convex hull; like "Qt Pp" the point list is the
// input and facets are triangles. Degenerate input throws, as qhull does.
#pragma once
#include <array>
#include <stdexcept>
#include <vector>

namespace visacd {
std::vector<std::array<int, 3>> hull_facets_for_ref(const std::vector<double>& coords);
}

typedef double coordT;
namespace orgQhull {
struct QhullPoint { int i; int id() const { return i; } };
struct QhullVertex { int i; QhullPoint point() const { return {i}; } };
struct QhullVertexSet {
  std::array<int, 3> v;
  int size() const { return 3; }
  struct It { const int* p; QhullVertex operator*() const { return {*p}; } It& operator++() { ++p; return *this; } bool operator!=(const It& o) const { return p != o.p; } };
  It begin() const { return {v.data()}; }
  It end() const { return {v.data() + 3}; }
};
struct QhullFacet {
  std::array<int, 3> v;
  bool isGood() const { return true; }
  QhullVertexSet vertices() const { return {v}; }
};
class Qhull {
 public:
  void runQhull(const char*, int dim, int n, const coordT* pts, const char*) {
    coords_.assign(pts, pts + (size_t)dim * n);
    auto f = visacd::hull_facets_for_ref(coords_);
    if (f.empty()) throw std::runtime_error("QH6154 qhull stand-in: degenerate input");
    for (auto& t : f) facets_.push_back({t});
  }
  coordT* pointCoordinateBegin() { return coords_.data(); }
  coordT* pointCoordinateEnd() { return coords_.data() + coords_.size(); }
  const std::vector<QhullFacet>& facetList() const { return facets_; }
 private:
  std::vector<coordT> coords_;
  std::vector<QhullFacet> facets_;
};
}  // namespace orgQhull

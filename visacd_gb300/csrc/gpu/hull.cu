// Convex hulls of many point sets in one launch: Mesh::compute_ch
// (lib/src/core.cpp:59-111) for every part of a batch, with this project's
// QuickHull (Barber et al. 1996) standing in for qhull "Qt Pp".
//
// The result must equal the host QuickHull (host/hull.cpp) triangle for
// triangle and in the same order: the hull's triangle list decides the random
// samples of the concavity metric (area-weighted draws over the triangles in
// order). So each part runs the same sequence of steps as the host, one warp
// per part:
//  * data-parallel across the 32 lanes, with the host's first-index tie
//    rules: the coordinate extremes, the farthest-from-line and
//    farthest-from-plane points of the initial simplex, the farthest outside
//    point of a face, the assignment of points to faces (the first face with
//    the largest distance above eps) and the stable scatter of each face's
//    outside list in point order (match-any ranks, so every list keeps the
//    host's order), the new faces' planes, the final compaction of live faces
//    in creation order and the orientation fix;
//  * sequential in lane 0, in the host's order: the depth-first flood fill of
//    visible faces, the horizon list and its loop order, face creation and
//    neighbour linking, the centroid sum of the orientation fix and the 2D
//    monotone chain of coplanar input.
// Faces are never reused: the host processes faces in creation order, and
// face ids here are creation indices, so both visit the same faces in the same
// order. Outside lists are append-only segments of a per-part pool.
// All arithmetic is FP64 with explicit round-to-nearest intrinsics in the
// host's operation order (no contraction), sqrt and division correctly
// rounded, so every distance, plane and decision equals the host's.
// Capacities (faces, pool, lists) are multiples of the part's point count;
// a part that outgrows them stops with a status code and the entry point runs
// it again with four times the room. Launches keep their work regions under
// 1 GiB, so large batches run as several launches.
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "geom64.cuh"

namespace vgpu {
namespace {

constexpr int kHullWarps = 4;  // parts in flight per block, one warp each
constexpr int kMaxHullMult = 16;  // with at most 2^22 points a part, every capacity fits in int32

enum : int32_t {
  kHullOk = 0,
  kHullFaceCap = 1,   // more faces than the face capacity
  kHullPoolCap = 2,   // outside-list pool full
  kHullListCap = 3,   // visible / stack / horizon list full
  kHullOutCap = 4,    // more live faces than 2n (cannot happen for a closed surface)
  kHullZeroNorm = 5,  // normalising a zero vector (the host throws there)
  kHullNumeric = 6,   // a face's outside point no longer lies outside it (non-finite planes)
};

struct D3 {
  double x, y, z;
};
struct __align__(16) HPlane {  // unit normal and offset of a face
  double x, y, z, w;
};
__device__ __forceinline__ D3 ld3(const double* P, int i) {
  return {P[3 * (int64_t)i], P[3 * (int64_t)i + 1], P[3 * (int64_t)i + 2]};
}
__device__ __forceinline__ D3 sub3(D3 a, D3 b) { return {ds(a.x, b.x), ds(a.y, b.y), ds(a.z, b.z)}; }
__device__ __forceinline__ double dot3(D3 a, D3 b) { return da(da(dm(a.x, b.x), dm(a.y, b.y)), dm(a.z, b.z)); }
__device__ __forceinline__ D3 cross3(D3 a, D3 b) {
  return {ds(dm(a.y, b.z), dm(a.z, b.y)), ds(dm(a.z, b.x), dm(a.x, b.z)), ds(dm(a.x, b.y), dm(a.y, b.x))};
}
__device__ __forceinline__ double norm3(D3 a) { return __dsqrt_rn(dot3(a, a)); }
__device__ __forceinline__ D3 div3(D3 a, double s) {
  return {__ddiv_rn(a.x, s), __ddiv_rn(a.y, s), __ddiv_rn(a.z, s)};
}
// dot(n, p) - off: the host's Hull::dist.
__device__ __forceinline__ double plane_dist(HPlane pl, D3 p) {
  return ds(da(da(dm(pl.x, p.x), dm(pl.y, p.y)), dm(pl.z, p.z)), pl.w);
}
// The host's add_face plane: unit normal of (b - a) x (c - a) (zero when the
// cross product is zero) and its offset at a.
__device__ __forceinline__ HPlane face_plane(const double* P, int a, int b, int c) {
  const D3 pa = ld3(P, a);
  D3 n = cross3(sub3(ld3(P, b), pa), sub3(ld3(P, c), pa));
  const double l = norm3(n);
  n = l > 0 ? div3(n, l) : D3{0.0, 0.0, 0.0};
  return HPlane{n.x, n.y, n.z, dot3(n, pa)};
}

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Warp-wide (value, index) reductions, every lane gets the result. The index
// breaks ties (smallest first), which is the host's "first in scan order".
__device__ __forceinline__ void warp_max_first(double& v, int& i) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double ov = __shfl_xor_sync(0xffffffffu, v, o);
    const int oi = __shfl_xor_sync(0xffffffffu, i, o);
    if (ov > v || (ov == v && oi < i)) {
      v = ov;
      i = oi;
    }
  }
}
__device__ __forceinline__ void warp_min_first(double& v, int& i) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double ov = __shfl_xor_sync(0xffffffffu, v, o);
    const int oi = __shfl_xor_sync(0xffffffffu, i, o);
    if (ov < v || (ov == v && oi < i)) {
      v = ov;
      i = oi;
    }
  }
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

}  // namespace

// Per-part capacities and the byte layout of its work region (host and device).
struct HullCaps {
  int64_t faces, pool, list, hor, n;
};
__host__ __device__ inline HullCaps hull_caps(int64_t n, int mult) {
  HullCaps c;
  c.n = n;
  c.faces = mult * (8 * n + 64);
  c.pool = mult * (16 * n + 256);
  c.list = mult * (2 * n + 16);
  c.hor = 3 * c.list;
  return c;
}
__host__ __device__ inline int64_t hull_a16(int64_t b) { return (b + 15) & ~(int64_t)15; }
__host__ __device__ inline int64_t hull_region_bytes(int64_t n, int mult) {
  const HullCaps c = hull_caps(n, mult);
  return hull_a16(c.faces * 32) + hull_a16(c.faces * 16) * 2 + hull_a16(c.faces * 8) + hull_a16(c.pool * 4) +
         3 * hull_a16(c.list * 4) + 3 * hull_a16(c.hor * 8) + hull_a16(c.hor * 4) + 2 * hull_a16(n * 4);
}

namespace {

struct HullWork {
  HPlane* plane;  // face: unit normal, offset
  int4* tv;        // face: v0, v1, v2, alive
  int4* nb;        // face: neighbour across (v[e], v[e+1]) for e = 0..2, visit stamp
  int2* outl;      // face: outside list (start in pool, count)
  int* pool;
  int* vis;        // visible faces of a step, in flood-fill order
  int* stack;
  int* voff;       // first orphan slot of each visible face
  int2* hor;       // horizon (face, edge) in discovery order
  int2* loop;      // horizon as a loop
  int2* hu;        // horizon edge endpoints (u, w); u = -1 once used
  int* fillc;      // scatter cursor of each new face
  int* orph;       // orphaned points of a step, in order
  int* obest;      // new face (0-based among the step's) of each orphan, -1 = inside
  HullCaps cap;
};

__device__ HullWork carve(char* base, int64_t n, int mult) {
  HullWork w;
  w.cap = hull_caps(n, mult);
  const HullCaps& c = w.cap;
  char* p = base;
  auto take = [&](int64_t bytes) {
    char* r = p;
    p += hull_a16(bytes);
    return r;
  };
  w.plane = (HPlane*)take(c.faces * 32);
  w.tv = (int4*)take(c.faces * 16);
  w.nb = (int4*)take(c.faces * 16);
  w.outl = (int2*)take(c.faces * 8);
  w.pool = (int*)take(c.pool * 4);
  w.vis = (int*)take(c.list * 4);
  w.stack = (int*)take(c.list * 4);
  w.voff = (int*)take(c.list * 4);
  w.hor = (int2*)take(c.hor * 8);
  w.loop = (int2*)take(c.hor * 8);
  w.hu = (int2*)take(c.hor * 8);
  w.fillc = (int*)take(c.hor * 4);
  w.orph = (int*)take(n * 4);
  w.obest = (int*)take(n * 4);
  return w;
}

__device__ __forceinline__ int comp(int4 v, int e) { return e == 0 ? v.x : (e == 1 ? v.y : v.z); }
__device__ __forceinline__ void set_comp(int4* p, int e, int x) {
  int* q = reinterpret_cast<int*>(p);
  q[e] = x;
}

// Assign the points pts[0..m) (pts == nullptr: the point ids 0..m-1 except the
// four in skip) to the faces f0..f0+L-1: each goes to the first face with the
// largest distance above eps, or nowhere; then every face's outside list is
// written as one pool segment, in point order. Returns the new pool top, or
// -1 when the pool is full.
__device__ int64_t assign_points(const double* P, HullWork& W, const int* pts, int m, int4 skip, int f0, int L,
                                 double eps, int64_t top, int lane) {
  // Pass 1: best face of each point, counts per face (outl[f].y).
  if (lane == 0)
    for (int q = 0; q < L; ++q) W.outl[f0 + q] = make_int2(0, 0);
  __syncwarp();
  for (int base = 0; base < m; base += 32) {
    const int k = base + lane;
    int bf = -2;
    if (k < m) {
      const int p = pts ? pts[k] : k;
      bf = -1;
      if (pts || (p != skip.x && p != skip.y && p != skip.z && p != skip.w)) {
        const D3 pp = ld3(P, p);
        double bd = eps;
        for (int q = 0; q < L; ++q) {
          const double d = plane_dist(W.plane[f0 + q], pp);
          if (d > bd) {
            bd = d;
            bf = q;
          }
        }
      }
      W.obest[k] = bf;
    }
    const unsigned mm = __match_any_sync(0xffffffffu, bf);
    if (bf >= 0 && (__ffs(mm) - 1) == lane) W.outl[f0 + bf].y += __popc(mm);
    __syncwarp();
  }
  // Segment starts.
  int64_t end = top;
  if (lane == 0) {
    for (int q = 0; q < L; ++q) {
      const int c = W.outl[f0 + q].y;
      W.outl[f0 + q].x = (int)end;
      W.fillc[q] = (int)end;
      end += c;
    }
  }
  end = __shfl_sync(0xffffffffu, end, 0);
  if (end > W.cap.pool) return -1;
  __syncwarp();
  // Pass 2: stable scatter.
  const unsigned lt = lanemask_lt();
  for (int base = 0; base < m; base += 32) {
    const int k = base + lane;
    const int bf = k < m ? W.obest[k] : -2;
    const unsigned mm = __match_any_sync(0xffffffffu, bf);
    if (bf >= 0) W.pool[W.fillc[bf] + __popc(mm & lt)] = pts ? pts[k] : k;
    __syncwarp();
    if (bf >= 0 && (__ffs(mm) - 1) == lane) W.fillc[bf] += __popc(mm);
    __syncwarp();
  }
  return end;
}

// Coplanar input: the host's flat_hull (2D monotone chain in the plane, closed
// as two opposite fans; no orientation fix). Uses the face arrays as scratch.
__device__ int flat_hull(const double* P, int n, HullWork& W, int32_t* tris, int& ntri, int lane) {
  ntri = 0;
  const D3 o = ld3(P, 0);
  double bd = -1.0;
  int ia = 0x7fffffff;
  for (int i = lane; i < n; i += 32) {
    const double d = norm3(sub3(ld3(P, i), o));
    if (d > bd) {
      bd = d;
      ia = i;
    }
  }
  warp_max_first(bd, ia);
  if (ia == 0x7fffffff) ia = 0;
  D3 u = sub3(ld3(P, ia), o);
  {
    const double l = norm3(u);
    if (l == 0) return kHullZeroNorm;
    u = div3(u, l);
  }
  double bc = -1.0;
  int ic = 0x7fffffff;
  for (int i = lane; i < n; i += 32) {
    const double d = norm3(cross3(u, sub3(ld3(P, i), o)));
    if (d > bc) {
      bc = d;
      ic = i;
    }
  }
  warp_max_first(bc, ic);
  if (!(bc > 0)) return kHullOk;
  D3 nrm = cross3(u, sub3(ld3(P, ic), o));
  nrm = div3(nrm, norm3(nrm));
  const D3 v = cross3(nrm, u);
  // Sort (x, y, index) lexicographically by rank counting: rank of i = number
  // of keys below it (keys are distinct through the index).
  double* qx = reinterpret_cast<double*>(W.plane);
  double* qy = qx + n;
  int* qi = reinterpret_cast<int*>(W.tv);
  int* h = qi + n;
  double* kx = reinterpret_cast<double*>(W.nb);  // the unsorted keys
  double* ky = kx + n;
  for (int i = lane; i < n; i += 32) {
    const D3 w = sub3(ld3(P, i), o);
    kx[i] = dot3(w, u);
    ky[i] = dot3(w, v);
  }
  __syncwarp();
  for (int i = lane; i < n; i += 32) {
    const double xi = kx[i], yi = ky[i];
    int r = 0;
    for (int j = 0; j < n; ++j) {
      const double xj = kx[j], yj = ky[j];
      r += (xj < xi || (xj == xi && (yj < yi || (yj == yi && j < i)))) ? 1 : 0;
    }
    qx[r] = xi;
    qy[r] = yi;
    qi[r] = i;
  }
  __syncwarp();
  int hs = 0;
  if (lane == 0) {
    auto crs = [&](int a, int b, int c) {
      return ds(dm(ds(qx[b], qx[a]), ds(qy[c], qy[a])), dm(ds(qy[b], qy[a]), ds(qx[c], qx[a])));
    };
    for (int pass = 0; pass < 2; ++pass) {
      const int start = hs;
      for (int k = 0; k < n; ++k) {
        const int i = pass == 0 ? k : n - 1 - k;
        while (hs >= start + 2 && crs(h[hs - 2], h[hs - 1], i) <= 0) --hs;
        h[hs++] = i;
      }
      --hs;
    }
  }
  hs = __shfl_sync(0xffffffffu, hs, 0);
  __syncwarp();
  if (hs < 3) return kHullOk;
  if (2 * (hs - 2) > 2 * n) return kHullOutCap;
  for (int k = 1 + lane; k + 1 < hs; k += 32) {
    const int a = qi[h[0]], b = qi[h[k]], c = qi[h[k + 1]];
    int32_t* t = tris + 6 * (int64_t)(k - 1);
    t[0] = a;
    t[1] = b;
    t[2] = c;
    t[3] = a;
    t[4] = c;
    t[5] = b;
  }
  ntri = 2 * (hs - 2);
  return kHullOk;
}

// One part: the host's convex_hull(pts, fix_normals) (host/hull.cpp).
__device__ int hull_one(const double* P, int n, HullWork& W, int fix, int32_t* tris, int& ntri, int lane) {
  ntri = 0;
  if (n < 3) return kHullOk;
  double ext = 0.0;
  for (int i = lane; i < n; i += 32) {
    const D3 p = ld3(P, i);
    ext = fmax(ext, fmax(fabs(p.x), fmax(fabs(p.y), fabs(p.z))));
  }
  ext = warp_max(ext);
  const double eps = dm(fmax(ext, 1e-300), 1e-11);
  // Coordinate extremes: first index of each axis' minimum and maximum.
  int ex[6];
  for (int a = 0; a < 3; ++a) {
    double lo = __longlong_as_double(0x7ff0000000000000LL), hi = -lo;
    int ilo = 0x7fffffff, ihi = 0x7fffffff;
    for (int i = lane; i < n; i += 32) {
      const double x = P[3 * (int64_t)i + a];
      if (x < lo) {
        lo = x;
        ilo = i;
      }
      if (x > hi) {
        hi = x;
        ihi = i;
      }
    }
    warp_min_first(lo, ilo);
    warp_max_first(hi, ihi);
    ex[2 * a] = ilo;
    ex[2 * a + 1] = ihi;
  }
  int i0 = ex[0], i1 = ex[1];
  double best = -1.0;
  for (int a = 0; a < 6; ++a)
    for (int b = a + 1; b < 6; ++b) {
      const double d = norm3(sub3(ld3(P, ex[a]), ld3(P, ex[b])));
      if (d > best) {
        best = d;
        i0 = ex[a];
        i1 = ex[b];
      }
    }
  if (best <= eps) return kHullOk;
  const D3 p0 = ld3(P, i0);
  const D3 dir = div3(sub3(ld3(P, i1), p0), best);
  double b2 = eps;
  int i2 = 0x7fffffff;
  for (int i = lane; i < n; i += 32) {
    const D3 w = sub3(ld3(P, i), p0);
    const double t = dot3(w, dir);
    const double d = norm3(D3{ds(w.x, dm(dir.x, t)), ds(w.y, dm(dir.y, t)), ds(w.z, dm(dir.z, t))});
    if (d > b2) {
      b2 = d;
      i2 = i;
    }
  }
  warp_max_first(b2, i2);
  if (i2 == 0x7fffffff) return kHullOk;  // collinear
  D3 nrm = cross3(sub3(ld3(P, i1), p0), sub3(ld3(P, i2), p0));
  {
    const double l = norm3(nrm);
    if (l == 0) return kHullZeroNorm;
    nrm = div3(nrm, l);
  }
  double b3 = eps;
  int i3 = 0x7fffffff;
  for (int i = lane; i < n; i += 32) {
    const double d = fabs(dot3(nrm, sub3(ld3(P, i), p0)));
    if (d > b3) {
      b3 = d;
      i3 = i;
    }
  }
  warp_max_first(b3, i3);
  if (i3 == 0x7fffffff) return flat_hull(P, n, W, tris, ntri, lane);
  if (dot3(nrm, sub3(ld3(P, i3), p0)) > 0) {
    const int t = i1;
    i1 = i2;
    i2 = t;
  }
  // The tetrahedron, faces outward, neighbours by shared reversed edges.
  if (lane < 4) {
    const int4 f = lane == 0 ? make_int4(i0, i1, i2, 1)
                             : (lane == 1 ? make_int4(i0, i3, i1, 1)
                                          : (lane == 2 ? make_int4(i1, i3, i2, 1) : make_int4(i2, i3, i0, 1)));
    W.tv[lane] = f;
    W.plane[lane] = face_plane(P, f.x, f.y, f.z);
  }
  __syncwarp();
  if (lane == 0) {
    for (int a = 0; a < 4; ++a) {
      int4 nbv = make_int4(-1, -1, -1, 0);
      const int4 va = W.tv[a];
      for (int e = 0; e < 3; ++e) {
        const int u = comp(va, e), w = comp(va, (e + 1) % 3);
        for (int b = 0; b < 4; ++b) {
          if (a == b) continue;
          const int4 vb = W.tv[b];
          for (int e2 = 0; e2 < 3; ++e2)
            if (comp(vb, e2) == w && comp(vb, (e2 + 1) % 3) == u) set_comp(&nbv, e, b);
        }
      }
      W.nb[a] = nbv;
    }
  }
  __syncwarp();
  int64_t top = assign_points(P, W, nullptr, n, make_int4(i0, i1, i2, i3), 0, 4, eps, 0, lane);
  if (top < 0) return kHullPoolCap;
  int nF = 4, cur = 0, iter = 0;
  for (;;) {
    while (cur < nF) {
      if (W.tv[cur].w && W.outl[cur].y > 0) break;
      ++cur;
    }
    if (cur >= nF) break;
    if (++iter > 4 * n + 64) break;
    // Farthest outside point of cur (first in list order among equals).
    const HPlane pc = W.plane[cur];
    const int2 ol = W.outl[cur];
    double bd = -1.0;
    int bpos = 0x7fffffff;
    for (int k = lane; k < ol.y; k += 32) {
      const double d = plane_dist(pc, ld3(P, W.pool[ol.x + k]));
      if (d > bd) {
        bd = d;
        bpos = k;
      }
    }
    warp_max_first(bd, bpos);
    if (bpos >= ol.y) return kHullNumeric;
    const int apex = W.pool[ol.x + bpos];
    const D3 pa = ld3(P, apex);
    // Lane 0: flood fill, horizon loop, new faces and links.
    int st = kHullOk, vn = 0, L = 0, norph = 0;
    if (lane == 0) {
      int sp = 0, hn = 0;
      W.stack[sp++] = cur;
      W.nb[cur].w = iter;
      while (sp > 0 && st == kHullOk) {
        const int f = W.stack[--sp];
        if (vn >= W.cap.list) {
          st = kHullListCap;
          break;
        }
        W.vis[vn] = f;
        W.voff[vn] = norph;
        norph += W.outl[f].y - (f == cur ? 1 : 0);
        ++vn;
        const int4 nbf = W.nb[f];
        for (int e = 0; e < 3; ++e) {
          const int g = comp(nbf, e);
          if (g < 0 || W.nb[g].w == iter) continue;
          if (plane_dist(W.plane[g], pa) > eps) {
            if (sp >= W.cap.list) {
              st = kHullListCap;
              break;
            }
            W.nb[g].w = iter;
            W.stack[sp++] = g;
          } else {
            if (hn >= W.cap.hor) {
              st = kHullListCap;
              break;
            }
            const int4 tf = W.tv[f];
            W.hor[hn] = make_int2(f, e);
            W.hu[hn] = make_int2(comp(tf, e), comp(tf, (e + 1) % 3));
            ++hn;
          }
        }
      }
      if (st == kHullOk) {
        // Order the horizon as a loop (the host's first-unused-match scan).
        bool ok = hn > 0;
        if (ok) {
          W.loop[0] = W.hor[0];
          int wlast = W.hu[0].y;
          W.hu[0].x = -1;
          L = 1;
          for (int k = 1; k < hn; ++k) {
            int found = -1;
            for (int hh = 0; hh < hn; ++hh)
              if (W.hu[hh].x == wlast) {
                found = hh;
                break;
              }
            if (found < 0) break;
            W.loop[L++] = W.hor[found];
            wlast = W.hu[found].y;
            W.hu[found].x = -1;
          }
          ok = L == hn;
        }
        if (!ok) {
          W.outl[cur].y = 0;  // numerically inconsistent horizon: drop cur's outside set
          L = 0;
        } else if (nF + L > W.cap.faces) {
          st = kHullFaceCap;
        } else {
          for (int k = 0; k < L; ++k) {
            const int2 fe = W.loop[k];
            const int4 tf = W.tv[fe.x];
            const int u = comp(tf, fe.y), w = comp(tf, (fe.y + 1) % 3);
            const int g = comp(W.nb[fe.x], fe.y);
            const int nfi = nF + k;
            W.tv[nfi] = make_int4(u, w, apex, 1);
            W.nb[nfi] = make_int4(g, nF + (k + 1) % L, nF + (k + L - 1) % L, 0);
            const int4 tg = W.tv[g];
            for (int e = 0; e < 3; ++e)
              if (comp(tg, e) == w && comp(tg, (e + 1) % 3) == u) {
                set_comp(&W.nb[g], e, nfi);
                break;
              }
          }
        }
      }
    }
    st = __shfl_sync(0xffffffffu, st, 0);
    if (st != kHullOk) return st;
    L = __shfl_sync(0xffffffffu, L, 0);
    if (L == 0) {
      ++cur;
      __syncwarp();
      continue;
    }
    vn = __shfl_sync(0xffffffffu, vn, 0);
    norph = __shfl_sync(0xffffffffu, norph, 0);
    __syncwarp();
    // New faces' planes; orphans of the visible faces in order (the apex
    // skipped); visible faces die.
    for (int k = lane; k < L; k += 32) {
      const int4 t = W.tv[nF + k];
      W.plane[nF + k] = face_plane(P, t.x, t.y, t.z);
    }
    for (int i = 0; i < vn; ++i) {
      const int f = W.vis[i];
      const int2 fl = W.outl[f];
      const int o0 = W.voff[i];
      if (f == cur) {
        for (int k = lane; k < fl.y; k += 32)
          if (k != bpos) W.orph[o0 + (k < bpos ? k : k - 1)] = W.pool[fl.x + k];
      } else {
        for (int k = lane; k < fl.y; k += 32) W.orph[o0 + k] = W.pool[fl.x + k];
      }
    }
    __syncwarp();
    for (int i = lane; i < vn; i += 32) {
      const int f = W.vis[i];
      W.tv[f].w = 0;
      W.outl[f].y = 0;
    }
    __syncwarp();
    top = assign_points(P, W, W.orph, norph, make_int4(-1, -1, -1, -1), nF, L, eps, top, lane);
    if (top < 0) return kHullPoolCap;
    nF += L;
    ++cur;
    __syncwarp();
  }
  // Live faces in creation order.
  int cnt = 0;
  for (int base = 0; base < nF; base += 32) {
    const int f = base + lane;
    const bool alive = f < nF && W.tv[f].w;
    const unsigned m = __ballot_sync(0xffffffffu, alive);
    if (cnt + __popc(m) > 2 * n) return kHullOutCap;
    if (alive) {
      const int4 t = W.tv[f];
      int32_t* o = tris + 3 * (int64_t)(cnt + __popc(m & lanemask_lt()));
      o[0] = t.x;
      o[1] = t.y;
      o[2] = t.z;
    }
    cnt += __popc(m);
  }
  ntri = cnt;
  if (fix) {
    // Centroid of all points, summed in index order as the host does.
    D3 c{0.0, 0.0, 0.0};
    if (lane == 0) {
      for (int i = 0; i < n; ++i) {
        const D3 p = ld3(P, i);
        c = D3{da(c.x, p.x), da(c.y, p.y), da(c.z, p.z)};
      }
      c = div3(c, (double)n);
    }
    c.x = __shfl_sync(0xffffffffu, c.x, 0);
    c.y = __shfl_sync(0xffffffffu, c.y, 0);
    c.z = __shfl_sync(0xffffffffu, c.z, 0);
    __syncwarp();
    for (int k = lane; k < cnt; k += 32) {
      int32_t* t = tris + 3 * (int64_t)k;
      const D3 v0 = ld3(P, t[0]);
      const D3 nn = cross3(sub3(ld3(P, t[1]), v0), sub3(ld3(P, t[2]), v0));
      if (dot3(nn, sub3(c, v0)) > 0) {
        const int s = t[1];
        t[1] = t[2];
        t[2] = s;
      }
    }
  }
  return kHullOk;
}

__global__ void __launch_bounds__(32 * kHullWarps)
    hull_kernel(const double* __restrict__ pts, const int64_t* __restrict__ poff, const int32_t* __restrict__ ids,
                int32_t nj, char* __restrict__ arena, const int64_t* __restrict__ roff, int mult, int fix,
                int32_t* __restrict__ tris, int32_t* __restrict__ counts, int32_t* __restrict__ pstatus) {
  const int lane = threadIdx.x & 31;
  const int nw = gridDim.x * kHullWarps;
  for (int j = blockIdx.x * kHullWarps + (threadIdx.x >> 5); j < nj; j += nw) {
    const int part = ids[j];
    const int64_t o = poff[part];
    const int n = (int)(poff[part + 1] - o);
    HullWork W = carve(arena + roff[j], n, mult);
    int ntri = 0;
    const int st = hull_one(pts + 3 * o, n, W, fix, tris + 6 * o, ntri, lane);
    if (lane == 0) {
      counts[part] = st == kHullOk ? ntri : 0;
      pstatus[part] = st;
    }
    __syncwarp();
  }
}

size_t hull_align256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace
}  // namespace vgpu

using namespace vgpu;

extern "C" int visacd_convex_hulls(visacd_ctx* ctx, const double* points, const int64_t* offsets, int32_t nparts,
                                   int32_t fix_normals, int32_t* tris, int32_t* counts) {
  VCHECK(ctx && offsets && (nparts == 0 || (tris && counts)), VISACD_ERR_INVALID_ARG,
         "convex_hulls: null argument");
  VCHECK(nparts >= 0, VISACD_ERR_INVALID_ARG, "convex_hulls: negative part count");
  if (nparts == 0) return VISACD_OK;
  VCHECK(offsets[0] == 0, VISACD_ERR_INVALID_ARG, "convex_hulls: offsets[0] must be 0");
  for (int32_t k = 0; k < nparts; ++k) {
    VCHECK(offsets[k + 1] >= offsets[k], VISACD_ERR_INVALID_ARG, "convex_hulls: offsets must not decrease");
    VCHECK(offsets[k + 1] - offsets[k] <= (1LL << 22), VISACD_ERR_INVALID_ARG,
           "convex_hulls: a part has more than 2^22 points");
  }
  const int64_t N = offsets[nparts];
  VCHECK(N == 0 || points, VISACD_ERR_INVALID_ARG, "convex_hulls: null points");
  for (int64_t i = 0; i < 3 * N; ++i)
    VCHECK(std::isfinite(points[i]), VISACD_ERR_INVALID_ARG, "convex_hulls: non-finite coordinate");
  VCUDA(cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->stream;
  // Fixed part: points, offsets, triangles, counts, status; then per launch
  // the part ids, region offsets and the regions.
  const size_t oPts = 0, oOff = oPts + hull_align256((size_t)N * 24), oTri = oOff + hull_align256((size_t)(nparts + 1) * 8),
               oCnt = oTri + hull_align256((size_t)N * 24), oSt = oCnt + hull_align256((size_t)nparts * 4),
               oIds = oSt + hull_align256((size_t)nparts * 4), oRoff = oIds + hull_align256((size_t)nparts * 4),
               oArena = oRoff + hull_align256((size_t)(nparts + 1) * 8);
  // Pending parts with their room multiplier, run in launches whose work
  // regions stay under kHullArenaCap (a part larger than that runs alone).
  constexpr int64_t kHullArenaCap = 1LL << 30;
  std::vector<std::pair<int32_t, int>> queue(nparts);
  for (int32_t k = 0; k < nparts; ++k) queue[k] = {k, 1};
  std::vector<int32_t> ids;
  std::vector<int64_t> roff;
  std::vector<int32_t> cnt_now(nparts), st_now(nparts);
  char* sent_to = nullptr;  // slot base the inputs were last uploaded to
  size_t head = 0;
  while (head < queue.size()) {
    // The next launch: parts of one multiplier, in queue order, under the cap.
    const int mult = queue[head].second;
    ids.clear();
    roff.assign(1, 0);
    while (head < queue.size() && queue[head].second == mult) {
      const int32_t k = queue[head].first;
      const int64_t r = hull_region_bytes(offsets[k + 1] - offsets[k], mult);
      if (!ids.empty() && roff.back() + r > kHullArenaCap) break;
      ids.push_back(k);
      roff.push_back(roff.back() + r);
      ++head;
    }
    VTRY(ensure_slot(ctx, kSlotConvexHull, oArena + (size_t)roff.back()));
    char* base = slot<char>(ctx, kSlotConvexHull);
    if (base != sent_to) {  // a slot that grew does not keep its contents
      if (N) VCUDA(cudaMemcpyAsync(base + oPts, points, (size_t)N * 24, cudaMemcpyHostToDevice, st));
      VCUDA(cudaMemcpyAsync(base + oOff, offsets, (size_t)(nparts + 1) * 8, cudaMemcpyHostToDevice, st));
      sent_to = base;
    }
    VCUDA(cudaMemcpyAsync(base + oIds, ids.data(), ids.size() * 4, cudaMemcpyHostToDevice, st));
    VCUDA(cudaMemcpyAsync(base + oRoff, roff.data(), roff.size() * 8, cudaMemcpyHostToDevice, st));
    const unsigned blocks =
        (unsigned)std::min<int64_t>(((int64_t)ids.size() + kHullWarps - 1) / kHullWarps, 16LL * ctx->sm_count);
    VLAUNCH(ctx, kKConvexHull, blocks, 32 * kHullWarps, 0, hull_kernel, (const double*)(base + oPts),
            (const int64_t*)(base + oOff), (const int32_t*)(base + oIds), (int32_t)ids.size(), base + oArena,
            (const int64_t*)(base + oRoff), mult, (int)fix_normals, (int32_t*)(base + oTri),
            (int32_t*)(base + oCnt), (int32_t*)(base + oSt));
    VCUDA(cudaMemcpyAsync(st_now.data(), base + oSt, (size_t)nparts * 4, cudaMemcpyDeviceToHost, st));
    VCUDA(cudaMemcpyAsync(cnt_now.data(), base + oCnt, (size_t)nparts * 4, cudaMemcpyDeviceToHost, st));
    const bool all = (int32_t)ids.size() == nparts;
    // The output has the device layout (6 int32 per point): one copy when every
    // part ran in this launch, one per part otherwise.
    if (all && N) VCUDA(cudaMemcpyAsync(tris, base + oTri, (size_t)N * 24, cudaMemcpyDeviceToHost, st));
    VCUDA(stream_wait(ctx));
    for (int32_t k : ids) {
      const int s = st_now[k];
      if (s == kHullOk) {
        counts[k] = cnt_now[k];
        const int64_t o = offsets[k];
        if (!all && cnt_now[k] > 0)
          VCUDA(cudaMemcpyAsync(tris + 6 * o, base + oTri + (size_t)o * 24, (size_t)cnt_now[k] * 12,
                                cudaMemcpyDeviceToHost, st));
      } else if (s == kHullFaceCap || s == kHullPoolCap || s == kHullListCap) {
        VCHECK(mult * 4 <= kMaxHullMult, VISACD_ERR_DEVICE,
               "convex_hulls: part %d outgrows %d times the default room", (int)k, mult);
        queue.push_back({k, mult * 4});
      } else {
        VCUDA(stream_wait(ctx));
        set_error("convex_hulls: part %d: %s", (int)k,
                  s == kHullZeroNorm   ? "zero-length normal"
                  : s == kHullNumeric ? "non-finite face plane"
                                      : "more hull triangles than twice its points");
        return VISACD_ERR_DEVICE;
      }
    }
    VCUDA(stream_wait(ctx));
  }
  return VISACD_OK;
}

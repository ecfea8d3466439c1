// FP64 geometry shared by kernels whose results must equal the host C++
// restatements bit for bit: explicit round-to-nearest intrinsics in the host's
// order of operations (no contraction into FMAs).
#pragma once

#include <cuda_runtime.h>

namespace vgpu {

__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double ds(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dot3(const double* a, const double* b) {
  return da(da(dm(a[0], b[0]), dm(a[1], b[1])), dm(a[2], b[2]));
}

// Closest point on triangle abc to p (host order of operations).
__device__ inline double point_tri_dist(const double* p, const double* a, const double* b, const double* c) {
  double ab[3] = {ds(b[0], a[0]), ds(b[1], a[1]), ds(b[2], a[2])};
  double ac[3] = {ds(c[0], a[0]), ds(c[1], a[1]), ds(c[2], a[2])};
  double ap[3] = {ds(p[0], a[0]), ds(p[1], a[1]), ds(p[2], a[2])};
  double cp[3];
  double d1 = dot3(ab, ap), d2 = dot3(ac, ap);
  if (d1 <= 0 && d2 <= 0) {
    cp[0] = a[0]; cp[1] = a[1]; cp[2] = a[2];
  } else {
    double bp[3] = {ds(p[0], b[0]), ds(p[1], b[1]), ds(p[2], b[2])};
    double d3 = dot3(ab, bp), d4 = dot3(ac, bp);
    double vc = ds(dm(d1, d4), dm(d3, d2));
    double cpv[3] = {ds(p[0], c[0]), ds(p[1], c[1]), ds(p[2], c[2])};
    double d5 = dot3(ab, cpv), d6 = dot3(ac, cpv);
    double vb = ds(dm(d5, d2), dm(d1, d6));
    double va = ds(dm(d3, d6), dm(d5, d4));
    if (d3 >= 0 && d4 <= d3) {
      cp[0] = b[0]; cp[1] = b[1]; cp[2] = b[2];
    } else if (vc <= 0 && d1 >= 0 && d3 <= 0) {
      double v = __ddiv_rn(d1, ds(d1, d3));
      for (int k = 0; k < 3; ++k) cp[k] = da(a[k], dm(ab[k], v));
    } else if (d6 >= 0 && d5 <= d6) {
      cp[0] = c[0]; cp[1] = c[1]; cp[2] = c[2];
    } else if (vb <= 0 && d2 >= 0 && d6 <= 0) {
      double w = __ddiv_rn(d2, ds(d2, d6));
      for (int k = 0; k < 3; ++k) cp[k] = da(a[k], dm(ac[k], w));
    } else if (va <= 0 && ds(d4, d3) >= 0 && ds(d5, d6) >= 0) {
      double w = __ddiv_rn(ds(d4, d3), da(ds(d4, d3), ds(d5, d6)));
      for (int k = 0; k < 3; ++k) cp[k] = da(b[k], dm(ds(c[k], b[k]), w));
    } else {
      double denom = __ddiv_rn(1.0, da(da(va, vb), vc));
      double v = dm(vb, denom), w = dm(vc, denom);
      for (int k = 0; k < 3; ++k) cp[k] = da(da(a[k], dm(ab[k], v)), dm(ac[k], w));
    }
  }
  double dx = ds(p[0], cp[0]), dy = ds(p[1], cp[1]), dz = ds(p[2], cp[2]);
  return __dsqrt_rn(da(da(dm(dx, dx), dm(dy, dy)), dm(dz, dz)));
}

// The concavity metric's point-triangle distance as the reference computes it
// (lib/include/hausdorff.hpp:97-212), in its operation order: the plane
// distance when the projection passes the barycentric test, else the std::min
// of the three edge distances (Pythagoras; DBL_MAX when the projection falls
// outside the edge) and the three vertex distances. On degenerate triangles
// (zero area) the plane normal is 0/0 and the result is NaN or an edge/vertex
// value; a NaN never lowers a minimum. Equal to the host's
// ref_point_triangle_distance bit for bit.
__device__ __forceinline__ double rsq(double x) { return dm(x, x); }
__device__ __forceinline__ double rmin(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ double ref_pp(const double* p, const double* q) {
  return __dsqrt_rn(da(da(rsq(ds(p[0], q[0])), rsq(ds(p[1], q[1]))), rsq(ds(p[2], q[2]))));
}
__device__ __forceinline__ double ref_pseg(const double* p, const double* s0, const double* s1) {
  const double BA0 = ds(p[0], s1[0]), BA1 = ds(p[1], s1[1]), BA2 = ds(p[2], s1[2]);
  const double BC0 = ds(s0[0], s1[0]), BC1 = ds(s0[1], s1[1]), BC2 = ds(s0[2], s1[2]);
  const double bc = __dsqrt_rn(da(da(rsq(BC0), rsq(BC1)), rsq(BC2)));
  const double proj = __ddiv_rn(da(da(dm(BA0, BC0), dm(BA1, BC1)), dm(BA2, BC2)), bc);
  const double ab = __dsqrt_rn(da(da(rsq(BA0), rsq(BA1)), rsq(BA2)));
  if (proj < 0 || proj > bc) return 1.7976931348623157e308;
  return __dsqrt_rn(ds(rsq(ab), rsq(proj)));
}
__device__ inline double ref_point_tri_dist(const double* p, const double* t0, const double* t1,
                                            const double* t2) {
  const double e1x = ds(t1[0], t0[0]), e1y = ds(t1[1], t0[1]), e1z = ds(t1[2], t0[2]);
  const double e2x = ds(t2[0], t0[0]), e2y = ds(t2[1], t0[1]), e2z = ds(t2[2], t0[2]);
  const double A = ds(dm(e1y, e2z), dm(e1z, e2y));
  const double B = ds(dm(e1z, e2x), dm(e1x, e2z));
  const double C = ds(dm(e1x, e2y), dm(e1y, e2x));
  const double nn = __dsqrt_rn(da(da(rsq(A), rsq(B)), rsq(C)));
  const double a = __ddiv_rn(A, nn), b = __ddiv_rn(B, nn), c = __ddiv_rn(C, nn);
  const double d = ds(0.0, da(da(dm(a, t0[0]), dm(b, t0[1])), dm(c, t0[2])));
  const double ev = da(da(da(dm(a, p[0]), dm(b, p[1])), dm(c, p[2])), d);
  const double dist = __ddiv_rn(fabs(ev), __dsqrt_rn(da(da(rsq(a), rsq(b)), rsq(c))));
  double pr[3] = {p[0], p[1], p[2]};
  if (ev > 1e-8) {
    pr[0] = ds(p[0], dm(a, dist));
    pr[1] = ds(p[1], dm(b, dist));
    pr[2] = ds(p[2], dm(c, dist));
  } else if (ev < -1e-8) {
    pr[0] = da(p[0], dm(a, dist));
    pr[1] = da(p[1], dm(b, dist));
    pr[2] = da(p[2], dm(c, dist));
  }
  {
    const double v2x = ds(pr[0], t0[0]), v2y = ds(pr[1], t0[1]), v2z = ds(pr[2], t0[2]);
    const double d00 = da(da(dm(e2x, e2x), dm(e2y, e2y)), dm(e2z, e2z));
    const double d01 = da(da(dm(e2x, e1x), dm(e2y, e1y)), dm(e2z, e1z));
    const double d02 = da(da(dm(e2x, v2x), dm(e2y, v2y)), dm(e2z, v2z));
    const double d11 = da(da(dm(e1x, e1x), dm(e1y, e1y)), dm(e1z, e1z));
    const double d12 = da(da(dm(e1x, v2x), dm(e1y, v2y)), dm(e1z, v2z));
    const double inv = __ddiv_rn(1.0, ds(dm(d00, d11), dm(d01, d01)));
    const double u = dm(ds(dm(d11, d02), dm(d01, d12)), inv);
    const double v = dm(ds(dm(d00, d12), dm(d01, d02)), inv);
    if ((u >= 0) && (v >= 0) && (da(u, v) <= 1)) return dist;
  }
  const double sab = ref_pseg(p, t0, t1), sbc = ref_pseg(p, t1, t2), sca = ref_pseg(p, t2, t0);
  const double pa = ref_pp(p, t0), pb = ref_pp(p, t1), pc = ref_pp(p, t2);
  return rmin(rmin(rmin(sab, sbc), sca), rmin(rmin(pa, pb), pc));
}

}  // namespace vgpu

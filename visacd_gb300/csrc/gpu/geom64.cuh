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

}  // namespace vgpu

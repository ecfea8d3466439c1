// SDF remeshing on the GPU: the iso-surface at distance `level` outside a
// mesh, on a grid of voxel size 1/scale — the cage / manifold step that
// replaces OpenVDB in lib/src/preprocess.cpp:18-67.
//
// Same algorithm and arithmetic as the host restatement (manifold_preprocess in
// csrc/host/remesh.cpp), so the output mesh is identical bit for bit:
//  1. sdf_tri_prep_kernel computes each triangle's set-up once (voxel box,
//     FP32 bounds and planes); the boxes are cut into work items of 1024
//     voxels; sdf_ub_kernel gives every band voxel an FP32 upper bound of its
//     distance, then sdf_dist_kernel gives every voxel centre in each
//     triangle's box grown by the band the exact FP64 point-triangle distance
//     (rounded to float) unless a lower bound rules it out, combined with
//     atomicMin (non-negative floats order like their bit patterns).
//  2. For each axis: sdf_cross_kernel marks, for every ray through voxel
//     centres (offset by 1.2345679e-6 / 2.3456789e-6 voxels) that crosses a
//     triangle at x, the first voxel whose centre lies beyond x (XOR toggle);
//     sdf_parity_kernel runs the prefix parity along each ray and adds a vote
//     where it is odd. Inside = at least two of the three votes.
//  3. Surface nets: a vertex per sign-changing cell at the mean of its edge
//     crossings (cells in linear order, exclusive scan), two triangles per
//     sign-changing grid edge whose four cells all have vertices (voxels in
//     linear order, x / y / z edges, exclusive scan).
#include "common.cuh"
#include "geom64.cuh"

namespace vgpu {

namespace {

constexpr float kSdfU = 5.9604645e-8f;  // 2^-24

struct SdfGrid {
  int org[3], dim[3];
  double band;
  float fiso;
  double scale;
  float margin;  // FP32 lower-bound margin (voxels): 1e-3 + 1e-6 max |grid coordinate|
};

__device__ __forceinline__ size_t vid(const SdfGrid& g, int i, int j, int k) {
  return ((size_t)k * g.dim[1] + j) * g.dim[0] + i;
}

__device__ __forceinline__ void load_tri(const double* __restrict__ P, const int32_t* __restrict__ T, int t,
                                         double (&A)[3], double (&B)[3], double (&C)[3]) {
  const int a = T[3 * (size_t)t], b = T[3 * (size_t)t + 1], c = T[3 * (size_t)t + 2];
  for (int k = 0; k < 3; ++k) {
    A[k] = P[3 * (size_t)a + k];
    B[k] = P[3 * (size_t)b + k];
    C[k] = P[3 * (size_t)c + k];
  }
}

__device__ __forceinline__ double min3(double a, double b, double c) { return fmin(fmin(a, b), c); }
__device__ __forceinline__ double max3(double a, double b, double c) { return fmax(fmax(a, b), c); }

// Lower-bound pre-filter of the exact distance: a voxel whose lower bound
// (FP32, less twice a margin of 1e-3 voxel plus 1e-6 of the largest grid
// coordinate, which covers the FP32 rounding of the plane evaluations) is not
// below the voxel's current minimum cannot lower it — the exact FP64 distance
// is at least as large, and rounding to float is monotone — so its FP64
// evaluation is skipped. The stored result is the same minimum as without the
// filter. The bound is the larger of the gap to the triangle's bounding box
// and sqrt(p^2 + s^2), with p the distance to the triangle's plane and s the
// largest distance beyond one of its edges in the plane: with n the unit
// normal and m_e the unit in-plane normal of edge e pointing away from the
// triangle (offset so that no vertex lies beyond it), every triangle point x
// has |q - x|^2 >= (n.(q - x))^2 + (m_e.(q - x))^2 >= p^2 + s_e^2.
// Per-triangle set-up of the band distances (one thread per triangle, once):
// the voxel box grown by the band, the FP32 bounding box, and the FP32 plane
// and edge planes of the lower bound.
struct SdfTri {
  int lo[3], ext[3];      // voxel box (ext[0] <= 0: nothing in the grid)
  float blo[3], bhi[3];   // bounding box rounded outwards
  float4 pl;              // unit normal, offset; w of fe[0] = -1e30 without a plane
  float4 fe[3];           // unit in-plane edge normals, offsets (no vertex beyond)
  int has_plane, pad[3];
};

constexpr int kSdfChunk = 1024;  // box voxels per work item of the distance passes

__global__ void sdf_tri_prep_kernel(const double* __restrict__ P, const int32_t* __restrict__ T, int nt, SdfGrid g,
                                    SdfTri* __restrict__ out, uint32_t* __restrict__ chunks) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += gridDim.x * blockDim.x) {
    double A[3], B[3], C[3];
    load_tri(P, T, t, A, B, C);
    SdfTri r;
    for (int a = 0; a < 3; ++a) {
      const double mn = min3(A[a], B[a], C[a]), mx = max3(A[a], B[a], C[a]);
      r.lo[a] = max(0, (int)floor(mn - g.band) - g.org[a]);
      const int hi = min(g.dim[a] - 1, (int)ceil(mx + g.band) - g.org[a]);
      r.ext[a] = hi - r.lo[a] + 1;
      r.blo[a] = __double2float_rd(mn);
      r.bhi[a] = __double2float_ru(mx);
    }
    if (r.ext[0] <= 0 || r.ext[1] <= 0 || r.ext[2] <= 0) r.ext[0] = 0;
    // unit normal and plane offset (FP32 copies; degenerate triangles get none)
    const double ux = B[0] - A[0], uy = B[1] - A[1], uz = B[2] - A[2];
    const double vx = C[0] - A[0], vy = C[1] - A[1], vz = C[2] - A[2];
    double nx = uy * vz - uz * vy, ny = uz * vx - ux * vz, nz = ux * vy - uy * vx;
    const double nl = sqrt(nx * nx + ny * ny + nz * nz);
    r.has_plane = nl > 1e-12;
    r.pl = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int e = 0; e < 3; ++e) r.fe[e] = make_float4(0.f, 0.f, 0.f, -1e30f);
    if (r.has_plane) {
      nx /= nl;
      ny /= nl;
      nz /= nl;
      r.pl = make_float4((float)nx, (float)ny, (float)nz, (float)-(nx * A[0] + ny * A[1] + nz * A[2]));
      const double* V[3] = {A, B, C};
      for (int e = 0; e < 3; ++e) {
        const double* P0 = V[e];
        const double* P1 = V[(e + 1) % 3];
        const double* P2 = V[(e + 2) % 3];
        const double ex = P1[0] - P0[0], ey = P1[1] - P0[1], ez = P1[2] - P0[2];
        double mx = ny * ez - nz * ey, my = nz * ex - nx * ez, mz = nx * ey - ny * ex;
        const double ml = sqrt(mx * mx + my * my + mz * mz);
        if (!(ml > 1e-12)) continue;
        mx /= ml;
        my /= ml;
        mz /= ml;
        if (mx * (P2[0] - P0[0]) + my * (P2[1] - P0[1]) + mz * (P2[2] - P0[2]) > 0) {
          mx = -mx;
          my = -my;
          mz = -mz;
        }
        const double top = fmax(fmax(mx * A[0] + my * A[1] + mz * A[2], mx * B[0] + my * B[1] + mz * B[2]),
                                mx * C[0] + my * C[1] + mz * C[2]);
        r.fe[e] = make_float4((float)mx, (float)my, (float)mz, (float)-top);
      }
    }
    out[t] = r;
    chunks[t] = r.ext[0] > 0 ? (uint32_t)((r.ext[0] * r.ext[1] * r.ext[2] + kSdfChunk - 1) / kSdfChunk) : 0u;
  }
}

// Work items of the distance passes: (triangle, chunk of kSdfChunk voxels of
// its box), numbered by the scanned chunk counts. Block b takes a contiguous
// range of items, so a triangle with a large box (the long triangles of a
// clipped part's cap) is spread over several blocks instead of holding one
// while the rest of the grid idles.
struct SdfItems {
  const uint64_t* off;  // nt + 1 scanned chunk counts
  int nt;
};

__device__ __forceinline__ void item_range(const SdfItems& W, long long& w0, long long& w1) {
  const long long total = (long long)W.off[W.nt];
  const long long per = (total + gridDim.x - 1) / gridDim.x;
  w0 = (long long)blockIdx.x * per;
  w1 = min(total, w0 + per);
}

// Triangle of item w (off[t] <= w < off[t + 1]).
__device__ __forceinline__ int item_triangle(const SdfItems& W, long long w) {
  int lo = 0, hi = W.nt;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if ((long long)W.off[mid] <= w) lo = mid;
    else hi = mid;
  }
  return lo;
}

// FP32 upper bound of the distance from q to triangle (A, B, C): the distance
// to a point of the triangle chosen in FP32 by the closest-point regions
// (Ericson, Real-Time Collision Detection 5.1.5), taken as A + v AB + w AC
// with v, w clamped to v, w >= 0, v + w <= 1 so that the exact point with
// these weights lies on the triangle; `slack` covers the FP32 rounding of the
// point and of the distance.
__device__ float tri_dist_ub32(float qx, float qy, float qz, const float (&A)[3], const float (&B)[3],
                               const float (&C)[3], float slack) {
  const float ab[3] = {B[0] - A[0], B[1] - A[1], B[2] - A[2]};
  const float ac[3] = {C[0] - A[0], C[1] - A[1], C[2] - A[2]};
  const float ap[3] = {qx - A[0], qy - A[1], qz - A[2]};
  const float bp[3] = {qx - B[0], qy - B[1], qz - B[2]};
  const float cp[3] = {qx - C[0], qy - C[1], qz - C[2]};
  auto dot = [](const float (&x)[3], const float (&y)[3]) { return x[0] * y[0] + x[1] * y[1] + x[2] * y[2]; };
  const float d1 = dot(ab, ap), d2 = dot(ac, ap), d3 = dot(ab, bp), d4 = dot(ac, bp), d5 = dot(ab, cp),
              d6 = dot(ac, cp);
  float v = 0.f, w = 0.f;
  const float vc = d1 * d4 - d3 * d2, vb = d5 * d2 - d1 * d6, va = d3 * d6 - d5 * d4;
  if (d1 <= 0.f && d2 <= 0.f) {
  } else if (d3 >= 0.f && d4 <= d3) {
    v = 1.f;
  } else if (vc <= 0.f && d1 >= 0.f && d3 <= 0.f) {
    v = d1 / (d1 - d3);
  } else if (d6 >= 0.f && d5 <= d6) {
    w = 1.f;
  } else if (vb <= 0.f && d2 >= 0.f && d6 <= 0.f) {
    w = d2 / (d2 - d6);
  } else if (va <= 0.f && (d4 - d3) >= 0.f && (d5 - d6) >= 0.f) {
    w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
    v = 1.f - w;
  } else {
    const float den = 1.f / (va + vb + vc);
    v = vb * den;
    w = vc * den;
  }
  v = fminf(fmaxf(v, 0.f), 1.f);  // NaN (degenerate triangle) becomes 0
  w = fminf(fmaxf(w, 0.f), 1.f - v);
  const float px = A[0] + v * ab[0] + w * ac[0], py = A[1] + v * ab[1] + w * ac[1], pz = A[2] + v * ab[2] + w * ac[2];
  const float ex = qx - px, ey = qy - py, ez = qz - pz;
  return __fadd_ru(__fmul_ru(__fsqrt_ru(__fadd_ru(__fadd_ru(__fmul_ru(ex, ex), __fmul_ru(ey, ey)), __fmul_ru(ez, ez))),
                             1.0f + 1.0f / 65536.0f),
                   slack);
}

// FP32 band voxel bound between the triangle's lower bound and its FP32 upper
// bound (first pass): ub[v] ends at or above the voxel's exact distance, so
// the exact pass can skip every triangle whose lower bound reaches it.
__device__ __forceinline__ float sdf_lower_bound(const SdfTri& r, float qx, float qy, float qz) {
  const float gx = fmaxf(fmaxf(r.blo[0] - qx, qx - r.bhi[0]), 0.f);
  const float gy = fmaxf(fmaxf(r.blo[1] - qy, qy - r.bhi[1]), 0.f);
  const float gz = fmaxf(fmaxf(r.blo[2] - qz, qz - r.bhi[2]), 0.f);
  float lb = sqrtf(gx * gx + gy * gy + gz * gz);
  if (r.has_plane) {
    const float pd = fabsf(r.pl.x * qx + r.pl.y * qy + r.pl.z * qz + r.pl.w);
    float se = 0.f;
    for (int e = 0; e < 3; ++e) se = fmaxf(se, r.fe[e].x * qx + r.fe[e].y * qy + r.fe[e].z * qz + r.fe[e].w);
    lb = fmaxf(lb, sqrtf(pd * pd + se * se));
  }
  return lb;
}

__global__ void __launch_bounds__(128) sdf_ub_kernel(const double* __restrict__ P, const int32_t* __restrict__ T,
                                                     SdfItems W, SdfGrid g, const SdfTri* __restrict__ prep,
                                                     uint32_t* __restrict__ ub) {
  long long w0, w1;
  item_range(W, w0, w1);
  int t = w0 < w1 ? item_triangle(W, w0) : 0;
  for (long long w = w0; w < w1; ++w) {
    while ((long long)W.off[t + 1] <= w) ++t;
    const SdfTri r = prep[t];
    double Ad[3], Bd[3], Cd[3];
    load_tri(P, T, t, Ad, Bd, Cd);
    const float A[3] = {(float)Ad[0], (float)Ad[1], (float)Ad[2]};
    const float B[3] = {(float)Bd[0], (float)Bd[1], (float)Bd[2]};
    const float C[3] = {(float)Cd[0], (float)Cd[1], (float)Cd[2]};
    // rounding of the vertices to float, of the chosen point and of its
    // distance: a few units of 2^-24 of the largest coordinate involved
    float mabs = 0.f;
    for (int a = 0; a < 3; ++a) mabs = fmaxf(mabs, fmaxf(fabsf(A[a]), fmaxf(fabsf(B[a]), fabsf(C[a]))));
    const int n = r.ext[0] * r.ext[1] * r.ext[2];
    const int c0 = (int)(w - (long long)W.off[t]) * kSdfChunk, c1 = min(n, c0 + kSdfChunk);
    for (int q0 = c0 + threadIdx.x; q0 < c1; q0 += blockDim.x) {
      const int i = r.lo[0] + q0 % r.ext[0], j = r.lo[1] + (q0 / r.ext[0]) % r.ext[1],
                k = r.lo[2] + q0 / (r.ext[0] * r.ext[1]);
      const size_t v = vid(g, i, j, k);
      const float qx = (float)(g.org[0] + i), qy = (float)(g.org[1] + j), qz = (float)(g.org[2] + k);
      const float lb = sdf_lower_bound(r, qx, qy, qz);
      const float cur = __uint_as_float(*(volatile const uint32_t*)&ub[v]);
      if (lb - 2.0f * g.margin >= cur) continue;
      const float qa = fmaxf(fabsf(qx), fmaxf(fabsf(qy), fabsf(qz)));
      const float slack = 64.0f * kSdfU * fmaxf(mabs, qa) + g.margin;
      atomicMin(&ub[v], __float_as_uint(tri_dist_ub32(qx, qy, qz, A, B, C, slack)));
    }
  }
}

// Each work item (a chunk of kSdfChunk box voxels) is filtered first; the
// voxels that pass are appended to a shared list and evaluated in FP64 by all
// threads together, so the FP64 pipe (slow on this part) runs with full warps
// instead of the few lanes that pass the filter in each warp.
__global__ void __launch_bounds__(128) sdf_dist_kernel(const double* __restrict__ P, const int32_t* __restrict__ T,
                                                       SdfItems W, SdfGrid g, const SdfTri* __restrict__ prep,
                                                       const uint32_t* __restrict__ ub, uint32_t* __restrict__ dist) {
  __shared__ int list[kSdfChunk];
  __shared__ int count;
  const int lane = threadIdx.x & 31;
  long long w0, w1;
  item_range(W, w0, w1);
  int t = w0 < w1 ? item_triangle(W, w0) : 0;
  for (long long w = w0; w < w1; ++w) {
    while ((long long)W.off[t + 1] <= w) ++t;
    const SdfTri& r = prep[t];
    const int ex0 = r.ext[0], ex1 = r.ext[1], ex2 = r.ext[2];
    const int lo0 = r.lo[0], lo1 = r.lo[1], lo2 = r.lo[2];
    const float blo0 = r.blo[0], blo1 = r.blo[1], blo2 = r.blo[2];
    const float bhi0 = r.bhi[0], bhi1 = r.bhi[1], bhi2 = r.bhi[2];
    const bool has_plane = r.has_plane != 0;
    const float4 pl = r.pl, fe0 = r.fe[0], fe1 = r.fe[1], fe2 = r.fe[2];
    double A[3], B[3], C[3];
    load_tri(P, T, t, A, B, C);
    const int n = ex0 * ex1 * ex2;
    const int c0 = (int)(w - (long long)W.off[t]) * kSdfChunk, c1 = min(n, c0 + kSdfChunk);
    if (threadIdx.x == 0) count = 0;
    __syncthreads();
    for (int base = c0; base < c1; base += blockDim.x) {
      const int q0 = base + threadIdx.x;
      bool keep = false;
      if (q0 < c1) {
        const int i = lo0 + q0 % ex0, j = lo1 + (q0 / ex0) % ex1, k = lo2 + q0 / (ex0 * ex1);
        const size_t v = vid(g, i, j, k);
        const float qx = (float)(g.org[0] + i), qy = (float)(g.org[1] + j), qz = (float)(g.org[2] + k);
        const float gx = fmaxf(fmaxf(blo0 - qx, qx - bhi0), 0.f);
        const float gy = fmaxf(fmaxf(blo1 - qy, qy - bhi1), 0.f);
        const float gz = fmaxf(fmaxf(blo2 - qz, qz - bhi2), 0.f);
        float lb = sqrtf(gx * gx + gy * gy + gz * gz);
        if (has_plane) {
          const float pd = fabsf(pl.x * qx + pl.y * qy + pl.z * qz + pl.w);
          float se = 0.f;
          se = fmaxf(se, fe0.x * qx + fe0.y * qy + fe0.z * qz + fe0.w);
          se = fmaxf(se, fe1.x * qx + fe1.y * qy + fe1.z * qz + fe1.w);
          se = fmaxf(se, fe2.x * qx + fe2.y * qy + fe2.z * qz + fe2.w);
          lb = fmaxf(lb, sqrtf(pd * pd + se * se));
        }
        const float cur = fminf(__uint_as_float(*(volatile const uint32_t*)&dist[v]), __uint_as_float(ub[v]));
        keep = lb - 2.0f * g.margin < cur;
      }
      // warp-aggregated append (at most kSdfChunk entries per item)
      const unsigned m = __ballot_sync(0xffffffffu, keep);
      int at = 0;
      if (lane == 0 && m) at = atomicAdd(&count, __popc(m));
      at = __shfl_sync(0xffffffffu, at, 0);
      if (keep) list[at + __popc(m & ((1u << lane) - 1u))] = q0;
    }
    __syncthreads();
    const int nc = count;
    for (int e = threadIdx.x; e < nc; e += blockDim.x) {
      const int q0 = list[e];
      const int i = lo0 + q0 % ex0, j = lo1 + (q0 / ex0) % ex1, k = lo2 + q0 / (ex0 * ex1);
      const double q[3] = {(double)(g.org[0] + i), (double)(g.org[1] + j), (double)(g.org[2] + k)};
      const float d = __double2float_rn(point_tri_dist(q, A, B, C));
      atomicMin(&dist[vid(g, i, j, k)], __float_as_uint(d));
    }
    __syncthreads();
  }
}

// Crossing of one ray (grid column (ku, kw) along axis ax) with a triangle:
// toggles the first voxel whose centre lies beyond the crossing.
__device__ __forceinline__ void cross_ray(const double (&A)[3], const double (&B)[3], const double (&C)[3],
                                          const SdfGrid& g, int ax, int u, int w, int ku, int kw,
                                          uint32_t* __restrict__ toggle) {
  const double ou = 1.2345679e-6, ow = 2.3456789e-6;
  const double y = da((double)(g.org[u] + ku), ou), z = da((double)(g.org[w] + kw), ow);
  const double e0 = ds(dm(ds(B[u], A[u]), ds(z, A[w])), dm(ds(B[w], A[w]), ds(y, A[u])));
  const double e1 = ds(dm(ds(C[u], B[u]), ds(z, B[w])), dm(ds(C[w], B[w]), ds(y, B[u])));
  const double e2 = ds(dm(ds(A[u], C[u]), ds(z, C[w])), dm(ds(A[w], C[w]), ds(y, C[u])));
  const bool in = (e0 > 0 && e1 > 0 && e2 > 0) || (e0 < 0 && e1 < 0 && e2 < 0);
  if (!in) return;
  const double sw = da(da(e0, e1), e2);
  const double x = __ddiv_rn(da(da(dm(e1, A[ax]), dm(e2, B[ax])), dm(e0, C[ax])), sw);
  // first voxel s whose centre org + s lies beyond x (integers compare exactly)
  int s = (int)floor(x - (double)g.org[ax]) + 1;
  while (s > 0 && (double)(g.org[ax] + s - 1) > x) --s;
  while (s < g.dim[ax] && !((double)(g.org[ax] + s) > x)) ++s;
  if (s < 0) s = 0;
  if (s >= g.dim[ax]) return;
  int gi[3];
  gi[ax] = s;
  gi[u] = ku;
  gi[w] = kw;
  atomicXor(&toggle[vid(g, gi[0], gi[1], gi[2])], 1u);
}

// The rays a triangle covers: its box projected on the grid plane.
__device__ __forceinline__ bool ray_box(const double (&A)[3], const double (&B)[3], const double (&C)[3],
                                        const SdfGrid& g, int u, int w, int& u0, int& w0, int& eu, int& ew) {
  u0 = max(0, (int)floor(min3(A[u], B[u], C[u]) - g.org[u]));
  const int u1 = min(g.dim[u] - 1, (int)ceil(max3(A[u], B[u], C[u]) - g.org[u]));
  w0 = max(0, (int)floor(min3(A[w], B[w], C[w]) - g.org[w]));
  const int w1 = min(g.dim[w] - 1, (int)ceil(max3(A[w], B[w], C[w]) - g.org[w]));
  eu = u1 - u0 + 1;
  ew = w1 - w0 + 1;
  return eu > 0 && ew > 0;
}

// Triangles covering at most kCrossSmall rays (nearly all): kCrossLanes lanes
// each, over its rays. Larger ones (the long triangles of clipped parts' caps,
// big faces): one block each (sdf_cross_wide_kernel).
constexpr int kCrossSmall = 32;
constexpr int kCrossLanes = 8;

__global__ void __launch_bounds__(128) sdf_cross_kernel(const double* __restrict__ P, const int32_t* __restrict__ T,
                                                        int nt, SdfGrid g, int ax, uint32_t* __restrict__ toggle,
                                                        int* __restrict__ wide, unsigned* __restrict__ n_wide) {
  const int u = (ax + 1) % 3, w = (ax + 2) % 3;
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  const int sub = gid % kCrossLanes;
  const int groups = (gridDim.x * blockDim.x) / kCrossLanes;
  for (int t = gid / kCrossLanes; t < nt; t += groups) {
    double A[3], B[3], C[3];
    load_tri(P, T, t, A, B, C);
    int u0, w0, eu, ew;
    if (!ray_box(A, B, C, g, u, w, u0, w0, eu, ew)) continue;
    if (eu * ew > kCrossSmall) {
      if (sub == 0) wide[atomicAdd(n_wide, 1u)] = t;
      continue;
    }
    for (int r = sub; r < eu * ew; r += kCrossLanes)
      cross_ray(A, B, C, g, ax, u, w, u0 + r % eu, w0 + r / eu, toggle);
  }
}

__global__ void __launch_bounds__(128) sdf_cross_wide_kernel(const double* __restrict__ P,
                                                             const int32_t* __restrict__ T, SdfGrid g, int ax,
                                                             const int* __restrict__ wide,
                                                             const unsigned* __restrict__ n_wide,
                                                             uint32_t* __restrict__ toggle) {
  const int u = (ax + 1) % 3, w = (ax + 2) % 3;
  const int nw = (int)*n_wide;
  for (int k = blockIdx.x; k < nw; k += gridDim.x) {
    const int t = wide[k];
    double A[3], B[3], C[3];
    load_tri(P, T, t, A, B, C);
    int u0, w0, eu, ew;
    if (!ray_box(A, B, C, g, u, w, u0, w0, eu, ew)) continue;
    for (int r = threadIdx.x; r < eu * ew; r += blockDim.x)
      cross_ray(A, B, C, g, ax, u, w, u0 + r % eu, w0 + r / eu, toggle);
  }
}

__global__ void sdf_parity_kernel(SdfGrid g, int ax, const uint32_t* __restrict__ toggle,
                                  uint8_t* __restrict__ votes) {
  const int u = (ax + 1) % 3, w = (ax + 2) % 3;
  const int ncol = g.dim[u] * g.dim[w];
  for (int col = blockIdx.x * blockDim.x + threadIdx.x; col < ncol; col += gridDim.x * blockDim.x) {
    int gi[3];
    gi[u] = col % g.dim[u];
    gi[w] = col / g.dim[u];
    uint32_t par = 0;
    for (int i = 0; i < g.dim[ax]; ++i) {
      gi[ax] = i;
      const size_t v = vid(g, gi[0], gi[1], gi[2]);
      par ^= toggle[v];
      if (par & 1u) votes[v] += 1;
    }
  }
}

__global__ void sdf_field_kernel(const uint32_t* __restrict__ dist, const uint8_t* __restrict__ votes, size_t n,
                                 float* __restrict__ f) {
  for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (size_t)gridDim.x * blockDim.x) {
    const float d = __uint_as_float(dist[v]);
    f[v] = votes[v] >= 2 ? -d : d;
  }
}

__constant__ int kCorner[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {1, 1, 0},
                                  {0, 0, 1}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};
__constant__ int kCedge[12][2] = {{0, 1}, {2, 3}, {4, 5}, {6, 7}, {0, 2}, {1, 3},
                                  {4, 6}, {5, 7}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};

__device__ __forceinline__ int corner_values(const SdfGrid& g, const float* __restrict__ f, int i, int j, int k,
                                             float (&cv)[8]) {
  int nin = 0;
  for (int c = 0; c < 8; ++c) {
    cv[c] = f[vid(g, i + kCorner[c][0], j + kCorner[c][1], k + kCorner[c][2])];
    nin += cv[c] < g.fiso;
  }
  return nin;
}

__global__ void sdf_cell_flag_kernel(SdfGrid g, const float* __restrict__ f, uint32_t* __restrict__ flag) {
  const int cx = g.dim[0] - 1, cy = g.dim[1] - 1, cz = g.dim[2] - 1;
  const size_t n = (size_t)cx * cy * cz;
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(c % cx), j = (int)((c / cx) % cy), k = (int)(c / ((size_t)cx * cy));
    float cv[8];
    const int nin = corner_values(g, f, i, j, k, cv);
    flag[c] = (nin != 0 && nin != 8) ? 1u : 0u;
  }
}

__global__ void sdf_cell_vertex_kernel(SdfGrid g, const float* __restrict__ f, const uint32_t* __restrict__ flag,
                                       const uint64_t* __restrict__ off, int32_t* __restrict__ cell_vertex,
                                       double* __restrict__ out_v) {
  const int cx = g.dim[0] - 1, cy = g.dim[1] - 1, cz = g.dim[2] - 1;
  const size_t n = (size_t)cx * cy * cz;
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    if (!flag[c]) {
      cell_vertex[c] = -1;
      continue;
    }
    const int i = (int)(c % cx), j = (int)((c / cx) % cy), k = (int)(c / ((size_t)cx * cy));
    float cv[8];
    corner_values(g, f, i, j, k, cv);
    double acc[3] = {0, 0, 0};
    int ncross = 0;
    for (int e = 0; e < 12; ++e) {
      const int c0 = kCedge[e][0], c1 = kCedge[e][1];
      if ((cv[c0] < g.fiso) == (cv[c1] < g.fiso)) continue;
      const double t = __ddiv_rn((double)__fsub_rn(g.fiso, cv[c0]), (double)__fsub_rn(cv[c1], cv[c0]));
      for (int a = 0; a < 3; ++a)
        acc[a] = da(acc[a], da((double)kCorner[c0][a], dm(t, (double)(kCorner[c1][a] - kCorner[c0][a]))));
      ++ncross;
    }
    const int vtx = (int)off[c];
    cell_vertex[c] = vtx;
    const int ijk[3] = {i, j, k};
    for (int a = 0; a < 3; ++a) {
      const double m = __ddiv_rn(acc[a], (double)ncross);
      out_v[3 * (size_t)vtx + a] = __ddiv_rn(da((double)(g.org[a] + ijk[a]), m), g.scale);
    }
  }
}

// Quads of interior voxel (i, j, k) in the host's order (+x, +y, +z edges),
// each as two triangles; returns the triangle count, writes them when out.
__device__ __forceinline__ int voxel_quads(const SdfGrid& g, const float* __restrict__ f,
                                           const int32_t* __restrict__ cv, int i, int j, int k,
                                           int32_t* __restrict__ out) {
  const int cx = g.dim[0] - 1, cy = g.dim[1] - 1;
  auto cid = [&](int a, int b, int c) { return ((size_t)c * cy + b) * cx + a; };
  const bool in0 = f[vid(g, i, j, k)] < g.fiso;
  int n = 0;
  auto emit = [&](int q0, int q1, int q2, int q3, bool flip) {
    if (q0 < 0 || q1 < 0 || q2 < 0 || q3 < 0) return;
    if (flip) {
      const int t = q1;
      q1 = q3;
      q3 = t;
    }
    if (out) {
      out[3 * n] = q0;
      out[3 * n + 1] = q1;
      out[3 * n + 2] = q2;
      out[3 * n + 3] = q0;
      out[3 * n + 4] = q2;
      out[3 * n + 5] = q3;
    }
    n += 2;
  };
  if (in0 != (f[vid(g, i + 1, j, k)] < g.fiso))
    emit(cv[cid(i, j - 1, k - 1)], cv[cid(i, j, k - 1)], cv[cid(i, j, k)], cv[cid(i, j - 1, k)], !in0);
  if (in0 != (f[vid(g, i, j + 1, k)] < g.fiso))
    emit(cv[cid(i - 1, j, k - 1)], cv[cid(i - 1, j, k)], cv[cid(i, j, k)], cv[cid(i, j, k - 1)], !in0);
  if (in0 != (f[vid(g, i, j, k + 1)] < g.fiso))
    emit(cv[cid(i - 1, j - 1, k)], cv[cid(i, j - 1, k)], cv[cid(i, j, k)], cv[cid(i - 1, j, k)], !in0);
  return n;
}

__global__ void sdf_quad_kernel(SdfGrid g, const float* __restrict__ f, const int32_t* __restrict__ cell_vertex,
                                uint32_t* __restrict__ count, const uint64_t* __restrict__ off,
                                int32_t* __restrict__ out_t) {
  const int ix = g.dim[0] - 2, iy = g.dim[1] - 2, iz = g.dim[2] - 2;
  const size_t n = (size_t)ix * iy * iz;
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (size_t)gridDim.x * blockDim.x) {
    const int i = 1 + (int)(r % ix), j = 1 + (int)((r / ix) % iy), k = 1 + (int)(r / ((size_t)ix * iy));
    if (off)
      voxel_quads(g, f, cell_vertex, i, j, k, out_t + 3 * (size_t)off[r]);
    else
      count[r] = (uint32_t)voxel_quads(g, f, cell_vertex, i, j, k, nullptr);
  }
}

__global__ void sdf_fill_kernel(uint32_t* __restrict__ p, size_t n, uint32_t v) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) p[i] = v;
}

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace
}  // namespace vgpu

using namespace vgpu;

extern "C" int visacd_sdf_remesh(visacd_ctx* ctx, const double* verts, int32_t nv, const int32_t* tris, int32_t nt,
                                 double scale, double level, int32_t* out_nv, int32_t* out_nt) {
  VCHECK(ctx && out_nv && out_nt, VISACD_ERR_INVALID_ARG, "sdf_remesh: null argument");
  VCHECK(nv >= 0 && nt >= 0 && (nt == 0 || (verts && tris)), VISACD_ERR_INVALID_ARG, "sdf_remesh: bad sizes");
  VCHECK(scale > 0, VISACD_ERR_INVALID_ARG, "sdf_remesh: scale must be positive");
  ctx->sdf_nv = ctx->sdf_nt = 0;
  *out_nv = *out_nt = 0;
  if (nt == 0 || nv == 0) return VISACD_OK;
  VCHECK(indices_in_range(tris, 3LL * nt, nv), VISACD_ERR_INVALID_ARG, "sdf_remesh: triangle index out of range");
  VCUDA(cudaSetDevice(ctx->device));
  // Grid (host arithmetic of manifold_preprocess).
  std::vector<double> P(3 * (size_t)nv);
  double lo[3] = {1e308, 1e308, 1e308}, hi[3] = {-1e308, -1e308, -1e308};
  for (int32_t i = 0; i < nv; ++i)
    for (int a = 0; a < 3; ++a) {
      const double x = verts[3 * (size_t)i + a] * scale;
      P[3 * (size_t)i + a] = x;
      lo[a] = std::min(lo[a], x);
      hi[a] = std::max(hi[a], x);
    }
  const double iso = level * scale;
  SdfGrid g;
  g.band = std::max(iso, 0.0) + 2.0;
  g.fiso = (float)iso;
  g.scale = scale;
  for (int a = 0; a < 3; ++a) {
    g.org[a] = (int)std::floor(lo[a] - g.band - 2.0);
    g.dim[a] = (int)std::ceil(hi[a] + g.band + 2.0) - g.org[a] + 1;
  }
  VCHECK(g.dim[0] >= 3 && g.dim[1] >= 3 && g.dim[2] >= 3, VISACD_ERR_INVALID_ARG, "sdf_remesh: degenerate grid");
  double qmax = 0;
  for (int a = 0; a < 3; ++a)
    qmax = std::max(qmax, std::max(std::fabs((double)g.org[a]), std::fabs((double)g.org[a] + g.dim[a])));
  g.margin = (float)(1e-3 + 1e-6 * qmax);
  const size_t nvox = (size_t)g.dim[0] * g.dim[1] * g.dim[2];
  VCHECK(nvox <= ((size_t)1 << 30), VISACD_ERR_CAPACITY, "sdf_remesh: grid of %zu voxels is too large", nvox);
  const size_t ncell = (size_t)(g.dim[0] - 1) * (g.dim[1] - 1) * (g.dim[2] - 1);
  const size_t nint = (size_t)(g.dim[0] - 2) * (g.dim[1] - 2) * (g.dim[2] - 2);
  // Scratch layout in one buffer.
  size_t at = 0;
  auto take = [&](size_t bytes) {
    const size_t o = at;
    at += align256(bytes);
    return o;
  };
  const size_t oP = take(P.size() * 8), oT = take(3 * (size_t)nt * 4), oPrep = take((size_t)nt * sizeof(SdfTri)),
               oWide = take(3 * (size_t)nt * 4), oNWide = take(16), oChunks = take((size_t)nt * 4),
               oChunkOff = take(((size_t)nt + 1) * 8),
               oDist = take(nvox * 4),
               oTog = take(nvox * 4), oVotes = take(nvox), oF = take(nvox * 4), oFlag = take(ncell * 4),
               oCoff = take((ncell + 1) * 8), oCv = take(ncell * 4), oQcnt = take(nint * 4),
               oQoff = take((nint + 1) * 8);
  VTRY(ensure_slot(ctx, kSlotSdf, at));
  char* base = slot<char>(ctx, kSlotSdf);
  double* dP = (double*)(base + oP);
  int32_t* dT = (int32_t*)(base + oT);
  uint32_t* dist = (uint32_t*)(base + oDist);
  uint32_t* tog = (uint32_t*)(base + oTog);
  uint8_t* votes = (uint8_t*)(base + oVotes);
  float* f = (float*)(base + oF);
  uint32_t* flag = (uint32_t*)(base + oFlag);
  uint64_t* coff = (uint64_t*)(base + oCoff);
  int32_t* cv = (int32_t*)(base + oCv);
  uint32_t* qcnt = (uint32_t*)(base + oQcnt);
  uint64_t* qoff = (uint64_t*)(base + oQoff);
  cudaStream_t st = ctx->stream;
  Stager up(ctx);
  VTRY(up.reserve(P.size() * 8 + 3 * (size_t)nt * 4, 2));
  VTRY(up.put(dP, P.data(), P.size() * 8));
  VTRY(up.put(dT, tris, 3 * (size_t)nt * 4));
  const unsigned gv = grid_for((int64_t)nvox, 256, 16 * (int64_t)ctx->sm_count);
  const float band_f = (float)g.band;
  uint32_t band_bits;
  std::memcpy(&band_bits, &band_f, 4);
  VLAUNCH(ctx, kKSdf, gv, 256, 0, sdf_fill_kernel, dist, nvox, band_bits);
  VCUDA(cudaMemsetAsync(votes, 0, nvox, st));
  SdfTri* prep = (SdfTri*)(base + oPrep);
  uint32_t* chunks = (uint32_t*)(base + oChunks);
  uint64_t* chunk_off = (uint64_t*)(base + oChunkOff);
  VLAUNCH(ctx, kKSdfDist, grid_for(nt, 128, 16 * (int64_t)ctx->sm_count), 128, 0, sdf_tri_prep_kernel, dP, dT, nt,
          g, prep, chunks);
  VTRY(exclusive_scan_u32_to_u64(ctx, chunks, chunk_off, nt));
  SdfItems items;
  items.off = chunk_off;
  items.nt = nt;
  const unsigned gw = (unsigned)(8 * (int64_t)ctx->sm_count);
  // First pass: FP32 upper bounds per voxel in the toggle buffer (free until
  // the crossings), then the exact pass.
  VLAUNCH(ctx, kKSdf, gv, 256, 0, sdf_fill_kernel, tog, nvox, band_bits);
  VLAUNCH(ctx, kKSdfDist, gw, 128, 0, sdf_ub_kernel, dP, dT, items, g, (const SdfTri*)prep, tog);
  VLAUNCH(ctx, kKSdfDist, gw, 128, 0, sdf_dist_kernel, dP, dT, items, g, (const SdfTri*)prep, (const uint32_t*)tog,
          dist);
  // Per axis: the triangles covering many rays are listed by the first
  // kernel and done one block each by the second (lists and counts per axis).
  int* wide = (int*)(base + oWide);
  unsigned* n_wide = (unsigned*)(base + oNWide);
  VCUDA(cudaMemsetAsync(n_wide, 0, 16, st));
  for (int ax = 0; ax < 3; ++ax) {
    VCUDA(cudaMemsetAsync(tog, 0, nvox * 4, st));
    VLAUNCH(ctx, kKSdfCross, grid_for((int64_t)kCrossLanes * nt, 128, 16 * (int64_t)ctx->sm_count), 128, 0,
            sdf_cross_kernel, dP, dT, nt, g, ax, tog, wide + (size_t)ax * nt, n_wide + ax);
    VLAUNCH(ctx, kKSdfCross, (unsigned)std::min<int64_t>(nt, 4 * (int64_t)ctx->sm_count), 128, 0,
            sdf_cross_wide_kernel, dP, dT, g, ax, (const int*)(wide + (size_t)ax * nt),
            (const unsigned*)(n_wide + ax), tog);
    const int u = (ax + 1) % 3, w = (ax + 2) % 3;
    VLAUNCH(ctx, kKSdfCross, grid_for((int64_t)g.dim[u] * g.dim[w], 128, 1 << 20), 128, 0, sdf_parity_kernel, g, ax,
            tog, votes);
  }
  VLAUNCH(ctx, kKSdf, gv, 256, 0, sdf_field_kernel, dist, votes, nvox, f);
  const unsigned gc = grid_for((int64_t)ncell, 256, 16 * (int64_t)ctx->sm_count);
  VLAUNCH(ctx, kKSdf, gc, 256, 0, sdf_cell_flag_kernel, g, f, flag);
  VTRY(exclusive_scan_u32_to_u64(ctx, flag, coff, (int64_t)ncell));
  const unsigned gq = grid_for((int64_t)nint, 256, 16 * (int64_t)ctx->sm_count);
  uint64_t totals[2];
  VCUDA(cudaMemcpyAsync(&totals[0], coff + ncell, 8, cudaMemcpyDeviceToHost, st));
  VCUDA(stream_wait(ctx));
  VCHECK(totals[0] < (1ull << 31), VISACD_ERR_CAPACITY, "sdf_remesh: too many vertices");
  VTRY(ensure_slot(ctx, kSlotSdfOut, align256(totals[0] * 24) + 256));
  double* out_v = slot<double>(ctx, kSlotSdfOut);
  VLAUNCH(ctx, kKSdf, gc, 256, 0, sdf_cell_vertex_kernel, g, f, flag, coff, cv, out_v);
  VLAUNCH(ctx, kKSdf, gq, 256, 0, sdf_quad_kernel, g, f, cv, qcnt, (const uint64_t*)nullptr,
          (int32_t*)nullptr);
  VTRY(exclusive_scan_u32_to_u64(ctx, qcnt, qoff, (int64_t)nint));
  VCUDA(cudaMemcpyAsync(&totals[1], qoff + nint, 8, cudaMemcpyDeviceToHost, st));
  VCUDA(stream_wait(ctx));
  VCHECK(totals[1] < (1ull << 31), VISACD_ERR_CAPACITY, "sdf_remesh: too many triangles");
  VTRY(ensure_slot(ctx, kSlotSdfTris, align256(totals[1] * 12) + 256));
  VLAUNCH(ctx, kKSdf, gq, 256, 0, sdf_quad_kernel, g, f, cv, qcnt, qoff, slot<int32_t>(ctx, kSlotSdfTris));
  ctx->sdf_nv = (int32_t)totals[0];
  ctx->sdf_nt = (int32_t)totals[1];
  *out_nv = ctx->sdf_nv;
  *out_nt = ctx->sdf_nt;
  return VISACD_OK;
}

extern "C" int visacd_sdf_fetch(visacd_ctx* ctx, double* verts, int32_t* tris) {
  VCHECK(ctx, VISACD_ERR_INVALID_ARG, "sdf_fetch: null context");
  VCUDA(cudaSetDevice(ctx->device));
  if (ctx->sdf_nv > 0) {
    VCHECK(verts, VISACD_ERR_INVALID_ARG, "sdf_fetch: null vertex buffer");
    VCUDA(cudaMemcpyAsync(verts, slot<double>(ctx, kSlotSdfOut), (size_t)ctx->sdf_nv * 24, cudaMemcpyDeviceToHost,
                          ctx->stream));
  }
  if (ctx->sdf_nt > 0) {
    VCHECK(tris, VISACD_ERR_INVALID_ARG, "sdf_fetch: null triangle buffer");
    VCUDA(cudaMemcpyAsync(tris, slot<int32_t>(ctx, kSlotSdfTris), (size_t)ctx->sdf_nt * 12, cudaMemcpyDeviceToHost,
                          ctx->stream));
  }
  VCUDA(stream_wait(ctx));
  return VISACD_OK;
}

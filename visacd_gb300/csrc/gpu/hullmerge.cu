// Hull merging on the GPU: exact minimum vertex-to-vertex distance between
// pairs of convex hulls, the mesh_dist gate of multimerge_ch
// (lib/src/postprocess.cpp:64-200 with lib/src/cost.cpp:125-159): a pair is a
// merge candidate only when its hulls come closer than the merge threshold.
//
// One block per requested pair (a, b): the vertices of b stream through shared
// memory in tiles, each thread keeps the smallest squared distance of its
// vertices of a, a block reduction takes the minimum and the square root is
// taken once. Squared distances use FP64 round-to-nearest intrinsics in the
// host's order ((dx^2 + dy^2) + dz^2), so the value equals the host's exact
// nearest-neighbour result bit for bit (the minimum of exact values, and the
// square root is monotone). A pair whose bounding boxes are farther apart than
// `cutoff` is not scanned and gets DBL_MAX, as does a pair with an empty hull
// (the host's kInf); the box gap is a lower bound of the distance, compared
// with a relative margin of 1e-12. Vertex pairs whose FP32 distance exceeds a
// thread's running minimum by more than the FP32 rounding bound skip the FP64
// evaluation (they cannot lower the minimum).
#include "common.cuh"
#include "geom64.cuh"

namespace vgpu {
namespace {

constexpr int kHdThreads = 256;
constexpr int kHdTile = 1024;

__device__ __forceinline__ double box_gap(const double* __restrict__ bb, int a, int b) {
  // bb: per hull lo xyz, hi xyz
  double g2 = 0.0;
  for (int k = 0; k < 3; ++k) {
    const double lo_a = bb[6 * a + k], hi_a = bb[6 * a + 3 + k];
    const double lo_b = bb[6 * b + k], hi_b = bb[6 * b + 3 + k];
    double d = 0.0;
    if (lo_b > hi_a) d = lo_b - hi_a;
    else if (lo_a > hi_b) d = lo_a - hi_b;
    g2 += d * d;
  }
  return sqrt(g2);
}

__global__ void __launch_bounds__(kHdThreads) hull_dist_kernel(const double* __restrict__ V,
                                                               const int64_t* __restrict__ off,
                                                               const double* __restrict__ bb,
                                                               const int32_t* __restrict__ pairs, int64_t P,
                                                               double cutoff, double* __restrict__ out) {
  __shared__ double tile[kHdTile * 3];
  __shared__ float tilef[kHdTile * 3];
  __shared__ double red[kHdThreads / 32];
  for (int64_t p = blockIdx.x; p < P; p += gridDim.x) {
    const int a = pairs[2 * p], b = pairs[2 * p + 1];
    const int64_t a0 = off[a], a1 = off[a + 1], b0 = off[b], b1 = off[b + 1];
    if (a1 == a0 || b1 == b0) {
      if (threadIdx.x == 0) out[p] = 1.7976931348623157e308;  // empty hull: the host's kInf
      continue;
    }
    if (cutoff < 1e300 && box_gap(bb, a, b) > cutoff * (1.0 + 1e-12)) {
      if (threadIdx.x == 0) out[p] = 1.7976931348623157e308;
      continue;
    }
    // FP32 pre-filter bound: coordinates rounded to float move by <= 2^-24 |x|;
    // with M the largest |coordinate| of the two hulls |d_f32 - d| <= M 2^-21.
    double M = 0;
    for (int k = 0; k < 6; ++k) M = fmax(M, fmax(fabs(bb[6 * a + k]), fabs(bb[6 * b + k])));
    const double eabs = M * 4.76837158203125e-7 + 1e-30;
    double best = 1.7976931348623157e308;
    float thr = 3.4e38f;  // FP32 squared distance above which a vertex pair cannot beat best
    for (int64_t t0 = b0; t0 < b1; t0 += kHdTile) {
      const int n = (int)min((int64_t)kHdTile, b1 - t0);
      __syncthreads();
      for (int i = threadIdx.x; i < 3 * n; i += blockDim.x) {
        tile[i] = V[3 * t0 + i];
        tilef[i] = (float)tile[i];
      }
      __syncthreads();
      for (int64_t i = a0 + threadIdx.x; i < a1; i += blockDim.x) {
        const double qx = V[3 * i], qy = V[3 * i + 1], qz = V[3 * i + 2];
        const float fx = (float)qx, fy = (float)qy, fz = (float)qz;
        for (int j = 0; j < n; ++j) {
          const float ex = tilef[3 * j] - fx, ey = tilef[3 * j + 1] - fy, ez = tilef[3 * j + 2] - fz;
          if (ex * ex + ey * ey + ez * ez > thr) continue;
          const double dx = ds(tile[3 * j], qx), dy = ds(tile[3 * j + 1], qy), dz = ds(tile[3 * j + 2], qz);
          const double d2 = da(da(dm(dx, dx), dm(dy, dy)), dm(dz, dz));
          if (d2 < best) {
            best = d2;
            const double r = __dsqrt_rn(best) + eabs;
            thr = __double2float_ru(r * r) * (1.0f + 1.0f / 65536.0f);
          }
        }
      }
    }
    for (int o = 16; o > 0; o >>= 1) best = fmin(best, __shfl_xor_sync(0xffffffffu, best, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = best;
    __syncthreads();
    if (threadIdx.x == 0) {
      double m = red[0];
      for (int w = 1; w < kHdThreads / 32; ++w) m = fmin(m, red[w]);
      out[p] = __dsqrt_rn(m);
    }
    __syncthreads();
  }
}

__global__ void hull_bbox_kernel(const double* __restrict__ V, const int64_t* __restrict__ off, int H,
                                 double* __restrict__ bb) {
  for (int h = blockIdx.x; h < H; h += gridDim.x) {
    double lo[3] = {1e308, 1e308, 1e308}, hi[3] = {-1e308, -1e308, -1e308};
    for (int64_t i = off[h] + threadIdx.x; i < off[h + 1]; i += blockDim.x)
      for (int k = 0; k < 3; ++k) {
        lo[k] = fmin(lo[k], V[3 * i + k]);
        hi[k] = fmax(hi[k], V[3 * i + k]);
      }
    for (int k = 0; k < 3; ++k)
      for (int o = 16; o > 0; o >>= 1) {
        lo[k] = fmin(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
        hi[k] = fmax(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
      }
    __shared__ double s[8][6];
    if ((threadIdx.x & 31) == 0)
      for (int k = 0; k < 3; ++k) {
        s[threadIdx.x >> 5][k] = lo[k];
        s[threadIdx.x >> 5][3 + k] = hi[k];
      }
    __syncthreads();
    if (threadIdx.x < 6) {
      double v = s[0][threadIdx.x];
      for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
        v = threadIdx.x < 3 ? fmin(v, s[w][threadIdx.x]) : fmax(v, s[w][threadIdx.x]);
      bb[6 * h + threadIdx.x] = v;
    }
    __syncthreads();
  }
}

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace
}  // namespace vgpu

using namespace vgpu;

extern "C" int visacd_hull_distances(visacd_ctx* ctx, const double* verts, const int64_t* offsets, int32_t H,
                                     const int32_t* pairs, int64_t P, double cutoff, double* out) {
  VCHECK(ctx && offsets && (P == 0 || (pairs && out)), VISACD_ERR_INVALID_ARG, "hull_distances: null argument");
  VCHECK(H >= 0 && P >= 0, VISACD_ERR_INVALID_ARG, "hull_distances: negative size");
  if (P == 0) return VISACD_OK;
  VCHECK(offsets[0] == 0, VISACD_ERR_INVALID_ARG, "hull_distances: offsets[0] must be 0");
  for (int32_t h = 0; h < H; ++h)
    VCHECK(offsets[h + 1] >= offsets[h], VISACD_ERR_INVALID_ARG, "hull_distances: offsets must not decrease");
  for (int64_t p = 0; p < 2 * P; ++p)
    VCHECK(pairs[p] >= 0 && pairs[p] < H, VISACD_ERR_INVALID_ARG, "hull_distances: hull index out of range");
  const int64_t nv = offsets[H];
  VCHECK(nv == 0 || verts, VISACD_ERR_INVALID_ARG, "hull_distances: null vertices");
  VCUDA(cudaSetDevice(ctx->device));
  const size_t oV = 0, oOff = align256((size_t)nv * 24), oBB = oOff + align256((size_t)(H + 1) * 8),
               oPairs = oBB + align256((size_t)H * 48), oOut = oPairs + align256((size_t)P * 8),
               total = oOut + align256((size_t)P * 8);
  VTRY(ensure_slot(ctx, kSlotHull, total));
  char* base = slot<char>(ctx, kSlotHull);
  cudaStream_t st = ctx->stream;
  if (nv) VCUDA(cudaMemcpyAsync(base + oV, verts, (size_t)nv * 24, cudaMemcpyHostToDevice, st));
  VCUDA(cudaMemcpyAsync(base + oOff, offsets, (size_t)(H + 1) * 8, cudaMemcpyHostToDevice, st));
  VCUDA(cudaMemcpyAsync(base + oPairs, pairs, (size_t)P * 8, cudaMemcpyHostToDevice, st));
  if (H > 0)
    VLAUNCH(ctx, kKHullDist, (unsigned)std::min<int64_t>(H, 4096), 256, 0, hull_bbox_kernel,
            (const double*)(base + oV), (const int64_t*)(base + oOff), H, (double*)(base + oBB));
  const unsigned grid = (unsigned)std::min<int64_t>(P, 64LL * ctx->sm_count);
  VLAUNCH(ctx, kKHullDist, grid, kHdThreads, 0, hull_dist_kernel, (const double*)(base + oV),
          (const int64_t*)(base + oOff), (const double*)(base + oBB), (const int32_t*)(base + oPairs), P,
          cutoff, (double*)(base + oOut));
  VCUDA(cudaMemcpyAsync(out, base + oOut, (size_t)P * 8, cudaMemcpyDeviceToHost, st));
  VCUDA(stream_wait(ctx));
  return VISACD_OK;
}

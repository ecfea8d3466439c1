// Free-space grid of a cage: for every cell of a uniform grid over the cage's
// bounding box, a lower bound B of the distance from the cell's centre to the
// cage's triangles. The visibility kernel walks a segment through it
// (traverse.cuh, trace_free): from a point x it may advance by
// B - |x - centre| - margin, because no cage triangle lies within
// B - |x - centre| of x; a segment whose whole length is covered this way
// cannot hit the cage, which is the answer the exact test gives for it.
// Segments it cannot cover (they cross the cage, or pass within a few cells
// of it) go through the BVH as before, so results do not change.
//
// The bound of a centre is the larger of two rigorous lower bounds:
//  * near: the smallest lower bound, over the triangles whose bounding box
//    lies within R of the centre, of the distance from the centre to the
//    triangle (plane distance and in-plane edge half-planes, minus a rounding
//    allowance; or the distance to the triangle's bounding box), capped at R
//    (triangles farther than R from the centre were not visited);
//  * far: h x the exact Euclidean distance, in cells, from the cell to the
//    nearest "surface" cell (one whose centre lies within a half diagonal of
//    a triangle: every cage point is in such a cell), minus a half diagonal.
// All roundings that matter are directed (down for bounds).
#include <atomic>
#include <cmath>

#include "bvh.cuh"

namespace vgpu {

namespace {

constexpr int kFgMaxDim = 256;          // cells per axis at most (EDT row buffers)
constexpr int kFgInf = 0x3fffffff;      // "no surface cell" squared distance
constexpr float kU32 = 5.9604645e-8f;   // 2^-24

__device__ __forceinline__ float fg_dot(float ax, float ay, float az, float bx, float by, float bz) {
  return ax * bx + ay * by + az * bz;
}

// A lower bound of the distance from x to triangle (A, B, C): the larger of
// the distance to the triangle's bounding box (directed roundings) and
// sqrt(plane distance^2 + in-plane distance to the nearest edge half-plane^2)
// less an allowance of 64 u k (|x - A| + longest edge), k = |e1| |e2| / |n|,
// far above the FP32 error of that expression. Nearly degenerate triangles
// (k > 1e4) use the box bound alone.
__device__ float fg_tri_lb(float x, float y, float z, float4 A, float4 B, float4 C) {
  // Box bound.
  const float bx0 = fminf(A.x, fminf(B.x, C.x)), bx1 = fmaxf(A.x, fmaxf(B.x, C.x));
  const float by0 = fminf(A.y, fminf(B.y, C.y)), by1 = fmaxf(A.y, fmaxf(B.y, C.y));
  const float bz0 = fminf(A.z, fminf(B.z, C.z)), bz1 = fmaxf(A.z, fmaxf(B.z, C.z));
  const float gx = fmaxf(0.f, fmaxf(__fsub_rd(bx0, x), __fsub_rd(x, bx1)));
  const float gy = fmaxf(0.f, fmaxf(__fsub_rd(by0, y), __fsub_rd(y, by1)));
  const float gz = fmaxf(0.f, fmaxf(__fsub_rd(bz0, z), __fsub_rd(z, bz1)));
  const float box = __fsqrt_rd(__fadd_rd(__fadd_rd(__fmul_rd(gx, gx), __fmul_rd(gy, gy)), __fmul_rd(gz, gz)));
  // Plane and edge half-planes.
  const float e1x = B.x - A.x, e1y = B.y - A.y, e1z = B.z - A.z;
  const float e2x = C.x - A.x, e2y = C.y - A.y, e2z = C.z - A.z;
  const float e3x = C.x - B.x, e3y = C.y - B.y, e3z = C.z - B.z;
  const float nx = e1y * e2z - e1z * e2y, ny = e1z * e2x - e1x * e2z, nz = e1x * e2y - e1y * e2x;
  const float nn = fg_dot(nx, ny, nz, nx, ny, nz);
  const float l1 = fg_dot(e1x, e1y, e1z, e1x, e1y, e1z), l2 = fg_dot(e2x, e2y, e2z, e2x, e2y, e2z);
  const float l3 = fg_dot(e3x, e3y, e3z, e3x, e3y, e3z);
  if (!(nn > 0.f) || !(l1 * l2 < 1e8f * nn)) return box;  // k > 1e4 (or degenerate)
  const float rn = rsqrtf(nn);
  const float k = sqrtf(l1 * l2) * rn * 1.0001f;
  const float rx = x - A.x, ry = y - A.y, rz = z - A.z;
  const float pd = fabsf(fg_dot(nx, ny, nz, rx, ry, rz)) * rn;
  // Outward in-plane edge normals m = e x n; |m| = |e| |n|.
  const float m1x = e1y * nz - e1z * ny, m1y = e1z * nx - e1x * nz, m1z = e1x * ny - e1y * nx;
  const float m3x = e3y * nz - e3z * ny, m3y = e3z * nx - e3x * nz, m3z = e3x * ny - e3y * nx;
  // Edge C -> A: e4 = A - C = -e2.
  const float m2x = -(e2y * nz - e2z * ny), m2y = -(e2z * nx - e2x * nz), m2z = -(e2x * ny - e2y * nx);
  const float o1 = fg_dot(m1x, m1y, m1z, rx, ry, rz) * rsqrtf(l1) * rn;
  const float o3 = fg_dot(m3x, m3y, m3z, x - B.x, y - B.y, z - B.z) * rsqrtf(l3 > 0.f ? l3 : 1.f) * rn;
  const float o2 = fg_dot(m2x, m2y, m2z, x - C.x, y - C.y, z - C.z) * rsqrtf(l2) * rn;
  const float out = fmaxf(0.f, fmaxf(o1, fmaxf(o2, o3)));
  const float d = sqrtf(pd * pd + out * out);
  const float r = fmaxf(fabsf(rx), fmaxf(fabsf(ry), fabsf(rz))) * 1.7321f;
  const float emax = sqrtf(fmaxf(l1, fmaxf(l2, l3)));
  const float slack = 64.f * kU32 * k * (r + emax) + 1e-30f;
  const float plane_lb = fmaxf(0.f, (d - slack) * (1.f - 64.f * kU32));
  return fmaxf(box, plane_lb);
}

struct FgParams {
  float ox, oy, oz;  // lower corner of cell (0, 0, 0)
  float h;           // cell size
  int nx, ny, nz;
  float R;           // near-band radius
};

// One warp per triangle: every cell whose centre lies within R of the
// triangle's bounding box (one extra cell of slack per side) takes the
// minimum of its near value and the triangle's bound at its centre.
__global__ void fg_near_kernel(const float4* __restrict__ tris, int32_t nt, FgParams g,
                               unsigned* __restrict__ near) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const float ih = 1.f / g.h;
  for (int64_t tri = warp; tri < nt; tri += nwarps) {
    const float4 A = tris[3 * tri], B = tris[3 * tri + 1], C = tris[3 * tri + 2];
    const float lo[3] = {fminf(A.x, fminf(B.x, C.x)) - g.R, fminf(A.y, fminf(B.y, C.y)) - g.R,
                         fminf(A.z, fminf(B.z, C.z)) - g.R};
    const float hi[3] = {fmaxf(A.x, fmaxf(B.x, C.x)) + g.R, fmaxf(A.y, fmaxf(B.y, C.y)) + g.R,
                         fmaxf(A.z, fmaxf(B.z, C.z)) + g.R};
    const float o[3] = {g.ox, g.oy, g.oz};
    const int dims[3] = {g.nx, g.ny, g.nz};
    int c0[3], c1[3];
    for (int a = 0; a < 3; ++a) {
      c0[a] = max(0, (int)floorf((lo[a] - o[a]) * ih - 0.5f) - 1);
      c1[a] = min(dims[a] - 1, (int)ceilf((hi[a] - o[a]) * ih - 0.5f) + 1);
    }
    const int sx = c1[0] - c0[0] + 1, sy = c1[1] - c0[1] + 1, sz = c1[2] - c0[2] + 1;
    if (sx <= 0 || sy <= 0 || sz <= 0) continue;
    const int total = sx * sy * sz;
    for (int k = lane; k < total; k += 32) {
      const int ix = c0[0] + k % sx, iy = c0[1] + (k / sx) % sy, iz = c0[2] + k / (sx * sy);
      // The centre exactly as the walk computes it.
      const float x = __fadd_rn(g.ox, __fmul_rn((float)ix + 0.5f, g.h));
      const float y = __fadd_rn(g.oy, __fmul_rn((float)iy + 0.5f, g.h));
      const float z = __fadd_rn(g.oz, __fmul_rn((float)iz + 0.5f, g.h));
      // Cells whose centre lies farther than R from the triangle's box keep
      // their value: the cap at R already bounds them.
      const float gx = fmaxf(0.f, fmaxf(lo[0] + g.R - x, x - (hi[0] - g.R)));
      const float gy = fmaxf(0.f, fmaxf(lo[1] + g.R - y, y - (hi[1] - g.R)));
      const float gz = fmaxf(0.f, fmaxf(lo[2] + g.R - z, z - (hi[2] - g.R)));
      if (gx * gx + gy * gy + gz * gz > 1.0001f * g.R * g.R) continue;
      const float lb = fg_tri_lb(x, y, z, A, B, C);
      atomicMin(&near[((int64_t)iz * g.ny + iy) * g.nx + ix], __float_as_uint(lb));
    }
  }
}

// EDT pass along x, one warp per row: squared distance (cells) to the nearest
// surface cell of the row (a surface cell: near value <= hd), kFgInf when
// the row has none. The nearest surface index at or before / at or after
// each cell comes from warp max / min scans, 32 cells at a time.
__global__ void fg_edt_x_kernel(const unsigned* __restrict__ near, FgParams g, float hd, int* __restrict__ d2) {
  constexpr unsigned full = 0xffffffffu;
  constexpr int kNone = 1 << 20;
  const int lane = threadIdx.x & 31;
  const int64_t rows = (int64_t)g.ny * g.nz;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int chunks = (g.nx + 31) >> 5;  // <= 8
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < rows; r += nwarps) {
    const int64_t base = r * g.nx;
    unsigned seeds[kFgMaxDim / 32];
    int last[kFgMaxDim / 32];
    int carry = -kNone;
#pragma unroll
    for (int m = 0; m < kFgMaxDim / 32; ++m) {
      if (m < chunks) {
        const int i = 32 * m + lane;
        const bool seed = i < g.nx && __uint_as_float(near[base + i]) <= hd;
        seeds[m] = __ballot_sync(full, seed);
        int x = seed ? i : -kNone;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_up_sync(full, x, o);
          if (lane >= o) x = max(x, y);
        }
        x = max(x, carry);
        last[m] = x;
        carry = __shfl_sync(full, x, 31);
      }
    }
    carry = 2 * kNone;
#pragma unroll
    for (int m = kFgMaxDim / 32 - 1; m >= 0; --m) {
      if (m < chunks) {
        const int i = 32 * m + lane;
        int x = ((seeds[m] >> lane) & 1u) ? i : 2 * kNone;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_down_sync(full, x, o);
          if (lane + o < 32) x = min(x, y);
        }
        x = min(x, carry);
        carry = __shfl_sync(full, x, 0);
        if (i < g.nx) {
          const int d = min(i - last[m], x - i);
          d2[base + i] = d >= kNone ? kFgInf : d * d;
        }
      }
    }
  }
}

// EDT pass along y (AXIS 1) or z (AXIS 2): lower envelope of the parabolas
// (q - p)^2 + f(p) over each line (Felzenszwalb and Huttenlocher, 2012), one
// line per thread. The envelope's parabolas live in shared memory, one column
// per thread, packed as (f << 8) | p (f < 2^24, p < 256); breakpoints are
// compared exactly by cross-multiplying their integer numerators and
// denominators. 32-bit arithmetic is exact here: finite values are squared
// cell distances of at most 3 x 255^2 < 2^18, so h = f + p^2 < 2^19 and every
// cross product stays below 2^27.
constexpr int kEdtThreads = 64;
template <int AXIS>
__global__ void __launch_bounds__(kEdtThreads) fg_edt_yz_kernel(FgParams g, int* __restrict__ d2) {
  extern __shared__ uint32_t env[];  // [line length][kEdtThreads]
  const int tid = threadIdx.x;
  const int n = AXIS == 1 ? g.ny : g.nz;
  const int64_t lines = AXIS == 1 ? (int64_t)g.nx * g.nz : (int64_t)g.nx * g.ny;
  const int64_t stride = AXIS == 1 ? g.nx : (int64_t)g.nx * g.ny;
  for (int64_t l = (int64_t)blockIdx.x * blockDim.x + tid; l < lines; l += (int64_t)gridDim.x * blockDim.x) {
    const int64_t base = AXIS == 1 ? (l / g.nx) * g.nx * g.ny + (l % g.nx) : l;
    int k = -1;
    // The line's values are read 8 at a time (independent loads in flight).
    int buf[8];
    for (int q = 0; q < n; ++q) {
      if ((q & 7) == 0) {
#pragma unroll
        for (int u = 0; u < 8; ++u) buf[u] = q + u < n ? d2[base + (int64_t)(q + u) * stride] : kFgInf;
      }
      int fq = buf[0];
#pragma unroll
      for (int u = 1; u < 8; ++u)
        if ((q & 7) == u) fq = buf[u];
      if (fq >= kFgInf) continue;
      const int hq = fq + q * q;
      while (k >= 1) {
        const uint32_t e0 = env[(k - 1) * kEdtThreads + tid], e1 = env[k * kEdtThreads + tid];
        const int v0 = (int)(e0 & 255u), v1 = (int)(e1 & 255u);
        const int h0 = (int)(e0 >> 8) + v0 * v0;
        const int h1 = (int)(e1 >> 8) + v1 * v1;
        // Drop v1 when the new parabola's breakpoint with it lies at or
        // before v1's own breakpoint with v0.
        if ((hq - h1) * (v1 - v0) <= (h1 - h0) * (q - v1)) --k;
        else break;
      }
      ++k;
      env[k * kEdtThreads + tid] = ((uint32_t)fq << 8) | (uint32_t)q;
    }
    if (k < 0) continue;  // no surface cell on this line: stays infinite
    int j = 0;
    for (int q = 0; q < n; ++q) {
      while (j < k) {
        const uint32_t e0 = env[j * kEdtThreads + tid], e1 = env[(j + 1) * kEdtThreads + tid];
        const int v0 = (int)(e0 & 255u), v1 = (int)(e1 & 255u);
        const int h0 = (int)(e0 >> 8) + v0 * v0;
        const int h1 = (int)(e1 >> 8) + v1 * v1;
        if (h1 - h0 < 2 * q * (v1 - v0)) ++j;
        else break;
      }
      const uint32_t e = env[j * kEdtThreads + tid];
      const int dq = q - (int)(e & 255u);
      const int val = dq * dq + (int)(e >> 8);
      d2[base + q * stride] = val >= kFgInf ? kFgInf : val;
    }
  }
}

// The bound of a cell's centre: B = max(min(near, R), h sqrt(d2) - hd),
// rounded down (hd: the half diagonal of a cell grown by delta, rounded up).
// A walk at point x in the cell takes B - |x - centre| (traverse.cuh).
__global__ void fg_final_kernel(const unsigned* __restrict__ near, const int* __restrict__ d2, int64_t cells,
                                float R, float h, float hd, float* __restrict__ lb) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < cells;
       c += (int64_t)gridDim.x * blockDim.x) {
    const float a = fminf(__uint_as_float(near[c]), R);
    const int e = d2[c];
    const float b = e >= kFgInf ? 3.0e38f : __fsub_rd(__fmul_rd(__fsqrt_rd((float)e), h), hd);
    lb[c] = fmaxf(a, b);
  }
}

}  // namespace

int free_grid_build(visacd_ctx* ctx, visacd_bvh* b, int64_t pairs) {
  if (b->free_built) return VISACD_OK;
  b->free_built = true;  // also when the grid is not usable: then it is not retried
  if (b->nt <= 0) return VISACD_OK;
  // Bounding box of the triangles, read back with the BVH build's counters
  // (order-preserving unsigned values).
  const unsigned* h = b->tri_bounds;
  float lo[3], hi[3];
  for (int a = 0; a < 3; ++a) {
    const unsigned ol = h[a], oh = h[3 + a];
    const unsigned bl = (ol & 0x80000000u) ? (ol & 0x7fffffffu) : ~ol;
    const unsigned bh = (oh & 0x80000000u) ? (oh & 0x7fffffffu) : ~oh;
    lo[a] = __uint_as_float_host(bl);
    hi[a] = __uint_as_float_host(bh);
    if (!std::isfinite(lo[a]) || !std::isfinite(hi[a]) || !(hi[a] >= lo[a])) return VISACD_OK;
  }
  const float ext = std::max(hi[0] - lo[0], std::max(hi[1] - lo[1], hi[2] - lo[2]));
  const float amax = std::max(std::max(std::fabs(lo[0]), std::fabs(hi[0])),
                              std::max(std::max(std::fabs(lo[1]), std::fabs(hi[1])),
                                       std::max(std::fabs(lo[2]), std::fabs(hi[2]))));
  if (!(ext > 0.f)) return VISACD_OK;
  // 192 cells along the longest side: fine enough that a cell's half
  // diagonal stays well below the usual part-to-cage gap. The grid's cost
  // follows its cells, so only calls with many pairs build one.
  (void)pairs;
  const float hcell = ext / 192.f;
  const float delta = hcell / 64.f;
  // The growth delta must cover the FP32 rounding of the walk's points and
  // cell indices (a few units in the last place of the coordinates).
  if (!(delta > 256.f * 5.9604645e-8f * (amax + ext))) return VISACD_OK;
  FgParams g;
  g.h = hcell;
  g.ox = lo[0] - 2.f * hcell;
  g.oy = lo[1] - 2.f * hcell;
  g.oz = lo[2] - 2.f * hcell;
  g.nx = (int)std::ceil((hi[0] - lo[0]) / hcell) + 4;
  g.ny = (int)std::ceil((hi[1] - lo[1]) / hcell) + 4;
  g.nz = (int)std::ceil((hi[2] - lo[2]) / hcell) + 4;
  if (g.nx > kFgMaxDim || g.ny > kFgMaxDim || g.nz > kFgMaxDim) return VISACD_OK;
  g.R = 2.f * hcell;
  const float hd = (0.8660254f * hcell + 1.7320508f * delta) * 1.0001f;
  const int64_t cells = (int64_t)g.nx * g.ny * g.nz;
  // Scratch: near values and squared distances (the context's SDF slot), the
  // grid itself on the BVH (it lives as long as the BVH).
  VTRY(ensure_slot(ctx, kSlotFreeGrid, (size_t)cells * 8));
  unsigned* near = slot<unsigned>(ctx, kSlotFreeGrid);
  int* d2 = reinterpret_cast<int*>(near + cells);
  float* lb = nullptr;
  VCUDA(cudaMallocAsync((void**)&lb, (size_t)cells * 4, b->stream));
  // The grid is attached to the BVH only once every launch went in.
  struct Guard {
    float*& p;
    cudaStream_t st;
    ~Guard() {
      if (p) cudaFreeAsync(p, st);
    }
  } guard{lb, b->stream};
  // near = 0x7f7f7f7f, a float far above any distance here (non-negative
  // floats order as unsigned integers, which the atomic minimum relies on).
  VCUDA(cudaMemsetAsync(near, 0x7f, (size_t)cells * 4, ctx->stream));
  VLAUNCH(ctx, kKGridNear, grid_for((int64_t)b->nt * 32, 256, 16LL * ctx->sm_count), 256, 0, fg_near_kernel,
          b->tris, b->nt, g, near);
  VLAUNCH(ctx, kKGridEdt, grid_for((int64_t)g.ny * g.nz * 32, 256, 16LL * ctx->sm_count), 256, 0,
          fg_edt_x_kernel, near, g, hd, d2);
  const int edt_smem = kFgMaxDim * kEdtThreads * 4;
  // The shared-memory opt-in is per device.
  static std::atomic<bool> edt_configured[64];
  const bool known = ctx->device >= 0 && ctx->device < 64;
  if (!known || !edt_configured[ctx->device].load()) {
    VCUDA(cudaFuncSetAttribute(fg_edt_yz_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, edt_smem));
    VCUDA(cudaFuncSetAttribute(fg_edt_yz_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, edt_smem));
    if (known) edt_configured[ctx->device].store(true);
  }
  // Each pass takes the shared memory its line length needs (an envelope
  // holds at most one parabola per cell of the line), so more blocks fit on
  // an SM than with the 256-cell maximum.
  VLAUNCH(ctx, kKGridEdt, grid_for((int64_t)g.nx * g.nz, kEdtThreads, 8LL * ctx->sm_count), kEdtThreads,
          g.ny * kEdtThreads * 4, fg_edt_yz_kernel<1>, g, d2);
  VLAUNCH(ctx, kKGridEdt, grid_for((int64_t)g.nx * g.ny, kEdtThreads, 8LL * ctx->sm_count), kEdtThreads,
          g.nz * kEdtThreads * 4, fg_edt_yz_kernel<2>, g, d2);
  VLAUNCH(ctx, kKGridFinal, grid_for(cells, 256, 8LL * ctx->sm_count), 256, 0, fg_final_kernel, near, d2, cells,
          g.R, g.h, hd, lb);
  // The bounds as a 3D texture: point sampling at cell coordinate u reads
  // cell floor(u), and the texture's block-linear layout keeps nearby cells
  // (in 3D) in the same cache lines; reads outside the grid return 0 (the
  // border), which stops a walk.
  {
    // The context's kept array and texture when the size matches; a kept one
    // of another size goes (after the work that may still read it).
    cudaArray_t arr = nullptr;
    cudaTextureObject_t tex = 0;
    if (ctx->grid_arr && ctx->grid_dims[0] == g.nx && ctx->grid_dims[1] == g.ny && ctx->grid_dims[2] == g.nz) {
      arr = ctx->grid_arr;
      tex = ctx->grid_tex;
    } else if (ctx->grid_arr) {
      cudaDestroyTextureObject(ctx->grid_tex);
      VCUDA(stream_wait(ctx));
      cudaFreeArray(ctx->grid_arr);
    }
    ctx->grid_arr = nullptr;
    ctx->grid_tex = 0;
    if (!arr) {
      cudaChannelFormatDesc fd = cudaCreateChannelDesc<float>();
      VCUDA(cudaMalloc3DArray(&arr, &fd, make_cudaExtent(g.nx, g.ny, g.nz)));
    }
    cudaMemcpy3DParms cp = {};
    cp.srcPtr = make_cudaPitchedPtr(lb, (size_t)g.nx * sizeof(float), g.nx, g.ny);
    cp.dstArray = arr;
    cp.extent = make_cudaExtent(g.nx, g.ny, g.nz);
    cp.kind = cudaMemcpyDeviceToDevice;
    cudaError_t e = cudaMemcpy3DAsync(&cp, ctx->stream);
    if (e == cudaSuccess && !tex) {
      cudaResourceDesc rd = {};
      rd.resType = cudaResourceTypeArray;
      rd.res.array.array = arr;
      cudaTextureDesc td = {};
      td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeBorder;
      td.borderColor[0] = td.borderColor[1] = td.borderColor[2] = td.borderColor[3] = 0.f;
      td.filterMode = cudaFilterModePoint;
      td.readMode = cudaReadModeElementType;
      td.normalizedCoords = 0;
      e = cudaCreateTextureObject(&tex, &rd, &td, nullptr);
    }
    if (e != cudaSuccess) {
      if (tex) cudaDestroyTextureObject(tex);
      cudaStreamSynchronize(ctx->stream);
      cudaFreeArray(arr);
      set_error("free_grid_build: %s", cudaGetErrorString(e));
      return VISACD_ERR_CUDA;
    }
    b->free_arr = arr;
    b->free_tex = tex;
  }
  b->free_lb = lb;
  lb = nullptr;  // owned by the BVH now
  b->fg_ox = g.ox;
  b->fg_oy = g.oy;
  b->fg_oz = g.oz;
  b->fg_h = g.h;
  b->fg_inv_h = 1.f / g.h;
  b->fg_margin = delta;
  b->fg_nx = g.nx;
  b->fg_ny = g.ny;
  b->fg_nz = g.nz;
  return VISACD_OK;
}

}  // namespace vgpu

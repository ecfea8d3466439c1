// Throughput probes for the rooflines of kernels that neither HBM nor the
// tensor cores bind:
//  * FP32 FMA: plane scoring and the traversal arithmetic. Independent FFMA
//    chains per thread so issue, not latency, limits it; packed f32x2 FMAs
//    (two FLOP pairs per instruction lane) as the scoring kernel uses them.
//  * Texture fetches: the free-space walk, one point-sampled tex3D<float> read
//    of its bound grid a step. Four independent fetch chains per thread from a
//    small 3D texture (cache-resident, like the walk's grid), two patterns:
//    coherent (a warp reads an 8 x 4 block of neighbouring texels, the best
//    case) and divergent (every lane walks its own line through the texture,
//    as the walk's lanes do).
#include "common.cuh"

namespace vgpu {

__global__ void fma_peak_kernel(float* __restrict__ out, int iters, float a, float b) {
  unsigned long long x[8];
  const unsigned long long A = ((unsigned long long)__float_as_uint(a) << 32) | __float_as_uint(a);
  const unsigned long long Bv = ((unsigned long long)__float_as_uint(b) << 32) | __float_as_uint(b);
#pragma unroll
  for (int k = 0; k < 8; ++k)
    x[k] = ((unsigned long long)__float_as_uint((float)(threadIdx.x + k)) << 32) |
           __float_as_uint((float)k);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) asm volatile("fma.rn.f32x2 %0, %0, %1, %2;" : "+l"(x[k]) : "l"(A), "l"(Bv));
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += __uint_as_float((unsigned)x[k]) + __uint_as_float((unsigned)(x[k] >> 32));
  if (s == 12345.678f) out[0] = s;  // keeps the chains live
}

constexpr int kTexDim = 32;

__global__ void tex_coherent_kernel(cudaTextureObject_t t, int iters, float* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const float x = (float)(lane & 7) + 0.5f, y = (float)(lane >> 3) + 0.5f;
  float z[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) z[k] = (float)((blockIdx.x * 7 + (threadIdx.x >> 5) * 3 + k * 5) % kTexDim) + 0.5f;
  float s = 0.f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      s += tex3D<float>(t, x, y, z[k]);
      z[k] += 1.f;
      if (z[k] > (float)kTexDim) z[k] -= (float)kTexDim;
    }
  }
  if (s == 12345.678f) out[0] = s;  // keeps the fetches live
}

__global__ void tex_divergent_kernel(cudaTextureObject_t t, int iters, float* __restrict__ out) {
  const unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
  const float dx = 0.37f + 0.01f * (id & 31), dy = 0.61f - 0.013f * (id & 15), dz = 0.29f + 0.007f * (id & 7);
  const float D = (float)kTexDim;
  float px[4], py[4], pz[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    px[k] = (float)((id * 13 + k * 7) % kTexDim);
    py[k] = (float)((id * 7 + k * 3) % kTexDim);
    pz[k] = (float)((id * 5 + k) % kTexDim);
  }
  float s = 0.f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      s += tex3D<float>(t, px[k], py[k], pz[k]);
      px[k] += dx;
      py[k] += dy;
      pz[k] += dz;
      if (px[k] >= D) px[k] -= D;
      if (py[k] >= D) py[k] -= D;
      if (pz[k] >= D) pz[k] -= D;
    }
  }
  if (s == 12345.678f) out[0] = s;
}

}  // namespace vgpu

using namespace vgpu;

extern "C" int visacd_measure_tex_peak(visacd_ctx* ctx, double* coherent_gfetch, double* divergent_gfetch) {
  VCHECK(ctx && coherent_gfetch && divergent_gfetch, VISACD_ERR_INVALID_ARG, "measure_tex_peak: null argument");
  VCUDA(cudaSetDevice(ctx->device));
  VTRY(ensure_slot(ctx, kSlotCounters, 256));
  float* out = slot<float>(ctx, kSlotCounters);
  cudaChannelFormatDesc fd = cudaCreateChannelDesc<float>();
  cudaArray_t arr = nullptr;
  VCUDA(cudaMalloc3DArray(&arr, &fd, make_cudaExtent(kTexDim, kTexDim, kTexDim)));
  cudaResourceDesc rd = {};
  rd.resType = cudaResourceTypeArray;
  rd.res.array.array = arr;
  cudaTextureDesc td = {};
  td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeBorder;
  td.filterMode = cudaFilterModePoint;
  td.readMode = cudaReadModeElementType;
  td.normalizedCoords = 0;
  cudaTextureObject_t tex = 0;
  cudaError_t e = cudaCreateTextureObject(&tex, &rd, &td, nullptr);
  if (e != cudaSuccess) {
    cudaFreeArray(arr);
    set_error("measure_tex_peak: %s", cudaGetErrorString(e));
    return VISACD_ERR_CUDA;
  }
  const int blocks = ctx->sm_count * 16, threads = 256, iters = 2048;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  double best[2] = {0, 0};
  e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  for (int mode = 0; mode < 2 && e == cudaSuccess; ++mode)
    for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {
      cudaEventRecord(e0, ctx->stream);
      if (mode == 0)
        tex_coherent_kernel<<<blocks, threads, 0, ctx->stream>>>(tex, iters, out);
      else
        tex_divergent_kernel<<<blocks, threads, 0, ctx->stream>>>(tex, iters, out);
      e = cudaGetLastError();
      if (e == cudaSuccess) e = cudaEventRecord(e1, ctx->stream);
      if (e == cudaSuccess) e = cudaEventSynchronize(e1);
      float ms = 0;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
      const double fetches = (double)blocks * threads * iters * 4;
      if (e == cudaSuccess && rep > 0) best[mode] = std::max(best[mode], fetches / (ms * 1e-3) / 1e9);
    }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaDestroyTextureObject(tex);
  cudaFreeArray(arr);
  VCUDA(e);
  ctx->launches += 8;
  *coherent_gfetch = best[0];
  *divergent_gfetch = best[1];
  return VISACD_OK;
}

extern "C" int visacd_measure_fp32_peak(visacd_ctx* ctx, double* tflops) {
  VCHECK(ctx && tflops, VISACD_ERR_INVALID_ARG, "measure_fp32_peak: null argument");
  VCUDA(cudaSetDevice(ctx->device));
  VTRY(ensure_slot(ctx, kSlotCounters, 256));
  float* out = slot<float>(ctx, kSlotCounters);
  const int blocks = ctx->sm_count * 8, threads = 256, iters = 4096;
  cudaEvent_t e0, e1;
  VCUDA(cudaEventCreate(&e0));
  VCUDA(cudaEventCreate(&e1));
  double best = 0;
  for (int rep = 0; rep < 4; ++rep) {
    VCUDA(cudaEventRecord(e0, ctx->stream));
    fma_peak_kernel<<<blocks, threads, 0, ctx->stream>>>(out, iters, 0.999f, 1e-3f);
    VCUDA(cudaGetLastError());
    VCUDA(cudaEventRecord(e1, ctx->stream));
    VCUDA(cudaEventSynchronize(e1));
    float ms = 0;
    VCUDA(cudaEventElapsedTime(&ms, e0, e1));
    // 8 chains x 2 lanes x 2 FLOP per FMA.
    double flop = (double)blocks * threads * iters * 8 * 2 * 2;
    if (rep > 0) best = std::max(best, flop / (ms * 1e-3) / 1e12);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  ctx->launches += 4;
  *tflops = best;
  return VISACD_OK;
}

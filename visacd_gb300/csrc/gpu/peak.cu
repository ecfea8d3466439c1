// FP32 FMA throughput probe: the denominator of the FP32-bound rooflines
// (plane scoring, traversal arithmetic). Independent FFMA chains per thread so
// issue, not latency, limits it; packed f32x2 FMAs (two FLOP pairs per
// instruction lane) as the scoring kernel uses them.
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

}  // namespace vgpu

using namespace vgpu;

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

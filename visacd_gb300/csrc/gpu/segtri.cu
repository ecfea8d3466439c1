// Independent segment-triangle tests: the visibility kernel's decision
// (FP32 filter with a rigorous rounding bound, FP64 re-decision of the
// undecided tests) applied to S given (segment, triangle) pairs. This is the
// precision form's measurement and test surface: the decisions equal the FP64
// oracle's on every input, grazing ones included, and the FP64 share is
// reported. Segment p -> q over t in [0.001 / |q - p|, 1] (the reference's
// tmin, lib/ptx/ray_segments.cu:99-100).
#include "common.cuh"
#include "traverse.cuh"

namespace vgpu {
namespace {

__global__ void seg_tri_kernel(const float* __restrict__ seg, const float* __restrict__ tri, int64_t S,
                               uint8_t* __restrict__ out, unsigned long long* __restrict__ n64) {
  unsigned rechecks = 0;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < S; k += (int64_t)gridDim.x * blockDim.x) {
    const float* sp = seg + 6 * k;
    const float* t = tri + 9 * k;
    Seg s;
    make_seg(s, make_float3(sp[0], sp[1], sp[2]), make_float3(sp[3], sp[4], sp[5]), -1, -1);
    s.exclude = false;
    const float4 a = make_float4(t[0], t[1], t[2], 0.f), b = make_float4(t[3], t[4], t[5], 0.f),
                 c = make_float4(t[6], t[7], t[8], 0.f);
    int r = tri_test32(s, a, b, c);
    if (r == 2) {
      ++rechecks;
      r = tri_test64(sp[0], sp[1], sp[2], sp[3], sp[4], sp[5], a, b, c) ? 1 : 0;
    }
    out[k] = (uint8_t)r;
  }
  for (int o = 16; o; o >>= 1) rechecks += __shfl_xor_sync(0xffffffffu, rechecks, o);
  if ((threadIdx.x & 31) == 0 && rechecks) atomicAdd(n64, (unsigned long long)rechecks);
}

}  // namespace
}  // namespace vgpu

using namespace vgpu;

extern "C" int visacd_segment_triangle_tests(visacd_ctx* ctx, const float* seg, const float* tri, int64_t S,
                                             uint8_t* hit_out, int64_t* n_fp64) {
  VCHECK(ctx && (S == 0 || (seg && tri && hit_out)), VISACD_ERR_INVALID_ARG, "segment_triangle_tests: null argument");
  VCHECK(S >= 0, VISACD_ERR_INVALID_ARG, "segment_triangle_tests: negative size");
  if (n_fp64) *n_fp64 = 0;
  if (S == 0) return VISACD_OK;
  VCUDA(cudaSetDevice(ctx->device));
  const size_t o_seg = 0, o_tri = ((size_t)S * 24 + 255) & ~size_t(255),
               o_out = o_tri + (((size_t)S * 36 + 255) & ~size_t(255)),
               o_cnt = o_out + (((size_t)S + 255) & ~size_t(255)), total = o_cnt + 256;
  VTRY(ensure_slot(ctx, kSlotSegTri, total));
  char* B = slot<char>(ctx, kSlotSegTri);
  cudaStream_t st = ctx->stream;
  VCUDA(cudaMemcpyAsync(B + o_seg, seg, (size_t)S * 24, cudaMemcpyHostToDevice, st));
  VCUDA(cudaMemcpyAsync(B + o_tri, tri, (size_t)S * 36, cudaMemcpyHostToDevice, st));
  VCUDA(cudaMemsetAsync(B + o_cnt, 0, 8, st));
  VLAUNCH(ctx, kKSegTri, grid_for(S, 256, 32LL * ctx->sm_count), 256, 0, seg_tri_kernel, (const float*)(B + o_seg),
          (const float*)(B + o_tri), S, (uint8_t*)(B + o_out), (unsigned long long*)(B + o_cnt));
  unsigned long long cnt = 0;
  VCUDA(cudaMemcpyAsync(hit_out, B + o_out, (size_t)S, cudaMemcpyDeviceToHost, st));
  VCUDA(cudaMemcpyAsync(&cnt, B + o_cnt, 8, cudaMemcpyDeviceToHost, st));
  VCUDA(stream_wait(ctx));
  if (n_fp64) *n_fp64 = (int64_t)cnt;
  return VISACD_OK;
}

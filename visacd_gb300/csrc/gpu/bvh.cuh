// Device-resident linear BVH shared by the builder and the visibility kernel.
#pragma once

#include <string.h>

#include "common.cuh"

// Node record (64 bytes, 4 x float4), each axis a (lo, hi) pair:
//   [0] L.lo.x L.hi.x L.lo.y L.hi.y
//   [1] L.lo.z L.hi.z R.lo.x R.hi.x
//   [2] R.lo.y R.hi.y R.lo.z R.hi.z
//   [3] left  right  (int bits; >= 0 internal node, < 0 leaf ~sorted_triangle)
// Leaf triangle record (48 bytes, 3 x float4): vertex xyz + vertex index bits.
struct visacd_bvh {
  int device = 0;
  int32_t nt = 0;
  int32_t nv = 0;
  int32_t depth = 0;
  float amax = 0.f;  // largest |vertex coordinate|
  // Bounds of the triangles' vertices as order-preserving unsigned values
  // (min xyz, max xyz), read back with the build's counters.
  unsigned tri_bounds[6] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u};
  float4* nodes = nullptr;
  float4* tris = nullptr;
  visacd_ctx* ctx = nullptr;       // owning context (null once it is destroyed)
  cudaStream_t stream = nullptr;   // the owner's stream (stream-ordered allocations)
  // Free-space grid (freegrid.cu), built on first use for a large visibility
  // call when this BVH is the cage: lb per cell, x fastest.
  bool free_built = false;
  float* free_lb = nullptr;
  cudaArray_t free_arr = nullptr;            // the same values as a 3D texture
  cudaTextureObject_t free_tex = 0;          // (point sampling, border 0)
  float fg_ox = 0.f, fg_oy = 0.f, fg_oz = 0.f, fg_h = 0.f, fg_inv_h = 0.f, fg_margin = 0.f;
  int32_t fg_nx = 0, fg_ny = 0, fg_nz = 0;
};

namespace vgpu {

inline float __uint_as_float_host(unsigned u) {
  float f;
  memcpy(&f, &u, 4);
  return f;
}

int bvh_build(visacd_ctx* ctx, const float* verts, int32_t nv, const uint32_t* tris, int32_t nt,
              int device_ptrs, visacd_bvh** out);
// Frees a BVH's device memory when its context goes away (the handle itself
// stays valid until visacd_bvh_destroy, and is rejected by queries).
void bvh_detach(visacd_bvh* b);
// Builds the BVH's free-space grid (once; a BVH whose grid would not be
// usable keeps none), its resolution sized for a call over `pairs` pairs. Uses the context's counter slot and pinned staging
// buffer (waits for the stream first), so it runs before a call takes them.
// Asynchronous after one small read-back.
int free_grid_build(visacd_ctx* ctx, visacd_bvh* b, int64_t pairs);

}  // namespace vgpu

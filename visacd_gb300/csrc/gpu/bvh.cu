// Linear BVH over a triangle mesh, built entirely on the device.
//
// Replaces the OptiX GAS build of the reference (lib/src/intersections.cpp:131-180).
//  1. tri_prep: per triangle centroid, conservatively widened AABB, index check.
//  2. morton: Morton code of the centroid, 10 to 21 bits per axis by triangle
//     count (morton_bits), sorted on exactly those bits.
//  3. stable LSD radix sort of (code, triangle) pairs (own kernels, ctx.cu).
//  4. karras_build: Karras (2012) "Maximizing parallelism in the construction of
//     BVHs, octrees and k-d trees" — each internal node finds its key range and
//     split from common-prefix lengths (ties broken by sorted position).
//  5. aabb_fit: bottom-up union with one atomic arrival counter per node.
//  6. node_layout: traversal records of 64 bytes (both child boxes with each
//     axis stored as a (lo, hi) pair for packed f32x2 slab tests, + child ids)
//     and leaf triangles of 48 bytes (3 vertices, vertex ids in .w).
#include <atomic>

#include "bvh.cuh"

namespace vgpu {

// Orderable uint encoding of a float (monotone for all non-NaN values).
__device__ __forceinline__ unsigned f2o(float f) {
  unsigned b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float o2f(unsigned o) {
  unsigned b = (o & 0x80000000u) ? (o & 0x7fffffffu) : ~o;
  return __uint_as_float(b);
}

struct BuildCounters {
  unsigned cmin[3];  // orderable centroid bounds
  unsigned cmax[3];
  unsigned amax;     // max |vertex coordinate| (float bits)
  unsigned bad_index;
  int depth;
  int pad;
  unsigned tb[6];    // orderable bounds of the triangles' vertices: min xyz, max xyz
};

// Order-preserving map of a float to unsigned (for atomic min / max).
__device__ __forceinline__ unsigned ord_f32(float f) {
  const unsigned b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

__global__ void vert_absmax_kernel(const float* __restrict__ v, int32_t nv,
                                   BuildCounters* __restrict__ c) {
  float m = 0.f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < 3LL * nv;
       i += (int64_t)gridDim.x * blockDim.x) {
    float x = fabsf(v[i]);
    if (x < INFINITY) m = fmaxf(m, x);
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(&c->amax, __float_as_uint(m));
}

__global__ void tri_prep_kernel(const float* __restrict__ v, int32_t nv,
                                const uint32_t* __restrict__ t, int32_t nt,
                                float* __restrict__ cent, BuildCounters* __restrict__ c) {
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  unsigned bad = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nt;
       i += (int64_t)gridDim.x * blockDim.x) {
    uint32_t i0 = t[3 * i], i1 = t[3 * i + 1], i2 = t[3 * i + 2];
    if (i0 >= (uint32_t)nv || i1 >= (uint32_t)nv || i2 >= (uint32_t)nv) {
      bad = 1;
      cent[3 * i] = cent[3 * i + 1] = cent[3 * i + 2] = 0.f;
      continue;
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      float x = (v[3 * (int64_t)i0 + a] + v[3 * (int64_t)i1 + a] + v[3 * (int64_t)i2 + a]) *
                (1.0f / 3.0f);
      cent[3 * i + a] = x;
      if (x == x && fabsf(x) < INFINITY) {
        lo[a] = fminf(lo[a], x);
        hi[a] = fmaxf(hi[a], x);
      }
    }
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) {
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
      hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
    }
  }
  bad = __reduce_or_sync(0xffffffffu, bad);
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      if (lo[a] <= hi[a]) {
        atomicMin(&c->cmin[a], f2o(lo[a]));
        atomicMax(&c->cmax[a], f2o(hi[a]));
      }
    }
    if (bad) atomicOr(&c->bad_index, 1u);
  }
}

__device__ __forceinline__ uint64_t spread21(uint64_t x) {
  x &= 0x1fffffull;
  x = (x | (x << 32)) & 0x1f00000000ffffull;
  x = (x | (x << 16)) & 0x1f0000ff0000ffull;
  x = (x | (x << 8)) & 0x100f00f00f00f00full;
  x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
  x = (x | (x << 2)) & 0x1249249249249249ull;
  return x;
}

__global__ void morton_kernel(const float* __restrict__ cent, int32_t n,
                              const BuildCounters* __restrict__ c, int bits, uint64_t* __restrict__ keys,
                              uint32_t* __restrict__ vals) {
  float lo[3], sc[3];
  const float top = (float)((1u << bits) - 1u);
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    lo[a] = o2f(c->cmin[a]);
    float ext = o2f(c->cmax[a]) - lo[a];
    sc[a] = ext > 0.f ? top / ext : 0.f;
  }
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    uint64_t q[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      float x = (cent[3 * i + a] - lo[a]) * sc[a];
      x = fminf(fmaxf(x, 0.f), top);  // NaN -> 0
      q[a] = (uint64_t)x;
    }
    keys[i] = (spread21(q[0]) << 2) | (spread21(q[1]) << 1) | spread21(q[2]);
    vals[i] = (uint32_t)i;
  }
}

// Common-prefix length of sorted keys i and j (ties broken by position).
__device__ __forceinline__ int delta(const uint64_t* __restrict__ k, int n, int i, int j) {
  if (j < 0 || j >= n) return -1;
  uint64_t a = k[i], b = k[j];
  if (a == b) return 64 + __clz((unsigned)(i ^ j));
  return __clzll(a ^ b);
}

// Children: >= 0 internal node, < 0 leaf ~sorted_position.
__global__ void karras_kernel(const uint64_t* __restrict__ keys, int32_t n,
                              int2* __restrict__ child, int* __restrict__ parent_int,
                              int* __restrict__ parent_leaf) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n - 1; i += gridDim.x * blockDim.x) {
    int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
    int dmin = delta(keys, n, i, i - d);
    int lmax = 2;
    while (delta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
      if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
    int j = i + l * d;
    int dnode = delta(keys, n, i, j);
    int s = 0;
    int t = l;
    do {
      t = (t + 1) >> 1;
      if (delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    int gamma = i + s * d + min(d, 0);
    int lo = min(i, j), hi = max(i, j);
    int left = (lo == gamma) ? ~gamma : gamma;
    int right = (hi == gamma + 1) ? ~(gamma + 1) : gamma + 1;
    child[i] = make_int2(left, right);
    if (left < 0) parent_leaf[~left] = i; else parent_int[left] = i;
    if (right < 0) parent_leaf[~right] = i; else parent_int[right] = i;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) parent_int[0] = -1;
}

// Leaf triangles in sorted order + their widened boxes.
__global__ void leaf_kernel(const float* __restrict__ v, int32_t nv,
                            const uint32_t* __restrict__ t,
                            const uint32_t* __restrict__ order, int32_t n,
                            BuildCounters* __restrict__ c, float4* __restrict__ tris,
                            float* __restrict__ leafbox) {
  float pad = __uint_as_float(c->amax) * 1.9073486e-6f + 1e-30f;  // 2^-19 * max|coord|
  // Bounds of all triangles' vertices (exact min / max; the free-space grid
  // of a cage is laid over them).
  float blo[3] = {INFINITY, INFINITY, INFINITY}, bhi[3] = {-INFINITY, -INFINITY, -INFINITY};
  bool any = false;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
    any = true;
    uint32_t tri = order[s];
    uint32_t id[3] = {t[3 * (int64_t)tri], t[3 * (int64_t)tri + 1], t[3 * (int64_t)tri + 2]};
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      // Out-of-range indices were flagged by tri_prep (the build then fails);
      // clamp here so this kernel never reads outside the vertex array.
      uint32_t vi = id[k] < (uint32_t)nv ? id[k] : 0u;
      float x = v[3 * (int64_t)vi], y = v[3 * (int64_t)vi + 1], z = v[3 * (int64_t)vi + 2];
      tris[3 * (int64_t)s + k] = make_float4(x, y, z, __int_as_float((int)id[k]));
      lo[0] = fminf(lo[0], x); hi[0] = fmaxf(hi[0], x);
      lo[1] = fminf(lo[1], y); hi[1] = fmaxf(hi[1], y);
      lo[2] = fminf(lo[2], z); hi[2] = fmaxf(hi[2], z);
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      leafbox[6 * (int64_t)s + a] = lo[a] - pad;
      leafbox[6 * (int64_t)s + 3 + a] = hi[a] + pad;
      blo[a] = fminf(blo[a], lo[a]);
      bhi[a] = fmaxf(bhi[a], hi[a]);
    }
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) {
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      blo[a] = fminf(blo[a], __shfl_xor_sync(0xffffffffu, blo[a], o));
      bhi[a] = fmaxf(bhi[a], __shfl_xor_sync(0xffffffffu, bhi[a], o));
    }
  }
  if (__any_sync(0xffffffffu, any) && (threadIdx.x & 31) == 0) {
    for (int a = 0; a < 3; ++a) {
      atomicMin(&c->tb[a], ord_f32(blo[a]));
      atomicMax(&c->tb[3 + a], ord_f32(bhi[a]));
    }
  }
}

__global__ void fit_kernel(const int2* __restrict__ child, const int* __restrict__ parent_int,
                           const int* __restrict__ parent_leaf, const float* __restrict__ leafbox,
                           float* __restrict__ nodebox, unsigned* __restrict__ visits, int* __restrict__ height,
                           int32_t n, BuildCounters* __restrict__ c) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
    int node = parent_leaf[s];
    for (int guard = 0; node >= 0 && guard < n + 1; ++guard) {
      __threadfence();
      if (atomicAdd(&visits[node], 1u) == 0u) break;
      int2 ch = child[node];
      // Height in edges (leaves 0); the root's is the tree depth.
      const int h = 1 + max(ch.x < 0 ? 0 : __ldcg(&height[ch.x]), ch.y < 0 ? 0 : __ldcg(&height[ch.y]));
      __stcg(&height[node], h);
      if (node == 0) atomicMax(&c->depth, h);
      float b[6];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        float l0 = ch.x < 0 ? __ldcg(&leafbox[6 * (int64_t)(~ch.x) + a]) : __ldcg(&nodebox[6 * (int64_t)ch.x + a]);
        float l1 = ch.y < 0 ? __ldcg(&leafbox[6 * (int64_t)(~ch.y) + a]) : __ldcg(&nodebox[6 * (int64_t)ch.y + a]);
        float h0 = ch.x < 0 ? __ldcg(&leafbox[6 * (int64_t)(~ch.x) + 3 + a]) : __ldcg(&nodebox[6 * (int64_t)ch.x + 3 + a]);
        float h1 = ch.y < 0 ? __ldcg(&leafbox[6 * (int64_t)(~ch.y) + 3 + a]) : __ldcg(&nodebox[6 * (int64_t)ch.y + 3 + a]);
        b[a] = fminf(l0, l1);
        b[3 + a] = fmaxf(h0, h1);
      }
#pragma unroll
      for (int a = 0; a < 6; ++a) __stcg(&nodebox[6 * (int64_t)node + a], b[a]);
      node = parent_int[node];
    }
  }
}

// The same fit for trees of up to kFitSmallMax leaves in one CTA: the
// topology (children, parents), the internal boxes, heights and arrival
// counters live in shared memory, so a level costs shared-memory latency
// instead of L2 round trips; the boxes go to global memory at the end. Boxes
// are minima and maxima of the children's, so they equal fit_kernel's.
constexpr int kFitSmallMax = 4096;
constexpr size_t kFitSmallBytesPerNode = 6 * 4 + 4 + 4 + 8 + 4;

__global__ void __launch_bounds__(1024) fit_small_kernel(const int2* __restrict__ child,
                                                         const int* __restrict__ parent_int,
                                                         const int* __restrict__ parent_leaf,
                                                         const float* __restrict__ leafbox,
                                                         float* __restrict__ nodebox, int32_t n,
                                                         BuildCounters* __restrict__ c) {
  extern __shared__ __align__(16) unsigned char fit_smem[];
  const int ni = n - 1;
  int2* ch_s = reinterpret_cast<int2*>(fit_smem);
  float* nb = reinterpret_cast<float*>(ch_s + ni);
  unsigned* vis = reinterpret_cast<unsigned*>(nb + 6 * ni);
  int* hgt = reinterpret_cast<int*>(vis + ni);
  int* par = hgt + ni;
  for (int i = threadIdx.x; i < ni; i += blockDim.x) {
    ch_s[i] = child[i];
    par[i] = parent_int[i];
    vis[i] = 0u;
  }
  __syncthreads();
  for (int s = threadIdx.x; s < n; s += blockDim.x) {
    int node = parent_leaf[s];
    for (int guard = 0; node >= 0 && guard < n + 1; ++guard) {
      __threadfence_block();
      if (atomicAdd(&vis[node], 1u) == 0u) break;
      __threadfence_block();
      const int2 ch = ch_s[node];
      const int h = 1 + max(ch.x < 0 ? 0 : hgt[ch.x], ch.y < 0 ? 0 : hgt[ch.y]);
      hgt[node] = h;
      if (node == 0) atomicMax(&c->depth, h);
      const float* lb = ch.x < 0 ? &leafbox[6 * (int64_t)(~ch.x)] : &nb[6 * ch.x];
      const float* rb = ch.y < 0 ? &leafbox[6 * (int64_t)(~ch.y)] : &nb[6 * ch.y];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        nb[6 * node + a] = fminf(lb[a], rb[a]);
        nb[6 * node + 3 + a] = fmaxf(lb[3 + a], rb[3 + a]);
      }
      node = par[node];
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 6 * ni; i += blockDim.x) nodebox[i] = nb[i];
}

__global__ void node_layout_kernel(const int2* __restrict__ child,
                                   const float* __restrict__ leafbox,
                                   const float* __restrict__ nodebox, int32_t n_internal,
                                   float4* __restrict__ nodes) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_internal;
       i += gridDim.x * blockDim.x) {
    int2 ch = child[i];
    const float* lb = ch.x < 0 ? &leafbox[6 * (int64_t)(~ch.x)] : &nodebox[6 * (int64_t)ch.x];
    const float* rb = ch.y < 0 ? &leafbox[6 * (int64_t)(~ch.y)] : &nodebox[6 * (int64_t)ch.y];
    // (lo, hi) per axis side by side: the traversal reads them as f32x2 pairs.
    nodes[4 * (int64_t)i + 0] = make_float4(lb[0], lb[3], lb[1], lb[4]);
    nodes[4 * (int64_t)i + 1] = make_float4(lb[2], lb[5], rb[0], rb[3]);
    nodes[4 * (int64_t)i + 2] = make_float4(rb[1], rb[4], rb[2], rb[5]);
    nodes[4 * (int64_t)i + 3] = make_float4(__int_as_float(ch.x), __int_as_float(ch.y), 0.f, 0.f);
  }
}

// Single-triangle mesh: one internal node whose two children are that leaf
// (the duplicate test is harmless and keeps the traversal branch-free).
__global__ void single_node_kernel(const float* __restrict__ leafbox, float4* __restrict__ nodes) {
  const float* lb = leafbox;
  nodes[0] = make_float4(lb[0], lb[3], lb[1], lb[4]);
  nodes[1] = make_float4(lb[2], lb[5], lb[0], lb[3]);
  nodes[2] = make_float4(lb[1], lb[4], lb[2], lb[5]);
  nodes[3] = make_float4(__int_as_float(~0), __int_as_float(~0), 0.f, 0.f);
}

int bvh_build(visacd_ctx* ctx, const float* verts, int32_t nv, const uint32_t* tris, int32_t nt,
              int device_ptrs, visacd_bvh** out) {
  VCHECK(ctx && out, VISACD_ERR_INVALID_ARG, "bvh_build: null argument");
  VCHECK(nv >= 0 && nt >= 0, VISACD_ERR_INVALID_ARG, "bvh_build: negative size");
  VCHECK(nt == 0 || (verts && tris && nv > 0), VISACD_ERR_INVALID_ARG,
         "bvh_build: missing vertices or triangles");
  VCHECK(nt < (1 << 30), VISACD_ERR_INVALID_ARG, "bvh_build: too many triangles");
  VCUDA(cudaSetDevice(ctx->device));
  *out = nullptr;
  visacd_bvh* b = new visacd_bvh();
  b->device = ctx->device;
  b->nt = nt;
  b->nv = nv;
  if (nt == 0) {
    b->ctx = ctx;
    b->stream = ctx->stream;
    ctx->bvhs.push_back(b);
    *out = b;
    return VISACD_OK;
  }
  const float* dv = verts;
  const uint32_t* dt = tris;
  if (!device_ptrs) {
    VTRY(ensure_slot(ctx, kSlotBuildVerts, (size_t)nv * 12));
    VTRY(ensure_slot(ctx, kSlotBuildTris, (size_t)nt * 12));
    Stager up(ctx);
    VTRY(up.reserve((size_t)nv * 12 + (size_t)nt * 12, 2));
    VTRY(up.put(ctx->buf[kSlotBuildVerts].p, verts, (size_t)nv * 12));
    VTRY(up.put(ctx->buf[kSlotBuildTris].p, tris, (size_t)nt * 12));
    dv = slot<float>(ctx, kSlotBuildVerts);
    dt = slot<uint32_t>(ctx, kSlotBuildTris);
  }
  const int n_int = nt > 1 ? nt - 1 : 1;
  // Scratch: centroids, keys x2, vals x2, child, parents, boxes, visits, counters.
  size_t off = 0;
  auto carve = [&](size_t bytes) {
    size_t o = off;
    off += (bytes + 255) & ~size_t(255);
    return o;
  };
  size_t o_cent = carve((size_t)nt * 12), o_k = carve((size_t)nt * 8), o_k2 = carve((size_t)nt * 8),
         o_v = carve((size_t)nt * 4), o_v2 = carve((size_t)nt * 4),
         o_child = carve((size_t)n_int * 8), o_pi = carve((size_t)n_int * 4),
         o_pl = carve((size_t)nt * 4), o_lb = carve((size_t)nt * 24),
         o_nb = carve((size_t)n_int * 24), o_vis = carve((size_t)n_int * 4), o_h = carve((size_t)n_int * 4),
         o_cnt = carve(sizeof(BuildCounters));
  VTRY(ensure_slot(ctx, kSlotTmpTris, off));
  char* base = slot<char>(ctx, kSlotTmpTris);
  float* cent = (float*)(base + o_cent);
  uint64_t *keys = (uint64_t*)(base + o_k), *keys2 = (uint64_t*)(base + o_k2);
  uint32_t *vals = (uint32_t*)(base + o_v), *vals2 = (uint32_t*)(base + o_v2);
  int2* child = (int2*)(base + o_child);
  int* pint = (int*)(base + o_pi);
  int* pleaf = (int*)(base + o_pl);
  float* leafbox = (float*)(base + o_lb);
  float* nodebox = (float*)(base + o_nb);
  unsigned* visits = (unsigned*)(base + o_vis);
  int* height = (int*)(base + o_h);
  BuildCounters* cnt = (BuildCounters*)(base + o_cnt);

  BuildCounters init;
  for (int a = 0; a < 3; ++a) {
    init.cmin[a] = 0xffffffffu;
    init.cmax[a] = 0u;
  }
  init.amax = 0;
  init.bad_index = 0;
  init.depth = 0;
  init.pad = 0;
  for (int a = 0; a < 3; ++a) {
    init.tb[a] = 0xffffffffu;
    init.tb[3 + a] = 0u;
  }
  BuildCounters* hcnt = nullptr;
  VTRY(pinned(ctx, sizeof(BuildCounters), (void**)&hcnt));
  *hcnt = init;
  VCUDA(cudaMemcpyAsync(cnt, hcnt, sizeof(BuildCounters), cudaMemcpyHostToDevice, ctx->stream));
  VCUDA(cudaMemsetAsync(visits, 0, (size_t)n_int * 4, ctx->stream));

  const unsigned g = grid_for(nt, 256, 8LL * ctx->sm_count);
  VLAUNCH(ctx, kKTriPrep, grid_for(3LL * nv, 256, 8LL * ctx->sm_count), 256, 0,
          vert_absmax_kernel, dv, nv, cnt);
  VLAUNCH(ctx, kKTriPrep, g, 256, 0, tri_prep_kernel, dv, nv, dt, nt, cent, cnt);
  const int mb = morton_bits(nt);
  VLAUNCH(ctx, kKMorton, g, 256, 0, morton_kernel, cent, nt, cnt, mb, keys, vals);
  VTRY(radix_sort_u64(ctx, keys, vals, keys2, vals2, nt, 3 * mb));

  size_t bytes_nodes = (size_t)n_int * 64, bytes_tris = (size_t)nt * 48;
  b->stream = ctx->stream;
  cudaError_t e1 = cudaMallocAsync((void**)&b->nodes, bytes_nodes, ctx->stream);
  cudaError_t e2 = e1 == cudaSuccess ? cudaMallocAsync((void**)&b->tris, bytes_tris, ctx->stream) : e1;
  if (e1 != cudaSuccess || e2 != cudaSuccess) {
    cudaGetLastError();
    if (b->nodes) cudaFreeAsync(b->nodes, ctx->stream);
    delete b;
    set_error("bvh_build: device allocation failed");
    return VISACD_ERR_NO_MEMORY;
  }
  VLAUNCH(ctx, kKNodeLayout, g, 256, 0, leaf_kernel, dv, nv, dt, vals, nt, cnt, b->tris, leafbox);
  if (nt == 1) {
    VLAUNCH(ctx, kKNodeLayout, 1, 1, 0, single_node_kernel, leafbox, b->nodes);
  } else {
    const unsigned gi = grid_for(n_int, 256, 8LL * ctx->sm_count);
    VLAUNCH(ctx, kKKarras, gi, 256, 0, karras_kernel, keys, nt, child, pint, pleaf);
    if (nt <= kFitSmallMax) {
      const size_t fit_smem = (size_t)n_int * kFitSmallBytesPerNode;
      static std::atomic<bool> fit_attr_set[64];
      if (ctx->device < 0 || ctx->device >= 64 || !fit_attr_set[ctx->device].load()) {
        VCUDA(cudaFuncSetAttribute(fit_small_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)(kFitSmallMax * kFitSmallBytesPerNode)));
        if (ctx->device >= 0 && ctx->device < 64) fit_attr_set[ctx->device].store(true);
      }
      VLAUNCH(ctx, kKFit, 1, 1024, fit_smem, fit_small_kernel, child, pint, pleaf, leafbox, nodebox, nt, cnt);
    } else {
      VLAUNCH(ctx, kKFit, g, 256, 0, fit_kernel, child, pint, pleaf, leafbox, nodebox, visits, height, nt,
            cnt);
    }
    VLAUNCH(ctx, kKNodeLayout, gi, 256, 0, node_layout_kernel, child, leafbox, nodebox, n_int,
            b->nodes);
  }
  VCUDA(cudaMemcpyAsync(hcnt, cnt, sizeof(BuildCounters), cudaMemcpyDeviceToHost, ctx->stream));
  VCUDA(stream_wait(ctx));
  if (hcnt->bad_index) {
    cudaFreeAsync(b->nodes, ctx->stream);
    cudaFreeAsync(b->tris, ctx->stream);
    delete b;
    set_error("bvh_build: a triangle references a vertex index >= %d", nv);
    return VISACD_ERR_INVALID_ARG;
  }
  b->depth = nt == 1 ? 1 : hcnt->depth;
  b->amax = __uint_as_float_host(hcnt->amax);
  for (int a = 0; a < 6; ++a) b->tri_bounds[a] = hcnt->tb[a];
  b->ctx = ctx;
  ctx->bvhs.push_back(b);
  *out = b;
  return VISACD_OK;
}

void bvh_detach(visacd_bvh* b) {
  if (b->nodes) cudaFreeAsync(b->nodes, b->stream);
  if (b->tris) cudaFreeAsync(b->tris, b->stream);
  if (b->free_lb) cudaFreeAsync(b->free_lb, b->stream);
  if (b->free_arr && b->ctx && !b->ctx->grid_arr) {
    // Kept on the context for the next grid of this size: work queued on the
    // context's stream reads it before any later copy into it.
    b->ctx->grid_arr = b->free_arr;
    b->ctx->grid_tex = b->free_tex;
    b->ctx->grid_dims[0] = b->fg_nx;
    b->ctx->grid_dims[1] = b->fg_ny;
    b->ctx->grid_dims[2] = b->fg_nz;
  } else {
    if (b->free_tex) cudaDestroyTextureObject(b->free_tex);
    if (b->free_arr) {
      cudaStreamSynchronize(b->stream);  // a queued walk may still read it
      cudaFreeArray(b->free_arr);
    }
  }
  b->free_tex = 0;
  b->free_arr = nullptr;
  b->nodes = b->tris = nullptr;
  b->free_lb = nullptr;
  b->ctx = nullptr;
  b->stream = nullptr;
}

}  // namespace vgpu

using namespace vgpu;

extern "C" int visacd_bvh_build(visacd_ctx* ctx, const float* verts, int32_t nv,
                                const uint32_t* tris, int32_t nt, int device_ptrs,
                                visacd_bvh** out) {
  return bvh_build(ctx, verts, nv, tris, nt, device_ptrs, out);
}

extern "C" int visacd_bvh_destroy(visacd_bvh* b) {
  if (!b) return VISACD_OK;
  cudaSetDevice(b->device);
  if (b->ctx) {
    auto& v = b->ctx->bvhs;
    v.erase(std::remove(v.begin(), v.end(), b), v.end());
    bvh_detach(b);
  }
  delete b;
  return VISACD_OK;
}

extern "C" int visacd_bvh_info(const visacd_bvh* b, int32_t* n_tris, int32_t* depth) {
  VCHECK(b, VISACD_ERR_INVALID_ARG, "bvh_info: null bvh");
  if (n_tris) *n_tris = b->nt;
  if (depth) *depth = b->depth;
  return VISACD_OK;
}

// Device side of plane scoring shared by the single-call and batched scoring
// kernels: the packed edge record, f32x2 helpers, the point-statistics and
// edge-packing kernels, the FP32 rounding band of a plane, the bulk-copy /
// mbarrier helpers and the FP64 side value (see score.cu for the design).
#pragma once

#include "common.cuh"

namespace vgpu {

constexpr int kScoreThreads = 256;
constexpr int kEdgeBlock = 256;  // edges per shared-memory block; 256 * (2^24 - 1) < 2^32
constexpr float kSideEps = 1e-6f;
// 3.0001u would do for the FMA chain; the extra covers the FP32 evaluation of
// S itself and the FP64 re-decision's own rounding.
constexpr float kBandFactor = 3.0e-7f;

struct __align__(16) EdgeRec {
  float x1, x2, y1, y2;
  float z1, z2;
  uint32_t q;
  uint32_t pad;
};
static_assert(sizeof(EdgeRec) == 32, "edge record must be 32 bytes");

__device__ __forceinline__ unsigned long long pack2(float a, float b) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ void unpack2(unsigned long long v, float& a, float& b) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ unsigned long long ffma2(unsigned long long a, unsigned long long b,
                                                    unsigned long long c) {
  unsigned long long d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}

// Largest |coordinate| over finite points, as float bits (non-negative floats
// order like unsigned ints).
static __global__ void point_stats_kernel(const float* __restrict__ pts, int32_t n,
                                   unsigned* __restrict__ stats) {
  float mx = 0.f, my = 0.f, mz = 0.f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float x = pts[3 * i], y = pts[3 * i + 1], z = pts[3 * i + 2];
    if (isfinite(x) && isfinite(y) && isfinite(z)) {
      mx = fmaxf(mx, fabsf(x));
      my = fmaxf(my, fabsf(y));
      mz = fmaxf(mz, fabsf(z));
    }
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    my = fmaxf(my, __shfl_xor_sync(0xffffffffu, my, o));
    mz = fmaxf(mz, __shfl_xor_sync(0xffffffffu, mz, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(&stats[0], __float_as_uint(mx));
    atomicMax(&stats[1], __float_as_uint(my));
    atomicMax(&stats[2], __float_as_uint(mz));
  }
}

// Exponent e with max|coord| < 2^e; edge lengths are below 2^(e+2), so with
// the quantum 2^(e - 22) every quantized length is below 2^24.
__device__ __host__ __forceinline__ int quantum_exp_from_cmax_bits(unsigned cbits) {
  int eb = (int)((cbits >> 23) & 0xffu);
  int e = eb >= 1 ? eb - 126 : -126;
  return e - 22;
}

__device__ __forceinline__ float edge_len32(float dx, float dy, float dz) {
  // IEEE single ops in a fixed order, no contraction: reproducible on the host.
  float s = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
  return __fsqrt_rn(s);
}

static __global__ void pack_edges_kernel(const float* __restrict__ pts, int32_t n,
                                  const uint32_t* __restrict__ edges, int64_t E,
                                  const unsigned* __restrict__ stats, EdgeRec* __restrict__ out,
                                  unsigned long long* __restrict__ skipped) {
  unsigned cmax = max(stats[0], max(stats[1], stats[2]));
  int qexp = quantum_exp_from_cmax_bits(cmax);
  unsigned long long nskip = 0;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E;
       e += (int64_t)gridDim.x * blockDim.x) {
    uint2 ij = reinterpret_cast<const uint2*>(edges)[e];
    EdgeRec r;
    r.pad = 0;
    bool ok = ij.x < (uint32_t)n && ij.y < (uint32_t)n;
    float x1 = 0, y1 = 0, z1 = 0, x2 = 0, y2 = 0, z2 = 0;
    if (ok) {
      x1 = pts[3 * (int64_t)ij.x];
      y1 = pts[3 * (int64_t)ij.x + 1];
      z1 = pts[3 * (int64_t)ij.x + 2];
      x2 = pts[3 * (int64_t)ij.y];
      y2 = pts[3 * (int64_t)ij.y + 1];
      z2 = pts[3 * (int64_t)ij.y + 2];
      ok = isfinite(x1) && isfinite(y1) && isfinite(z1) && isfinite(x2) && isfinite(y2) &&
           isfinite(z2);
    }
    if (ok) {
      float len = edge_len32(__fsub_rn(x2, x1), __fsub_rn(y2, y1), __fsub_rn(z2, z1));
      r.x1 = x1; r.x2 = x2; r.y1 = y1; r.y2 = y2; r.z1 = z1; r.z2 = z2;
      r.q = __float2uint_rn(ldexpf(len, -qexp));
    } else {
      r.x1 = r.x2 = r.y1 = r.y2 = r.z1 = r.z2 = 0.f;
      r.q = 0;
      ++nskip;
    }
    out[e] = r;
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) nskip += __shfl_xor_sync(0xffffffffu, nskip, o);
  if ((threadIdx.x & 31) == 0 && nskip) atomicAdd(skipped, nskip);
}

// Negated thresholds: crossing is certain when s < nhi, possible when s < nlo,
// with s = max(min(v1, v2), -max(v1, v2)) (negative iff signs differ; then
// -s = min(|v1|, |v2|)).
__device__ __forceinline__ void plane_thresholds(float4 pl, const unsigned* stats, float& nlo,
                                                 float& nhi) {
  float X = __uint_as_float(stats[0]), Y = __uint_as_float(stats[1]),
        Z = __uint_as_float(stats[2]);
  float S = fabsf(pl.x) * X + fabsf(pl.y) * Y + fabsf(pl.z) * Z + fabsf(pl.w);
  float B = S * kBandFactor;
  nhi = -(kSideEps + B);
  nlo = -(kSideEps - B);
}

// Per-plane state of the streaming scorer. A pair (v1, v2) of FP32 plane values
// is a certain crossing when the signs differ and m = min(|v1|, |v2|) > th
// (th = eps + B, the negated nhi above); it lies in the rounding band when
// m is in [eps - B, th]. With dh = th - m (FP32), "m > th" is the sign bit of
// dh, so the certain test is one logic op on sign bits: bit 31 of
// (v1 ^ v2) & dh. For m <= th,
// dh >= +0 and its bits order like the values, while dh < 0 has bit 31 set;
// so the smallest dh (as unsigned bits) over a block is at most the bits of
// th - (eps - B) exactly when some pair of the block may be in the band. Such
// blocks are re-decided in FP64; this flags every pair the sign-aware band
// test would (and pairs with equal signs too).
struct PlaneAcc {
  unsigned long long a2, b2, c2, d2;  // coefficients duplicated into f32x2 pairs
  float th;                           // eps + B
  uint32_t wbits;                     // bits of (eps + B) - (eps - B)
};

__device__ __forceinline__ PlaneAcc plane_acc(float4 pl, const unsigned* stats) {
  PlaneAcc a;
  a.a2 = pack2(pl.x, pl.x);
  a.b2 = pack2(pl.y, pl.y);
  a.c2 = pack2(pl.z, pl.z);
  a.d2 = pack2(pl.w, pl.w);
  float nlo, nhi;
  plane_thresholds(pl, stats, nlo, nhi);
  a.th = -nhi;
  a.wbits = __float_as_uint(__fsub_rn(-nhi, -nlo));
  return a;
}

// One shared-memory block of cnt edge records against K planes: acc[k] gets
// the quantised length of every certain crossing, dmin[k] the smallest dh
// bits (the band flag). Per (plane, edge): 3 packed FMAs, the FP32 add and
// the multiply-add of the masked length on the FMA pipe; min-abs, the sign
// logic, the shift and the unsigned min on the integer side. (Moving the
// shift to the FMA pipe as a high-word multiply measured slower: that pipe
// then limits.)
template <int K>
__device__ __forceinline__ void score_edge_block(const ulonglong2* __restrict__ s, int cnt,
                                                 const PlaneAcc (&pa)[K], uint32_t (&acc)[K],
                                                 uint32_t (&dmin)[K]) {
#pragma unroll 2
  for (int e = 0; e < cnt; ++e) {
    const ulonglong2 r0 = s[2 * e];      // (x1,x2), (y1,y2)
    const ulonglong2 r1 = s[2 * e + 1];  // (z1,z2), (q,pad)
    const uint32_t q = (uint32_t)(r1.y & 0xffffffffull);
#pragma unroll
    for (int k = 0; k < K; ++k) {
      unsigned long long v = ffma2(pa[k].c2, r1.x, pa[k].d2);
      v = ffma2(pa[k].b2, r0.y, v);
      v = ffma2(pa[k].a2, r0.x, v);
      float v1, v2;
      unpack2(v, v1, v2);
      const float m = fminf(fabsf(v1), fabsf(v2));
      const float dh = __fsub_rn(pa[k].th, m);
      const uint32_t c = (__float_as_uint(v1) ^ __float_as_uint(v2)) & __float_as_uint(dh);
      acc[k] += (c >> 31) * q;
      dmin[k] = min(dmin[k], __float_as_uint(dh));
    }
  }
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes,
                                          uint64_t* bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
  asm volatile(
      "cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// Bounded wait on an mbarrier phase; returns false if the phase never completed.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity) {
  for (int it = 0; it < (1 << 22); ++it) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 "
        "%0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

// FP64 side value of a point, in the fixed order the oracle uses. Products of
// two floats are exact in double, so contraction would not change them; the
// explicit intrinsics pin the order of the three additions.
__device__ __forceinline__ double side_value64(float4 pl, float x, float y, float z) {
  double ax = __dmul_rn((double)pl.x, (double)x);
  double by = __dmul_rn((double)pl.y, (double)y);
  double cz = __dmul_rn((double)pl.z, (double)z);
  return __dadd_rn(__dadd_rn(__dadd_rn(ax, by), cz), (double)pl.w);
}

}  // namespace vgpu

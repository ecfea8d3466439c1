// Device side of the segment visibility test, shared by the single-part and
// the batched visibility kernels: segment setup, conservative packed slab test,
// FP32 segment-triangle test with its rounding bound, FP64 re-decision, and the
// warp-packet any-hit traversal (see vis.cu for the design notes).
#pragma once

#include <math.h>

#include "bvh.cuh"

namespace vgpu {

constexpr int kVisThreads = 128;
constexpr int kStack = 64;
constexpr float kU = 5.9604645e-8f;  // 2^-24
constexpr float kTmin = 0.001f;      // reference tmin (ray_segments.cu:99)

struct VisCounters {
  unsigned long long work;
  unsigned long long pairs, edges, self_hits, cage_hits, rechecks, degenerate;
  unsigned long long node_visits, tri_tests;  // per-warp node fetches, per-lane triangle tests
  unsigned pmin[3], pmax[3];  // orderable point bounds
  unsigned long long n_rows;  // rows of the tile space (masked mode)
  unsigned long long certified, trace_steps;  // free-space walks: segments cleared, grid reads
  unsigned long long walk_work;               // tile counter of the walk kernel
  unsigned long long pending;                 // tiles the walk left to the traversal
};

// A cage's free-space grid as the visibility kernel reads it (freegrid.cu).
struct FreeGridView {
  const float* lb;          // null: no grid
  cudaTextureObject_t tex;  // the same bounds as a 3D texture (border 0)
  float ox, oy, oz, h_up, inv_h, margin;  // h_up: the cell size times (1 + 1e-6)
  int32_t nx, ny, nz;
};

// Lower bound of the distance to the cage from the point at cell coordinates
// (u, v, w) (x = o + u h): the bound B of the centre of the cell the point
// falls in, less h x the point's distance to that centre in cells. Outside
// the grid the texture's border gives B = 0, so the result is negative.
__device__ __forceinline__ float free_bound(const FreeGridView& g, float u, float v, float w) {
  const float B = tex3D<float>(g.tex, u, v, w);
  // u - floor(u) is exact; so is subtracting 0.5 from it.
  const float rx = (u - floorf(u)) - 0.5f, ry = (v - floorf(v)) - 0.5f, rz = (w - floorf(w)) - 0.5f;
  // |r| from the hardware reciprocal square root (2 ulp), rounded up through
  // the factor folded into h_up = h (1 + 1e-6).
  const float q = rx * rx + ry * ry + rz * rz;
  return B - q * rsqrtf(q + 1e-30f) * g.h_up;
}

constexpr int kTraceSteps = 32;  // rounds (two grid reads each) before a segment goes to the BVH

// Free-space walk of the segment p -> q (d = q - p rounded, len its FP32
// length) through a cage's grid, from both ends at once (two independent
// chains of dependent reads). The point at t has cell coordinates
// u0 + t du with u0 = (p - o) / h and du = d / h; from it the walk may
// advance by (lb - margin) / |q - p| in either direction, lb = free_bound:
// no cage triangle lies within lb of the point. The margin covers the FP32
// rounding of those coordinates against the true point of the segment (below
// 2e-4 cells for grids of at most 256 cells a side), of the cell centres, a
// cell read on either side of a face the point lies on, and leaves every
// covered point at least that far from the cage. True when the two covered
// parts [0, t] and [s, 1] meet: the segment cannot hit the cage. Roundings
// are directed so that the parts covered are never overstated. `steps`
// counts the grid reads.
__device__ __forceinline__ bool trace_free(const FreeGridView& g, float px, float py, float pz, float dx,
                                           float dy, float dz, float len, unsigned long long& steps) {
  // 1 / |q - p| rounded down; |q - p| <= len (1 + 17u).
  const float inv_len = __frcp_rd(__fmul_ru(len, 1.000001f));
  const float u0 = (px - g.ox) * g.inv_h, v0 = (py - g.oy) * g.inv_h, w0 = (pz - g.oz) * g.inv_h;
  const float du = dx * g.inv_h, dv = dy * g.inv_h, dw = dz * g.inv_h;
  float t = 0.f, s = 1.f;
  for (int k = 0; k < kTraceSteps; ++k) {
    const float lb0 = free_bound(g, fmaf(t, du, u0), fmaf(t, dv, v0), fmaf(t, dw, w0));
    const float lb1 = free_bound(g, fmaf(s, du, u0), fmaf(s, dv, v0), fmaf(s, dw, w0));
    steps += 2;
    if (!(lb0 > g.margin) || !(lb1 > g.margin)) return false;
    t = __fadd_rd(t, __fmul_rd(__fsub_rd(lb0, g.margin), inv_len));
    s = __fsub_ru(s, __fmul_rd(__fsub_rd(lb1, g.margin), inv_len));
    if (t >= s) return true;
  }
  return false;
}

struct Seg {
  unsigned long long ox2, oy2, oz2;  // (o, o) pairs for packed slab tests
  unsigned long long ix2, iy2, iz2;  // (1/d, 1/d) pairs
  float dx, dy, dz;
  float kw;      // Ew = kw * L^2
  int vi, vj;    // endpoint vertex ids (q = pts[vj])
  bool exclude;  // skip triangles incident to vi or vj (self test)
};

__device__ __forceinline__ unsigned f2o_v(float f) {
  unsigned b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float o2f_v(unsigned o) {
  unsigned b = (o & 0x80000000u) ? (o & 0x7fffffffu) : ~o;
  return __uint_as_float(b);
}

__device__ __forceinline__ float max3f(float a, float b, float c) {
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
__device__ __forceinline__ float min3f(float a, float b, float c) {
  float r;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}

__device__ __forceinline__ unsigned long long pk2(float a, float b) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ float lo2(unsigned long long v) {
  float a, b;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
  return a;
}
__device__ __forceinline__ void up2(unsigned long long v, float& a, float& b) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ unsigned long long sub2(unsigned long long a, unsigned long long b) {
  unsigned long long r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ unsigned long long mul2(unsigned long long a, unsigned long long b) {
  unsigned long long r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}

__device__ __forceinline__ float inv_guard(float d) {
  float ad = fabsf(d);
  float g = ad < 1e-30f ? copysignf(1e-30f, d) : d;
  return __frcp_rn(g);
}

__device__ __forceinline__ void make_seg(Seg& s, float3 p, float3 q, int vi, int vj) {
  s.ox2 = pk2(p.x, p.x);
  s.oy2 = pk2(p.y, p.y);
  s.oz2 = pk2(p.z, p.z);
  s.dx = __fsub_rn(q.x, p.x);
  s.dy = __fsub_rn(q.y, p.y);
  s.dz = __fsub_rn(q.z, p.z);
  float ix = inv_guard(s.dx), iy = inv_guard(s.dy), iz = inv_guard(s.dz);
  s.ix2 = pk2(ix, ix);
  s.iy2 = pk2(iy, iy);
  s.iz2 = pk2(iz, iz);
  float d1 = fabsf(s.dx) + fabsf(s.dy) + fabsf(s.dz);
  s.kw = 17.0f * kU * d1 * (1.0f + 4.0f * kU);
  s.vi = vi;
  s.vj = vj;
  s.exclude = true;
}

__device__ __forceinline__ float seg_len(const Seg& s) {
  return __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(s.dx, s.dx), __fmul_rn(s.dy, s.dy)),
                              __fmul_rn(s.dz, s.dz)));
}

// Conservative slab test of the segment (t in [0, 1]) against a box given as
// (lo, hi) pairs per axis; one packed sub + mul per axis.
__device__ __forceinline__ bool box_hit(const Seg& s, unsigned long long bx, unsigned long long by,
                                        unsigned long long bz) {
  float t0x, t1x, t0y, t1y, t0z, t1z;
  up2(mul2(sub2(bx, s.ox2), s.ix2), t0x, t1x);
  up2(mul2(sub2(by, s.oy2), s.iy2), t0y, t1y);
  up2(mul2(sub2(bz, s.oz2), s.iz2), t0z, t1z);
  float tn = max3f(fminf(t0x, t1x), fminf(t0y, t1y), fmaxf(fminf(t0z, t1z), 0.f));
  float tf = min3f(fmaxf(t0x, t1x), fmaxf(t0y, t1y), fminf(fmaxf(t0z, t1z), 1.f));
  tf = fmaf(fabsf(tf), 4e-6f, tf);
  return tn <= tf;
}

// FP64 segment-triangle decision from the FP32 inputs; identical formula to the
// oracle. Explicit round-to-nearest intrinsics keep contraction out.
static __device__ __noinline__ bool tri_test64(float ox, float oy, float oz, float qx, float qy, float qz,
                                        float4 a, float4 b, float4 c) {
  double Ax = __dsub_rn(a.x, ox), Ay = __dsub_rn(a.y, oy), Az = __dsub_rn(a.z, oz);
  double Bx = __dsub_rn(b.x, ox), By = __dsub_rn(b.y, oy), Bz = __dsub_rn(b.z, oz);
  double Cx = __dsub_rn(c.x, ox), Cy = __dsub_rn(c.y, oy), Cz = __dsub_rn(c.z, oz);
  double Dx = __dsub_rn(qx, ox), Dy = __dsub_rn(qy, oy), Dz = __dsub_rn(qz, oz);
  double BCx = __dsub_rn(__dmul_rn(By, Cz), __dmul_rn(Bz, Cy));
  double BCy = __dsub_rn(__dmul_rn(Bz, Cx), __dmul_rn(Bx, Cz));
  double BCz = __dsub_rn(__dmul_rn(Bx, Cy), __dmul_rn(By, Cx));
  double CAx = __dsub_rn(__dmul_rn(Cy, Az), __dmul_rn(Cz, Ay));
  double CAy = __dsub_rn(__dmul_rn(Cz, Ax), __dmul_rn(Cx, Az));
  double CAz = __dsub_rn(__dmul_rn(Cx, Ay), __dmul_rn(Cy, Ax));
  double ABx = __dsub_rn(__dmul_rn(Ay, Bz), __dmul_rn(Az, By));
  double ABy = __dsub_rn(__dmul_rn(Az, Bx), __dmul_rn(Ax, Bz));
  double ABz = __dsub_rn(__dmul_rn(Ax, By), __dmul_rn(Ay, Bx));
  double Wa = __dadd_rn(__dadd_rn(__dmul_rn(Dx, BCx), __dmul_rn(Dy, BCy)), __dmul_rn(Dz, BCz));
  double Wb = __dadd_rn(__dadd_rn(__dmul_rn(Dx, CAx), __dmul_rn(Dy, CAy)), __dmul_rn(Dz, CAz));
  double Wc = __dadd_rn(__dadd_rn(__dmul_rn(Dx, ABx), __dmul_rn(Dy, ABy)), __dmul_rn(Dz, ABz));
  double det = __dadd_rn(__dadd_rn(Wa, Wb), Wc);
  if (!(det != 0.0)) return false;
  bool inside = (Wa >= 0.0 && Wb >= 0.0 && Wc >= 0.0) || (Wa <= 0.0 && Wb <= 0.0 && Wc <= 0.0);
  if (!inside) return false;
  double vol = __dadd_rn(__dadd_rn(__dmul_rn(Ax, BCx), __dmul_rn(Ay, BCy)), __dmul_rn(Az, BCz));
  double len = __dsqrt_rn(
      __dadd_rn(__dadd_rn(__dmul_rn(Dx, Dx), __dmul_rn(Dy, Dy)), __dmul_rn(Dz, Dz)));
  double tmin = (double)kTmin;
  double lhs = __dmul_rn(vol, len), rhs = __dmul_rn(tmin, det);
  if (det > 0.0) return lhs >= rhs && vol <= det;
  return lhs <= rhs && vol >= det;
}

// FP32 filter: 1 certain hit, 0 certain miss, 2 undecided (needs FP64).
__device__ __forceinline__ int tri_test32(const Seg& s, float4 a, float4 b, float4 c) {
  const float ox = lo2(s.ox2), oy = lo2(s.oy2), oz = lo2(s.oz2);
  float Ax = __fsub_rn(a.x, ox), Ay = __fsub_rn(a.y, oy), Az = __fsub_rn(a.z, oz);
  float Bx = __fsub_rn(b.x, ox), By = __fsub_rn(b.y, oy), Bz = __fsub_rn(b.z, oz);
  float Cx = __fsub_rn(c.x, ox), Cy = __fsub_rn(c.y, oy), Cz = __fsub_rn(c.z, oz);
  float L = max3f(max3f(fabsf(Ax), fabsf(Ay), fabsf(Az)), max3f(fabsf(Bx), fabsf(By), fabsf(Bz)),
                  max3f(fabsf(Cx), fabsf(Cy), fabsf(Cz)));
  float BCx = By * Cz - Bz * Cy, BCy = Bz * Cx - Bx * Cz, BCz = Bx * Cy - By * Cx;
  float CAx = Cy * Az - Cz * Ay, CAy = Cz * Ax - Cx * Az, CAz = Cx * Ay - Cy * Ax;
  float ABx = Ay * Bz - Az * By, ABy = Az * Bx - Ax * Bz, ABz = Ax * By - Ay * Bx;
  float Wa = s.dx * BCx + s.dy * BCy + s.dz * BCz;
  float Wb = s.dx * CAx + s.dy * CAy + s.dz * CAz;
  float Wc = s.dx * ABx + s.dy * ABy + s.dz * ABz;
  float L2 = L * L;
  float Ew = s.kw * L2;
  float mx = max3f(Wa, Wb, Wc), mn = min3f(Wa, Wb, Wc);
  if (mx > Ew && mn < -Ew) return 0;  // edge functions of strictly opposite sign
  bool allpos = mn > Ew, allneg = mx < -Ew;
  if (!(allpos || allneg)) return 2;
  float sg = allpos ? 1.f : -1.f;
  float det_s = sg * ((Wa + Wb) + Wc);
  float vol_s = sg * (Ax * BCx + Ay * BCy + Az * BCz);
  float Ev = 49.0f * kU * L2 * L;
  float Edet = 3.0f * Ew + 2.02f * kU * det_s;
  float g1 = det_s - vol_s;
  float e1 = Edet + Ev + 2.0f * kU * fabsf(g1);
  const float len = seg_len(s);
  float g2 = vol_s * len - kTmin * det_s;
  float e2 = (Ev + 6.0f * kU * fabsf(vol_s)) * len + kTmin * (Edet + 2.0f * kU * det_s) +
             2.0f * kU * fabsf(g2);
  if (g1 < -e1 || g2 < -e2) return 0;
  if (g1 > e1 && g2 > e2) return 1;
  return 2;
}

__device__ __forceinline__ bool leaf_hit(const float4* __restrict__ tris, int leaf, const Seg& s,
                                         const float* __restrict__ pts, unsigned& rechecks) {
  float4 a = __ldg(&tris[3 * leaf]), b = __ldg(&tris[3 * leaf + 1]), c = __ldg(&tris[3 * leaf + 2]);
  if (s.exclude) {
    int ia = __float_as_int(a.w), ib = __float_as_int(b.w), ic = __float_as_int(c.w);
    if (ia == s.vi || ia == s.vj || ib == s.vi || ib == s.vj || ic == s.vi || ic == s.vj)
      return false;
  }
  int r = tri_test32(s, a, b, c);
  if (r == 2) {
    ++rechecks;
    const float* q = pts + 3 * (int64_t)s.vj;
    return tri_test64(lo2(s.ox2), lo2(s.oy2), lo2(s.oz2), q[0], q[1], q[2], a, b, c);
  }
  return r == 1;
}

// Warp-packet any-hit traversal. Every lane carries its own segment; the warp
// walks one path through the BVH: a child is visited when any still-active
// lane's segment overlaps its box (ballot), node records are fetched at a
// warp-uniform address (one broadcast transaction), and a lane retires at its
// first hit. The stack is per warp and lives in registers: entry k is held by
// lane k mod 32, in the first register for k < 32 and the second above, so a
// push is a select and a pop one shuffle (no shared memory, no warp barrier).
// Lanes retire only at leaf tests, so the warp checks for an early exit only
// after those. Returns this lane's hit flag; `visits` grows by the node
// records fetched. `status_bits` collects stack-overflow / iteration-overrun
// conditions (the lane is then reported as hit and the call fails on the
// host).
static __device__ bool packet_any_hit(const float4* __restrict__ nodes, const float4* __restrict__ tris,
                                      int nt, const Seg& s, const float* __restrict__ pts, bool active,
                                      unsigned& rechecks, unsigned& status_bits, unsigned& visits,
                                      unsigned& tri_tests) {
  static_assert(kStack == 64, "two stack registers per lane");
  const unsigned full = 0xffffffffu;
  bool hit = false;
  if (nt <= 0) return false;
  if (!__ballot_sync(full, active)) return false;
  const int lane = threadIdx.x & 31;
  int stk0 = 0, stk1 = 0;
  int node = 0, sp = 0;
  const int max_iter = 4 * nt + 64;
  for (int it = 0; it < max_iter; ++it) {
    const ulonglong2* nd = reinterpret_cast<const ulonglong2*>(nodes) + 4 * node;
    const ulonglong2 n0 = __ldg(nd), n1 = __ldg(nd + 1), n2 = __ldg(nd + 2);
    const int2 lr = __ldg(reinterpret_cast<const int2*>(nd + 3));
    const int l = lr.x, r = lr.y;
    const bool hl = active && box_hit(s, n0.x, n0.y, n1.x);
    const bool hr = active && box_hit(s, n1.y, n2.x, n2.y);
    const unsigned bl = __ballot_sync(full, hl);
    const unsigned br = __ballot_sync(full, hr);
    int next = -1;
    bool leaf = false;
    if (bl) {
      if (l < 0) {
        leaf = true;
        if (hl) {
          ++tri_tests;
          if (leaf_hit(tris, ~l, s, pts, rechecks)) {
            hit = true;
            active = false;
          }
        }
      } else {
        next = l;
      }
    }
    if (br) {
      if (r < 0) {
        leaf = true;
        if (hr && active) {
          ++tri_tests;
          if (leaf_hit(tris, ~r, s, pts, rechecks)) {
            hit = true;
            active = false;
          }
        }
      } else if (next < 0) {
        next = r;
      } else {
        if (sp >= kStack) {
          visits += it + 1;
          status_bits |= kStatusStackOverflow;
          return true;
        }
        if (sp < 32) {
          stk0 = lane == sp ? r : stk0;
        } else {
          stk1 = lane == sp - 32 ? r : stk1;
        }
        ++sp;
      }
    }
    if (leaf && !__ballot_sync(full, active)) {
      visits += it + 1;
      return hit;
    }
    if (next < 0) {
      if (sp == 0) {
        visits += it + 1;
        return hit;
      }
      --sp;
      next = __shfl_sync(full, sp < 32 ? stk0 : stk1, sp & 31);
    }
    node = next;
  }
  visits += max_iter;
  status_bits |= kStatusTraversalOverrun;
  return true;
}

__device__ __forceinline__ int64_t row_start(int64_t i, int64_t n) {
  return i * (2 * n - i - 1) / 2;
}

// Morton order of n device points into perm (vis.cu); synchronizes.
int vis_morton_order(visacd_ctx* ctx, const float* d_pts, int32_t n, uint32_t* perm);

}  // namespace vgpu

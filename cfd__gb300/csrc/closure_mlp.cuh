// closure_mlp.cuh — the learned closure's 6 -> 32 -> 32 -> 1 MLP for one warp
// of 32 cells on the tensor cores (mma.sync.m16n8k16, bf16 operands, fp32
// accumulation).  Used by the fused closure step and by closure_eval.
//
// Fragment conventions of m16n8k16 (PTX ISA, "Matrix fragments for mma"):
// g = lane / 4, t = lane % 4;
//   A (16x16, row-major): a0 = (row g, k 2t..2t+1), a1 = (row g+8, k 2t..),
//                         a2 = (row g, k 2t+8..),   a3 = (row g+8, k 2t+8..)
//   B (16x8, col-major):  b0 = (k 2t..2t+1, col g), b1 = (k 2t+8.., col g)
//   C (16x8, fp32):       c0,c1 = (row g, cols 2t, 2t+1), c2,c3 = (row g+8, ...)
// Two adjacent n8 output tiles of one layer are exactly the k16 A fragment of
// the next layer (c0c1 | c2c3 of tile 2k and 2k+1), so hidden activations
// never leave registers.  Biases initialise the accumulators.
#pragma once
#include <cstdint>
#include <cuda_bf16.h>

#include "closure_tc.cuh"

namespace lbm {

// Weights in fragment order (built on the host by closure_pack).
struct MlpFrag {
  uint4 tcb[TC_B_BYTES / 16];   // B operands of the tcgen05 path (closure_tc.cuh)
  uint2 w1[4][32];      // layer 1: nt 0..3, k 0..15 (inputs 0..5, rest zero)
  uint2 w2[4][2][32];   // layer 2: nt 0..3, kt 0..1
  uint2 w3[2][32];      // layer 3: n 0 only (n 1..7 zero), kt 0..1
  float b1[32], b2[32], b3;
  float w3b[33];                // output weights and bias, bf16-rounded (CTA engine's CUDA-core layer)
  float mean[6], inv_std[6];
  float nu_scale, nu_max;
  float lo[6], hi[6];           // raw-feature range of the training set
  int coef;                     // output is Cs^2 (1) or nu_t (0)
};

// The network's per-feature constants and output bounds, passed by value in
// the step kernels' parameters (read from the constant bank, no loads).
struct CloConst {
  float lo[6], hi[6], mean[6], inv_std[6];
  float nu_scale, nu_max;
};

// Raw features inside the trained range (false also for NaN features).
__device__ __forceinline__ bool closure_in_range(const CloConst& K, const float (&f)[6]) {
  bool ok = true;
#pragma unroll
  for (int a = 0; a < 6; ++a) ok = ok && f[a] >= K.lo[a] && f[a] <= K.hi[a];
  return ok;
}

// Raw features inside the trained range (false also for NaN features).
__device__ __forceinline__ bool closure_in_range(const MlpFrag& F, const float (&f)[6]) {
  bool ok = true;
#pragma unroll
  for (int a = 0; a < 6; ++a) ok = ok && f[a] >= __ldg(&F.lo[a]) && f[a] <= __ldg(&F.hi[a]);
  return ok;
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint2 b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b.x), "r"(b.y));
}

// ReLU of two floats packed as bf16x2 (lo = a, hi = b), round to nearest.
__device__ __forceinline__ uint32_t relu_bf16x2(float a, float b) {
  uint32_t r;
  asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;\n" : "=r"(r) : "f"(b), "f"(a));
  return r;
}

// Weight and bias reads as volatile loads: they stay where the network is
// evaluated instead of being hoisted above the caller's population loads,
// where they would hold ~45 registers through the pull.  Generic addressing
// (the fragments may sit in global or shared memory).
__device__ __forceinline__ uint2 ld_w(const uint2* p) {
  uint2 r;
  asm volatile("ld.v2.u32 {%0,%1}, [%2];\n" : "=r"(r.x), "=r"(r.y) : "l"(p));
  return r;
}
__device__ __forceinline__ float2 ld_b(const float* p) {
  float2 r;
  asm volatile("ld.v2.f32 {%0,%1}, [%2];\n" : "=f"(r.x), "=f"(r.y) : "l"(p));
  return r;
}
__device__ __forceinline__ float ld_b1(const float* p) {
  float r;
  asm volatile("ld.f32 %0, [%1];\n" : "=f"(r) : "l"(p));
  return r;
}

__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
  uint32_t r;
  asm("cvt.rn.bf16x2.f32 %0, %1, %2;\n" : "=r"(r) : "f"(b), "f"(a));
  return r;
}

// y (pre-softplus output) of this lane's cell.  Every lane of the warp must
// call it (the mma is warp-collective); x holds the lane's normalised
// features (zeros for lanes without a cell).  The warp's 32 cells are two
// 16-row tiles; each weight fragment is loaded once and used for both.
__device__ __forceinline__ float warp_mlp(const MlpFrag& F, const float (&x)[6]) {
  const int lane = threadIdx.x & 31;
  const int g = lane >> 2, t = lane & 3;
  const uint32_t f01 = pack_bf16x2(x[0], x[1]);
  const uint32_t f23 = pack_bf16x2(x[2], x[3]);
  const uint32_t f45 = pack_bf16x2(x[4], x[5]);
  // layer-1 A fragments: rows g and g+8 of each tile, k pair t (pairs 3..7 zero)
  uint32_t a0[2], a1[2];
#pragma unroll
  for (int mt = 0; mt < 2; ++mt) {
    const int src_lo = mt * 16 + g, src_hi = src_lo + 8;
    const uint32_t lo0 = __shfl_sync(0xffffffffu, f01, src_lo), lo1 = __shfl_sync(0xffffffffu, f23, src_lo),
                   lo2 = __shfl_sync(0xffffffffu, f45, src_lo);
    const uint32_t hi0 = __shfl_sync(0xffffffffu, f01, src_hi), hi1 = __shfl_sync(0xffffffffu, f23, src_hi),
                   hi2 = __shfl_sync(0xffffffffu, f45, src_hi);
    a0[mt] = t == 0 ? lo0 : (t == 1 ? lo1 : (t == 2 ? lo2 : 0u));
    a1[mt] = t == 0 ? hi0 : (t == 1 ? hi1 : (t == 2 ? hi2 : 0u));
  }
  // layer 1: 4 n8 tiles of 32 hidden units
  uint32_t h1[2][4][2];
#pragma unroll
  for (int nt = 0; nt < 4; ++nt) {
    const float2 b = ld_b(&F.b1[nt * 8 + 2 * t]);
    const uint2 w = ld_w(&F.w1[nt][lane]);
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
      float c[4] = {b.x, b.y, b.x, b.y};
      mma_bf16(c, a0[mt], a1[mt], 0u, 0u, w);
      h1[mt][nt][0] = relu_bf16x2(c[0], c[1]);
      h1[mt][nt][1] = relu_bf16x2(c[2], c[3]);
    }
  }
  // layer 2
  uint32_t h2[2][4][2];
#pragma unroll
  for (int nt = 0; nt < 4; ++nt) {
    const float2 b = ld_b(&F.b2[nt * 8 + 2 * t]);
    const uint2 w0 = ld_w(&F.w2[nt][0][lane]), w1 = ld_w(&F.w2[nt][1][lane]);
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
      float c[4] = {b.x, b.y, b.x, b.y};
      mma_bf16(c, h1[mt][0][0], h1[mt][0][1], h1[mt][1][0], h1[mt][1][1], w0);
      mma_bf16(c, h1[mt][2][0], h1[mt][2][1], h1[mt][3][0], h1[mt][3][1], w1);
      h2[mt][nt][0] = relu_bf16x2(c[0], c[1]);
      h2[mt][nt][1] = relu_bf16x2(c[2], c[3]);
    }
  }
  // layer 3 (output in column 0): (row g, col 2t) and (row g+8, col 2t)
  const float b3 = ld_b1(&F.b3);
  const uint2 v0 = ld_w(&F.w3[0][lane]), v1 = ld_w(&F.w3[1][lane]);
  float y0[2], y2[2];
#pragma unroll
  for (int mt = 0; mt < 2; ++mt) {
    float c[4] = {b3, b3, b3, b3};
    mma_bf16(c, h2[mt][0][0], h2[mt][0][1], h2[mt][1][0], h2[mt][1][1], v0);
    mma_bf16(c, h2[mt][2][0], h2[mt][2][1], h2[mt][3][0], h2[mt][3][1], v1);
    y0[mt] = c[0];
    y2[mt] = c[2];
  }
  // cell r of the warp: tile r/16, row r%16 -> lane 4 (r%8) holds it
  const int mt = lane >> 4, rr = lane & 15, srcl = 4 * (rr & 7);
  const float v00 = __shfl_sync(0xffffffffu, y0[0], srcl), v02 = __shfl_sync(0xffffffffu, y2[0], srcl);
  const float v10 = __shfl_sync(0xffffffffu, y0[1], srcl), v12 = __shfl_sync(0xffffffffu, y2[1], srcl);
  const bool hi = rr >= 8;
  return mt == 0 ? (hi ? v02 : v00) : (hi ? v12 : v10);
}

__device__ __forceinline__ float sqrt_approx(float v) {
  float r;
  asm("sqrt.approx.f32 %0, %1;\n" : "=f"(r) : "f"(v));
  return r;
}

// The raw features x0..x3 and x5 of one cell from its non-equilibrium
// stress Pi (components xx, yy, zz, xy, xz, yz), 1/rho and delta = rho - 1;
// x4 = omega0 is per run and set by the caller.  Approximate sqrt, log and
// division (the network does not need IEEE rounding).  Shared by the fused
// step and the sample builder so training and inference see the same
// numbers.
__device__ __forceinline__ void closure_features(float xx, float yy, float zz, float xy, float xz, float yz,
                                                 float rinv, float delta, float (&f)[6]) {
  const float off = xy * xy + xz * xz + yz * yz;
  const float pp = xx * xx + yy * yy + zz * zz + 2.0f * off;
  const float qs = sqrt_approx(2.0f * pp);
  f[0] = __logf(qs * rinv + 1e-9f);
  f[1] = __fdividef(xx + yy + zz, qs + 1e-12f);
  const float det = xx * (yy * zz - yz * yz) - xy * (xy * zz - yz * xz) + xz * (xy * yz - yy * xz);
  f[2] = __fdividef(det, qs * qs * qs + 1e-30f);
  f[3] = __fdividef(off, 0.5f * pp + 1e-30f);
  f[5] = 100.0f * delta;
}

// nu_t from the network output: nu_scale * softplus(y); NaN when the cell
// must fall back (not finite, negative or above nu_max).
__device__ __forceinline__ float closure_nu(float nu_scale, float nu_max, float y) {
  const float sp = y > 20.0f ? y : __logf(1.0f + __expf(y));
  const float nu = nu_scale * sp;
  return (nu >= 0.0f && nu <= nu_max) ? nu : __int_as_float(0x7fc00000);
}
__device__ __forceinline__ float closure_nu(const MlpFrag& F, float y) { return closure_nu(F.nu_scale, F.nu_max, y); }
__device__ __forceinline__ float closure_nu(const CloConst& K, float y) { return closure_nu(K.nu_scale, K.nu_max, y); }

}  // namespace lbm

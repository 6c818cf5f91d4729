// lbm_core.cuh — D3Q19 tables and the per-cell collide shared by every step
// kernel of the GB300 solver.
//
// The arithmetic restates the reference's generated step body
// (src/core/emit/ir.js:493-533, blocks :166-478) operation by operation: the
// files that include this header are compiled with -fmad=false and IEEE
// division/sqrt, so each fp32 operation rounds exactly where the shader text
// writes it.  That makes the fp32 path bit-identical to the CPU oracle.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>

#include <cmath>

namespace lbm {

constexpr int Q = 19;

// Cell classes (src/core/emit/ir.js:71-80).
enum : uint32_t {
  FLUIDO = 0, SOLIDO = 1, ENTRADA = 2, SAIDA = 3, SOLIDO_MOVEL = 4,
  ESPELHO_Y = 5, ESPELHO_Z = 6, PAREDE = 7
};

__host__ __device__ constexpr bool is_solid(uint32_t t) {
  return t == SOLIDO || t == SOLIDO_MOVEL || t == PAREDE;
}

// Velocity set with opposite pairs adjacent (src/core/lattice.js:57-79).
__host__ __device__ constexpr int cx(int i) {
  return (i == 1 || i == 7 || i == 9 || i == 11 || i == 13) ? 1
       : (i == 2 || i == 8 || i == 10 || i == 12 || i == 14) ? -1 : 0;
}
__host__ __device__ constexpr int cy(int i) {
  return (i == 3 || i == 7 || i == 10 || i == 15 || i == 17) ? 1
       : (i == 4 || i == 8 || i == 9 || i == 16 || i == 18) ? -1 : 0;
}
__host__ __device__ constexpr int cz(int i) {
  return (i == 5 || i == 11 || i == 14 || i == 15 || i == 18) ? 1
       : (i == 6 || i == 12 || i == 13 || i == 16 || i == 17) ? -1 : 0;
}
__host__ __device__ constexpr int ci(int i, int a) { return a == 0 ? cx(i) : (a == 1 ? cy(i) : cz(i)); }
// opp(0) = 0, opp(i) = ((i-1)^1)+1 (src/core/lattice.js:89)
__host__ __device__ constexpr int opp(int i) { return i == 0 ? 0 : (((i - 1) ^ 1) + 1); }
// Specular reflection across axis `ax` (espelharIdx, src/core/emit/ir.js:86-93).
__host__ __device__ constexpr int mirror_idx(int i, int ax) {
  int j = 0;
  for (int k = 0; k < Q; ++k) {
    const int a0 = ax == 0 ? -cx(i) : cx(i);
    const int a1 = ax == 1 ? -cy(i) : cy(i);
    const int a2 = ax == 2 ? -cz(i) : cz(i);
    if (cx(k) == a0 && cy(k) == a1 && cz(k) == a2) j = k;
  }
  return j;
}

// Weights as the shader literals (num(), src/core/emit/ir.js:99-106) for fp32,
// the exact rationals rounded once for fp64.
template <typename R> struct Lit;
template <> struct Lit<float> {
  __host__ __device__ static constexpr float w(int i) {
    return i == 0 ? 0.333333333f : (i <= 6 ? 0.0555555556f : 0.0277777778f);
  }
  // 2 w_i / c_s^2 (src/core/emit/ir.js:185)
  __host__ __device__ static constexpr float sixw(int i) {
    return i == 0 ? 0.0f : (i <= 6 ? 0.333333333f : 0.166666667f);
  }
  __host__ __device__ static constexpr float bl_exp() { return 0.1428571429f; }
};
template <> struct Lit<double> {
  __host__ __device__ static constexpr double w(int i) {
    return i == 0 ? 1.0 / 3.0 : (i <= 6 ? 1.0 / 18.0 : 1.0 / 36.0);
  }
  __host__ __device__ static constexpr double sixw(int i) { return i == 0 ? 0.0 : 2.0 * w(i) * 3.0; }
  __host__ __device__ static constexpr double bl_exp() { return 0.1428571429; }
};

__device__ __forceinline__ float r_sqrt(float v) { return sqrtf(v); }
__device__ __forceinline__ double r_sqrt(double v) { return sqrt(v); }

// Inlet boundary-layer factor of row z (src/core/emit/wgsl.js:217-220):
//   blf = zc < BL ? pow(zc / max(BL, 1), 1/7) : 1,  zc = z + 1/2.
// It depends on z and BL only, so the library evaluates it on the host once
// per configuration (bl_factor_host, the host's libm pow) and the kernels read
// it from a per-z table: the power function leaves the device, and a host
// restatement of the shader computes the same value bit for bit.
template <typename R>
inline R bl_factor_host(float bl_thickness, int z) {
  const R bl = R(bl_thickness);
  const R uInletBL = bl > R(1.0) ? bl : R(1.0);
  const R zc = R(z) + R(0.5);
  if (!(zc < bl)) return R(1.0);
  return std::pow(zc / uInletBL, Lit<R>::bl_exp());
}

// Kernel-side copy of lbm_params (src/core/emit/wgsl.js:123-135).
struct Params {
  float omega_plus, magic, les_cs;
  float belt[3], inlet[3];
  float sponge_start, sponge_len, bl;
  int32_t closure;
};

// c_i . v with the term order dotC emits (src/core/emit/ir.js:116-126).
template <typename R>
__device__ __forceinline__ R dotc(int i, R vx, R vy, R vz) {
  const int a = cx(i), b = cy(i), c = cz(i);
  R acc = R(0);
  bool first = true;
  if (a != 0) { acc = a > 0 ? vx : -vx; first = false; }
  if (b != 0) { if (first) { acc = b > 0 ? vy : -vy; first = false; } else acc = b > 0 ? acc + vy : acc - vy; }
  if (c != 0) { if (first) { acc = c > 0 ? vz : -vz; } else acc = c > 0 ? acc + vz : acc - vz; }
  return acc;
}

// Signed sum over the directions with coefficient k(i) != 0, index order,
// as the emitter joins the terms (src/core/emit/ir.js:201-208, :272-282).
template <typename R, typename K>
__device__ __forceinline__ R signed_sum(const R* v, K coef) {
  R acc = R(0);
  bool first = true;
#pragma unroll
  for (int i = 0; i < Q; ++i) {
    const int c = coef(i);
    if (c == 0) continue;
    if (first) { acc = c > 0 ? v[i] : -v[i]; first = false; }
    else acc = c > 0 ? acc + v[i] : acc - v[i];
  }
  return acc;
}

// ---------------------------------------------------------- arithmetic modes
// Two restatements of the shader's arithmetic, both reproduced bit for bit by
// the CPU oracle:
//  * STRICT (FAST = false): the generated shader text read literally, one IEEE
//    operation per written operator, no contraction (src/core/emit/ir.js).
//  * FAST (FAST = true): the same formulas with fused multiply-adds at fixed
//    places, u = m * (1/rho) (one reciprocal instead of three divisions) and
//    omega- = (tau - 1/2) / (Lambda + (tau - 1/2)/2), which is
//    1 / (Lambda / (1/omega+ - 1/2) + 1/2) with 1/omega+ = tau exactly
//    (src/core/emit/ir.js:297-299).  Rounding differs from STRICT by ~1 ulp per
//    operation; the fp64 reference form always runs STRICT.
// Explicit fmaf() stays fused under -fmad=false, so both modes are fixed
// sequences of IEEE operations.
template <typename R>
__device__ __forceinline__ R fma_r(R a, R b, R c) { return fma(a, b, c); }
template <>
__device__ __forceinline__ float fma_r<float>(float a, float b, float c) { return fmaf(a, b, c); }

// Equilibrium of one direction (src/core/emit/ir.js:216-232).  uu15 = 1.5 uu
// is used by FAST only.
template <typename R, bool FAST>
__device__ __forceinline__ R equilibrium(int i, R delta, R rho, R ux, R uy, R uz, R uu, R uu15) {
  if constexpr (FAST) {
    if (i == 0) return Lit<R>::w(0) * fma_r<R>(-rho, uu15, delta);
    const R cu = dotc<R>(i, ux, uy, uz);
    const R a = fma_r<R>(cu, fma_r<R>(R(4.5), cu, R(3.0)), -uu15);
    return Lit<R>::w(i) * fma_r<R>(rho, a, delta);
  }
  if (i == 0) return Lit<R>::w(0) * (delta - R(1.5) * rho * uu);
  const R cu = dotc<R>(i, ux, uy, uz);
  return Lit<R>::w(i) * (delta + rho * (R(3.0) * cu + R(4.5) * cu * cu - R(1.5) * uu));
}

// Pulled moments (src/core/emit/ir.js:192-213), STRICT: the emitter's
// index-order sums and three divisions.
template <typename R>
__device__ __forceinline__ void moments_strict(const R* g, R& delta, R& rho, R& ux, R& uy, R& uz, R& uu) {
  delta = g[0];
#pragma unroll
  for (int i = 1; i < Q; ++i) delta = delta + g[i];
  rho = R(1.0) + delta;
  const R mx = signed_sum<R>(g, [](int i) { return cx(i); });
  const R my = signed_sum<R>(g, [](int i) { return cy(i); });
  const R mz = signed_sum<R>(g, [](int i) { return cz(i); });
  ux = mx / rho;
  uy = my / rho;
  uz = mz / rho;
  uu = ux * ux + uy * uy + uz * uz;
}

// Signed sum over the nine opposite pairs (k = 0..8, odd member i = 2k+1)
// with coefficient coef(i) of the odd member, pair order.
template <typename R, typename K>
__device__ __forceinline__ R pair_sum(const R* v, K coef) {
  R acc = R(0);
  bool first = true;
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    const int c = coef(2 * k + 1);
    if (c == 0) continue;
    if (first) { acc = c > 0 ? v[k] : -v[k]; first = false; }
    else acc = c > 0 ? acc + v[k] : acc - v[k];
  }
  return acc;
}

// FAST moments from the pair sums s_k = g_i + g_j and differences
// d_k = g_i - g_j (j = opp i): delta = g0 + sum s, rho u = sum c_i d_k,
// u = (rho u) (1/rho).  s and d are reused by the pair-form collision.
template <typename R>
__device__ __forceinline__ void moments_fast(const R* g, R* sp, R* dp, R& delta, R& rho, R& ux, R& uy, R& uz,
                                             R& uu, R& rinv) {
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    sp[k] = g[2 * k + 1] + g[2 * k + 2];
    dp[k] = g[2 * k + 1] - g[2 * k + 2];
  }
  delta = g[0];
#pragma unroll
  for (int k = 0; k < 9; ++k) delta = delta + sp[k];
  rho = R(1.0) + delta;
  const R mx = pair_sum<R>(dp, [](int i) { return cx(i); });
  const R my = pair_sum<R>(dp, [](int i) { return cy(i); });
  const R mz = pair_sum<R>(dp, [](int i) { return cz(i); });
  rinv = R(1.0) / rho;
  ux = mx * rinv;
  uy = my * rinv;
  uz = mz * rinv;
  uu = fma_r<R>(uz, uz, fma_r<R>(uy, uy, ux * ux));
}

// FAST moments of populations held times a power-of-two scale S (the 16-bit
// form stores S g_i): the pair sums, delta and rho u come out exactly S times
// the unscaled ones (scaling by a power of two commutes with rounding), and
//   rho = fma(S delta, 1/S, 1) = RN(1 + delta),
//   u   = (S rho u) (RN(1/rho) / S) = RN((rho u) RN(1/rho))
// round as the unscaled operations do: the results are bit-identical to
// moments_fast on the unscaled values.  delta_s = S delta.
template <typename R>
__device__ __forceinline__ void moments_fast_scaled(const R* g, R inv_scale, R* sp, R* dp, R& delta_s, R& rho, R& ux,
                                                    R& uy, R& uz, R& uu, R& rinv) {
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    sp[k] = g[2 * k + 1] + g[2 * k + 2];
    dp[k] = g[2 * k + 1] - g[2 * k + 2];
  }
  delta_s = g[0];
#pragma unroll
  for (int k = 0; k < 9; ++k) delta_s = delta_s + sp[k];
  rho = fma_r<R>(delta_s, inv_scale, R(1.0));
  const R mx = pair_sum<R>(dp, [](int i) { return cx(i); });
  const R my = pair_sum<R>(dp, [](int i) { return cy(i); });
  const R mz = pair_sum<R>(dp, [](int i) { return cz(i); });
  rinv = R(1.0) / rho;
  const R rinvs = rinv * inv_scale;
  ux = mx * rinvs;
  uy = my * rinvs;
  uz = mz * rinvs;
  uu = fma_r<R>(uz, uz, fma_r<R>(uy, uy, ux * ux));
}

// Warp-uniform values derived from Params once per launch on the host (same
// IEEE operations the per-cell code would do, so results do not change):
//   tau0 = 1/omega+, tau0^2, 18 Cs^2 (src/core/emit/ir.js:290-293);
//   with Cs = 0 the LES root is exactly tau0 (sqrt(RN(t^2)) = t in binary
//   round-to-nearest), so omega+ and omega- are uniform too;
//   the sponge's free-stream targets (src/core/emit/ir.js:464-476).
template <typename R>
struct Uni {
  R tau0, tau0sq, c18;
  R omegaP0, omegaM0;      // STRICT, Cs = 0
  R omegaP0f, omegaM0f;    // FAST, Cs = 0
  R sp_start, sp_len;
  R sp_t[Q];               // STRICT sponge targets
  R sp_tf[Q];              // FAST sponge targets
  R sp_tfs[Q];             // FAST sponge targets times the storage scale
  int les_on;
};

template <typename R>
__host__ __device__ inline R dotc_h(int i, R vx, R vy, R vz) {
  const int a = cx(i), b = cy(i), c = cz(i);
  R acc = R(0);
  bool first = true;
  if (a != 0) { acc = a > 0 ? vx : -vx; first = false; }
  if (b != 0) { if (first) { acc = b > 0 ? vy : -vy; first = false; } else acc = b > 0 ? acc + vy : acc - vy; }
  if (c != 0) { if (first) { acc = c > 0 ? vz : -vz; } else acc = c > 0 ? acc + vz : acc - vz; }
  return acc;
}

inline float fma_h(float a, float b, float c) { return std::fmaf(a, b, c); }
inline double fma_h(double a, double b, double c) { return std::fma(a, b, c); }

// Host side (built with -ffp-contract=off; fusion only where fma_h is called).
template <typename R>
inline Uni<R> make_uni(const Params& P, R scale = R(1.0)) {
  Uni<R> u;
  const R cs = R(P.les_cs);
  const R magic = R(P.magic);
  u.tau0 = R(1.0) / R(P.omega_plus);
  u.tau0sq = u.tau0 * u.tau0;
  u.c18 = R(18.0) * cs * cs;
  u.les_on = !(cs == R(0.0));
  u.omegaP0 = R(1.0) / u.tau0;
  u.omegaM0 = R(1.0) / (magic / (R(1.0) / u.omegaP0 - R(0.5)) + R(0.5));
  u.omegaP0f = R(1.0) / u.tau0;
  const R tm = u.tau0 - R(0.5);
  u.omegaM0f = tm / fma_h(R(0.5), tm, magic);
  u.sp_start = R(P.sponge_start);
  u.sp_len = R(P.sponge_len) > R(1.0) ? R(P.sponge_len) : R(1.0);
  const R ix = R(P.inlet[0]), iy = R(P.inlet[1]), iz = R(P.inlet[2]);
  const R uuInf = ix * ix + iy * iy + iz * iz;
  const R uuInfF = fma_h(iz, iz, fma_h(iy, iy, ix * ix));
  const R uu15f = R(1.5) * uuInfF;
  u.sp_t[0] = Lit<R>::w(0) * (R(-1.5) * uuInf);
  u.sp_tf[0] = Lit<R>::w(0) * (-uu15f);
  for (int i = 1; i < Q; ++i) {
    const R si = dotc_h<R>(i, ix, iy, iz);
    u.sp_t[i] = Lit<R>::w(i) * (R(3.0) * si + R(4.5) * si * si - R(1.5) * uuInf);
    u.sp_tf[i] = Lit<R>::w(i) * fma_h(si, fma_h(R(4.5), si, R(3.0)), -uu15f);
  }
  for (int i = 0; i < Q; ++i) u.sp_tfs[i] = u.sp_tf[i] * scale;   // exact: scale is a power of two
  return u;
}

// ---- FAST fluid path in three pieces (the learned closure runs its network
// between the first and the last) ----

// Pair form of the shifted equilibrium (c_j = -c_i, w_j = w_i):
//   e_i + e_j = 2 w (delta + rho (4.5 cu^2 - 1.5 uu)),  e_i - e_j = 6 w rho cu;
// ns = (g_i + g_j) - (e_i + e_j), nd = (g_i - g_j) - (e_i - e_j).
// Fused as: B = fma(-rho, 1.5 uu, delta) once per cell (e0 = w0 B), then per
// pair E = fma(4.5 rho cu, cu, B), ns = fma(-2w, E, s), nd = fma(-6 w rho, cu, d):
// four operations a pair.
template <typename R>
__device__ __forceinline__ void fluid_neq_fast(const R* sp, const R* dp, R delta, R rho, R ux, R uy, R uz, R uu,
                                               R& e0, R* ns, R* nd) {
  const R uu15 = R(1.5) * uu;
  const R B = fma_r<R>(-rho, uu15, delta);
  e0 = Lit<R>::w(0) * B;
  const R a45 = R(4.5) * rho;
  const R r6a = (R(6.0) * Lit<R>::w(1)) * rho, r6d = (R(6.0) * Lit<R>::w(7)) * rho;
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    const int i = 2 * k + 1;
    const R cu = dotc<R>(i, ux, uy, uz);
    const R E = fma_r<R>(a45 * cu, cu, B);
    ns[k] = fma_r<R>(-(R(2.0) * Lit<R>::w(i)), E, sp[k]);
    nd[k] = fma_r<R>(-(i <= 6 ? r6a : r6d), cu, dp[k]);
  }
}

// Pi_ab = sum over pairs of c_ia c_ib ns (src/core/emit/ir.js:269-282, pair form)
template <typename R>
struct PiT {
  R xx, yy, zz, xy, xz, yz;
};
template <typename R>
__device__ __forceinline__ PiT<R> pi_fast(const R* ns) {
  PiT<R> p;
  p.xx = pair_sum<R>(ns, [](int i) { return cx(i) * cx(i); });
  p.yy = pair_sum<R>(ns, [](int i) { return cy(i) * cy(i); });
  p.zz = pair_sum<R>(ns, [](int i) { return cz(i) * cz(i); });
  p.xy = pair_sum<R>(ns, [](int i) { return cx(i) * cy(i); });
  p.xz = pair_sum<R>(ns, [](int i) { return cx(i) * cz(i); });
  p.yz = pair_sum<R>(ns, [](int i) { return cy(i) * cz(i); });
  return p;
}

// Smagorinsky relaxation rates (src/core/emit/ir.js:284-299), FAST form.
template <typename R>
__device__ __forceinline__ void smag_rates_fast(const Params& P, const Uni<R>& U, const R* ns, R rinv, R& omegaP,
                                                R& omegaM) {
  omegaP = U.omegaP0f;
  omegaM = U.omegaM0f;
  if (U.les_on) {
    const PiT<R> q = pi_fast<R>(ns);
    const R pd = fma_r<R>(q.zz, q.zz, fma_r<R>(q.yy, q.yy, q.xx * q.xx));
    const R po = fma_r<R>(q.yz, q.yz, fma_r<R>(q.xz, q.xz, q.xy * q.xy));
    const R pp = fma_r<R>(R(2.0), po, pd);
    const R qs = r_sqrt(R(2.0) * pp);
    const R tauT = R(0.5) * (U.tau0 + r_sqrt(fma_r<R>(U.c18 * qs, rinv, U.tau0sq)));
    omegaP = R(1.0) / tauT;
    const R tm = tauT - R(0.5);
    omegaM = tm / fma_r<R>(R(0.5), tm, R(P.magic));
  }
}

// The same relaxation with a per-cell coefficient: c18 = 18 Cs^2 (the
// learned closure's coefficient form), whatever U.les_on says.
template <typename R>
__device__ __forceinline__ void smag_rates_c18(const Params& P, const Uni<R>& U, const R* ns, R rinv, R c18,
                                               R& omegaP, R& omegaM) {
  const PiT<R> q = pi_fast<R>(ns);
  const R pd = fma_r<R>(q.zz, q.zz, fma_r<R>(q.yy, q.yy, q.xx * q.xx));
  const R po = fma_r<R>(q.yz, q.yz, fma_r<R>(q.xz, q.xz, q.xy * q.xy));
  const R pp = fma_r<R>(R(2.0), po, pd);
  const R qs = r_sqrt(R(2.0) * pp);
  const R tauT = R(0.5) * (U.tau0 + r_sqrt(fma_r<R>(c18 * qs, rinv, U.tau0sq)));
  omegaP = R(1.0) / tauT;
  const R tm = tauT - R(0.5);
  omegaM = tm / fma_r<R>(R(0.5), tm, R(P.magic));
}

// Relaxation rates of a FLUIDO cell for collide(): the Smagorinsky rates by
// default; the held closure steps supply their own (lbm_kernels.cuh).
struct SmagRates {
  template <typename R>
  __device__ __forceinline__ void operator()(const Params& P, const Uni<R>& U, const R* ns, R rinv, R& omegaP,
                                             R& omegaM) const {
    smag_rates_fast<R>(P, U, ns, rinv, omegaP, omegaM);
  }
};

// TRT per pair and the sponge blend (src/core/emit/ir.js:304-323, :458-478).
// spt: the sponge targets in the units of g (U.sp_tf, or U.sp_tfs for
// populations held times the storage scale).
template <typename R, typename Emit>
__device__ __forceinline__ void trt_emit_fast(const Uni<R>& U, int x, const R* g, R e0, const R* ns, const R* nd,
                                              R omegaP, R omegaM, const R* spt, Emit&& emit) {
  R sig2 = R(0.0);
  if (R(x) > U.sp_start) {
    const R sx = (R(x) - U.sp_start) / U.sp_len;
    const R sigma = sx < R(1.0) ? sx : R(1.0);
    sig2 = sigma * sigma;
  }
  const R o0 = fma_r<R>(-omegaP, g[0] - e0, g[0]);
  const R hP = R(0.5) * omegaP, hM = R(0.5) * omegaM;
  // One branch per cell (warps run along x, so a warp is either inside the
  // sponge or not) instead of a select per output.
  if (sig2 != R(0.0)) {
    const R oms = R(1.0) - sig2;
    emit(0, fma_r<R>(spt[0], sig2, o0 * oms));
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      const int i = 2 * k + 1, j = i + 1;
      const R oi = fma_r<R>(-hM, nd[k], fma_r<R>(-hP, ns[k], g[i]));
      const R oj = fma_r<R>(hM, nd[k], fma_r<R>(-hP, ns[k], g[j]));
      emit(i, fma_r<R>(spt[i], sig2, oi * oms));
      emit(j, fma_r<R>(spt[j], sig2, oj * oms));
    }
    return;
  }
  emit(0, o0);
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    const int i = 2 * k + 1, j = i + 1;
    emit(i, fma_r<R>(-hM, nd[k], fma_r<R>(-hP, ns[k], g[i])));
    emit(j, fma_r<R>(hM, nd[k], fma_r<R>(-hP, ns[k], g[j])));
  }
}

// Everything after the pull for one non-solid cell: the boundary branches and
// the fluid collide with LES, TRT and sponge (src/core/emit/ir.js:505-530).
// g: pulled populations.  Each post-collision population is handed to
// emit(i, value) as soon as it exists (i is a compile-time constant after
// unrolling), so no output array stays live.  blf: the per-z inlet
// boundary-layer factors (bl_factor_host), null when every factor is 1.
// SC (FAST only): g, sp, dp and delta are held times the power-of-two `scale`
// (moments_fast_scaled) and the emitted values are too; every operation on
// them is the unscaled one times the scale, exactly.
// rates(P, U, ns, rinv, omegaP, omegaM): the FLUIDO cell's relaxation rates
// in the FAST form (SmagRates: Smagorinsky).
template <typename R, bool FAST, bool SC = false, typename Emit, typename Rates = SmagRates>
__device__ __forceinline__ void collide(const Params& P, const Uni<R>& U, uint32_t ct, int x, int z, const R* g,
                                        const R* sp, const R* dp, R delta, R rho, R ux, R uy, R uz, R uu, R rinv,
                                        const R* blf_tab, Emit&& emit, R scale = R(1.0), Rates rates = Rates()) {
  static_assert(FAST || !SC, "the scaled form is a FAST restatement");
  if (ct == ESPELHO_Y) {
#pragma unroll
    for (int i = 0; i < Q; ++i) emit(i, g[mirror_idx(i, 1)]);
    return;
  }
  if (ct == ESPELHO_Z) {
#pragma unroll
    for (int i = 0; i < Q; ++i) emit(i, g[mirror_idx(i, 2)]);
    return;
  }
  if (ct == ENTRADA) {
    // blocoEntrada with the boundary-layer factor of the kernel header
    // (src/core/emit/ir.js:405-422; src/core/emit/wgsl.js:217-220)
    const R blf = blf_tab ? blf_tab[z] : R(1.0);
    const R ex = R(P.inlet[0]) * blf, ey = R(P.inlet[1]) * blf, ez = R(P.inlet[2]) * blf;
    if constexpr (FAST) {
      const R uuIn = fma_r<R>(ez, ez, fma_r<R>(ey, ey, ex * ex));
      const R uu15 = R(1.5) * uuIn;
#pragma unroll
      for (int i = 0; i < Q; ++i) {
        const R e = equilibrium<R, true>(i, R(0.0), R(1.0), ex, ey, ez, uuIn, uu15);
        emit(i, SC ? e * scale : e);
      }
      return;
    }
    const R deltaIn = R(0.0), rhoIn = R(1.0);
    const R uuIn = ex * ex + ey * ey + ez * ez;
    emit(0, Lit<R>::w(0) * (deltaIn - R(1.5) * rhoIn * uuIn));
#pragma unroll
    for (int i = 1; i < Q; ++i) {
      const R c = dotc<R>(i, ex, ey, ez);
      emit(i, Lit<R>::w(i) * (deltaIn + rhoIn * (R(3.0) * c + R(4.5) * c * c - R(1.5) * uuIn)));
    }
    return;
  }
  const R uu15 = R(1.5) * uu;
  if (ct == SAIDA) {
    // blocoSaida with the pulled u (src/core/emit/ir.js:432-444, :512-515)
    if constexpr (FAST) {
      const R o0 = Lit<R>::w(0) * (-uu15);
      emit(0, SC ? o0 * scale : o0);
#pragma unroll
      for (int i = 1; i < Q; ++i) {
        const R c = dotc<R>(i, ux, uy, uz);
        const R o = Lit<R>::w(i) * fma_r<R>(c, fma_r<R>(R(4.5), c, R(3.0)), -uu15);
        emit(i, SC ? o * scale : o);
      }
      return;
    }
    emit(0, Lit<R>::w(0) * (R(-1.5) * uu));
#pragma unroll
    for (int i = 1; i < Q; ++i) {
      const R c = dotc<R>(i, ux, uy, uz);
      emit(i, Lit<R>::w(i) * (R(3.0) * c + R(4.5) * c * c - R(1.5) * uu));
    }
    return;
  }
  // FLUIDO: equilibrium, Smagorinsky LES (src/core/emit/ir.js:262-301)
  if constexpr (FAST) {
    R e0, ns[9], nd[9], omegaP, omegaM;
    if constexpr (SC) {
      // scaled: e = (S rho) a + S delta and the LES term's (S c18 qs) (rinv / S)
      // are S times / exactly the unscaled operations
      fluid_neq_fast<R>(sp, dp, delta, rho * scale, ux, uy, uz, uu, e0, ns, nd);
      rates(P, U, ns, rinv * (R(1.0) / scale), omegaP, omegaM);
      trt_emit_fast<R>(U, x, g, e0, ns, nd, omegaP, omegaM, U.sp_tfs, emit);
    } else {
      fluid_neq_fast<R>(sp, dp, delta, rho, ux, uy, uz, uu, e0, ns, nd);
      rates(P, U, ns, rinv, omegaP, omegaM);
      trt_emit_fast<R>(U, x, g, e0, ns, nd, omegaP, omegaM, U.sp_tf, emit);
    }
    return;
  }
  R e[Q];
#pragma unroll
  for (int i = 0; i < Q; ++i) e[i] = equilibrium<R, false>(i, delta, rho, ux, uy, uz, uu, R(0.0));
  R omegaP = U.omegaP0, omegaM = U.omegaM0;
  if (U.les_on) {
    R n[Q];
#pragma unroll
    for (int i = 0; i < Q; ++i) n[i] = g[i] - e[i];
    const R pxx = signed_sum<R>(n, [](int i) { return cx(i) * cx(i); });
    const R pyy = signed_sum<R>(n, [](int i) { return cy(i) * cy(i); });
    const R pzz = signed_sum<R>(n, [](int i) { return cz(i) * cz(i); });
    const R pxy = signed_sum<R>(n, [](int i) { return cx(i) * cy(i); });
    const R pxz = signed_sum<R>(n, [](int i) { return cx(i) * cz(i); });
    const R pyz = signed_sum<R>(n, [](int i) { return cy(i) * cz(i); });
    const R pp = pxx * pxx + pyy * pyy + pzz * pzz + R(2.0) * (pxy * pxy + pxz * pxz + pyz * pyz);
    const R qs = r_sqrt(R(2.0) * pp);
    const R tauT = R(0.5) * (U.tau0 + r_sqrt(U.tau0sq + U.c18 * qs / rho));
    omegaP = R(1.0) / tauT;
    omegaM = R(1.0) / (R(P.magic) / (R(1.0) / omegaP - R(0.5)) + R(0.5));
  }
  // Sponge weight (src/core/emit/ir.js:458-463): zero for x <= start, where
  // the blend a (1 - 0) + b 0 leaves every population unchanged.
  R sig2 = R(0.0);
  if (R(x) > U.sp_start) {
    const R sx = (R(x) - U.sp_start) / U.sp_len;
    const R sigma = sx < R(1.0) ? sx : R(1.0);
    sig2 = sigma * sigma;
  }
  // TRT per opposite pair (src/core/emit/ir.js:304-323), mix(a, b, t) = a (1 - t) + b t;
  // one branch per cell for the sponge, as in trt_emit_fast
  if (sig2 != R(0.0)) {
    const R oms = R(1.0) - sig2;
    emit(0, (g[0] - omegaP * (g[0] - e[0])) * oms + U.sp_t[0] * sig2);
#pragma unroll
    for (int i = 1; i < Q; i += 2) {
      const int j = i + 1;
      const R p = R(0.5) * ((g[i] + g[j]) - (e[i] + e[j]));
      const R m = R(0.5) * ((g[i] - g[j]) - (e[i] - e[j]));
      emit(i, (g[i] - omegaP * p - omegaM * m) * oms + U.sp_t[i] * sig2);
      emit(j, (g[j] - omegaP * p + omegaM * m) * oms + U.sp_t[j] * sig2);
    }
    return;
  }
  emit(0, g[0] - omegaP * (g[0] - e[0]));
#pragma unroll
  for (int i = 1; i < Q; i += 2) {
    const int j = i + 1;
    const R p = R(0.5) * ((g[i] + g[j]) - (e[i] + e[j]));
    const R m = R(0.5) * ((g[i] - g[j]) - (e[i] - e[j]));
    emit(i, g[i] - omegaP * p - omegaM * m);
    emit(j, g[j] - omegaP * p + omegaM * m);
  }
}

// ---------------------------------------------------------------- storage
// Population storage forms.  Arithmetic is float (or double for the fp64 reference form).
// kScaled: the stored value is the population times kScale (a power of two);
// ld_raw / st_raw move the stored value without the scale.
struct StF32 {
  static constexpr bool kSR = false;   // stores rounded to nearest
  using store_t = float;
  using real = float;
  static constexpr bool kScaled = false;
  static constexpr float kScale = 1.0f;
  static __device__ __forceinline__ float ld(const float* p) { return *p; }
  static __device__ __forceinline__ float ld_raw(const float* p) { return *p; }
  static __device__ __forceinline__ void st_raw(float* p, float v) { *p = v; }
  static __device__ __forceinline__ void st(float* p, float v) { *p = v; }
  static __device__ __forceinline__ float from_double(double v) { return (float)v; }
  // value from the aligned 32-bit word a pipelined copy brought in
  static __device__ __forceinline__ float from_word(uint32_t w, uint32_t) { return __uint_as_float(w); }
};
struct StF64 {
  static constexpr bool kSR = false;   // stores rounded to nearest
  using store_t = double;
  using real = double;
  static constexpr bool kScaled = false;
  static constexpr double kScale = 1.0;
  static __device__ __forceinline__ double ld(const double* p) { return *p; }
  static __device__ __forceinline__ double ld_raw(const double* p) { return *p; }
  static __device__ __forceinline__ void st_raw(double* p, double v) { *p = v; }
  static __device__ __forceinline__ void st(double* p, double v) { *p = v; }
  static __device__ __forceinline__ double from_double(double v) { return v; }
};
// fp16 holding g_i * 2^10: the scale lifts the ~1e-5 free-stream deviations
// out of the fp16 subnormal range.  Scaling by a power of two is exact.
struct StF16S {
  static constexpr bool kSR = false;   // stores rounded to nearest
  using store_t = uint16_t;
  using real = float;
  static constexpr bool kScaled = true;
  static constexpr float kScale = 1024.0f;
  static __device__ __forceinline__ float ld(const uint16_t* p) {
    return __half2float(__ushort_as_half(*p)) * (1.0f / 1024.0f);
  }
  static __device__ __forceinline__ float ld_raw(const uint16_t* p) { return __half2float(__ushort_as_half(*p)); }
  static __device__ __forceinline__ void st_raw(uint16_t* p, float v) { *p = __half_as_ushort(__float2half_rn(v)); }
  static __device__ __forceinline__ float from_word(uint32_t w, uint32_t shift) {
    return __half2float(__ushort_as_half((unsigned short)(w >> shift))) * (1.0f / 1024.0f);
  }
  static __device__ __forceinline__ void st(uint16_t* p, float v) {
    *p = __half_as_ushort(__float2half_rn(v * 1024.0f));
  }
  static __device__ __forceinline__ float from_double(double v) { return (float)v; }
};
struct StBF16S {
  static constexpr bool kSR = false;   // stores rounded to nearest
  using store_t = uint16_t;
  using real = float;
  static constexpr bool kScaled = false;
  static constexpr float kScale = 1.0f;
  static __device__ __forceinline__ float ld(const uint16_t* p) {
    return __bfloat162float(__ushort_as_bfloat16(*p));
  }
  static __device__ __forceinline__ float ld_raw(const uint16_t* p) { return ld(p); }
  static __device__ __forceinline__ void st_raw(uint16_t* p, float v) { *p = __bfloat16_as_ushort(__float2bfloat16_rn(v)); }
  static __device__ __forceinline__ float from_word(uint32_t w, uint32_t shift) {
    return __bfloat162float(__ushort_as_bfloat16((unsigned short)(w >> shift)));
  }
  static __device__ __forceinline__ void st(uint16_t* p, float v) {
    *p = __bfloat16_as_ushort(__float2bfloat16_rn(v));
  }
  static __device__ __forceinline__ float from_double(double v) { return (float)v; }
};

// Stochastic rounding of the 16-bit stores (LBM_F16SR, LBM_BF16SR).  A
// stored value v (fp32, in the stored scale) keeps its top bits; the dropped
// low bits B (13 for fp16, 16 for bf16) round it up in magnitude with
// probability B / 2^bits: r, uniform on [0, 2^bits), is added to the fp32 bit
// pattern (sign and magnitude, so the carry goes into the magnitude for
// either sign) and the result is truncated (round toward zero).  r comes from
// a hash of the colliding cell, the step count and the direction, so a run is
// reproducible and the oracle restates it bit for bit.
__host__ __device__ __forceinline__ uint32_t sr_seed(int64_t step) {
  return (uint32_t)((uint64_t)step * 0x632BE5ABull);
}
__host__ __device__ __forceinline__ uint32_t sr_cell_hash(uint32_t cell, uint32_t seed) {
  uint32_t h = cell * 0x9E3779B1u + seed;
  h ^= h >> 16;
  h *= 0x7FEB352Du;
  h ^= h >> 15;
  h *= 0x846CA68Bu;
  h ^= h >> 16;
  return h;
}
// per direction i: an odd multiplier; r = top `bits` bits of h * sr_mult(i)
__host__ __device__ constexpr uint32_t sr_mult(int i) { return 0x9E3779B1u * (2u * (uint32_t)i + 1u); }

struct StF16SR : StF16S {
  static constexpr bool kSR = true;
  static constexpr int kSRBits = 13;
  // vs: the value times 2^10 (the stored scale)
  static __device__ __forceinline__ void st_sr(uint16_t* p, float vs, uint32_t r) {
    *p = __half_as_ushort(__float2half_rz(__uint_as_float(__float_as_uint(vs) + r)));
  }
};
struct StBF16SR : StBF16S {
  static constexpr bool kSR = true;
  static constexpr int kSRBits = 16;
  static __device__ __forceinline__ void st_sr(uint16_t* p, float vs, uint32_t r) {
    *p = __bfloat16_as_ushort(__float2bfloat16_rz(__uint_as_float(__float_as_uint(vs) + r)));
  }
};

// ------------------------------------------------------------- link words
// Per-cell 32-bit word the in-place kernel reads instead of 18 neighbour
// types (the reference gathers tipo[] for every direction,
// src/core/emit/ir.js:176-186):
//   bits 0..17  bit (k-1): the upstream cell x - c_k is solid (1, 4 or 7)
//   bits 18..20 the cell's own class
//   bit 21      slow path: some upstream solid is SOLIDO_MOVEL, or the
//               upstream solids mix SOLIDO and PAREDE (read tipo[] per link)
//   bit 22      every upstream solid is SOLIDO (the body): all bounce-back
//               links count in the force
constexpr uint32_t LINK_CLASS_SHIFT = 18;
constexpr uint32_t LINK_SLOW = 1u << 21;
constexpr uint32_t LINK_BODY = 1u << 22;

}  // namespace lbm

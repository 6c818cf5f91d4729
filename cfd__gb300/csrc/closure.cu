// closure.cu — training and evaluation of the learned eddy-viscosity closure
// (include/lbm_closure.h).
//
// Training is fp32 on the CUDA cores, deterministic:
//   k_sample   minibatch indices from a counter-based hash (splitmix64)
//   k_fwd_bwd  one thread per sample: forward, loss, backward; the block's
//              activations go to shared memory and its threads then form
//              the weight-gradient sums over the block's samples (one entry
//              per thread at a time), written as per-block partials
//   k_sum      fixed-order sum of the partials -> gradient, loss
//   k_adam     Adam with bias correction, one thread per parameter
// Evaluation uses the tensor-core MLP the fused step uses (closure_mlp.cuh).
#include <cuda_runtime.h>

#include <algorithm>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/lbm.h"
#include "../../include/lbm_closure.h"
#include "closure_mlp.cuh"

extern "C" int lbm_internal_fail(int code, const char* msg);

using namespace lbm;

namespace {

constexpr int NI = CLOSURE_IN, NH = CLOSURE_H;
constexpr int NP = NH * NI + NH + NH * NH + NH + NH + 1;   // 1313
constexpr int OW1 = 0, OB1 = OW1 + NH * NI, OW2 = OB1 + NH, OB2 = OW2 + NH * NH, OW3 = OB2 + NH, OB3 = OW3 + NH;
constexpr int TB = 64;   // samples per training block

static_assert(sizeof(closure_weights) == sizeof(float) * (NP + 4 * NI + 3), "closure_weights layout");

__device__ __forceinline__ float softplus(float y) { return y > 20.0f ? y : log1pf(expf(y)); }
__device__ __forceinline__ float sigmoid(float y) { return 1.0f / (1.0f + expf(-y)); }

__device__ __forceinline__ unsigned long long splitmix64(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__global__ void k_sample(int* idx, int b, long long m, unsigned long long seed, int step) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < b) idx[i] = (int)(splitmix64(seed ^ ((unsigned long long)step << 32) ^ (unsigned long long)i) % (unsigned long long)m);
}

// feats: m x 6 raw; norm: mean[6], inv_std[6], nu_scale; P: parameters.
__global__ void __launch_bounds__(TB) k_fwd_bwd(const float* __restrict__ feats, const float* __restrict__ target,
                                                const int* __restrict__ idx, int nb_samples, long long m,
                                                const float* __restrict__ P, const float* __restrict__ norm,
                                                float inv_batch, float* __restrict__ gpart,
                                                float* __restrict__ lpart) {
  __shared__ float W[NP];
  __shared__ float X[TB][NI], H1[TB][NH], DH1[TB][NH], H2[TB][NH], DY[TB];
  __shared__ float L[TB];
  const int tid = threadIdx.x;
  for (int e = tid; e < NP; e += TB) W[e] = P[e];
  __syncthreads();
  const int s = blockIdx.x * TB + tid;
  const bool valid = s < nb_samples;
  float x[NI], h1[NH], h2[NH];
  float loss = 0.0f, dy = 0.0f;
  if (valid) {
    const long long i = idx ? (long long)idx[s] : (long long)s;
#pragma unroll
    for (int a = 0; a < NI; ++a) x[a] = (feats[i * NI + a] - norm[a]) * norm[NI + a];
#pragma unroll
    for (int j = 0; j < NH; ++j) {
      float v = W[OB1 + j];
#pragma unroll
      for (int a = 0; a < NI; ++a) v = fmaf(W[OW1 + j * NI + a], x[a], v);
      h1[j] = fmaxf(v, 0.0f);
    }
#pragma unroll 4
    for (int k = 0; k < NH; ++k) {
      float v = W[OB2 + k];
#pragma unroll
      for (int j = 0; j < NH; ++j) v = fmaf(W[OW2 + k * NH + j], h1[j], v);
      h2[k] = fmaxf(v, 0.0f);
    }
    float y = W[OB3];
#pragma unroll
    for (int k = 0; k < NH; ++k) y = fmaf(W[OW3 + k], h2[k], y);
    const float scale = norm[2 * NI];
    const float r = (scale * softplus(y) - target[i]) / scale;
    loss = r * r;
    dy = 2.0f * r * sigmoid(y) * inv_batch;
  } else {
#pragma unroll
    for (int a = 0; a < NI; ++a) x[a] = 0.0f;
#pragma unroll
    for (int j = 0; j < NH; ++j) { h1[j] = 0.0f; h2[j] = 0.0f; }
  }
#pragma unroll
  for (int a = 0; a < NI; ++a) X[tid][a] = x[a];
#pragma unroll
  for (int j = 0; j < NH; ++j) { H1[tid][j] = h1[j]; H2[tid][j] = h2[j]; }
  DY[tid] = dy;
  L[tid] = loss;
  // dh1_j = sum_k W2[k][j] dh2_k relu'(h1_j), dh2_k = dy W3[k] relu'(h2_k)
#pragma unroll 4
  for (int j = 0; j < NH; ++j) {
    float v = 0.0f;
#pragma unroll
    for (int k = 0; k < NH; ++k) v = fmaf(W[OW2 + k * NH + j], h2[k] > 0.0f ? dy * W[OW3 + k] : 0.0f, v);
    DH1[tid][j] = h1[j] > 0.0f ? v : 0.0f;
  }
  __syncthreads();
  // weight-gradient sums over this block's samples
  float* out = gpart + (size_t)blockIdx.x * NP;
  for (int e = tid; e < NP; e += TB) {
    float acc = 0.0f;
    if (e < OB1) {
      const int j = e / NI, a = e % NI;
      for (int q = 0; q < TB; ++q) acc = fmaf(DH1[q][j], X[q][a], acc);
    } else if (e < OW2) {
      const int j = e - OB1;
      for (int q = 0; q < TB; ++q) acc += DH1[q][j];
    } else if (e < OB2) {
      const int k = (e - OW2) / NH, j = (e - OW2) % NH;
      const float w3 = W[OW3 + k];
      for (int q = 0; q < TB; ++q) acc = fmaf(H2[q][k] > 0.0f ? DY[q] * w3 : 0.0f, H1[q][j], acc);
    } else if (e < OW3) {
      const int k = e - OB2;
      const float w3 = W[OW3 + k];
      for (int q = 0; q < TB; ++q) acc += H2[q][k] > 0.0f ? DY[q] * w3 : 0.0f;
    } else if (e < OB3) {
      const int k = e - OW3;
      for (int q = 0; q < TB; ++q) acc = fmaf(DY[q], H2[q][k], acc);
    } else {
      for (int q = 0; q < TB; ++q) acc += DY[q];
    }
    out[e] = acc;
  }
  if (tid == 0) {
    float a = 0.0f;
    for (int q = 0; q < TB; ++q) a += L[q];
    lpart[blockIdx.x] = a;
  }
}

// Fixed-order sums: grad[e] = sum_b gpart[b][e]; loss = sum_b lpart[b] / n
__global__ void k_sum(const float* __restrict__ gpart, const float* __restrict__ lpart, int nblk, float inv_n,
                      float* __restrict__ grad, float* __restrict__ loss_out) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < NP) {
    float acc = 0.0f;
    for (int b = 0; b < nblk; ++b) acc += gpart[(size_t)b * NP + e];
    grad[e] = acc;
  }
  if (e == 0 && loss_out) {
    float a = 0.0f;
    for (int b = 0; b < nblk; ++b) a += lpart[b];
    *loss_out = a * inv_n;
  }
}

__global__ void k_adam(float* __restrict__ P, float* __restrict__ M, float* __restrict__ V,
                       const float* __restrict__ grad, float lr, float b1, float b2, float eps, float c1, float c2) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= NP) return;
  const float g = grad[e];
  const float m = b1 * M[e] + (1.0f - b1) * g;
  const float v = b2 * V[e] + (1.0f - b2) * g * g;
  M[e] = m;
  V[e] = v;
  P[e] -= lr * (m * c1) / (sqrtf(v * c2) + eps);
}

// nu_t of feature rows through the step's warp engine (fragments read from
// global memory, as in the fused step).
__global__ void __launch_bounds__(128) k_eval(const float* __restrict__ feats, long long m,
                                              const MlpFrag* __restrict__ F, float* __restrict__ nu) {
  const long long i = (long long)blockIdx.x * 128 + threadIdx.x;
  float x[6];
#pragma unroll
  for (int a = 0; a < 6; ++a) x[a] = i < m ? feats[i * 6 + a] : 0.0f;
  const bool inside = closure_in_range(*F, x);
#pragma unroll
  for (int a = 0; a < 6; ++a) x[a] = i < m ? (x[a] - F->mean[a]) * F->inv_std[a] : 0.0f;
  const float y = warp_mlp(*F, x);
  if (i < m) nu[i] = inside ? closure_nu(*F, y) : __int_as_float(0x7fc00000);
}

// The same through the CTA-wide tcgen05 MLP: persistent CTAs walk tiles of
// 128 rows (set up once per CTA, closure_tc.cuh).
__global__ void __launch_bounds__(128) k_eval_tc(const float* __restrict__ feats, long long m,
                                                 const MlpFrag* __restrict__ F, float* __restrict__ nu,
                                                 unsigned* __restrict__ err) {
  __shared__ TcPersist S;
  const int tid = threadIdx.x;
  const uint32_t tmem = tcp_setup(S, F->tcb, F->w3b, tid);
  uint32_t phase = 0;
  bool dead = false;
  const long long ntiles = (m + TC_ROWS - 1) / TC_ROWS;
  for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const long long i = t * TC_ROWS + tid;
    float x[6];
#pragma unroll
    for (int a = 0; a < 6; ++a) x[a] = i < m ? feats[i * 6 + a] : 0.0f;
    const bool inside = closure_in_range(*F, x);
#pragma unroll
    for (int a = 0; a < 6; ++a) x[a] = i < m ? (x[a] - F->mean[a]) * F->inv_std[a] : 0.0f;
    const float y = tcp_mlp(S, tmem, tid, x, phase, dead);
    if (i < m) nu[i] = inside ? closure_nu(*F, y) : __int_as_float(0x7fc00000);
  }
  tcp_teardown(S, tmem, tid, phase, dead);
  if (tid == 0 && S.err) atomicOr(err, 1u);
}

// ---- training samples from a fine run ----
// Pass 1: per coarse cell, the 2x2x2 block means of u and delta of the fine
// macros (x, y, z, delta per fine cell) and the residual stress
// tau_ab = <(u_a - <u_a>)(u_b - <u_b>)> = <u_a u_b> - <u_a><u_b>;
// out[11]: u(3), delta, tau(xx, yy, zz, xy, xz, yz), 1 if all eight fine
// cells are FLUIDO else 0.
__global__ void k_filter(const float4* __restrict__ mac, const uint8_t* __restrict__ tipo, int nx, int ny, int nz,
                         float* __restrict__ out) {
  const int cx_ = nx / 2, cy_ = ny / 2, cz_ = nz / 2;
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nc = (long long)cx_ * cy_ * cz_;
  if (c >= nc) return;
  const int X = (int)(c % cx_), Y = (int)((c / cx_) % cy_), Z = (int)(c / ((long long)cx_ * cy_));
  // block values, then the mean and the centred second moments (the
  // residual stress is a small difference of large terms: centring first
  // keeps it accurate in fp32)
  float4 v[8];
  bool ok = true;
  for (int q = 0; q < 8; ++q) {
    const int dx = q & 1, dy = (q >> 1) & 1, dz = q >> 2;
    const long long f = ((long long)(2 * Z + dz) * ny + (2 * Y + dy)) * nx + (2 * X + dx);
    ok = ok && tipo[f] == 0;
    v[q] = mac[f];
  }
  float s[10];
  float mx = 0.f, my = 0.f, mz = 0.f, mw = 0.f;
  for (int q = 0; q < 8; ++q) { mx += v[q].x; my += v[q].y; mz += v[q].z; mw += v[q].w; }
  mx *= 0.125f; my *= 0.125f; mz *= 0.125f; mw *= 0.125f;
  s[0] = mx; s[1] = my; s[2] = mz; s[3] = mw;
  for (int a = 4; a < 10; ++a) s[a] = 0.f;
  for (int q = 0; q < 8; ++q) {
    const float ax = v[q].x - mx, ay = v[q].y - my, az = v[q].z - mz;
    s[4] += ax * ax; s[5] += ay * ay; s[6] += az * az;
    s[7] += ax * ay; s[8] += ax * az; s[9] += ay * az;
  }
  for (int a = 4; a < 10; ++a) s[a] *= 0.125f;
  float* o = out + c * 11;
  for (int a = 0; a < 10; ++a) o[a] = s[a];
  o[10] = ok ? 1.0f : 0.0f;
}

// Pass 2: strain rate of the filtered velocity by central differences on the
// coarse grid, residual stress tau_ab = <u_a u_b> - <u_a><u_b>, target
// nu_t = max(0, -tau^d:S / (2 S:S)) (0 where |S| < s_min), and the features of the coarse
// non-equilibrium stress Pi = -(2/3) rho (tau0c + 3 nu_t) S.  Rows for coarse
// cells x0 <= X < x1 (all Y, Z), X fastest; target NaN where the cell or a
// face neighbour is not fluid.
__global__ void k_samples(const float* __restrict__ fil, int cx_, int cy_, int cz_, float tau0c, float omega0c,
                          float s_min, int x0, int x1, float* __restrict__ feats, float* __restrict__ target) {
  const int wx = x1 - x0;
  const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nr = (long long)wx * cy_ * cz_;
  if (r >= nr) return;
  const int X = x0 + (int)(r % wx), Y = (int)((r / wx) % cy_), Z = (int)(r / ((long long)wx * cy_));
  float* fo = feats + r * 6;
  auto at = [&](int x, int y, int z) { return fil + (((long long)z * cy_ + y) * cx_ + x) * 11; };
  bool ok = X > 0 && X < cx_ - 1 && Y > 0 && Y < cy_ - 1 && Z > 0 && Z < cz_ - 1;
  if (ok) {
    ok = at(X, Y, Z)[10] != 0.f && at(X - 1, Y, Z)[10] != 0.f && at(X + 1, Y, Z)[10] != 0.f &&
         at(X, Y - 1, Z)[10] != 0.f && at(X, Y + 1, Z)[10] != 0.f && at(X, Y, Z - 1)[10] != 0.f &&
         at(X, Y, Z + 1)[10] != 0.f;
  }
  if (!ok) {
    for (int a = 0; a < 6; ++a) fo[a] = 0.f;
    target[r] = __int_as_float(0x7fc00000);
    return;
  }
  // G[a][b] = d u_b / d x_a
  float G[3][3];
  const float* xm = at(X - 1, Y, Z); const float* xp = at(X + 1, Y, Z);
  const float* ym = at(X, Y - 1, Z); const float* yp = at(X, Y + 1, Z);
  const float* zm = at(X, Y, Z - 1); const float* zp = at(X, Y, Z + 1);
  for (int b = 0; b < 3; ++b) {
    G[0][b] = 0.5f * (xp[b] - xm[b]);
    G[1][b] = 0.5f * (yp[b] - ym[b]);
    G[2][b] = 0.5f * (zp[b] - zm[b]);
  }
  const float sxx = G[0][0], syy = G[1][1], szz = G[2][2];
  const float sxy = 0.5f * (G[0][1] + G[1][0]), sxz = 0.5f * (G[0][2] + G[2][0]), syz = 0.5f * (G[1][2] + G[2][1]);
  const float* c = at(X, Y, Z);
  const float txx = c[4], tyy = c[5], tzz = c[6], txy = c[7], txz = c[8], tyz = c[9];
  const float tr3 = (txx + tyy + tzz) * (1.0f / 3.0f);
  const float ss = sxx * sxx + syy * syy + szz * szz + 2.0f * (sxy * sxy + sxz * sxz + syz * syz);
  const float ts = (txx - tr3) * sxx + (tyy - tr3) * syy + (tzz - tr3) * szz +
                   2.0f * (txy * sxy + txz * sxz + tyz * syz);
  // |S| = sqrt(2 S:S) below s_min: no eddy viscosity (the ratio is
  // ill-conditioned there and the dissipation nu_t |S|^2 negligible)
  const float nut = (2.0f * ss > s_min * s_min && ss > 1e-30f) ? fmaxf(0.0f, -ts / (2.0f * ss)) : 0.0f;
  const float delta = c[3], rho = 1.0f + delta;
  const float k = -(2.0f / 3.0f) * rho * (tau0c + 3.0f * nut);
  float f[6];
  closure_features(k * sxx, k * syy, k * szz, k * sxy, k * sxz, k * syz, 1.0f / rho, delta, f);
  f[4] = omega0c;
  for (int a = 0; a < 6; ++a) fo[a] = f[a];
  target[r] = nut;
}

int cfail(int code, const std::string& m) { return lbm_internal_fail(code, m.c_str()); }

#define CCK(call, what)                                                                                   \
  do {                                                                                                    \
    cudaError_t _e = (call);                                                                              \
    if (_e != cudaSuccess) {                                                                              \
      cudaGetLastError();                                                                                 \
      return cfail(_e == cudaErrorMemoryAllocation ? LBM_ENOMEM : LBM_ECUDA,                              \
                   std::string(what) + ": " + cudaGetErrorString(_e));                                    \
    }                                                                                                     \
  } while (0)

struct Mem {
  std::vector<void*> p;
  ~Mem() {
    for (void* q : p) cudaFree(q);
  }
  template <typename T>
  cudaError_t get(T** out, size_t bytes) {
    cudaError_t e = cudaMalloc((void**)out, bytes);
    if (e == cudaSuccess) p.push_back(*out);
    return e;
  }
};

uint16_t f32_to_bf16(float f) {   // round to nearest even
  uint32_t x;
  memcpy(&x, &f, 4);
  if ((x & 0x7f800000u) == 0x7f800000u && (x & 0x7fffffu)) return (uint16_t)((x >> 16) | 0x40u);
  x += 0x7fffu + ((x >> 16) & 1u);
  return (uint16_t)(x >> 16);
}

uint32_t pack2(float lo, float hi) { return (uint32_t)f32_to_bf16(lo) | ((uint32_t)f32_to_bf16(hi) << 16); }

unsigned long long splitmix64_h(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

}  // namespace

namespace lbm {

// Weights -> tensor-core fragments (see closure_mlp.cuh for the layout).
void closure_pack(const closure_weights* w, MlpFrag* F) {
  memset(F, 0, sizeof *F);
  for (int lane = 0; lane < 32; ++lane) {
    const int g = lane >> 2, t = lane & 3;
    for (int nt = 0; nt < 4; ++nt) {
      const int n = nt * 8 + g;
      auto w1 = [&](int k) { return k < NI ? w->w1[n * NI + k] : 0.0f; };
      F->w1[nt][lane] = make_uint2(pack2(w1(2 * t), w1(2 * t + 1)), pack2(w1(2 * t + 8), w1(2 * t + 9)));
      for (int kt = 0; kt < 2; ++kt) {
        const int k = kt * 16 + 2 * t;
        F->w2[nt][kt][lane] = make_uint2(pack2(w->w2[n * NH + k], w->w2[n * NH + k + 1]),
                                         pack2(w->w2[n * NH + k + 8], w->w2[n * NH + k + 9]));
      }
    }
    for (int kt = 0; kt < 2; ++kt) {
      const int k = kt * 16 + 2 * t;
      const bool col0 = g == 0;   // output column 0 only
      F->w3[kt][lane] = make_uint2(col0 ? pack2(w->w3[k], w->w3[k + 1]) : 0u,
                                   col0 ? pack2(w->w3[k + 8], w->w3[k + 9]) : 0u);
    }
  }
  for (int j = 0; j < NH; ++j) { F->b1[j] = w->b1[j]; F->b2[j] = w->b2[j]; }
  F->b3 = w->b3;
  // tcgen05 B operands, K-major core-matrix layout, bias in column K-slot kb
  uint8_t* tb = reinterpret_cast<uint8_t*>(F->tcb);
  auto put = [&](uint32_t base, int n, int k, int K, float v) {
    const uint16_t h = f32_to_bf16(v);
    memcpy(tb + base + tc_off(n, k, K), &h, 2);
  };
  for (int n = 0; n < NH; ++n) {
    for (int k = 0; k < NI; ++k) put(0, n, k, TC_K1, w->w1[n * NI + k]);
    put(0, n, NI, TC_K1, w->b1[n]);
    for (int k = 0; k < NH; ++k) put(TC_B1_BYTES, n, k, TC_K2, w->w2[n * NH + k]);
    put(TC_B1_BYTES, n, NH, TC_K2, w->b2[n]);
  }
  auto bf16f = [](float v) {
    const uint32_t u = (uint32_t)f32_to_bf16(v) << 16;
    float f;
    memcpy(&f, &u, 4);
    return f;
  };
  for (int k = 0; k < NH; ++k) F->w3b[k] = bf16f(w->w3[k]);
  F->w3b[NH] = bf16f(w->b3);
  for (int a = 0; a < NI; ++a) {
    F->mean[a] = w->mean[a];
    F->inv_std[a] = w->std[a] != 0.0f ? 1.0f / w->std[a] : 0.0f;
  }
  F->nu_scale = w->nu_scale;
  F->nu_max = w->nu_max;
  for (int a = 0; a < NI; ++a) { F->lo[a] = w->lo[a]; F->hi[a] = w->hi[a]; }
  F->coef = w->coef != 0;
}

// Rows of closure_samples (see include/lbm_closure.h); scratch is allocated
// here.  Returns a CUDA error or cudaSuccess.
cudaError_t closure_samples_launch(const float4* mac, const uint8_t* tipo, int nx, int ny, int nz, float tau0c,
                                   float s_min, int x0, int x1, float* feats_dev, float* target_dev, cudaStream_t s) {
  const int cx_ = nx / 2, cy_ = ny / 2, cz_ = nz / 2;
  const long long nc = (long long)cx_ * cy_ * cz_;
  float* fil = nullptr;
  cudaError_t e = cudaMalloc(&fil, sizeof(float) * 11 * (size_t)nc);
  if (e != cudaSuccess) return e;
  k_filter<<<(unsigned)((nc + 255) / 256), 256, 0, s>>>(mac, tipo, nx, ny, nz, fil);
  const long long nr = (long long)(x1 - x0) * cy_ * cz_;
  k_samples<<<(unsigned)((nr + 255) / 256), 256, 0, s>>>(fil, cx_, cy_, cz_, tau0c, 1.0f / tau0c, s_min, x0, x1,
                                                       feats_dev, target_dev);
  e = cudaGetLastError();
  cudaError_t e2 = cudaStreamSynchronize(s);
  cudaFree(fil);
  return e != cudaSuccess ? e : e2;
}

}  // namespace lbm

extern "C" {

int closure_grad(const float* feats, const float* target, size_t m, const closure_weights* w, float* loss,
                 float* grad) {
  if (!feats || !target || !w || !grad || m == 0) return cfail(LBM_EINVAL, "null argument or no samples");
  if (m > (1u << 30)) return cfail(LBM_EINVAL, "too many samples");
  Mem mem;
  float *d_f, *d_t, *d_p, *d_norm, *d_gp, *d_lp, *d_g, *d_l;
  const int nblk = (int)((m + TB - 1) / TB);
  CCK(mem.get(&d_f, sizeof(float) * m * NI), "features");
  CCK(mem.get(&d_t, sizeof(float) * m), "targets");
  CCK(mem.get(&d_p, sizeof(float) * NP), "parameters");
  CCK(mem.get(&d_norm, sizeof(float) * (2 * NI + 1)), "normalisation");
  CCK(mem.get(&d_gp, sizeof(float) * NP * (size_t)nblk), "gradient partials");
  CCK(mem.get(&d_lp, sizeof(float) * nblk), "loss partials");
  CCK(mem.get(&d_g, sizeof(float) * NP), "gradient");
  CCK(mem.get(&d_l, sizeof(float)), "loss");
  float norm[2 * NI + 1];
  for (int a = 0; a < NI; ++a) { norm[a] = w->mean[a]; norm[NI + a] = w->std[a] != 0.0f ? 1.0f / w->std[a] : 0.0f; }
  norm[2 * NI] = w->nu_scale;
  CCK(cudaMemcpy(d_f, feats, sizeof(float) * m * NI, cudaMemcpyHostToDevice), "upload");
  CCK(cudaMemcpy(d_t, target, sizeof(float) * m, cudaMemcpyHostToDevice), "upload");
  CCK(cudaMemcpy(d_p, w->w1, sizeof(float) * NP, cudaMemcpyHostToDevice), "upload");
  CCK(cudaMemcpy(d_norm, norm, sizeof norm, cudaMemcpyHostToDevice), "upload");
  k_fwd_bwd<<<nblk, TB>>>(d_f, d_t, nullptr, (int)m, (long long)m, d_p, d_norm, 1.0f / (float)m, d_gp, d_lp);
  k_sum<<<(NP + 127) / 128, 128>>>(d_gp, d_lp, nblk, 1.0f / (float)m, d_g, d_l);
  CCK(cudaGetLastError(), "gradient kernels");
  CCK(cudaMemcpy(grad, d_g, sizeof(float) * NP, cudaMemcpyDeviceToHost), "download");
  if (loss) CCK(cudaMemcpy(loss, d_l, sizeof(float), cudaMemcpyDeviceToHost), "download");
  return LBM_OK;
}

int closure_train(const float* feats, const float* target, size_t m, const closure_cfg* cfg, closure_weights* w,
                  float* loss_out) {
  if (!feats || !target || !cfg || !w || m == 0) return cfail(LBM_EINVAL, "null argument or no samples");
  if (cfg->steps < 0 || cfg->batch < 1 || cfg->batch > (1 << 24)) return cfail(LBM_EINVAL, "bad steps or batch");
  if (m > (1u << 30)) return cfail(LBM_EINVAL, "too many samples");
  if (cfg->init) {
    // He-uniform hidden layers, small output layer, zero biases
    unsigned long long s = cfg->seed;
    auto uni = [&](float a) {
      s = splitmix64_h(s);
      return a * (2.0f * (float)((s >> 11) * (1.0 / 9007199254740992.0)) - 1.0f);
    };
    for (int e = 0; e < NH * NI; ++e) w->w1[e] = uni(std::sqrt(6.0f / NI));
    for (int e = 0; e < NH * NH; ++e) w->w2[e] = uni(std::sqrt(6.0f / NH));
    for (int e = 0; e < NH; ++e) w->w3[e] = uni(std::sqrt(6.0f / NH) * 0.1f);
    for (int e = 0; e < NH; ++e) { w->b1[e] = 0.0f; w->b2[e] = 0.0f; }
    w->b3 = 0.0f;
  }
  Mem mem;
  const int B = cfg->batch;
  const int nblk = (B + TB - 1) / TB;
  float *d_f, *d_t, *d_p, *d_m, *d_v, *d_norm, *d_gp, *d_lp, *d_g, *d_loss;
  int* d_idx;
  CCK(mem.get(&d_f, sizeof(float) * m * NI), "features");
  CCK(mem.get(&d_t, sizeof(float) * m), "targets");
  CCK(mem.get(&d_p, sizeof(float) * NP), "parameters");
  CCK(mem.get(&d_m, sizeof(float) * NP), "adam m");
  CCK(mem.get(&d_v, sizeof(float) * NP), "adam v");
  CCK(mem.get(&d_norm, sizeof(float) * (2 * NI + 1)), "normalisation");
  CCK(mem.get(&d_gp, sizeof(float) * NP * (size_t)nblk), "gradient partials");
  CCK(mem.get(&d_lp, sizeof(float) * nblk), "loss partials");
  CCK(mem.get(&d_g, sizeof(float) * NP), "gradient");
  CCK(mem.get(&d_loss, sizeof(float) * std::max(1, cfg->steps)), "loss history");
  CCK(mem.get(&d_idx, sizeof(int) * B), "minibatch");
  float norm[2 * NI + 1];
  for (int a = 0; a < NI; ++a) { norm[a] = w->mean[a]; norm[NI + a] = w->std[a] != 0.0f ? 1.0f / w->std[a] : 0.0f; }
  norm[2 * NI] = w->nu_scale;
  CCK(cudaMemcpy(d_f, feats, sizeof(float) * m * NI, cudaMemcpyHostToDevice), "upload");
  CCK(cudaMemcpy(d_t, target, sizeof(float) * m, cudaMemcpyHostToDevice), "upload");
  CCK(cudaMemcpy(d_p, w->w1, sizeof(float) * NP, cudaMemcpyHostToDevice), "upload");
  CCK(cudaMemcpy(d_norm, norm, sizeof norm, cudaMemcpyHostToDevice), "upload");
  CCK(cudaMemset(d_m, 0, sizeof(float) * NP), "clear");
  CCK(cudaMemset(d_v, 0, sizeof(float) * NP), "clear");
  double b1t = 1.0, b2t = 1.0;
  for (int step = 0; step < cfg->steps; ++step) {
    k_sample<<<(B + 255) / 256, 256>>>(d_idx, B, (long long)m, cfg->seed, step);
    k_fwd_bwd<<<nblk, TB>>>(d_f, d_t, d_idx, B, (long long)m, d_p, d_norm, 1.0f / (float)B, d_gp, d_lp);
    k_sum<<<(NP + 127) / 128, 128>>>(d_gp, d_lp, nblk, 1.0f / (float)B, d_g, d_loss + step);
    b1t *= cfg->beta1;
    b2t *= cfg->beta2;
    k_adam<<<(NP + 127) / 128, 128>>>(d_p, d_m, d_v, d_g, cfg->lr, cfg->beta1, cfg->beta2, cfg->eps,
                                      (float)(1.0 / (1.0 - b1t)), (float)(1.0 / (1.0 - b2t)));
  }
  CCK(cudaGetLastError(), "training kernels");
  CCK(cudaMemcpy(w->w1, d_p, sizeof(float) * NP, cudaMemcpyDeviceToHost), "download");
  if (loss_out && cfg->steps > 0)
    CCK(cudaMemcpy(loss_out, d_loss, sizeof(float) * cfg->steps, cudaMemcpyDeviceToHost), "download");
  return LBM_OK;
}

int closure_eval(const closure_weights* w, const float* feats, size_t m, int engine, float* nu_out) {
  if (!w || !feats || !nu_out || m == 0) return cfail(LBM_EINVAL, "null argument or no samples");
  if (engine != 0 && engine != 1) return cfail(LBM_EINVAL, "engine must be 0 or 1");
  MlpFrag F;
  closure_pack(w, &F);
  Mem mem;
  float *d_f, *d_nu;
  MlpFrag* d_F;
  unsigned* d_err;
  CCK(mem.get(&d_f, sizeof(float) * m * NI), "features");
  CCK(mem.get(&d_nu, sizeof(float) * m), "output");
  CCK(mem.get(&d_F, sizeof(MlpFrag)), "fragments");
  CCK(mem.get(&d_err, sizeof(unsigned)), "error flag");
  CCK(cudaMemcpy(d_f, feats, sizeof(float) * m * NI, cudaMemcpyHostToDevice), "upload");
  CCK(cudaMemcpy(d_F, &F, sizeof F, cudaMemcpyHostToDevice), "upload");
  CCK(cudaMemset(d_err, 0, sizeof(unsigned)), "clear");
  if (engine == 1) {
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long tiles = ((long long)m + TC_ROWS - 1) / TC_ROWS;
    const unsigned grid = (unsigned)std::max<long long>(1, std::min<long long>(tiles, 4LL * sms));
    k_eval_tc<<<grid, TC_ROWS>>>(d_f, (long long)m, d_F, d_nu, d_err);
  }
  else k_eval<<<(unsigned)((m + 127) / 128), 128>>>(d_f, (long long)m, d_F, d_nu);
  CCK(cudaGetLastError(), "eval kernel");
  unsigned err = 0;
  CCK(cudaMemcpy(&err, d_err, sizeof err, cudaMemcpyDeviceToHost), "download");
  if (err) return cfail(LBM_ETIMEDOUT, "tensor-core MLP: an mbarrier wait gave up");
  CCK(cudaMemcpy(nu_out, d_nu, sizeof(float) * m, cudaMemcpyDeviceToHost), "download");
  return LBM_OK;
}

}  // extern "C"

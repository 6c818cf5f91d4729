// vis.cu — visualisation compute on headless device buffers
// (include/lbm_vis.h): the smoke volume's advection step and the streak
// particles, reading a solver context's macros and cell types.
//
// Built with -fmad=false: every operation is rounded as written, which is
// what the oracle (oracle/vis_oracle.py) restates.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdio>
#include <string>

#include "../../include/lbm.h"
#include "../../include/lbm_vis.h"
#include "lbm_kernels.cuh"

extern "C" int lbm_internal_fail(int code, const char* msg);

using namespace lbm;

struct vis_fumaca {
  lbm_ctx* ctx;
  int nx, ny, nz;
  int64_t N;
  __half* vol[3];   // current, next, intermediate
};

struct vis_esteiras {
  lbm_ctx* ctx;
  size_t n;
  vis_part* parts;
};

namespace {

int vfail(int code, const std::string& m) { return lbm_internal_fail(code, m.c_str()); }

#define VCK(call, what)                                                                     \
  do {                                                                                      \
    cudaError_t _e = (call);                                                                \
    if (_e != cudaSuccess) {                                                                \
      cudaGetLastError();                                                                   \
      return vfail(_e == cudaErrorMemoryAllocation ? LBM_ENOMEM : LBM_ECUDA,                \
                   std::string(what) + ": " + cudaGetErrorString(_e));                      \
    }                                                                                       \
  } while (0)

struct Grid {
  int nx, ny, nz;
};

__device__ __forceinline__ bool solid_at(const uint8_t* tipo, Grid g, int x, int y, int z) {
  x = min(max(x, 0), g.nx - 1);
  y = min(max(y, 0), g.ny - 1);
  z = min(max(z, 0), g.nz - 1);
  const uint8_t t = tipo[((int64_t)z * g.ny + y) * g.nx + x];
  return t == 1 || t == 4 || t == 7;
}

__device__ __forceinline__ float ldv(const __half* v, Grid g, int x, int y, int z) {
  return __half2float(v[((int64_t)z * g.ny + y) * g.nx + x]);
}

// Trilinear sample at lattice position p (cell centres at i + 0.5) with
// clamp-to-edge: t = p - 0.5, corners floor(t) and floor(t) + 1 clamped to
// the grid, weights f = t - floor(t); interpolated along x, then y, then z
// as a + f (b - a).
__device__ __forceinline__ float sample3(const __half* v, Grid g, float px, float py, float pz) {
  const float tx = px - 0.5f, ty = py - 0.5f, tz = pz - 0.5f;
  const float bx = floorf(tx), by = floorf(ty), bz = floorf(tz);
  const float fx = tx - bx, fy = ty - by, fz = tz - bz;
  const int x0 = min(max((int)bx, 0), g.nx - 1), x1 = min(max((int)bx + 1, 0), g.nx - 1);
  const int y0 = min(max((int)by, 0), g.ny - 1), y1 = min(max((int)by + 1, 0), g.ny - 1);
  const int z0 = min(max((int)bz, 0), g.nz - 1), z1 = min(max((int)bz + 1, 0), g.nz - 1);
  auto lerp = [](float a, float b, float f) { return a + f * (b - a); };
  const float c00 = lerp(ldv(v, g, x0, y0, z0), ldv(v, g, x1, y0, z0), fx);
  const float c10 = lerp(ldv(v, g, x0, y1, z0), ldv(v, g, x1, y1, z0), fx);
  const float c01 = lerp(ldv(v, g, x0, y0, z1), ldv(v, g, x1, y0, z1), fx);
  const float c11 = lerp(ldv(v, g, x0, y1, z1), ldv(v, g, x1, y1, z1), fx);
  return lerp(lerp(c00, c10, fy), lerp(c01, c11, fy), fz);
}

__device__ __forceinline__ bool inside(Grid g, float px, float py, float pz) {
  return px >= 0.5f && py >= 0.5f && pz >= 0.5f && px <= (float)g.nx - 0.5f && py <= (float)g.ny - 0.5f &&
         pz <= (float)g.nz - 0.5f;
}

// Rake emission at a cell centre (src/render/fumaca.js:96-132).
__device__ __forceinline__ float rake_at(const vis_rake& R, const vis_fumo& F, float px, float py, float pz) {
  const float meia = fmaxf(1.5f, F.avanco * 0.6f);
  const float dx = fabsf(px - R.x);
  if (dx > meia) return 0.0f;
  if (py < R.y0 || py > R.y1) return 0.0f;
  if (pz < R.z0 || pz > R.z1) return 0.0f;
  const float ay = (py - R.y0) / R.passo_y, az = (pz - R.z0) / R.passo_z;
  const float fy = fabsf((ay - floorf(ay)) - 0.5f) * R.passo_y;
  const float fz = fabsf((az - floorf(az)) - 0.5f) * R.passo_z;
  const float r = sqrtf(fy * fy + fz * fz) / fmaxf(R.raio, 1e-3f);
  return F.taxa * expf(-r * r * 5.5f) * (1.0f - 0.35f * dx / meia);
}

// Pass 1: semi-Lagrangian back-trace of the current volume into the
// intermediate one (src/render/fumaca.js:147-160).
__global__ void k_recuar(const __half* __restrict__ cur, __half* __restrict__ mid, const float4* __restrict__ mac,
                         const uint8_t* __restrict__ tipo, Grid g, float dt) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= g.nx || y >= g.ny) return;
  const int64_t c = ((int64_t)z * g.ny + y) * g.nx + x;
  if (solid_at(tipo, g, x, y, z)) { mid[c] = __float2half_rn(0.0f); return; }
  const float px = (float)x + 0.5f, py = (float)y + 0.5f, pz = (float)z + 0.5f;
  const float4 u = mac[c];
  const float ax = px - u.x * dt, ay = py - u.y * dt, az = pz - u.z * dt;
  float d = sample3(cur, g, ax, ay, az);
  if (!inside(g, ax, ay, az)) d = 0.0f;
  mid[c] = __float2half_rn(d);
}

// Pass 2: MacCormack correction, eight-corner limiter, dissipation, domain
// cut-off, rake (src/render/fumaca.js:186-218).
__global__ void k_corrigir(const __half* __restrict__ cur, const __half* __restrict__ mid,
                           __half* __restrict__ nxt, const float4* __restrict__ mac,
                           const uint8_t* __restrict__ tipo, Grid g, vis_rake R, vis_fumo F) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= g.nx || y >= g.ny) return;
  const int64_t c = ((int64_t)z * g.ny + y) * g.nx + x;
  if (solid_at(tipo, g, x, y, z)) { nxt[c] = __float2half_rn(0.0f); return; }
  const float px = (float)x + 0.5f, py = (float)y + 0.5f, pz = (float)z + 0.5f;
  const float4 u = mac[c];
  const float ax = px - u.x * F.dt, ay = py - u.y * F.dt, az = pz - u.z * F.dt;
  const float chapeu = __half2float(mid[c]);
  const float voltando = sample3(mid, g, px + u.x * F.dt, py + u.y * F.dt, pz + u.z * F.dt);
  const float original = __half2float(cur[c]);
  float d = chapeu + 0.5f * (original - voltando);
  const float bx = floorf(ax - 0.5f), by = floorf(ay - 0.5f), bz = floorf(az - 0.5f);
  float lo = 1e30f, hi = -1e30f;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const int qx = min(max((int)(bx + (float)(k & 1)), 0), g.nx - 1);
    const int qy = min(max((int)(by + (float)((k >> 1) & 1)), 0), g.ny - 1);
    const int qz = min(max((int)(bz + (float)((k >> 2) & 1)), 0), g.nz - 1);
    const float v = ldv(cur, g, qx, qy, qz);
    lo = fminf(lo, v);
    hi = fmaxf(hi, v);
  }
  d = fminf(fmaxf(d, lo), hi) * F.dissipacao;
  if (!inside(g, ax, ay, az)) d = 0.0f;
  d = fmaxf(d, rake_at(R, F, px, py, pz));
  nxt[c] = __float2half_rn(fminf(fmaxf(d, 0.0f), 4.0f));
}

// The respawn hash of the particles (src/render/renderer.js:55-59).
__device__ __forceinline__ float hash01(uint32_t n) {
  uint32_t x = n * 747796405u + 2891336453u;
  x = ((x >> ((x >> 28u) + 4u)) ^ x) * 277803737u;
  return __uint2float_rn((x >> 22u) ^ x) / 4294967296.0f;
}

__device__ __forceinline__ float4 nearest(const float4* mac, Grid g, float px, float py, float pz) {
  const int x = min(max((int)px, 0), g.nx - 1);
  const int y = min(max((int)py, 0), g.ny - 1);
  const int z = min(max((int)pz, 0), g.nz - 1);
  return mac[((int64_t)z * g.ny + y) * g.nx + x];
}

// One frame of the streak particles (src/render/renderer.js:61-116); RAS:
// the ground streaks (src/render/rasante.js:95-149).
template <bool RAS>
__global__ void k_esteiras(vis_part* __restrict__ parts, long long n, const float4* __restrict__ mac, Grid g,
                           float dt_quadro, int nsub, uint32_t quadro, float altura) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  vis_part P = parts[i];
  const float4 m = nearest(mac, g, P.pos[0], P.pos[1], P.pos[2]);
  const int ns = max(nsub, 1);
  const float dt = dt_quadro / (float)ns;
  float x = P.pos[0], y = P.pos[1], z = P.pos[2];
  for (int k = 0; k < ns; ++k) {
    const float4 u = nearest(mac, g, x, y, z);
    x = x + u.x * dt;
    y = y + u.y * dt;
    z = z + u.z * dt;
  }
  float w = P.pos[3] - 1.0f;
  const float fx = (float)g.nx, fy = (float)g.ny, fz = (float)g.nz;
  const bool fora = x >= fx - 1.0f || x < 1.0f || y < 1.0f || y >= fy - 1.0f || z < (RAS ? 0.4f : 0.5f) ||
                    z >= fz - 1.0f;
  const bool presa = sqrtf(m.x * m.x + m.y * m.y + m.z * m.z) < 1e-5f;
  if (fora || presa || w <= 0.0f) {
    const uint32_t s = (uint32_t)i * 3u + quadro * 7919u;
    if (RAS) {
      const float h = hash01(s + 2u);
      x = 1.5f + hash01(s) * 4.0f;
      y = 1.0f + hash01(s + 1u) * (fy - 2.0f);
      z = 0.6f + h * h * h * altura;
      w = 150.0f + hash01(s + 5u) * 320.0f;
    } else {
      x = 2.0f + hash01(s) * 3.0f;
      y = 2.0f + hash01(s + 1u) * (fy - 4.0f);
      z = 0.5f + hash01(s + 2u) * (fz - 2.0f);
      w = 220.0f + hash01(s + 5u) * 260.0f;
    }
    P.ant[0] = x; P.ant[1] = y; P.ant[2] = z; P.ant[3] = 0.0f;
  } else {
    P.ant[0] = P.pos[0]; P.ant[1] = P.pos[1]; P.ant[2] = P.pos[2]; P.ant[3] = 1.0f;
  }
  P.pos[0] = x; P.pos[1] = y; P.pos[2] = z; P.pos[3] = w;
  parts[i] = P;
}

// ---- ray-march of the smoke volume (src/render/fumaca.js:257-349) ----
struct V3 {
  float x, y, z;
};
__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float dot3(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 normalize3(V3 a) {
  const float l = sqrtf(dot3(a, a));
  return v3(a.x / l, a.y / l, a.z / l);
}
__device__ __forceinline__ float fract(float x) { return x - floorf(x); }

// clip space (ndc.x, ndc.y, depth) -> world through the inverse view-projection
__device__ __forceinline__ V3 world_of(const float* m, float nx_, float ny_, float z) {
  float h[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) h[i] = ((m[i] * nx_ + m[4 + i] * ny_) + m[8 + i] * z) + m[12 + i];
  return v3(h[0] / h[3], h[1] / h[3], h[2] / h[3]);
}

__device__ __forceinline__ float hash12(float px, float py) {
  float p3x = fract(px * 0.1031f), p3y = fract(py * 0.1031f), p3z = fract(px * 0.1031f);
  const float d = p3x * (p3y + 33.33f) + p3y * (p3z + 33.33f) + p3z * (p3x + 33.33f);
  p3x = p3x + d; p3y = p3y + d; p3z = p3z + d;
  return fract((p3x + p3y) * p3z);
}

__device__ __forceinline__ float density_at(const __half* vol, Grid g, float k, V3 w) {
  const float px = w.x / k + (float)g.nx * 0.5f, py = w.y / k + (float)g.ny * 0.5f, pz = w.z / k;
  const float ux = px / (float)g.nx, uy = py / (float)g.ny, uz = pz / (float)g.nz;
  if (ux < 0.0f || uy < 0.0f || uz < 0.0f || ux > 1.0f || uy > 1.0f || uz > 1.0f) return 0.0f;
  return sample3(vol, g, px, py, pz);
}

__global__ void k_render(const __half* __restrict__ vol, Grid g, vis_camera cam, float4* __restrict__ img) {
  const int ix = blockIdx.x * blockDim.x + threadIdx.x;
  const int iy = blockIdx.y * blockDim.y + threadIdx.y;
  if (ix >= cam.largura || iy >= cam.altura) return;
  const float fx = (float)ix + 0.5f, fy = (float)iy + 0.5f;
  const float ndx = fx / (float)cam.largura * 2.0f - 1.0f;
  const float ndy = 1.0f - fy / (float)cam.altura * 2.0f;
  float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
  const V3 origem = v3(cam.olho[0], cam.olho[1], cam.olho[2]);
  const V3 alvo = world_of(cam.inv_view_proj, ndx, ndy, 1.0f);
  const V3 dir = normalize3(alvo - origem);
  const float k = (1.0f / (float)g.nx) * 2.0f;
  const V3 lo = v3(-(float)g.nx * 0.5f * k, -(float)g.ny * 0.5f * k, 0.0f);
  const V3 hi = v3((float)g.nx * 0.5f * k, (float)g.ny * 0.5f * k, (float)g.nz * k);
  // slab test (src/render/comum.js:81-89)
  const float ivx = 1.0f / dir.x, ivy = 1.0f / dir.y, ivz = 1.0f / dir.z;
  const float ax = (lo.x - origem.x) * ivx, bx = (hi.x - origem.x) * ivx;
  const float ay = (lo.y - origem.y) * ivy, by = (hi.y - origem.y) * ivy;
  const float az = (lo.z - origem.z) * ivz, bz = (hi.z - origem.z) * ivz;
  const float tmin = fmaxf(fmaxf(fminf(ax, bx), fminf(ay, by)), fminf(az, bz));
  const float tmax = fminf(fminf(fmaxf(ax, bx), fmaxf(ay, by)), fmaxf(az, bz));
  const float t0 = fmaxf(tmin, 0.0f), t1 = tmax;
  if (t1 > t0) {
    const int np = cam.passos, nl = cam.passos_luz;
    const float ds = (t1 - t0) / (float)np;
    const float sigma = cam.densidade, gg = cam.g;
    const V3 luz_dir = normalize3(v3(cam.luz[0], cam.luz[1], cam.luz[2]));
    // Henyey-Greenstein
    const float g2 = gg * gg;
    const float dd = 1.0f + g2 - 2.0f * gg * dot3(dir, luz_dir);
    const float fase = (1.0f - g2) / (12.566370614f * fmaxf(dd * sqrtf(dd), 1e-4f));
    const float jitter = hash12(fx + cam.quadro * 0.618f, fy + cam.quadro * 0.618f) * ds;
    float T = 1.0f, Lr = 0.0f, Lg = 0.0f, Lb = 0.0f;
    float s = t0 + jitter;
    const float dl = (hi.z - lo.z) / (float)nl * 0.9f;
    for (int i = 0; i < np; ++i) {
      if (T < 0.01f) break;
      const V3 w = origem + dir * s;
      const float d = density_at(vol, g, k, w);
      s = s + ds;
      if (d <= 0.001f) continue;
      const float st = d * sigma;
      const float atenua = 1.0f - expf(-st * ds);
      float tau = 0.0f;
      for (int j = 1; j <= nl; ++j) tau = tau + density_at(vol, g, k, w + luz_dir * ((float)j * dl)) * sigma * dl;
      const float luz = expf(-tau);
      const float ambiente = 0.16f + 0.10f * expf(-tau * 0.35f);
      const float c = T * atenua * (luz * fase * 3.6f + ambiente) * cam.luz[3];
      Lr = Lr + c * 0.96f;
      Lg = Lg + c * 0.97f;
      Lb = Lb + c * 1.0f;
      T = T * expf(-st * ds);
    }
    out = make_float4(Lr, Lg, Lb, 1.0f - T);
  }
  img[(size_t)iy * cam.largura + ix] = out;
}

// Surface Cp per triangle (src/render/renderer.js:168-180, at the centroid).
__global__ void k_cp(const float* __restrict__ pos, const uint32_t* __restrict__ idx, long long nt,
                     const float4* __restrict__ mac, const uint8_t* __restrict__ tipo, Grid g, float u_ref,
                     float* __restrict__ cp) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  const uint32_t a = idx[3 * t], b = idx[3 * t + 1], c = idx[3 * t + 2];
  const V3 v0 = v3(pos[3 * a], pos[3 * a + 1], pos[3 * a + 2]);
  const V3 v1 = v3(pos[3 * b], pos[3 * b + 1], pos[3 * b + 2]);
  const V3 v2 = v3(pos[3 * c], pos[3 * c + 1], pos[3 * c + 2]);
  const V3 e1 = v1 - v0, e2 = v2 - v0;
  const V3 n = normalize3(v3(e1.y * e2.z - e1.z * e2.y, e1.z * e2.x - e1.x * e2.z, e1.x * e2.y - e1.y * e2.x));
  const V3 cen = v3(((v0.x + v1.x) + v2.x) / 3.0f, ((v0.y + v1.y) + v2.y) / 3.0f, ((v0.z + v1.z) + v2.z) / 3.0f);
  V3 fora = cen + n * 1.8f;
  if (solid_at(tipo, g, (int)fora.x, (int)fora.y, (int)fora.z)) fora = cen - n * 1.8f;
  const float4 m = nearest(mac, g, fora.x, fora.y, fora.z);
  cp[t] = m.w / fmaxf(1.5f * u_ref * u_ref, 1e-12f);
}

}  // namespace

extern "C" {

int vis_fumaca_create(lbm_ctx* ctx, vis_fumaca** out) {
  if (!ctx || !out) return vfail(LBM_EINVAL, "null argument");
  *out = nullptr;
  CtxView v;
  int r = ctx_view(ctx, &v);
  if (r) return r;
  vis_fumaca* f = new vis_fumaca();
  f->ctx = ctx;
  f->nx = v.nx; f->ny = v.ny; f->nz = v.nz;
  f->N = v.N;
  for (int k = 0; k < 3; ++k) {
    cudaError_t e = cudaMalloc(&f->vol[k], sizeof(__half) * (size_t)v.N);
    if (e != cudaSuccess) {
      cudaGetLastError();
      for (int j = 0; j < k; ++j) cudaFree(f->vol[j]);
      delete f;
      return vfail(LBM_ENOMEM, std::string("smoke volume: ") + cudaGetErrorString(e));
    }
  }
  *out = f;
  return vis_fumaca_limpar(f);
}

int vis_fumaca_destroy(vis_fumaca* f) {
  if (!f) return vfail(LBM_EINVAL, "null smoke volume");
  CtxView v;
  if (ctx_view(f->ctx, &v) == LBM_OK) cudaStreamSynchronize(v.stream);
  for (int k = 0; k < 3; ++k) cudaFree(f->vol[k]);
  delete f;
  return LBM_OK;
}

int vis_fumaca_limpar(vis_fumaca* f) {
  if (!f) return vfail(LBM_EINVAL, "null smoke volume");
  CtxView v;
  int r = ctx_view(f->ctx, &v);
  if (r) return r;
  for (int k = 0; k < 3; ++k)
    VCK(cudaMemsetAsync(f->vol[k], 0, sizeof(__half) * (size_t)f->N, v.stream), "smoke clear");
  VCK(cudaStreamSynchronize(v.stream), "smoke clear sync");
  return LBM_OK;
}

int vis_fumaca_passo(vis_fumaca* f, const vis_rake* rake, const vis_fumo* params) {
  if (!f || !rake || !params) return vfail(LBM_EINVAL, "null argument");
  CtxView v;
  int r = ctx_view(f->ctx, &v);
  if (r) return r;
  const Grid g{f->nx, f->ny, f->nz};
  const dim3 block(32, 4), grid((f->nx + 31) / 32, (f->ny + 3) / 4, f->nz);
  k_recuar<<<grid, block, 0, v.stream>>>(f->vol[0], f->vol[2], v.macros, v.tipo, g, params->dt);
  k_corrigir<<<grid, block, 0, v.stream>>>(f->vol[0], f->vol[2], f->vol[1], v.macros, v.tipo, g, *rake, *params);
  VCK(cudaGetLastError(), "smoke kernels");
  __half* t = f->vol[0];
  f->vol[0] = f->vol[1];
  f->vol[1] = t;
  return LBM_OK;
}

int vis_fumaca_ler(vis_fumaca* f, uint16_t* out, size_t n) {
  if (!f || !out) return vfail(LBM_EINVAL, "null argument");
  if ((int64_t)n != f->N) return vfail(LBM_EINVAL, "density array must hold N values");
  CtxView v;
  int r = ctx_view(f->ctx, &v);
  if (r) return r;
  VCK(cudaMemcpyAsync(out, f->vol[0], sizeof(__half) * n, cudaMemcpyDeviceToHost, v.stream), "smoke download");
  VCK(cudaStreamSynchronize(v.stream), "smoke download sync");
  return LBM_OK;
}

int vis_fumaca_definir(vis_fumaca* f, const uint16_t* in, size_t n) {
  if (!f || !in) return vfail(LBM_EINVAL, "null argument");
  if ((int64_t)n != f->N) return vfail(LBM_EINVAL, "density array must hold N values");
  CtxView v;
  int r = ctx_view(f->ctx, &v);
  if (r) return r;
  VCK(cudaMemcpyAsync(f->vol[0], in, sizeof(__half) * n, cudaMemcpyHostToDevice, v.stream), "smoke upload");
  VCK(cudaStreamSynchronize(v.stream), "smoke upload sync");
  return LBM_OK;
}

int vis_esteiras_create(lbm_ctx* ctx, size_t n, vis_esteiras** out) {
  if (!ctx || !out || n == 0) return vfail(LBM_EINVAL, "null argument or no particles");
  *out = nullptr;
  CtxView v;
  int r = ctx_view(ctx, &v);
  if (r) return r;
  vis_esteiras* e = new vis_esteiras();
  e->ctx = ctx;
  e->n = n;
  cudaError_t ce = cudaMalloc(&e->parts, sizeof(vis_part) * n);
  if (ce != cudaSuccess) {
    cudaGetLastError();
    delete e;
    return vfail(LBM_ENOMEM, std::string("particles: ") + cudaGetErrorString(ce));
  }
  VCK(cudaMemsetAsync(e->parts, 0, sizeof(vis_part) * n, v.stream), "particles clear");
  VCK(cudaStreamSynchronize(v.stream), "particles clear sync");
  *out = e;
  return LBM_OK;
}

int vis_esteiras_destroy(vis_esteiras* e) {
  if (!e) return vfail(LBM_EINVAL, "null particles");
  CtxView v;
  if (ctx_view(e->ctx, &v) == LBM_OK) cudaStreamSynchronize(v.stream);
  cudaFree(e->parts);
  delete e;
  return LBM_OK;
}

int vis_esteiras_definir(vis_esteiras* e, const vis_part* in, size_t n) {
  if (!e || !in) return vfail(LBM_EINVAL, "null argument");
  if (n != e->n) return vfail(LBM_EINVAL, "particle count differs");
  CtxView v;
  int r = ctx_view(e->ctx, &v);
  if (r) return r;
  VCK(cudaMemcpyAsync(e->parts, in, sizeof(vis_part) * n, cudaMemcpyHostToDevice, v.stream), "particles upload");
  VCK(cudaStreamSynchronize(v.stream), "particles upload sync");
  return LBM_OK;
}

int vis_esteiras_ler(vis_esteiras* e, vis_part* out, size_t n) {
  if (!e || !out) return vfail(LBM_EINVAL, "null argument");
  if (n != e->n) return vfail(LBM_EINVAL, "particle count differs");
  CtxView v;
  int r = ctx_view(e->ctx, &v);
  if (r) return r;
  VCK(cudaMemcpyAsync(out, e->parts, sizeof(vis_part) * n, cudaMemcpyDeviceToHost, v.stream), "particles download");
  VCK(cudaStreamSynchronize(v.stream), "particles download sync");
  return LBM_OK;
}

int vis_esteiras_passo(vis_esteiras* e, float dt_quadro, int nsub, uint32_t quadro) {
  if (!e) return vfail(LBM_EINVAL, "null particles");
  if (nsub < 1 || nsub > 4096) return vfail(LBM_EINVAL, "sub-steps must be 1..4096");
  CtxView v;
  int r = ctx_view(e->ctx, &v);
  if (r) return r;
  const Grid g{v.nx, v.ny, v.nz};
  k_esteiras<false><<<(unsigned)((e->n + 127) / 128), 128, 0, v.stream>>>(e->parts, (long long)e->n, v.macros, g,
                                                                         dt_quadro, nsub, quadro, 0.0f);
  VCK(cudaGetLastError(), "particle kernel");
  return LBM_OK;
}

int vis_rasantes_passo(vis_esteiras* e, float dt_quadro, int nsub, uint32_t quadro, float altura) {
  if (!e) return vfail(LBM_EINVAL, "null particles");
  if (nsub < 1 || nsub > 4096) return vfail(LBM_EINVAL, "sub-steps must be 1..4096");
  CtxView v;
  int r = ctx_view(e->ctx, &v);
  if (r) return r;
  const Grid g{v.nx, v.ny, v.nz};
  k_esteiras<true><<<(unsigned)((e->n + 127) / 128), 128, 0, v.stream>>>(e->parts, (long long)e->n, v.macros, g,
                                                                        dt_quadro, nsub, quadro, altura);
  VCK(cudaGetLastError(), "ground streak kernel");
  return LBM_OK;
}

int vis_cp_triangulos(lbm_ctx* ctx, const float* pos, size_t nv, const uint32_t* idx, size_t nt, float u_ref,
                      float* cp_out) {
  if (!ctx || !pos || !idx || !cp_out || nv == 0 || nt == 0) return vfail(LBM_EINVAL, "null argument or empty mesh");
  for (size_t i = 0; i < 3 * nt; ++i)
    if (idx[i] >= nv) return vfail(LBM_EINVAL, "triangle index out of range");
  CtxView v;
  int r = ctx_view(ctx, &v);
  if (r) return r;
  float *d_pos = nullptr, *d_cp = nullptr;
  uint32_t* d_idx = nullptr;
  cudaError_t e = cudaMalloc(&d_pos, sizeof(float) * 3 * nv);
  if (e == cudaSuccess) e = cudaMalloc(&d_idx, sizeof(uint32_t) * 3 * nt);
  if (e == cudaSuccess) e = cudaMalloc(&d_cp, sizeof(float) * nt);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_pos, pos, sizeof(float) * 3 * nv, cudaMemcpyHostToDevice, v.stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_idx, idx, sizeof(uint32_t) * 3 * nt, cudaMemcpyHostToDevice, v.stream);
  if (e == cudaSuccess) {
    const Grid g{v.nx, v.ny, v.nz};
    k_cp<<<(unsigned)((nt + 127) / 128), 128, 0, v.stream>>>(d_pos, d_idx, (long long)nt, v.macros, v.tipo, g, u_ref,
                                                             d_cp);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(cp_out, d_cp, sizeof(float) * nt, cudaMemcpyDeviceToHost, v.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(v.stream);
  cudaFree(d_pos);
  cudaFree(d_idx);
  cudaFree(d_cp);
  VCK(e, "surface Cp");
  return LBM_OK;
}

int vis_fumaca_render(vis_fumaca* f, const vis_camera* cam, float* rgba, size_t n) {
  if (!f || !cam || !rgba) return vfail(LBM_EINVAL, "null argument");
  if (cam->largura < 1 || cam->altura < 1 || cam->largura > 16384 || cam->altura > 16384)
    return vfail(LBM_EINVAL, "image size must be 1..16384 per side");
  if (cam->passos < 1 || cam->passos > 4096 || cam->passos_luz < 1 || cam->passos_luz > 256)
    return vfail(LBM_EINVAL, "march steps must be 1..4096 (light 1..256)");
  const size_t px = (size_t)cam->largura * (size_t)cam->altura;
  if (n != 4 * px) return vfail(LBM_EINVAL, "rgba must hold largura * altura * 4 floats");
  CtxView v;
  int r = ctx_view(f->ctx, &v);
  if (r) return r;
  float4* d_img = nullptr;
  VCK(cudaMalloc(&d_img, sizeof(float4) * px), "image");
  const Grid g{f->nx, f->ny, f->nz};
  const dim3 block(16, 8), grid((cam->largura + 15) / 16, (cam->altura + 7) / 8);
  k_render<<<grid, block, 0, v.stream>>>(f->vol[0], g, *cam, d_img);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(rgba, d_img, sizeof(float4) * px, cudaMemcpyDeviceToHost, v.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(v.stream);
  cudaFree(d_img);
  VCK(e, "smoke render");
  return LBM_OK;
}

}  // extern "C"

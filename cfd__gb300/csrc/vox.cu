// vox.cu — triangle-mesh voxelizer on the GPU (include/vox.h).
//
// Restates voxelizar() of the reference (src/geom/voxel.js:376-433):
//   raster  one warp per triangle walks the triangle's banded box
//           (:194-201); per voxel the squared point-triangle distance
//           (Ericson, :105-151) feeds the distance band, and where it is
//           <= 0.75 the Akenine-Moller separating-axis test (:61-98) marks
//           the shell (:213-221).  Both predicates are evaluated in fp32 with
//           a certified error bound; a pair whose margin falls inside the
//           bound is appended to a short list and decided by k_tiebreak in
//           fp64 with the reference's own operation order, so the shell is
//           bit-identical to the reference's fp64 result.
//   seal    26-neighbourhood dilation of the shell as separable x/y/z box
//           maxima on 1-bit-per-cell rows (:244-267).
//   flood   6-connected exterior fill from the six faces (:278-327) as a
//           monotone fixed-point iteration on bit rows: each pass takes seeds
//           from the rows above/below in y and z, then propagates them along
//           the whole row in one carry sweep per direction.
//   skin    one non-cascading 6-neighbour growth of the exterior into
//           non-shell voxels (:333-355).
//   classes FLUIDO / CASCA / DENTRO and the signed narrow-band distance
//           (:401-415).
// Built with -fmad=false: the fp64 tie-break must not fuse, and the fp32
// bounds below assume no fusion either.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/lbm.h"
#include "../../include/vox.h"

extern "C" int lbm_internal_fail(int code, const char* msg);

namespace {

constexpr float kU = 5.9604645e-8f;  // 2^-24, unit roundoff of fp32

struct Tri {
  float v[9];          // a, b, c
  int box[6];          // x0, y0, z0, x1, y1, z1 (inclusive)
  float kappa;         // |ab|^2 |ac|^2 / |ab x ac|^2 (shape factor), or -1: degenerate
  int id;
};

struct Deferred {
  int tri;
  int pad;
  long long cell;
};

__device__ __forceinline__ float mn3(float a, float b, float c) { return fminf(fminf(a, b), c); }
__device__ __forceinline__ float mx3(float a, float b, float c) { return fmaxf(fmaxf(a, b), c); }

// ---------------------------------------------------------------- fp32 path
// Squared distance point-triangle, Ericson 5.1.5, the reference's branch
// structure (src/geom/voxel.js:105-151) in fp32.
__device__ float dist2_f32(const float* p, const float* a, const float* b, const float* c) {
  const float abx = b[0] - a[0], aby = b[1] - a[1], abz = b[2] - a[2];
  const float acx = c[0] - a[0], acy = c[1] - a[1], acz = c[2] - a[2];
  const float apx = p[0] - a[0], apy = p[1] - a[1], apz = p[2] - a[2];
  const float d1 = abx * apx + aby * apy + abz * apz;
  const float d2 = acx * apx + acy * apy + acz * apz;
  if (d1 <= 0 && d2 <= 0) return apx * apx + apy * apy + apz * apz;
  const float bpx = p[0] - b[0], bpy = p[1] - b[1], bpz = p[2] - b[2];
  const float d3 = abx * bpx + aby * bpy + abz * bpz;
  const float d4 = acx * bpx + acy * bpy + acz * bpz;
  if (d3 >= 0 && d4 <= d3) return bpx * bpx + bpy * bpy + bpz * bpz;
  const float vc = d1 * d4 - d3 * d2;
  if (vc <= 0 && d1 >= 0 && d3 <= 0) {
    const float v = d1 / (d1 - d3);
    const float qx = apx - v * abx, qy = apy - v * aby, qz = apz - v * abz;
    return qx * qx + qy * qy + qz * qz;
  }
  const float cpx = p[0] - c[0], cpy = p[1] - c[1], cpz = p[2] - c[2];
  const float d5 = abx * cpx + aby * cpy + abz * cpz;
  const float d6 = acx * cpx + acy * cpy + acz * cpz;
  if (d6 >= 0 && d5 <= d6) return cpx * cpx + cpy * cpy + cpz * cpz;
  const float vb = d5 * d2 - d1 * d6;
  if (vb <= 0 && d2 >= 0 && d6 <= 0) {
    const float w = d2 / (d2 - d6);
    const float qx = apx - w * acx, qy = apy - w * acy, qz = apz - w * acz;
    return qx * qx + qy * qy + qz * qz;
  }
  const float va = d3 * d6 - d5 * d4;
  if (va <= 0 && (d4 - d3) >= 0 && (d5 - d6) >= 0) {
    const float w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
    const float qx = bpx + w * (cpx - bpx), qy = bpy + w * (cpy - bpy), qz = bpz + w * (cpz - bpz);
    return qx * qx + qy * qy + qz * qz;
  }
  const float den = 1.0f / (va + vb + vc);
  const float v = vb * den, w = vc * den;
  const float qx = apx - (v * abx + w * acx);
  const float qy = apy - (v * aby + w * acy);
  const float qz = apz - (v * abz + w * acz);
  return qx * qx + qy * qy + qz * qz;
}

// Separating-axis test in fp32 on coordinates relative to the voxel centre.
// Returns 0: certainly disjoint, 1: certainly overlapping, 2: too close to
// call.  Bounds (Vs = largest |coordinate| + 1, u = 2^-24), each a few times
// the forward error of the expression it guards:
//   edge x box axes   |(min|max) - r|  error <= 24 u Vs^2  -> 32 u Vs^2
//   box axes          |coord - 1/2|    error <=  u Vs      -> 4 u Vs
//   triangle normal   ||d| - r|        error <= 240 u Vs^3 -> 320 u Vs^3
__device__ int sat_f32(const float* v0, const float* v1, const float* v2, float Vs) {
  const float e0[3] = {v1[0] - v0[0], v1[1] - v0[1], v1[2] - v0[2]};
  const float e1[3] = {v2[0] - v1[0], v2[1] - v1[1], v2[2] - v1[2]};
  const float e2[3] = {v0[0] - v2[0], v0[1] - v2[1], v0[2] - v2[2]};
  const float bax = 32.0f * kU * Vs * Vs;
  bool unsure = false;
  // margin > 0 means the axis separates
  auto axis = [&](float a, float b, float fa, float fb, int i, int j) -> bool {
    const float p0 = a * v0[i] + b * v0[j];
    const float p1 = a * v1[i] + b * v1[j];
    const float p2 = a * v2[i] + b * v2[j];
    const float r = fa * 0.5f + fb * 0.5f;
    const float m = fmaxf(mn3(p0, p1, p2) - r, -r - mx3(p0, p1, p2));
    if (m > bax) return true;          // certainly separating
    if (m > -bax) unsure = true;
    return false;
  };
  const float* es[3] = {e0, e1, e2};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float* e = es[k];
    const float fx = fabsf(e[0]), fy = fabsf(e[1]), fz = fabsf(e[2]);
    if (axis(e[2], -e[1], fz, fy, 1, 2)) return 0;
    if (axis(-e[2], e[0], fz, fx, 0, 2)) return 0;
    if (axis(e[1], -e[0], fy, fx, 0, 1)) return 0;
  }
  const float bb = 4.0f * kU * Vs;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float m = fmaxf(mn3(v0[k], v1[k], v2[k]) - 0.5f, -0.5f - mx3(v0[k], v1[k], v2[k]));
    if (m > bb) return 0;
    if (m > -bb) unsure = true;
  }
  const float n0 = e0[1] * e1[2] - e0[2] * e1[1];
  const float n1 = e0[2] * e1[0] - e0[0] * e1[2];
  const float n2 = e0[0] * e1[1] - e0[1] * e1[0];
  const float d = n0 * v0[0] + n1 * v0[1] + n2 * v0[2];
  const float r = fabsf(n0) * 0.5f + fabsf(n1) * 0.5f + fabsf(n2) * 0.5f;
  const float bn = 320.0f * kU * Vs * Vs * Vs;
  const float m = fabsf(d) - r;
  if (m > bn) return 0;
  if (m > -bn) unsure = true;
  return unsure ? 2 : 1;
}

// ---------------------------------------------------------------- fp64 path
// The reference's own arithmetic (JavaScript doubles), used for the few
// pairs the fp32 path cannot decide.
__device__ double dmin3(double a, double b, double c) { double m = a < b ? a : b; return m < c ? m : c; }
__device__ double dmax3(double a, double b, double c) { double m = a > b ? a : b; return m > c ? m : c; }

__device__ bool sat_axis_f64(double a, double b, double fa, double fb, int i, int j, const double* v0,
                             const double* v1, const double* v2) {
  const double p0 = a * v0[i] + b * v0[j];
  const double p1 = a * v1[i] + b * v1[j];
  const double p2 = a * v2[i] + b * v2[j];
  const double mn = dmin3(p0, p1, p2), mx = dmax3(p0, p1, p2);
  const double r = fa * 0.5 + fb * 0.5;
  return !(mn > r || mx < -r);
}

__device__ bool tri_box_f64(const double* v0, const double* v1, const double* v2) {
  const double e0[3] = {v1[0] - v0[0], v1[1] - v0[1], v1[2] - v0[2]};
  const double e1[3] = {v2[0] - v1[0], v2[1] - v1[1], v2[2] - v1[2]};
  const double e2[3] = {v0[0] - v2[0], v0[1] - v2[1], v0[2] - v2[2]};
  const double* es[3] = {e0, e1, e2};
  for (int k = 0; k < 3; ++k) {
    const double* e = es[k];
    const double fx = fabs(e[0]), fy = fabs(e[1]), fz = fabs(e[2]);
    if (!sat_axis_f64(e[2], -e[1], fz, fy, 1, 2, v0, v1, v2)) return false;
    if (!sat_axis_f64(-e[2], e[0], fz, fx, 0, 2, v0, v1, v2)) return false;
    if (!sat_axis_f64(e[1], -e[0], fy, fx, 0, 1, v0, v1, v2)) return false;
  }
  for (int k = 0; k < 3; ++k) {
    if (dmin3(v0[k], v1[k], v2[k]) > 0.5) return false;
    if (dmax3(v0[k], v1[k], v2[k]) < -0.5) return false;
  }
  const double n[3] = {e0[1] * e1[2] - e0[2] * e1[1], e0[2] * e1[0] - e0[0] * e1[2], e0[0] * e1[1] - e0[1] * e1[0]};
  const double d = n[0] * v0[0] + n[1] * v0[1] + n[2] * v0[2];
  const double r = fabs(n[0]) * 0.5 + fabs(n[1]) * 0.5 + fabs(n[2]) * 0.5;
  return fabs(d) <= r;
}

__device__ double dist2_f64(const double* p, const double* a, const double* b, const double* c) {
  const double abx = b[0] - a[0], aby = b[1] - a[1], abz = b[2] - a[2];
  const double acx = c[0] - a[0], acy = c[1] - a[1], acz = c[2] - a[2];
  const double apx = p[0] - a[0], apy = p[1] - a[1], apz = p[2] - a[2];
  const double d1 = abx * apx + aby * apy + abz * apz;
  const double d2 = acx * apx + acy * apy + acz * apz;
  if (d1 <= 0 && d2 <= 0) return apx * apx + apy * apy + apz * apz;
  const double bpx = p[0] - b[0], bpy = p[1] - b[1], bpz = p[2] - b[2];
  const double d3 = abx * bpx + aby * bpy + abz * bpz;
  const double d4 = acx * bpx + acy * bpy + acz * bpz;
  if (d3 >= 0 && d4 <= d3) return bpx * bpx + bpy * bpy + bpz * bpz;
  const double vc = d1 * d4 - d3 * d2;
  if (vc <= 0 && d1 >= 0 && d3 <= 0) {
    const double v = d1 / (d1 - d3);
    const double qx = apx - v * abx, qy = apy - v * aby, qz = apz - v * abz;
    return qx * qx + qy * qy + qz * qz;
  }
  const double cpx = p[0] - c[0], cpy = p[1] - c[1], cpz = p[2] - c[2];
  const double d5 = abx * cpx + aby * cpy + abz * cpz;
  const double d6 = acx * cpx + acy * cpy + acz * cpz;
  if (d6 >= 0 && d5 <= d6) return cpx * cpx + cpy * cpy + cpz * cpz;
  const double vb = d5 * d2 - d1 * d6;
  if (vb <= 0 && d2 >= 0 && d6 <= 0) {
    const double w = d2 / (d2 - d6);
    const double qx = apx - w * acx, qy = apy - w * acy, qz = apz - w * acz;
    return qx * qx + qy * qy + qz * qz;
  }
  const double va = d3 * d6 - d5 * d4;
  if (va <= 0 && (d4 - d3) >= 0 && (d5 - d6) >= 0) {
    const double w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
    const double qx = bpx + w * (cpx - bpx), qy = bpy + w * (cpy - bpy), qz = bpz + w * (cpz - bpz);
    return qx * qx + qy * qy + qz * qz;
  }
  const double den = 1 / (va + vb + vc);
  const double v = vb * den, w = vc * den;
  const double qx = apx - (v * abx + w * acx);
  const double qy = apy - (v * aby + w * acy);
  const double qz = apz - (v * abz + w * acz);
  return qx * qx + qy * qy + qz * qz;
}

// ---------------------------------------------------------------- kernels
// One warp per triangle; lanes stride over the voxels of its banded box.
__global__ void k_raster(const Tri* __restrict__ tris, int ntri, int nx, int ny, uint8_t* __restrict__ flags,
                         unsigned* __restrict__ dist2, Deferred* __restrict__ def, unsigned long long* ndef,
                         long long cap, unsigned long long* npairs) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= ntri) return;
  const Tri T = tris[warp];
  const int bx = T.box[3] - T.box[0] + 1, by = T.box[4] - T.box[1] + 1, bz = T.box[5] - T.box[2] + 1;
  const long long nvox = (long long)bx * by * bz;
  if (lane == 0) atomicAdd(npairs, (unsigned long long)nvox);
  if (T.kappa < 0.0f) return;   // ill-conditioned triangle: k_raster_f64 takes all of it
  const float* a = T.v;
  const float* b = T.v + 3;
  const float* c = T.v + 6;
  for (long long k = lane; k < nvox; k += 32) {
    const int x = T.box[0] + (int)(k % bx);
    const int y = T.box[1] + (int)((k / bx) % by);
    const int z = T.box[2] + (int)(k / ((long long)bx * by));
    const long long cell = ((long long)z * ny + y) * nx + x;
    const float p[3] = {x + 0.5f, y + 0.5f, z + 0.5f};
    const float d2 = dist2_f32(p, a, b, c);
    if (d2 >= 0.0f) atomicMin(dist2 + cell, __float_as_uint(d2));
    const float la[3] = {a[0] - p[0], a[1] - p[1], a[2] - p[2]};
    const float lb[3] = {b[0] - p[0], b[1] - p[1], b[2] - p[2]};
    const float lc[3] = {c[0] - p[0], c[1] - p[1], c[2] - p[2]};
    float V = 0.0f;
#pragma unroll
    for (int q = 0; q < 3; ++q) V = fmaxf(V, fmaxf(fabsf(la[q]), fmaxf(fabsf(lb[q]), fabsf(lc[q]))));
    const float Vs = V + 1.0f;
    bool defer = false;
    {
      // d2 error: the point-triangle distance conditions like the triangle's
      // shape (kappa); 128 u kappa (6 Vs)^2 covers the branch that divides.
      const float bd2 = 128.0f * kU * T.kappa * 36.0f * Vs * Vs;
      if (!(d2 - bd2 <= 0.75f)) continue;     // certainly d2 > 0.75: no shell
      const int s = sat_f32(la, lb, lc, Vs);
      if (s == 0) continue;                   // certainly no overlap
      if (s == 1 && d2 + bd2 <= 0.75f) {      // certainly shell
        flags[cell] = 1;
        continue;
      }
      defer = true;
    }
    const unsigned long long slot = atomicAdd(ndef, 1ull);
    if ((long long)slot < cap) {
      def[slot].tri = warp;
      def[slot].cell = cell;
    }
  }
}

// Deferred pairs: the reference's fp64 predicate (src/geom/voxel.js:207-221).
__global__ void k_tiebreak(const Tri* __restrict__ tris, const Deferred* __restrict__ def, long long n, int nx,
                           int ny, uint8_t* __restrict__ flags) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const Deferred D = def[i];
  const Tri& T = tris[D.tri];
  const long long cell = D.cell;
  const int x = (int)(cell % nx), y = (int)((cell / nx) % ny), z = (int)(cell / ((long long)nx * ny));
  const double p[3] = {x + 0.5, y + 0.5, z + 0.5};
  const double a[3] = {T.v[0], T.v[1], T.v[2]}, b[3] = {T.v[3], T.v[4], T.v[5]}, c[3] = {T.v[6], T.v[7], T.v[8]};
  const double d2 = dist2_f64(p, a, b, c);
  if (d2 <= 0.75) {
    const double la[3] = {a[0] - p[0], a[1] - p[1], a[2] - p[2]};
    const double lb[3] = {b[0] - p[0], b[1] - p[1], b[2] - p[2]};
    const double lc[3] = {c[0] - p[0], c[1] - p[1], c[2] - p[2]};
    if (tri_box_f64(la, lb, lc)) flags[cell] = 1;
  }
}

__global__ void k_fill_u32(unsigned* __restrict__ p, unsigned v, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

// Ill-conditioned triangles (slivers, near-degenerate): the whole banded box
// in the reference's fp64 arithmetic, distance band included.
__global__ void k_raster_f64(const Tri* __restrict__ tris, const int* __restrict__ list, int n, int nx, int ny,
                             uint8_t* __restrict__ flags, unsigned* __restrict__ dist2) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= n) return;
  const Tri& T = tris[list[warp]];
  const int bx = T.box[3] - T.box[0] + 1, by = T.box[4] - T.box[1] + 1, bz = T.box[5] - T.box[2] + 1;
  const long long nvox = (long long)bx * by * bz;
  const double a[3] = {T.v[0], T.v[1], T.v[2]}, b[3] = {T.v[3], T.v[4], T.v[5]}, c[3] = {T.v[6], T.v[7], T.v[8]};
  for (long long k = lane; k < nvox; k += 32) {
    const int x = T.box[0] + (int)(k % bx);
    const int y = T.box[1] + (int)((k / bx) % by);
    const int z = T.box[2] + (int)(k / ((long long)bx * by));
    const long long cell = ((long long)z * ny + y) * nx + x;
    const double p[3] = {x + 0.5, y + 0.5, z + 0.5};
    const double d2 = dist2_f64(p, a, b, c);
    if (d2 >= 0.0) atomicMin(dist2 + cell, __float_as_uint((float)d2));
    if (d2 <= 0.75) {
      const double la[3] = {a[0] - p[0], a[1] - p[1], a[2] - p[2]};
      const double lb[3] = {b[0] - p[0], b[1] - p[1], b[2] - p[2]};
      const double lc[3] = {c[0] - p[0], c[1] - p[1], c[2] - p[2]};
      if (tri_box_f64(la, lb, lc)) flags[cell] = 1;
    }
  }
}

// ---- 1-bit rows: word w of row (y, z) holds x = 32 w .. 32 w + 31
__device__ __forceinline__ unsigned valid_mask(int w, int W, int nx) {
  const int rem = nx - 32 * (W - 1);
  return (w == W - 1 && rem < 32) ? ((1u << rem) - 1u) : 0xffffffffu;
}

__global__ void k_pack(const uint8_t* __restrict__ flags, unsigned* __restrict__ S, int nx, int W, long long nwords) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nwords) return;
  const long long row = i / W;
  const int w = (int)(i % W);
  unsigned bits = 0;
  for (int b = 0; b < 32; ++b) {
    const int x = 32 * w + b;
    if (x < nx && flags[row * nx + x] == 1) bits |= 1u << b;
  }
  S[i] = bits;
}

// x dilation by one (clamped at the row ends)
__global__ void k_dil_x(const unsigned* __restrict__ in, unsigned* __restrict__ out, int nx, int W, long long nwords) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nwords) return;
  const int w = (int)(i % W);
  const unsigned s = in[i];
  const unsigned lo = w > 0 ? in[i - 1] >> 31 : 0u;
  const unsigned hi = w < W - 1 ? in[i + 1] << 31 : 0u;
  out[i] = (s | (s << 1) | (s >> 1) | lo | hi) & valid_mask(w, W, nx);
}

// y or z dilation by one (clamped): stride = W (y) or W*ny (z)
__global__ void k_dil_rows(const unsigned* __restrict__ in, unsigned* __restrict__ out, int W, int ny, int nz,
                           int axis, long long nwords) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nwords) return;
  const long long row = i / W;
  const int y = (int)(row % ny), z = (int)(row / ny);
  unsigned v = in[i];
  if (axis == 1) {
    if (y > 0) v |= in[i - W];
    if (y < ny - 1) v |= in[i + W];
  } else {
    const long long st = (long long)W * ny;
    if (z > 0) v |= in[i - st];
    if (z < nz - 1) v |= in[i + st];
  }
  out[i] = v;
}

// Exterior seeds: the six faces, minus the barrier.
__global__ void k_flood_init(const unsigned* __restrict__ B, unsigned* __restrict__ E, int nx, int ny, int nz, int W,
                             long long nwords) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nwords) return;
  const long long row = i / W;
  const int w = (int)(i % W);
  const int y = (int)(row % ny), z = (int)(row / ny);
  const unsigned vm = valid_mask(w, W, nx);
  unsigned s;
  if (y == 0 || y == ny - 1 || z == 0 || z == nz - 1) {
    s = vm;
  } else {
    s = 0;
    if (w == 0) s |= 1u;
    if (w == (nx - 1) / 32) s |= 1u << ((nx - 1) % 32);
  }
  E[i] = s & ~B[i] & vm;
}

// Fill the free runs of a word upward (toward higher bits) from the seeds:
// U = S | (F & ((F + S) ^ F ^ S)), S a subset of F.
__device__ __forceinline__ unsigned fill_up(unsigned F, unsigned S) { return S | (F & ((F + S) ^ F ^ S)); }

// One monotone pass: seeds from the 4 y/z neighbour rows, then full
// propagation along x (upward sweep, then downward sweep with bit reversal).
// Rows are updated in place; reading a neighbour mid-update only sees a
// subset of its final bits, so the fixed point is the reference's set.
__global__ void k_flood_pass(const unsigned* __restrict__ B, unsigned* E, int nx, int ny, int nz, int W,
                             int* changed) {
  const long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= (long long)ny * nz) return;
  const int y = (int)(row % ny), z = (int)(row / ny);
  unsigned* e = E + row * W;
  const unsigned* b = B + row * W;
  const long long sy = W, sz = (long long)W * ny;
  bool any = false;
  unsigned carry = 0;
  // upward sweep (x increasing); seeds gathered on the fly
  for (int w = 0; w < W; ++w) {
    const unsigned F = ~b[w] & valid_mask(w, W, nx);
    unsigned s = e[w];
    if (y > 0) s |= e[w - sy];
    if (y < ny - 1) s |= e[w + sy];
    if (z > 0) s |= e[w - sz];
    if (z < nz - 1) s |= e[w + sz];
    s = (s | carry) & F;
    const unsigned u = fill_up(F, s);
    carry = (u >> 31) & 1u;
    if (u != e[w]) { e[w] = u; any = true; }
  }
  carry = 0;
  for (int w = W - 1; w >= 0; --w) {
    const unsigned F = ~b[w] & valid_mask(w, W, nx);
    const unsigned s = (e[w] | (carry << 31)) & F;
    const unsigned u = __brev(fill_up(__brev(F), __brev(s)));
    carry = u & 1u;
    if (u != e[w]) { e[w] = u; any = true; }
  }
  if (any) *changed = 1;
}

// Skin recovery: E |= (6-neighbours of E_before) & ~S.
__global__ void k_skin(const unsigned* __restrict__ E0, const unsigned* __restrict__ S, unsigned* __restrict__ E,
                       int nx, int ny, int nz, int W, long long nwords) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nwords) return;
  const long long row = i / W;
  const int w = (int)(i % W);
  const int y = (int)(row % ny), z = (int)(row / ny);
  const unsigned e = E0[i];
  unsigned g = (e << 1) | (e >> 1);
  if (w > 0) g |= E0[i - 1] >> 31;
  if (w < W - 1) g |= E0[i + 1] << 31;
  if (y > 0) g |= E0[i - W];
  if (y < ny - 1) g |= E0[i + W];
  const long long st = (long long)W * ny;
  if (z > 0) g |= E0[i - st];
  if (z < nz - 1) g |= E0[i + st];
  E[i] = (e | (g & ~S[i])) & valid_mask(w, W, nx);
}

// Classes (src/geom/voxel.js:401-407) and the signed band distance (:409-415).
__global__ void k_classify(const unsigned* __restrict__ S, const unsigned* __restrict__ E,
                           const unsigned* __restrict__ dist2, int nx, int W, long long N, float fora_banda,
                           uint8_t* __restrict__ tipo, float* __restrict__ sdf, unsigned long long* counts) {
  const long long cell = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned nc = 0, nd = 0;
  if (cell < N) {
    const long long row = cell / nx;
    const int x = (int)(cell % nx);
    const long long wi = row * W + (x >> 5);
    const unsigned bit = 1u << (x & 31);
    uint8_t t = 0;
    if (S[wi] & bit) { t = 1; nc = 1; }
    else if (!(E[wi] & bit)) { t = 2; nd = 1; }
    tipo[cell] = t;
    if (sdf) {
      const float d2 = __uint_as_float(dist2[cell]);
      const float d = isinf(d2) ? fora_banda : sqrtf(d2);
      sdf[cell] = t == 0 ? d : -d;
    }
  }
  nc = __reduce_add_sync(0xffffffffu, nc);
  nd = __reduce_add_sync(0xffffffffu, nd);
  if ((threadIdx.x & 31) == 0) {
    if (nc) atomicAdd(counts, (unsigned long long)nc);
    if (nd) atomicAdd(counts + 1, (unsigned long long)nd);
  }
}

struct DevBuf {
  std::vector<void*> ptrs;
  ~DevBuf() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <typename T>
  cudaError_t alloc(T** p, size_t bytes) {
    cudaError_t e = cudaMalloc((void**)p, bytes);
    if (e == cudaSuccess) ptrs.push_back(*p);
    return e;
  }
};

int vfail(int code, const std::string& msg) { return lbm_internal_fail(code, msg.c_str()); }

#define VCK(call, what)                                                                                     \
  do {                                                                                                      \
    cudaError_t _e = (call);                                                                                \
    if (_e != cudaSuccess) {                                                                                \
      cudaGetLastError();                                                                                   \
      return vfail(_e == cudaErrorMemoryAllocation ? LBM_ENOMEM : LBM_ECUDA,                                \
                   std::string(what) + ": " + cudaGetErrorString(_e));                                      \
    }                                                                                                       \
  } while (0)

inline unsigned blocks(long long n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

extern "C" int vox_voxelize(const float* pos, size_t nvert, const uint32_t* idx, size_t ntri, const lbm_dims* dims,
                            float band, int seal, uint8_t* tipo_out, float* sdf_out, vox_stats* stats) {
  if (!dims || !tipo_out || (ntri && (!pos || !idx))) return vfail(LBM_EINVAL, "null argument");
  const int nx = dims->nx, ny = dims->ny, nz = dims->nz;
  if (nx < 1 || ny < 1 || nz < 1) return vfail(LBM_EINVAL, "grid dimensions must be >= 1");
  if (!(band >= 0.0f) || !std::isfinite(band)) return vfail(LBM_EINVAL, "band must be finite and >= 0");
  const long long N = (long long)nx * ny * nz;
  const double banda = band;

  // Triangle prepass on the host in fp64, the reference's bbox arithmetic
  // (src/geom/voxel.js:185-201).
  std::vector<Tri> tris;
  tris.reserve(ntri);
  long long fora = 0;
  for (size_t t = 0; t < ntri; ++t) {
    const uint32_t i0 = idx[3 * t], i1 = idx[3 * t + 1], i2 = idx[3 * t + 2];
    if (i0 >= nvert || i1 >= nvert || i2 >= nvert) {
      char buf[128];
      snprintf(buf, sizeof buf, "triangle %zu references vertex %u beyond %zu", t, std::max(i0, std::max(i1, i2)), nvert);
      return vfail(LBM_EINVAL, buf);
    }
    Tri T;
    const uint32_t ids[3] = {i0, i1, i2};
    double v[9];
    for (int q = 0; q < 3; ++q)
      for (int a = 0; a < 3; ++a) {
        T.v[3 * q + a] = pos[3 * (size_t)ids[q] + a];
        v[3 * q + a] = (double)T.v[3 * q + a];
      }
    const double sum = v[0] + v[1] + v[2] + v[3] + v[4] + v[5] + v[6] + v[7] + v[8];
    if (!std::isfinite(sum)) continue;
    const int n[3] = {nx, ny, nz};
    int r0[3], r1[3];
    for (int a = 0; a < 3; ++a) {
      const double lo = std::floor(std::min(std::min(v[a], v[3 + a]), v[6 + a]) - banda);
      const double hi = std::ceil(std::max(std::max(v[a], v[3 + a]), v[6 + a]) + banda);
      const double l = lo > 0 ? lo : 0;
      const double u = hi < n[a] - 1 ? hi : n[a] - 1;
      r0[a] = l > 2147483647.0 ? 2147483647 : (int)l;
      r1[a] = u < -2147483647.0 ? -2147483647 : (int)u;
    }
    if (r1[0] < r0[0] || r1[1] < r0[1] || r1[2] < r0[2]) { fora++; continue; }
    for (int a = 0; a < 3; ++a) { T.box[a] = r0[a]; T.box[3 + a] = r1[a]; }
    // shape factor of the distance computation
    const double ab[3] = {v[3] - v[0], v[4] - v[1], v[5] - v[2]};
    const double ac[3] = {v[6] - v[0], v[7] - v[1], v[8] - v[2]};
    const double cr[3] = {ab[1] * ac[2] - ab[2] * ac[1], ab[2] * ac[0] - ab[0] * ac[2], ab[0] * ac[1] - ab[1] * ac[0]};
    const double A = cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2];
    const double L = (ab[0] * ab[0] + ab[1] * ab[1] + ab[2] * ab[2]) * (ac[0] * ac[0] + ac[1] * ac[1] + ac[2] * ac[2]);
    const double kappa = A > 0 ? L / A : INFINITY;
    // shape factor above 16: the fp32 distance loses too many digits; such
    // triangles (slivers, near-degenerate) go to the fp64 kernel whole
    T.kappa = (kappa <= 16.0) ? (float)std::max(1.0, kappa) : -1.0f;
    T.id = (int)t;
    tris.push_back(T);
  }

  cudaStream_t st;
  VCK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "stream");
  struct StreamGuard { cudaStream_t s; ~StreamGuard() { cudaStreamSynchronize(s); cudaStreamDestroy(s); } } sg{st};
  cudaEvent_t ev[4];
  for (auto& e : ev) VCK(cudaEventCreate(&e), "event");
  struct EvGuard { cudaEvent_t* e; ~EvGuard() { for (int i = 0; i < 4; ++i) cudaEventDestroy(e[i]); } } eg{ev};

  DevBuf mem;
  const int W = (nx + 31) / 32;
  const long long rows = (long long)ny * nz;
  const long long nwords = rows * W;
  const long long cap = std::max<long long>(1 << 16, (long long)tris.size() * 8);
  Tri* d_tris = nullptr;
  uint8_t* d_flags = nullptr;
  unsigned* d_dist2 = nullptr;
  Deferred* d_def = nullptr;
  unsigned long long* d_cnt = nullptr;   // [0] deferred, [1] pairs, [2] casca, [3] dentro
  unsigned *S, *B, *T1, *E, *E0;
  int* d_changed = nullptr;
  uint8_t* d_tipo = nullptr;
  float* d_sdf = nullptr;
  VCK(mem.alloc(&d_tris, sizeof(Tri) * std::max<size_t>(1, tris.size())), "triangle upload");
  VCK(mem.alloc(&d_flags, (size_t)N), "shell flags");
  VCK(mem.alloc(&d_dist2, sizeof(unsigned) * (size_t)N), "distance band");
  VCK(mem.alloc(&d_def, sizeof(Deferred) * (size_t)cap), "deferred pairs");
  VCK(mem.alloc(&d_cnt, 4 * sizeof(unsigned long long)), "counters");
  VCK(mem.alloc(&S, 4 * (size_t)nwords), "bit rows");
  VCK(mem.alloc(&B, 4 * (size_t)nwords), "bit rows");
  VCK(mem.alloc(&T1, 4 * (size_t)nwords), "bit rows");
  VCK(mem.alloc(&E, 4 * (size_t)nwords), "bit rows");
  VCK(mem.alloc(&E0, 4 * (size_t)nwords), "bit rows");
  VCK(mem.alloc(&d_changed, sizeof(int)), "flag");
  VCK(mem.alloc(&d_tipo, (size_t)N), "classes");
  if (sdf_out) VCK(mem.alloc(&d_sdf, sizeof(float) * (size_t)N), "signed distance");

  VCK(cudaEventRecord(ev[0], st), "event");
  if (!tris.empty())
    VCK(cudaMemcpyAsync(d_tris, tris.data(), sizeof(Tri) * tris.size(), cudaMemcpyHostToDevice, st), "triangle upload");
  VCK(cudaMemsetAsync(d_flags, 0, (size_t)N, st), "clear");
  k_fill_u32<<<blocks(N, 256), 256, 0, st>>>(d_dist2, 0x7f800000u, N);   // +inf (Float32Array.fill(Infinity))
  VCK(cudaMemsetAsync(d_cnt, 0, 4 * sizeof(unsigned long long), st), "clear");
  const int ntr = (int)tris.size();
  std::vector<int> f64list;
  long long f64pairs = 0;
  for (int t = 0; t < ntr; ++t)
    if (tris[t].kappa < 0.0f) {
      f64list.push_back(t);
      f64pairs += (long long)(tris[t].box[3] - tris[t].box[0] + 1) * (tris[t].box[4] - tris[t].box[1] + 1) *
                  (tris[t].box[5] - tris[t].box[2] + 1);
    }
  int* d_f64 = nullptr;
  VCK(mem.alloc(&d_f64, sizeof(int) * std::max<size_t>(1, f64list.size())), "fp64 triangle list");
  if (!f64list.empty()) {
    VCK(cudaMemcpyAsync(d_f64, f64list.data(), sizeof(int) * f64list.size(), cudaMemcpyHostToDevice, st),
        "fp64 list upload");
    k_raster_f64<<<blocks((long long)f64list.size() * 32, 128), 128, 0, st>>>(d_tris, d_f64, (int)f64list.size(),
                                                                           nx, ny, d_flags, d_dist2);
    VCK(cudaGetLastError(), "fp64 raster launch");
  }
  if (ntr > 0) {
    k_raster<<<blocks((long long)ntr * 32, 128), 128, 0, st>>>(d_tris, ntr, nx, ny, d_flags, d_dist2, d_def, d_cnt,
                                                               cap, d_cnt + 1);
    VCK(cudaGetLastError(), "raster launch");
  }
  unsigned long long h_cnt[4];
  VCK(cudaMemcpyAsync(h_cnt, d_cnt, sizeof h_cnt, cudaMemcpyDeviceToHost, st), "counter download");
  VCK(cudaStreamSynchronize(st), "raster");
  const long long ndef = (long long)h_cnt[0];
  if (ndef > cap) {
    char buf[160];
    snprintf(buf, sizeof buf, "%lld undecided (triangle, voxel) pairs exceed the list of %lld", ndef, cap);
    return vfail(LBM_ENOMEM, buf);
  }
  if (ndef > 0) {
    k_tiebreak<<<blocks(ndef, 128), 128, 0, st>>>(d_tris, d_def, ndef, nx, ny, d_flags);
    VCK(cudaGetLastError(), "tie-break launch");
  }
  VCK(cudaEventRecord(ev[1], st), "event");

  const int tb = 256;
  k_pack<<<blocks(nwords, tb), tb, 0, st>>>(d_flags, S, nx, W, nwords);
  if (seal) {
    k_dil_x<<<blocks(nwords, tb), tb, 0, st>>>(S, T1, nx, W, nwords);
    k_dil_rows<<<blocks(nwords, tb), tb, 0, st>>>(T1, E0, W, ny, nz, 1, nwords);
    k_dil_rows<<<blocks(nwords, tb), tb, 0, st>>>(E0, B, W, ny, nz, 2, nwords);
  } else {
    VCK(cudaMemcpyAsync(B, S, 4 * (size_t)nwords, cudaMemcpyDeviceToDevice, st), "barrier copy");
  }
  k_flood_init<<<blocks(nwords, tb), tb, 0, st>>>(B, E, nx, ny, nz, W, nwords);
  VCK(cudaGetLastError(), "flood init launch");
  // Fixed-point iteration, bounded: every pass that changes nothing ends it.
  const int max_pass = 200000;
  int passes = 0;
  bool converged = false;
  while (passes < max_pass) {
    VCK(cudaMemsetAsync(d_changed, 0, sizeof(int), st), "flag clear");
    for (int k = 0; k < 4; ++k) {
      k_flood_pass<<<blocks(rows, 128), 128, 0, st>>>(B, E, nx, ny, nz, W, d_changed);
      ++passes;
    }
    int h_changed = 1;
    VCK(cudaMemcpyAsync(&h_changed, d_changed, sizeof(int), cudaMemcpyDeviceToHost, st), "flag download");
    VCK(cudaStreamSynchronize(st), "flood pass");
    if (!h_changed) { converged = true; break; }
  }
  if (!converged) return vfail(LBM_ETIMEDOUT, "exterior flood did not converge within 200000 passes");
  if (seal) {
    VCK(cudaMemcpyAsync(E0, E, 4 * (size_t)nwords, cudaMemcpyDeviceToDevice, st), "exterior copy");
    k_skin<<<blocks(nwords, tb), tb, 0, st>>>(E0, S, E, nx, ny, nz, W, nwords);
  }
  VCK(cudaEventRecord(ev[2], st), "event");
  k_classify<<<blocks(N, tb), tb, 0, st>>>(S, E, d_dist2, nx, W, N, band + 1.0f, d_tipo, d_sdf, d_cnt + 2);
  VCK(cudaGetLastError(), "classify launch");
  VCK(cudaMemcpyAsync(tipo_out, d_tipo, (size_t)N, cudaMemcpyDeviceToHost, st), "classes download");
  if (sdf_out) VCK(cudaMemcpyAsync(sdf_out, d_sdf, sizeof(float) * (size_t)N, cudaMemcpyDeviceToHost, st), "sdf download");
  VCK(cudaMemcpyAsync(h_cnt, d_cnt, sizeof h_cnt, cudaMemcpyDeviceToHost, st), "counter download");
  VCK(cudaEventRecord(ev[3], st), "event");
  VCK(cudaStreamSynchronize(st), "voxelize");
  if (stats) {
    stats->n_cells = N;
    stats->n_casca = (long long)h_cnt[2];
    stats->n_dentro = (long long)h_cnt[3];
    stats->n_solido = stats->n_casca + stats->n_dentro;
    stats->triangulo_fora = fora;
    stats->oco_suspeito = ((double)stats->n_dentro < (double)stats->n_casca * 0.25) && stats->n_casca > 500;
    stats->flood_iterations = passes;
    stats->n_pairs = (long long)h_cnt[1];
    stats->n_deferred = ndef + f64pairs;
    cudaEventElapsedTime(&stats->ms_raster, ev[0], ev[1]);
    cudaEventElapsedTime(&stats->ms_flood, ev[1], ev[2]);
    cudaEventElapsedTime(&stats->ms_total, ev[0], ev[3]);
    stats->_pad = 0;
  }
  return LBM_OK;
}

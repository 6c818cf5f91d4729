// lbm_noalloc.cu — momentum-exchange force that allocates nothing.
//
// lbm_forces() sums per-block partial forces in a scratch buffer the solver
// context allocates with cudaMalloc.  Some callers cannot allocate device
// memory at the point where they need a force: real-time loops that must not
// take the implicit device synchronisation of cudaMalloc/cudaFree, and hosts
// that hand the library memory from their own pool (a JavaScript/N-API host
// owning its buffers, a framework allocator).  lbm_forces_noalloc() gives
// them the same force from buffers they already own, with its scratch in the
// file-scope device array below.  Its address is looked up per device
// ordinal, so the device's primary context is the one supported.
//
// Scratch: g_noalloc_partials holds one partial force (3 doubles) per
// (y, z) row of cells, for at most kNoAllocMaxRows rows (1.5 MiB, held by every
// GPU that loads the library until the process exits).  Every call writes all
// the partials it reads, so nothing has to be cleared between calls; the
// array keeps the last call's contents.  Two calls that overlap on the GPU
// (different streams, or different host threads) share the array and race.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "../../include/lbm.h"
#include "lbm_kernels.cuh"

extern "C" int lbm_internal_fail(int code, const char* msg);

namespace {

using namespace lbm;

constexpr int kNoAllocMaxRows = 65536;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_partials[3 * kNoAllocMaxRows];

// One block per (y, z) row; threads stride along x.  Same per-link value as
// k_forces: FLUIDO cells, links whose downstream neighbour is SOLIDO,
// q = 2 (g_i + w_i) in fp32, fp64 accumulation.
__global__ void k_forces_rows(const float* __restrict__ pop, const uint8_t* __restrict__ tipo, int nx, int ny, int nz,
                              long long N, double* __restrict__ partials) {
  const int row = blockIdx.x;
  const int y = row % ny, z = row / ny;
  double fx = 0, fy = 0, fz = 0;
  for (int x = threadIdx.x; x < nx; x += blockDim.x) {
    const int64_t cell = ((int64_t)z * ny + y) * nx + x;
    if (tipo[cell] != FLUIDO) continue;
    const Wrap w = wrap3(x, y, z, nx, ny, nz);
#pragma unroll
    for (int i = 1; i < Q; ++i) {
      if (tipo[nbr(i, +1, x, y, z, w, nx, ny)] != SOLIDO) continue;
      const float q = 2.0f * (pop[(int64_t)i * N + cell] + Lit<float>::w(i));
      fx += (double)(cx(i) * q);
      fy += (double)(cy(i) * q);
      fz += (double)(cz(i) * q);
    }
  }
  __shared__ double sh[3][32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    fx += __shfl_down_sync(0xffffffffu, fx, o);
    fy += __shfl_down_sync(0xffffffffu, fy, o);
    fz += __shfl_down_sync(0xffffffffu, fz, o);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) { sh[0][wid] = fx; sh[1][wid] = fy; sh[2][wid] = fz; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0, b = 0, c = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) { a += sh[0][k]; b += sh[1][k]; c += sh[2][k]; }
    partials[3 * row + 0] = a;
    partials[3 * row + 1] = b;
    partials[3 * row + 2] = c;
  }
}

// Fixed-order single-block sum of the row partials into out[3].
__global__ void k_sum_rows(const double* __restrict__ partials, int nrows, double* __restrict__ out) {
  __shared__ double sh[3][256];
  const int t = threadIdx.x;
  double a = 0, b = 0, c = 0;
  for (int i = t; i < nrows; i += 256) {
    a += partials[3 * i];
    b += partials[3 * i + 1];
    c += partials[3 * i + 2];
  }
  sh[0][t] = a; sh[1][t] = b; sh[2][t] = c;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (t < s) { sh[0][t] += sh[0][t + s]; sh[1][t] += sh[1][t + s]; sh[2][t] += sh[2][t + s]; }
    __syncthreads();
  }
  if (t == 0) { out[0] = sh[0][0]; out[1] = sh[1][0]; out[2] = sh[2][0]; }
}

// Device address of the scratch array, looked up once per device with that
// device current (in host code the symbol is only a host-side stand-in).
std::mutex g_mu;
void* g_scratch_addr[kMaxDevices] = {};

int scratch_for_current_device(double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return lbm_internal_fail(LBM_ECUDA, "cudaGetDevice failed");
  if (dev < 0 || dev >= kMaxDevices) return lbm_internal_fail(LBM_EINVAL, "device ordinal beyond 64");
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_partials);
    if (e != cudaSuccess || !p) {
      char buf[160];
      snprintf(buf, sizeof buf, "cudaGetSymbolAddress of the force scratch failed: %s", cudaGetErrorString(e));
      return lbm_internal_fail(LBM_ECUDA, buf);
    }
    g_scratch_addr[dev] = p;
  }
  *out = static_cast<double*>(g_scratch_addr[dev]);
  return LBM_OK;
}

}  // namespace

extern "C" int lbm_forces_noalloc(const float* pop, const uint8_t* tipo, const lbm_dims* dims, double* f_out,
                                  void* stream) {
  if (!pop || !tipo || !dims || !f_out) return lbm_internal_fail(LBM_EINVAL, "null argument");
  const int nx = dims->nx, ny = dims->ny, nz = dims->nz;
  if (nx < 1 || ny < 1 || nz < 1) return lbm_internal_fail(LBM_EINVAL, "grid dimensions must be >= 1");
  const long long rows = (long long)ny * nz;
  if (rows > kNoAllocMaxRows) {
    char buf[200];
    snprintf(buf, sizeof buf,
             "ny*nz = %lld rows exceeds the %d rows the built-in force scratch holds; use lbm_forces", rows,
             kNoAllocMaxRows);
    return lbm_internal_fail(LBM_EINVAL, buf);
  }
  double* scratch = nullptr;
  int r = scratch_for_current_device(&scratch);
  if (r) return r;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const long long N = (long long)nx * ny * nz;
  k_forces_rows<<<(unsigned)rows, 128, 0, s>>>(pop, tipo, nx, ny, nz, N, scratch);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) {
    k_sum_rows<<<1, 256, 0, s>>>(scratch, (int)rows, f_out);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) {
    char buf[160];
    snprintf(buf, sizeof buf, "force kernel launch failed: %s", cudaGetErrorString(e));
    return lbm_internal_fail(LBM_ECUDA, buf);
  }
  return LBM_OK;
}

// lbm_api.cu — the C ABI of include/lbm.h: solver contexts, the link-word
// builder, deterministic reductions and the dispatch into the per-storage
// kernel instantiations (lbm_inst_*.cu).
//
// Member-by-member counterpart of the reference's SolverWebGPU
// (src/backend/webgpu/solver.js:36-528); each function cites its member.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/lbm.h"
#include "../../include/lbm_closure.h"
#include "../../include/lbm_state.h"
#include "lbm_kernels.cuh"

using namespace lbm;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  char buf[256];
  snprintf(buf, sizeof buf, "%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
  return fail(LBM_ECUDA, buf);
}

#define CK(call, what)                                 \
  do {                                                 \
    cudaError_t _e = (call);                           \
    if (_e != cudaSuccess) return cuda_fail(_e, what); \
  } while (0)

// Per-cell link words (see LINK_* in lbm_core.cuh).
__global__ void k_links(const uint8_t* __restrict__ tipo, uint32_t* __restrict__ link, int nx, int ny, int nz) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= nx || y >= ny) return;
  const int64_t cell = ((int64_t)z * ny + y) * nx + x;
  const Wrap w = wrap3(x, y, z, nx, ny, nz);
  uint32_t bits = 0;
  bool has_body = false, has_wall = false, has_belt = false;
#pragma unroll
  for (int k = 1; k < Q; ++k) {
    const uint32_t t = tipo[nbr(k, -1, x, y, z, w, nx, ny)];
    if (is_solid(t)) {
      bits |= 1u << (k - 1);
      has_body |= t == SOLIDO;
      has_wall |= t == PAREDE;
      has_belt |= t == SOLIDO_MOVEL;
    }
  }
  uint32_t lw = bits | ((uint32_t)tipo[cell] << LINK_CLASS_SHIFT);
  if (has_belt || (has_body && has_wall)) lw |= LINK_SLOW;
  if (has_body && !has_wall && !has_belt) lw |= LINK_BODY;
  link[cell] = lw;
}

// Deterministic single-block sum of n triples: each thread walks a fixed
// stride, then a fixed tree.  out[3].
// Per step k: the kForceSlots copies of the fused force summed in slot order.
__global__ void k_sum_slots(const double* __restrict__ slots, int n, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3 * n) return;
  const int k = i / 3, a = i % 3;
  const double* h = slots + (size_t)k * 3 * kForceSlots;
  double f = 0.0;
  for (int q = 0; q < kForceSlots; ++q) f += h[3 * q + a];
  out[i] = f;
}

__global__ void k_reduce3(const double* __restrict__ part, int64_t n, double* __restrict__ out) {
  __shared__ double sh[3][256];
  const int t = threadIdx.x;
  double a = 0, b = 0, c = 0;
  for (int64_t i = t; i < n; i += 256) {
    a += part[3 * i];
    b += part[3 * i + 1];
    c += part[3 * i + 2];
  }
  sh[0][t] = a; sh[1][t] = b; sh[2][t] = c;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (t < s) {
      sh[0][t] += sh[0][t + s];
      sh[1][t] += sh[1][t + s];
      sh[2][t] += sh[2][t + s];
    }
    __syncthreads();
  }
  if (t == 0) { out[0] = sh[0][0]; out[1] = sh[1][0]; out[2] = sh[2][0]; }
}

}  // namespace

namespace lbm {
// Link-word builder for other units (batched tunnels).
cudaError_t launch_links(const uint8_t* tipo, uint32_t* link, int nx, int ny, int nz, cudaStream_t s) {
  const int bx = nx < 64 ? ((nx + 31) / 32) * 32 : 64;
  k_links<<<dim3((nx + bx - 1) / bx, ny, nz), dim3(bx, 1, 1), 0, s>>>(tipo, link, nx, ny, nz);
  return cudaGetLastError();
}
cudaError_t launch_reduce3(const double* part, int64_t n, double* out, cudaStream_t s) {
  k_reduce3<<<1, 256, 0, s>>>(part, n, out);
  return cudaGetLastError();
}
// The nz inlet boundary-layer factors of thickness bl in the arithmetic type
// of the storage form (double for the fp64 reference form, else float), as
// raw bytes; returns whether any factor differs from 1.
bool bl_table(float bl, int nz, bool f64, std::vector<unsigned char>& out) {
  const size_t el = f64 ? sizeof(double) : sizeof(float);
  out.assign(el * (size_t)nz, 0);
  bool any = false;
  for (int z = 0; z < nz; ++z) {
    if (f64) {
      const double v = bl_factor_host<double>(bl, z);
      any |= v != 1.0;
      memcpy(out.data() + el * z, &v, el);
    } else {
      const float v = bl_factor_host<float>(bl, z);
      any |= v != 1.0f;
      memcpy(out.data() + el * z, &v, el);
    }
  }
  return any;
}
}  // namespace lbm

struct lbm_ctx {
  lbm_dims dims{};
  int64_t N = 0;
  int storage = LBM_F32;
  int flags = 0;
  bool inplace = true;
  bool aos = false;       // in-place set in the AoSoA layout (lbm_kernels.cuh, elem_off)
  int aos_b = 32;         // its block width (cells along x)
  int nxp = 0;            // its row length: nx rounded up to the block width (nx for SoA)
  int64_t nset = 0;       // cells per population slot, padding included
  Ops ops{};
  void* pop = nullptr;    // in-place set, or ping-pong front
  void* pop2 = nullptr;   // ping-pong back
  uint8_t* tipo = nullptr;
  uint32_t* link = nullptr;
  float4* macros = nullptr;
  void* blf = nullptr;         // nz inlet boundary-layer factors (arithmetic type)
  bool blf_on = false;         // some factor differs from 1
  bool blf_set = false;        // blf holds the factors of thickness blf_bl
  float blf_bl = 0.0f;
  double* partials = nullptr;
  int64_t npart = 0;
  double* red = nullptr;       // 3 doubles
  double* fbuf = nullptr;      // per-step fused forces
  int64_t fbuf_cap = 0;        // in steps
  double* stage = nullptr;     // N doubles for set/get
  double* hpin = nullptr;      // pinned host staging for force read-backs
  cudaEvent_t mac_evt = nullptr;   // completion of the last asynchronous macros read-back
  // asynchronous force read-backs: a ring of events, one per ticket
  static constexpr int kTickets = 16;
  cudaEvent_t frc_evt[kTickets] = {};
  int64_t frc_ticket = 0;          // last issued
  double* fsum = nullptr;          // 3 doubles per step, summed on the device
  int64_t fsum_cap = 0;
  int64_t hpin_cap = 0;        // in doubles
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  Params P{};
  bool configured = false, types_set = false, state_set = false;
  int64_t steps = 0;
  int block_x = 0, block_y = 1;
  int occ = 8;
  int pipe = 0;
  int64_t dev_bytes = 0;
  // learned closure
  lbm::MlpFrag* clo = nullptr;            // fragments of the network (device)
  unsigned long long* clo_fb = nullptr;   // fallback counter (device), then the timeout flag
  int64_t clo_steps = 0;                  // network evaluations since the last stats call
  int64_t n_fluido = 0;                   // FLUIDO cells of the current types
  int clo_engine = 0;                     // 0 warp mma.sync, 1 CTA tcgen05
  float* clo_nu = nullptr;                // held nu_t per cell (closure evaluated every k > 1 steps)
  int clo_since = -1;                     // steps since the last evaluation; -1: evaluate next
  int clo_coef = 0;                       // the network gives Cs^2 (1) or nu_t (0)
  lbm::CloConst clo_k{};                  // feature range, normalisation, output bounds
};

namespace lbm {
void closure_pack(const closure_weights* w, MlpFrag* F);
cudaError_t closure_samples_launch(const float4* mac, const uint8_t* tipo, int nx, int ny, int nz, float tau0c,
                                   float s_min, int x0, int x1, float* feats_dev, float* target_dev, cudaStream_t s);
}

namespace {

// Launch shapes chosen by lbm_autotune, per (nx, ny, nz, storage, flags,
// layout), for this process: a context created later with the same key
// starts with the measured shape.
struct Shape {
  int bx, by, occ, pipe;
};
using ShapeKey = std::tuple<int, int, int, int, int, int>;
std::mutex g_tune_mu;
std::map<ShapeKey, Shape> g_tuned;
// Layouts chosen by lbm_autotune_layout, per (nx, ny, nz, storage, flags).
using LayoutKey = std::tuple<int, int, int, int, int>;
std::map<LayoutKey, bool> g_layout;

Ops ops_for(int storage) {
  switch (storage) {
    case LBM_F32: return ops_f32();
    case LBM_F64: return ops_f64();
    case LBM_F16S: return ops_f16s();
    case LBM_F16SR: return ops_f16sr();
    case LBM_BF16SR: return ops_bf16sr();
    default: return ops_bf16s();
  }
}

bool is_sr(int storage) { return storage == LBM_F16SR || storage == LBM_BF16SR; }

Launch cell_launch(const lbm_ctx* c) {
  // The in-place step is compiled for at most 128 threads per block.
  int bx = c->block_x;
  if (bx <= 0) {
    bx = 64;
    const int rx = ((c->dims.nx + 31) / 32) * 32;
    if (rx < bx) bx = rx;
  }
  int by = c->block_y > 0 ? c->block_y : 1;
  while (bx * by > 128) by = std::max(1, by / 2);
  Launch L;
  L.occ = c->occ;
  L.pipe = c->pipe;
  L.block = dim3(bx, by, 1);
  L.grid = dim3((c->dims.nx + bx - 1) / bx, (c->dims.ny + by - 1) / by, c->dims.nz);
  return L;
}

// Population set layout as reported by lbm_get_info and stored in a
// checkpoint: 0 in-place SoA, 1 ping-pong, 2 in-place AoSoA in blocks of 32
// cells, 3 in blocks of 64.
int layout_code(const lbm_ctx* c) {
  if (!c->inplace) return 1;
  if (!c->aos) return 0;
  return c->aos_b == 64 ? 3 : 2;
}

Dev dev_of(const lbm_ctx* c) {
  Dev d;
  d.nx = c->dims.nx; d.ny = c->dims.ny; d.nz = c->dims.nz;
  d.N = c->N;
  d.pop = c->pop; d.pop2 = c->pop2;
  d.tipo = c->tipo; d.link = c->link;
  d.macros = c->macros;
  d.force = nullptr;
  d.blf = c->blf_on ? c->blf : nullptr;
  d.aos = c->aos ? c->aos_b : 0;
  d.nxp = c->nxp;
  d.seed = sr_seed(c->steps);
  d.seed_base = nullptr;
  return d;
}

int dalloc(lbm_ctx* c, void** p, size_t bytes, const char* what) {
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    char buf[256];
    snprintf(buf, sizeof buf, "device allocation of %.3f GB for %s failed (%dx%dx%d): %s",
             bytes / 1e9, what, c->dims.nx, c->dims.ny, c->dims.nz, cudaGetErrorString(e));
    *p = nullptr;
    return fail(LBM_ENOMEM, buf);
  }
  c->dev_bytes += (int64_t)bytes;
  return LBM_OK;
}

int ensure_macros(lbm_ctx* c) {
  if (c->macros) return LBM_OK;
  return dalloc(c, (void**)&c->macros, sizeof(float4) * (size_t)c->N, "macros");
}

int ensure_partials(lbm_ctx* c, int64_t n) {
  if (c->npart >= n) return LBM_OK;
  if (c->partials) { cudaFree(c->partials); c->dev_bytes -= 3 * sizeof(double) * c->npart; c->partials = nullptr; }
  int r = dalloc(c, (void**)&c->partials, 3 * sizeof(double) * (size_t)n, "reduction partials");
  if (r) { c->npart = 0; return r; }
  c->npart = n;
  return LBM_OK;
}

int ensure_stage(lbm_ctx* c) {
  if (c->stage) return LBM_OK;
  return dalloc(c, (void**)&c->stage, sizeof(double) * (size_t)c->N, "state staging");
}

int parity(const lbm_ctx* c) { return c->inplace ? (int)(c->steps & 1) : 0; }

// Pinned host staging of at least n doubles: a device-to-host copy into
// pinned memory is a plain DMA, without the driver's pageable bounce buffer.
int ensure_pinned(lbm_ctx* c, int64_t n) {
  if (c->hpin_cap >= n) return LBM_OK;
  if (c->hpin) { cudaFreeHost(c->hpin); c->hpin = nullptr; c->hpin_cap = 0; }
  const int64_t cap = std::max<int64_t>(n, 64);
  cudaError_t e = cudaHostAlloc((void**)&c->hpin, sizeof(double) * (size_t)cap, cudaHostAllocDefault);
  if (e != cudaSuccess) {
    cudaGetLastError();
    c->hpin = nullptr;
    return fail(LBM_ENOMEM, std::string("pinned host staging: ") + cudaGetErrorString(e));
  }
  c->hpin_cap = cap;
  return LBM_OK;
}

int check_ready(lbm_ctx* c, bool need_cfg) {
  if (!c) return fail(LBM_EINVAL, "null context");
  if (!c->types_set) return fail(LBM_ESTATE, "cell types not set (call lbm_set_types first)");
  if (need_cfg && !c->configured) return fail(LBM_ESTATE, "parameters not set (call lbm_configure first)");
  return LBM_OK;
}

// One step; mac/frc select the kernel variant.  force: 3 doubles or null.
int launch_step(lbm_ctx* c, bool mac, double* force) {
  Dev d = dev_of(c);
  d.force = force;
  if (c->P.closure >= 1) {
    if (!c->clo) return fail(LBM_ESTATE, "closure >= 1 but no network set (call lbm_set_closure first)");
    if (!c->inplace || (c->flags & LBM_FLAG_STRICT) || !c->ops.step_closure)
      return fail(LBM_ENOTSUP, "the learned closure runs in the in-place FAST step with fp32 arithmetic only");
    if ((int64_t)Q * c->N >= (int64_t)INT32_MAX)
      return fail(LBM_ENOTSUP, "the learned closure addresses the set with 32-bit indices (19 N < 2^31 cells)");
    const int every = c->P.closure;
    int mode = 0;
    if (every > 1) {
      if (!c->clo_nu) {
        int r = dalloc(c, (void**)&c->clo_nu, sizeof(float) * (size_t)c->N, "held eddy viscosity");
        if (r) return r;
        c->clo_since = -1;
      }
      mode = (c->clo_since < 0 || c->clo_since >= every - 1) ? 1 : 2;
    }
    CloArgs A;
    A.F = c->clo;
    A.nfb = c->clo_fb;
    A.err = reinterpret_cast<unsigned*>(c->clo_fb + 1);
    A.nu = c->clo_nu;
    A.omega0 = 1.0f / make_uni<float>(c->P).tau0;
    A.coef = c->clo_coef;
    A.K = c->clo_k;
    cudaError_t e = c->ops.step_closure(d, c->P, parity(c), mac, force != nullptr, c->clo_engine, mode, A,
                                        cell_launch(c), c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "closure step kernel launch");
    c->steps++;
    if (mode != 2) c->clo_steps++;
    if (every > 1) c->clo_since = mode == 1 ? 0 : c->clo_since + 1;
    return LBM_OK;
  }
  cudaError_t e = c->ops.step(d, c->P, parity(c), c->inplace, mac, force != nullptr, !(c->flags & LBM_FLAG_STRICT),
                              cell_launch(c), c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "step kernel launch");
  if (!c->inplace) std::swap(c->pop, c->pop2);
  c->steps++;
  return LBM_OK;
}

}  // namespace

extern "C" {

const char* lbm_last_error(void) { return g_err.c_str(); }

// Shared error channel for the other units of the library (voxelizer).
int lbm_internal_fail(int code, const char* msg) { return fail(code, msg); }

int lbm_create(const lbm_dims* dims, int storage, int flags, lbm_ctx** out) {
  if (!dims || !out) return fail(LBM_EINVAL, "null argument");
  *out = nullptr;
  if (dims->nx < 1 || dims->ny < 1 || dims->nz < 1) return fail(LBM_EINVAL, "grid dimensions must be >= 1");
  if (dims->ny > 65535 * 256 || dims->nz > 65535) return fail(LBM_EINVAL, "grid too large for the launch shape");
  if (storage < LBM_F32 || storage > LBM_BF16SR) return fail(LBM_EINVAL, "unknown storage form");
  if (is_sr(storage) && (flags & LBM_FLAG_PINGPONG))
    return fail(LBM_ENOTSUP, "the stochastically rounded storage forms use the in-place set only");
  if (flags & ~(LBM_FLAG_WRITE_MACROS | LBM_FLAG_PINGPONG | LBM_FLAG_STRICT | LBM_FLAG_SOA | LBM_FLAG_AOS))
    return fail(LBM_EINVAL, "unknown flag bits");
  if ((flags & LBM_FLAG_SOA) && (flags & LBM_FLAG_AOS)) return fail(LBM_EINVAL, "LBM_FLAG_SOA and LBM_FLAG_AOS together");
  lbm_ctx* c = new lbm_ctx();
  c->dims = *dims;
  c->N = (int64_t)dims->nx * dims->ny * dims->nz;
  c->storage = storage;
  c->flags = flags;
  c->inplace = !(flags & LBM_FLAG_PINGPONG);
  // AoSoA where the in-place FAST step can use it (fp32 arithmetic, 32-bit
  // element offsets over the padded rows), in blocks of 32 cells for fp32
  // and 64 for the 16-bit forms (one 128-byte line per slot row), rows
  // padded to a multiple of the block; the default unless the layout asked
  // for or the one lbm_autotune_layout measured faster for this grid says
  // otherwise (measured on GB300: faster than SoA for every form)
  const bool is16 = storage != LBM_F32 && storage != LBM_F64;
  const int ab = is16 ? 64 : 32;
  const int nxp_a = (dims->nx + ab - 1) / ab * ab;
  const bool aos_ok = c->inplace && !(flags & LBM_FLAG_STRICT) && storage != LBM_F64 &&
                      (int64_t)Q * nxp_a * dims->ny * dims->nz < (int64_t)INT32_MAX;
  bool want_aos = true;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_layout.find(LayoutKey(dims->nx, dims->ny, dims->nz, storage, flags & ~LBM_FLAG_WRITE_MACROS));
    if (it != g_layout.end()) want_aos = it->second;
  }
  if (flags & LBM_FLAG_AOS) want_aos = true;
  if (flags & LBM_FLAG_SOA) want_aos = false;
  c->aos = aos_ok && want_aos;
  c->aos_b = ab;
  c->nxp = c->aos ? nxp_a : dims->nx;
  c->nset = (int64_t)c->nxp * dims->ny * dims->nz;
  c->ops = ops_for(storage);
  const size_t set_bytes = (size_t)c->nset * Q * c->ops.elem_bytes;
  int r = dalloc(c, &c->pop, set_bytes, "populations");
  if (!r && !c->inplace) r = dalloc(c, &c->pop2, set_bytes, "second population set");
  if (!r) r = dalloc(c, (void**)&c->tipo, (size_t)c->N, "cell types");
  if (!r && c->inplace) r = dalloc(c, (void**)&c->link, sizeof(uint32_t) * (size_t)c->N, "link words");
  if (!r) r = dalloc(c, (void**)&c->red, 3 * sizeof(double), "reduction result");
  if (!r) r = dalloc(c, &c->blf, sizeof(double) * (size_t)dims->nz, "inlet boundary-layer factors");
  if (!r && (flags & LBM_FLAG_WRITE_MACROS)) r = ensure_macros(c);
  if (r) { lbm_destroy(c); return r; }
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tuned.find(ShapeKey(dims->nx, dims->ny, dims->nz, storage, flags & ~LBM_FLAG_WRITE_MACROS, c->aos));
    if (it != g_tuned.end()) {
      c->block_x = it->second.bx; c->block_y = it->second.by; c->occ = it->second.occ; c->pipe = it->second.pipe;
    }
  }
  cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { lbm_destroy(c); return cuda_fail(e, "cudaStreamCreate"); }
  c->own_stream = true;
  // Rest state: g = 0 everywhere (src/core/lattice.js:32-34).
  e = cudaMemsetAsync(c->pop, 0, set_bytes, c->stream);
  if (e == cudaSuccess && c->pop2) e = cudaMemsetAsync(c->pop2, 0, set_bytes, c->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(c->tipo, 0, (size_t)c->N, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) { lbm_destroy(c); return cuda_fail(e, "initial clear"); }
  *out = c;
  return LBM_OK;
}

int lbm_destroy(lbm_ctx* c) {
  if (!c) return fail(LBM_EINVAL, "null context");
  if (c->stream) cudaStreamSynchronize(c->stream);
  void* ps[] = {c->pop, c->pop2, c->tipo, c->link, c->macros, c->partials, c->red, c->fbuf, c->stage, c->clo, c->clo_fb,
                c->clo_nu, c->blf};
  for (void* p : ps)
    if (p) cudaFree(p);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  if (c->hpin) cudaFreeHost(c->hpin);
  if (c->mac_evt) cudaEventDestroy(c->mac_evt);
  for (int k = 0; k < lbm_ctx::kTickets; ++k)
    if (c->frc_evt[k]) cudaEventDestroy(c->frc_evt[k]);
  if (c->fsum) cudaFree(c->fsum);
  delete c;
  return LBM_OK;
}

int lbm_set_stream(lbm_ctx* c, void* s) {
  if (!c) return fail(LBM_EINVAL, "null context");
  CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
  if (c->own_stream) cudaStreamDestroy(c->stream);
  c->stream = static_cast<cudaStream_t>(s);
  c->own_stream = false;
  return LBM_OK;
}

int lbm_configure(lbm_ctx* c, const lbm_params* p) {
  if (!c || !p) return fail(LBM_EINVAL, "null argument");
  if (p->closure < 0 || p->closure > 4096) return fail(LBM_EINVAL, "closure must be 0 (Smagorinsky) or 1..4096");
  Params P;
  P.omega_plus = p->omega_plus; P.magic = p->magic; P.les_cs = p->les_cs;
  for (int a = 0; a < 3; ++a) { P.belt[a] = p->belt_u[a]; P.inlet[a] = p->inlet_u[a]; }
  P.sponge_start = p->sponge_start; P.sponge_len = p->sponge_len; P.bl = p->bl_thickness;
  P.closure = p->closure;
  // The boundary-layer table depends on the thickness alone: rebuilt only
  // when it changes (a ramp re-configures the inlet before every step).
  if (!c->blf_set || memcmp(&c->blf_bl, &p->bl_thickness, sizeof(float)) != 0) {
    std::vector<unsigned char> tab;
    const bool on = bl_table(p->bl_thickness, c->dims.nz, c->storage == LBM_F64, tab);
    if (on) {
      CK(cudaMemcpyAsync(c->blf, tab.data(), tab.size(), cudaMemcpyHostToDevice, c->stream), "boundary-layer table upload");
      CK(cudaStreamSynchronize(c->stream), "boundary-layer table upload sync");
    }
    c->blf_on = on;
    c->blf_bl = p->bl_thickness;
    c->blf_set = true;
  }
  c->P = P;
  c->configured = true;
  c->clo_since = -1;
  return LBM_OK;
}

int lbm_set_types(lbm_ctx* c, const uint32_t* tipo, size_t n) {
  if (!c || !tipo) return fail(LBM_EINVAL, "null argument");
  if ((int64_t)n != c->N) {
    char buf[128];
    snprintf(buf, sizeof buf, "cell-type field has %zu entries, expected %lld", n, (long long)c->N);
    return fail(LBM_EINVAL, buf);
  }
  std::vector<uint8_t> t8((size_t)n);
  for (size_t i = 0; i < n; ++i) {
    if (tipo[i] > 7u) {
      char buf[128];
      snprintf(buf, sizeof buf, "cell type %u at index %zu is not a CELULA code (0..7)", tipo[i], i);
      return fail(LBM_EINVAL, buf);
    }
    t8[i] = (uint8_t)tipo[i];
  }
  int64_t nf = 0;
  for (size_t i = 0; i < n; ++i) nf += t8[i] == LBM_FLUIDO;
  c->n_fluido = nf;
  c->clo_since = -1;
  CK(cudaMemcpyAsync(c->tipo, t8.data(), n, cudaMemcpyHostToDevice, c->stream), "types upload");
  if (c->inplace) {
    Launch L = cell_launch(c);
    k_links<<<L.grid, L.block, 0, c->stream>>>(c->tipo, c->link, c->dims.nx, c->dims.ny, c->dims.nz);
    CK(cudaGetLastError(), "link kernel launch");
  }
  CK(cudaStreamSynchronize(c->stream), "types upload sync");
  c->types_set = true;
  return LBM_OK;
}

int lbm_init_equilibrium(lbm_ctx* c) {
  int r = check_ready(c, true);
  if (r) return r;
  c->steps = 0;
  c->clo_since = -1;
  CK(c->ops.init(dev_of(c), c->P, c->inplace, cell_launch(c), c->stream), "init kernel launch");
  c->state_set = true;
  return LBM_OK;
}

int lbm_set_populations(lbm_ctx* c, const double* g, size_t n) {
  if (!c || !g) return fail(LBM_EINVAL, "null argument");
  if ((int64_t)n != Q * c->N) return fail(LBM_EINVAL, "population array must hold 19*N values");
  int r = ensure_stage(c);
  if (r) return r;
  c->steps = 0;
  c->clo_since = -1;
  for (int k = 0; k < Q; ++k) {
    CK(cudaMemcpyAsync(c->stage, g + (size_t)k * c->N, sizeof(double) * c->N, cudaMemcpyHostToDevice, c->stream),
       "population upload");
    CK(c->ops.put_dir(dev_of(c), c->stage, k, 0, c->inplace, cell_launch(c), c->stream), "population scatter");
  }
  CK(cudaStreamSynchronize(c->stream), "population upload sync");
  c->state_set = true;
  return LBM_OK;
}

int lbm_get_populations(lbm_ctx* c, double* g, size_t n) {
  if (!c || !g) return fail(LBM_EINVAL, "null argument");
  if ((int64_t)n != Q * c->N) return fail(LBM_EINVAL, "population array must hold 19*N values");
  int r = ensure_stage(c);
  if (r) return r;
  for (int k = 0; k < Q; ++k) {
    CK(c->ops.get_dir(dev_of(c), c->stage, k, parity(c), c->inplace, cell_launch(c), c->stream), "population gather");
    CK(cudaMemcpyAsync(g + (size_t)k * c->N, c->stage, sizeof(double) * c->N, cudaMemcpyDeviceToHost, c->stream),
       "population download");
    CK(cudaStreamSynchronize(c->stream), "population download sync");
  }
  return LBM_OK;
}

int lbm_step(lbm_ctx* c, int n) {
  int r = check_ready(c, true);
  if (r) return r;
  if (n < 0) return fail(LBM_EINVAL, "negative step count");
  const bool want_mac = (c->flags & LBM_FLAG_WRITE_MACROS) != 0;
  if (want_mac && (r = ensure_macros(c))) return r;
  for (int k = 0; k < n; ++k) {
    r = launch_step(c, want_mac && k == n - 1, nullptr);
    if (r) return r;
  }
  return LBM_OK;
}

int lbm_step_forces(lbm_ctx* c, int n, double* out_f) {
  int r = check_ready(c, true);
  if (r) return r;
  if (n < 0 || (n > 0 && !out_f)) return fail(LBM_EINVAL, "bad step count or null output");
  if (n == 0) return LBM_OK;
  const bool want_mac = (c->flags & LBM_FLAG_WRITE_MACROS) != 0;
  if (want_mac && (r = ensure_macros(c))) return r;
  const size_t per = 3 * (size_t)kForceSlots;   // doubles per step
  if (c->fbuf_cap < n) {
    if (c->fbuf) { cudaFree(c->fbuf); c->dev_bytes -= sizeof(double) * per * c->fbuf_cap; c->fbuf = nullptr; c->fbuf_cap = 0; }
    r = dalloc(c, (void**)&c->fbuf, sizeof(double) * per * (size_t)n, "per-step forces");
    if (r) return r;
    c->fbuf_cap = n;
  }
  CK(cudaMemsetAsync(c->fbuf, 0, sizeof(double) * per * (size_t)n, c->stream), "force buffer clear");
  for (int k = 0; k < n; ++k) {
    r = launch_step(c, want_mac && k == n - 1, c->fbuf + per * (size_t)k);
    if (r) return r;
  }
  if ((r = ensure_pinned(c, (int64_t)(per * (size_t)n)))) return r;
  CK(cudaMemcpyAsync(c->hpin, c->fbuf, sizeof(double) * per * (size_t)n, cudaMemcpyDeviceToHost, c->stream),
     "force download");
  CK(cudaStreamSynchronize(c->stream), "force download sync");
  for (int k = 0; k < n; ++k) {
    const double* h = c->hpin + per * (size_t)k;
    double f[3] = {0.0, 0.0, 0.0};
    for (int q = 0; q < kForceSlots; ++q)
      for (int a = 0; a < 3; ++a) f[a] += h[3 * q + a];
    for (int a = 0; a < 3; ++a) out_f[3 * (size_t)k + a] = f[a];
  }
  return LBM_OK;
}

int lbm_step_forces_async(lbm_ctx* c, int n, double* out_f, int64_t* ticket) {
  int r = check_ready(c, true);
  if (r) return r;
  if (n < 1 || !out_f || !ticket) return fail(LBM_EINVAL, "bad step count or null output");
  const int64_t t = c->frc_ticket + 1;
  const int slot = (int)(t % lbm_ctx::kTickets);
  if (c->frc_evt[slot]) {
    // the ticket that used this event 16 calls ago must have finished
    const cudaError_t q = cudaEventQuery(c->frc_evt[slot]);
    if (q == cudaErrorNotReady) { cudaGetLastError(); return fail(LBM_ESTATE, "16 asynchronous force read-backs already in flight"); }
    if (q != cudaSuccess) return cuda_fail(q, "force event");
  } else {
    CK(cudaEventCreateWithFlags(&c->frc_evt[slot], cudaEventDisableTiming), "event create");
  }
  const bool want_mac = (c->flags & LBM_FLAG_WRITE_MACROS) != 0;
  if (want_mac && (r = ensure_macros(c))) return r;
  const size_t per = 3 * (size_t)kForceSlots;
  if (c->fbuf_cap < n) {
    if (c->fbuf) { cudaFree(c->fbuf); c->dev_bytes -= sizeof(double) * per * c->fbuf_cap; c->fbuf = nullptr; c->fbuf_cap = 0; }
    r = dalloc(c, (void**)&c->fbuf, sizeof(double) * per * (size_t)n, "per-step forces");
    if (r) return r;
    c->fbuf_cap = n;
  }
  if (c->fsum_cap < n) {
    if (c->fsum) { cudaFree(c->fsum); c->dev_bytes -= sizeof(double) * 3 * c->fsum_cap; c->fsum = nullptr; c->fsum_cap = 0; }
    r = dalloc(c, (void**)&c->fsum, sizeof(double) * 3 * (size_t)n, "per-step force sums");
    if (r) return r;
    c->fsum_cap = n;
  }
  CK(cudaMemsetAsync(c->fbuf, 0, sizeof(double) * per * (size_t)n, c->stream), "force buffer clear");
  for (int k = 0; k < n; ++k) {
    r = launch_step(c, want_mac && k == n - 1, c->fbuf + per * (size_t)k);
    if (r) return r;
  }
  k_sum_slots<<<(3 * n + 127) / 128, 128, 0, c->stream>>>(c->fbuf, n, c->fsum);
  CK(cudaGetLastError(), "force sum launch");
  CK(cudaMemcpyAsync(out_f, c->fsum, sizeof(double) * 3 * (size_t)n, cudaMemcpyDeviceToHost, c->stream),
     "force download");
  CK(cudaEventRecord(c->frc_evt[slot], c->stream), "event record");
  c->frc_ticket = t;
  *ticket = t;
  return LBM_OK;
}

int lbm_forces_done(lbm_ctx* c, int64_t ticket, int wait, int* done) {
  if (!c || !done) return fail(LBM_EINVAL, "null argument");
  if (ticket < 1 || ticket > c->frc_ticket) return fail(LBM_EINVAL, "unknown ticket");
  if (ticket <= c->frc_ticket - lbm_ctx::kTickets) { *done = 1; return LBM_OK; }   // older than the ring: finished
  cudaEvent_t ev = c->frc_evt[ticket % lbm_ctx::kTickets];
  if (wait) {
    CK(cudaEventSynchronize(ev), "force read-back wait");
    *done = 1;
    return LBM_OK;
  }
  const cudaError_t q = cudaEventQuery(ev);
  if (q == cudaSuccess) { *done = 1; return LBM_OK; }
  if (q == cudaErrorNotReady) { cudaGetLastError(); *done = 0; return LBM_OK; }
  return cuda_fail(q, "force read-back");
}

int lbm_update_macros(lbm_ctx* c) {
  int r = check_ready(c, false);
  if (r) return r;
  if ((r = ensure_macros(c))) return r;
  CK(c->ops.macros(dev_of(c), parity(c), c->inplace, cell_launch(c), c->stream), "macros kernel launch");
  return LBM_OK;
}

int lbm_read_macros(lbm_ctx* c, float* out, size_t n) {
  if (!c || !out) return fail(LBM_EINVAL, "null argument");
  if ((int64_t)n != 4 * c->N) return fail(LBM_EINVAL, "macros array must hold 4*N floats");
  int r = ensure_macros(c);
  if (r) return r;
  CK(cudaMemcpyAsync(out, c->macros, sizeof(float4) * (size_t)c->N, cudaMemcpyDeviceToHost, c->stream),
     "macros download");
  CK(cudaStreamSynchronize(c->stream), "macros download sync");
  return LBM_OK;
}

int lbm_forces(lbm_ctx* c, double f[3]) {
  int r = check_ready(c, false);
  if (r) return r;
  if (!f) return fail(LBM_EINVAL, "null output");
  Launch L = cell_launch(c);
  const int64_t nb = (int64_t)L.grid.x * L.grid.y * L.grid.z;
  if ((r = ensure_partials(c, nb))) return r;
  CK(c->ops.forces(dev_of(c), parity(c), c->inplace, c->partials, L, c->stream), "force kernel launch");
  k_reduce3<<<1, 256, 0, c->stream>>>(c->partials, nb, c->red);
  CK(cudaGetLastError(), "reduce kernel launch");
  if ((r = ensure_pinned(c, 3))) return r;
  CK(cudaMemcpyAsync(c->hpin, c->red, 3 * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "force download");
  CK(cudaStreamSynchronize(c->stream), "force sync");
  memcpy(f, c->hpin, 3 * sizeof(double));
  return LBM_OK;
}

int lbm_mass(lbm_ctx* c, double* sum) {
  int r = check_ready(c, false);
  if (r) return r;
  if (!sum) return fail(LBM_EINVAL, "null output");
  Launch L = cell_launch(c);
  const int64_t nb = (int64_t)L.grid.x * L.grid.y * L.grid.z;
  if ((r = ensure_partials(c, nb))) return r;
  CK(c->ops.mass(dev_of(c), parity(c), c->inplace, c->partials, L, c->stream), "mass kernel launch");
  k_reduce3<<<1, 256, 0, c->stream>>>(c->partials, nb, c->red);
  CK(cudaGetLastError(), "reduce kernel launch");
  double out[3];
  CK(cudaMemcpyAsync(out, c->red, 3 * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "mass download");
  CK(cudaStreamSynchronize(c->stream), "mass sync");
  *sum = out[0];
  return LBM_OK;
}

static_assert(sizeof(lbm_state_header) == 48, "lbm_state_header layout");

int lbm_state_bytes(lbm_ctx* c, size_t* bytes) {
  if (!c || !bytes) return fail(LBM_EINVAL, "null argument");
  *bytes = sizeof(lbm_state_header) + (size_t)Q * (size_t)c->nset * (size_t)c->ops.elem_bytes;
  return LBM_OK;
}

int lbm_save_state(lbm_ctx* c, void* dst, size_t bytes) {
  if (!c || !dst) return fail(LBM_EINVAL, "null argument");
  int r = check_ready(c, false);
  if (r) return r;
  if (!c->state_set) return fail(LBM_ESTATE, "no state yet (initialise or set populations first)");
  size_t need = 0;
  lbm_state_bytes(c, &need);
  if (bytes < need) return fail(LBM_EINVAL, "checkpoint buffer too small (see lbm_state_bytes)");
  lbm_state_header h;
  memset(&h, 0, sizeof h);
  h.magic = LBM_STATE_MAGIC;
  h.version = LBM_STATE_VERSION;
  h.nx = c->dims.nx; h.ny = c->dims.ny; h.nz = c->dims.nz;
  h.storage = c->storage;
  h.layout = layout_code(c);
  h.parity = parity(c);
  h.steps = c->steps;
  h.payload_bytes = need - sizeof h;
  memcpy(dst, &h, sizeof h);
  CK(cudaMemcpyAsync(static_cast<char*>(dst) + sizeof h, c->pop, h.payload_bytes, cudaMemcpyDeviceToHost, c->stream),
     "state download");
  CK(cudaStreamSynchronize(c->stream), "state download sync");
  return LBM_OK;
}

int lbm_load_state(lbm_ctx* c, const void* src, size_t bytes) {
  if (!c || !src) return fail(LBM_EINVAL, "null argument");
  if (bytes < sizeof(lbm_state_header)) return fail(LBM_EINVAL, "checkpoint shorter than its header");
  lbm_state_header h;
  memcpy(&h, src, sizeof h);
  if (h.magic != LBM_STATE_MAGIC || h.version != LBM_STATE_VERSION) return fail(LBM_EINVAL, "not a checkpoint of this library");
  size_t need = 0;
  lbm_state_bytes(c, &need);
  if (h.nx != c->dims.nx || h.ny != c->dims.ny || h.nz != c->dims.nz)
    return fail(LBM_EINVAL, "checkpoint grid differs from the context's");
  if (h.storage != c->storage) return fail(LBM_EINVAL, "checkpoint storage form differs from the context's");
  if (h.layout != layout_code(c))
    return fail(LBM_EINVAL, "checkpoint layout differs from the context's");
  if (h.payload_bytes + sizeof h != need || bytes < need) return fail(LBM_EINVAL, "checkpoint size does not match");
  if (c->inplace && h.parity != (int)(h.steps & 1)) return fail(LBM_EINVAL, "checkpoint parity and step count disagree");
  CK(cudaMemcpyAsync(c->pop, static_cast<const char*>(src) + sizeof h, h.payload_bytes, cudaMemcpyHostToDevice, c->stream),
     "state upload");
  CK(cudaStreamSynchronize(c->stream), "state upload sync");
  c->steps = h.steps;
  c->clo_since = -1;
  c->state_set = true;
  return LBM_OK;
}

int lbm_read_macros_async(lbm_ctx* c, float* out, size_t n) {
  if (!c || !out) return fail(LBM_EINVAL, "null argument");
  if ((int64_t)n != 4 * c->N) return fail(LBM_EINVAL, "macros array must hold 4*N floats");
  int r = check_ready(c, false);
  if (r) return r;
  if ((r = ensure_macros(c))) return r;
  if (!c->mac_evt) CK(cudaEventCreateWithFlags(&c->mac_evt, cudaEventDisableTiming), "event create");
  CK(c->ops.macros(dev_of(c), parity(c), c->inplace, cell_launch(c), c->stream), "macros kernel launch");
  CK(cudaMemcpyAsync(out, c->macros, sizeof(float4) * (size_t)c->N, cudaMemcpyDeviceToHost, c->stream),
     "macros download");
  CK(cudaEventRecord(c->mac_evt, c->stream), "event record");
  return LBM_OK;
}

int lbm_macros_ready(lbm_ctx* c, int* ready) {
  if (!c || !ready) return fail(LBM_EINVAL, "null argument");
  if (!c->mac_evt) { *ready = 1; return LBM_OK; }
  const cudaError_t e = cudaEventQuery(c->mac_evt);
  if (e == cudaSuccess) { *ready = 1; return LBM_OK; }
  if (e == cudaErrorNotReady) { cudaGetLastError(); *ready = 0; return LBM_OK; }
  return cuda_fail(e, "macros read-back");
}

}  // extern "C"

namespace lbm {
// Device view of a context for the other units of the library (visualisation).
int ctx_view(lbm_ctx* c, CtxView* v) {
  if (!c || !v) return fail(LBM_EINVAL, "null argument");
  int r = check_ready(c, false);
  if (r) return r;
  if ((r = ensure_macros(c))) return r;
  v->nx = c->dims.nx; v->ny = c->dims.ny; v->nz = c->dims.nz;
  v->N = c->N;
  v->macros = c->macros;
  v->tipo = c->tipo;
  v->stream = c->stream;
  return LBM_OK;
}
}  // namespace lbm

extern "C" {

int lbm_sync(lbm_ctx* c) {
  if (!c) return fail(LBM_EINVAL, "null context");
  CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
  return LBM_OK;
}

int lbm_set_closure(lbm_ctx* c, const closure_weights* w) {
  if (!c || !w) return fail(LBM_EINVAL, "null argument");
  if (!c->ops.step_closure || !c->inplace || (c->flags & LBM_FLAG_STRICT))
    return fail(LBM_ENOTSUP, "the learned closure runs in the in-place FAST step with fp32 arithmetic only");
  lbm::MlpFrag F;
  lbm::closure_pack(w, &F);
  c->clo_coef = w->coef != 0;
  for (int a = 0; a < 6; ++a) {
    c->clo_k.lo[a] = F.lo[a];
    c->clo_k.hi[a] = F.hi[a];
    c->clo_k.mean[a] = F.mean[a];
    c->clo_k.inv_std[a] = F.inv_std[a];
  }
  c->clo_k.nu_scale = F.nu_scale;
  c->clo_k.nu_max = F.nu_max;
  if (!c->clo) {
    int r = dalloc(c, (void**)&c->clo, sizeof(lbm::MlpFrag), "closure network");
    if (r) return r;
    r = dalloc(c, (void**)&c->clo_fb, 2 * sizeof(unsigned long long), "closure counter");
    if (r) return r;
    CK(cudaMemsetAsync(c->clo_fb, 0, 2 * sizeof(unsigned long long), c->stream), "closure counter clear");
  }
  CK(cudaMemcpyAsync(c->clo, &F, sizeof F, cudaMemcpyHostToDevice, c->stream), "closure upload");
  CK(cudaStreamSynchronize(c->stream), "closure upload sync");
  c->clo_since = -1;
  return LBM_OK;
}

int lbm_closure_engine(lbm_ctx* c, int engine) {
  if (!c) return fail(LBM_EINVAL, "null context");
  if (engine != 0 && engine != 1) return fail(LBM_EINVAL, "engine must be 0 (warp mma.sync) or 1 (CTA tcgen05)");
  c->clo_engine = engine;
  return LBM_OK;
}

int closure_samples(lbm_ctx* c, float tau0_coarse, float s_min, int x0, int x1, float* feats, float* target,
                    size_t rows) {
  if (!c || !feats || !target) return fail(LBM_EINVAL, "null argument");
  int r = check_ready(c, false);
  if (r) return r;
  const int cx_ = c->dims.nx / 2, cy_ = c->dims.ny / 2, cz_ = c->dims.nz / 2;
  if (cx_ < 3 || cy_ < 3 || cz_ < 3) return fail(LBM_EINVAL, "fine grid too small for a 2x coarse grid");
  if (x0 < 0 || x1 > cx_ || x0 >= x1) return fail(LBM_EINVAL, "bad coarse x range");
  const size_t nr = (size_t)(x1 - x0) * cy_ * cz_;
  if (rows != nr) return fail(LBM_EINVAL, "rows must be (x1 - x0) * (ny/2) * (nz/2)");
  if (!(tau0_coarse > 0.5f)) return fail(LBM_EINVAL, "tau0_coarse must exceed 1/2");
  if (!(s_min >= 0.0f)) return fail(LBM_EINVAL, "s_min must be >= 0");
  if ((r = lbm_update_macros(c))) return r;
  float *df = nullptr, *dt = nullptr;
  if ((r = dalloc(c, (void**)&df, sizeof(float) * 6 * nr, "sample features"))) return r;
  if ((r = dalloc(c, (void**)&dt, sizeof(float) * nr, "sample targets"))) {
    cudaFree(df); c->dev_bytes -= sizeof(float) * 6 * nr;
    return r;
  }
  cudaError_t e = lbm::closure_samples_launch(c->macros, c->tipo, c->dims.nx, c->dims.ny, c->dims.nz, tau0_coarse,
                                              s_min, x0, x1, df, dt, c->stream);
  if (e == cudaSuccess) e = cudaMemcpy(feats, df, sizeof(float) * 6 * nr, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(target, dt, sizeof(float) * nr, cudaMemcpyDeviceToHost);
  cudaFree(df);
  cudaFree(dt);
  c->dev_bytes -= sizeof(float) * 7 * nr;
  if (e != cudaSuccess) return cuda_fail(e, "closure samples");
  return LBM_OK;
}

int lbm_closure_stats(lbm_ctx* c, int64_t* fallback_cells, int64_t* fluid_cells) {
  if (!c || !fallback_cells || !fluid_cells) return fail(LBM_EINVAL, "null argument");
  unsigned long long fb[2] = {0, 0};
  if (c->clo_fb) {
    CK(cudaMemcpyAsync(fb, c->clo_fb, sizeof fb, cudaMemcpyDeviceToHost, c->stream), "closure counter download");
    CK(cudaMemsetAsync(c->clo_fb, 0, sizeof fb, c->stream), "closure counter clear");
    CK(cudaStreamSynchronize(c->stream), "closure counter sync");
  }
  *fallback_cells = (int64_t)fb[0];
  *fluid_cells = c->n_fluido * c->clo_steps;
  c->clo_steps = 0;
  if (fb[1]) return fail(LBM_ETIMEDOUT, "closure step: a tensor-core mbarrier wait gave up (those cells fell back)");
  return LBM_OK;
}

int lbm_get_info(lbm_ctx* c, lbm_info* info) {
  if (!c || !info) return fail(LBM_EINVAL, "null argument");
  info->n_cells = c->N;
  info->device_bytes = c->dev_bytes;
  info->storage = c->storage;
  info->flags = c->flags;
  info->steps = c->steps;
  info->parity = (int)(c->steps & 1);
  info->block_x = (int)cell_launch(c).block.x;
  info->layout = layout_code(c);
  return LBM_OK;
}

int lbm_set_launch(lbm_ctx* c, int block_x, int min_blocks) {
  if (!c) return fail(LBM_EINVAL, "null context");
  // min_blocks 4/8/16 with block_x = 64 selects the pipelined step with that
  // many cells per thread along z
  if (min_blocks != 0 && min_blocks != 6 && min_blocks != 8 && min_blocks != 9 && min_blocks != 20 &&
      min_blocks != 21 && min_blocks != 104 && min_blocks != 108 && min_blocks != 116)
    return fail(LBM_EINVAL,
                "min_blocks must be 0, 6, 8, 9 (AoSoA: addresses kept from load to store), 20 or 21 (SoA addressing "
                "variants), or 100 + cells per thread (4, 8, 16) for the pipelined step");
  int r = lbm_set_block(c, block_x);
  if (r) return r;
  if (min_blocks >= 100) { c->pipe = min_blocks - 100; c->occ = 8; }
  else { c->pipe = 0; c->occ = min_blocks == 0 ? 8 : min_blocks; }
  return LBM_OK;
}

int lbm_autotune(lbm_ctx* c, int steps, int* block_x, int* block_y, int* variant, float* ms_per_step) {
  int r = check_ready(c, true);
  if (r) return r;
  if (!c->inplace) return fail(LBM_ENOTSUP, "the tuner times the in-place step");
  if (!c->state_set) return fail(LBM_ESTATE, "no state yet (initialise or set populations first)");
  if (steps < 2 || steps > 100000) return fail(LBM_EINVAL, "steps must be in [2, 100000]");
  // candidates: threads along x and y of the block (<= 128), the register-cap
  // variant (8 or 6 resident blocks; the AoSoA step is built for 8), the
  // addressing variants (AoSoA: 9; SoA: 20, 21), and for the SoA set the
  // pipelined step (cells per thread along z)
  const bool fits32 = (int64_t)Q * c->N < (int64_t)INT32_MAX;
  std::vector<Shape> cand;
  for (int bx : {32, 64, 128})
    for (int by : {1, 2, 4})
      if (bx * by <= 128) {
        cand.push_back({bx, by, 8, 0});
        if (c->aos) cand.push_back({bx, by, 9, 0});
        if (!c->aos && c->storage != LBM_F64 && fits32) {
          cand.push_back({bx, by, 20, 0});
          cand.push_back({bx, by, 21, 0});
        }
      }
  if (!c->aos && c->storage != LBM_F64) {
    cand.push_back({64, 1, 6, 0});
    cand.push_back({128, 1, 6, 0});
    if (fits32 && !is_sr(c->storage))   // the pipelined step has no stochastic rounding
      for (int kz : {4, 8, 16}) cand.push_back({64, 1, 8, kz});
  }
  // the state is saved and put back: the trials advance a copy of it
  const size_t set_bytes = (size_t)c->nset * Q * c->ops.elem_bytes;
  void* keep = nullptr;
  cudaError_t e = cudaMalloc(&keep, set_bytes);
  if (e != cudaSuccess) { cudaGetLastError(); return fail(LBM_ENOMEM, "no device memory for the tuner's copy of the state"); }
  const Shape saved{c->block_x, c->block_y, c->occ, c->pipe};
  const int64_t steps0 = c->steps;
  const int since0 = c->clo_since;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  Shape best = saved;
  float best_ms = 1e30f;
  e = cudaMemcpyAsync(keep, c->pop, set_bytes, cudaMemcpyDeviceToDevice, c->stream);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  for (size_t q = 0; q < cand.size() && e == cudaSuccess && !r; ++q) {
    c->block_x = cand[q].bx; c->block_y = cand[q].by; c->occ = cand[q].occ; c->pipe = cand[q].pipe;
    for (int k = 0; k < 2 && !r; ++k) r = launch_step(c, false, nullptr);   // warm-up
    e = cudaEventRecord(e0, c->stream);
    for (int k = 0; k < steps && !r && e == cudaSuccess; ++k) r = launch_step(c, false, nullptr);
    if (e == cudaSuccess) e = cudaEventRecord(e1, c->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (!r && e == cudaSuccess && ms / steps < best_ms) { best_ms = ms / steps; best = cand[q]; }
  }
  cudaError_t e2 = cudaMemcpyAsync(c->pop, keep, set_bytes, cudaMemcpyDeviceToDevice, c->stream);
  if (e2 == cudaSuccess) e2 = cudaStreamSynchronize(c->stream);
  cudaFree(keep);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  c->steps = steps0;
  c->clo_since = since0;
  if (r) { c->block_x = saved.bx; c->block_y = saved.by; c->occ = saved.occ; c->pipe = saved.pipe; return r; }
  if (e != cudaSuccess) return cuda_fail(e, "tuner");
  if (e2 != cudaSuccess) return cuda_fail(e2, "tuner state restore");
  c->block_x = best.bx; c->block_y = best.by; c->occ = best.occ; c->pipe = best.pipe;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tuned[ShapeKey(c->dims.nx, c->dims.ny, c->dims.nz, c->storage, c->flags & ~LBM_FLAG_WRITE_MACROS, c->aos)] = best;
  }
  if (block_x) *block_x = best.bx;
  if (block_y) *block_y = best.by;
  if (variant) *variant = best.pipe ? 100 + best.pipe : best.occ;
  if (ms_per_step) *ms_per_step = best_ms;
  return LBM_OK;
}

int lbm_autotune_layout(const lbm_dims* dims, int storage, int flags, int steps, int* layout, float* ms_aos,
                        float* ms_soa) {
  if (!dims || !layout) return fail(LBM_EINVAL, "null argument");
  if (steps < 2 || steps > 100000) return fail(LBM_EINVAL, "steps must be in [2, 100000]");
  flags &= ~(LBM_FLAG_SOA | LBM_FLAG_AOS | LBM_FLAG_WRITE_MACROS);
  float ms[2] = {0.f, 0.f};
  int lay[2] = {0, 0};
  // the same free stream in an all-fluid box of this grid, once per layout
  for (int q = 0; q < 2; ++q) {
    lbm_ctx* c = nullptr;
    int r = lbm_create(dims, storage, flags | (q == 0 ? LBM_FLAG_AOS : LBM_FLAG_SOA), &c);
    if (r) return r;
    lay[q] = layout_code(c);
    lbm_params p{};
    p.omega_plus = 1.9f; p.magic = 0.1875f; p.les_cs = 0.1f;
    p.inlet_u[0] = 0.05f;
    p.sponge_start = (float)dims->nx + 10.0f; p.sponge_len = 4.0f;
    std::vector<uint32_t> t((size_t)c->N, 0u);
    r = lbm_configure(c, &p);
    if (!r) r = lbm_set_types(c, t.data(), t.size());
    if (!r) r = lbm_init_equilibrium(c);
    if (!r) r = lbm_step(c, 2);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaSuccess;
    if (!r) e = cudaEventCreate(&e0);
    if (!r && e == cudaSuccess) e = cudaEventCreate(&e1);
    if (!r && e == cudaSuccess) e = cudaEventRecord(e0, c->stream);
    if (!r && e == cudaSuccess) r = lbm_step(c, steps);
    if (!r && e == cudaSuccess) e = cudaEventRecord(e1, c->stream);
    if (!r && e == cudaSuccess) e = cudaEventSynchronize(e1);
    if (!r && e == cudaSuccess) e = cudaEventElapsedTime(&ms[q], e0, e1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    lbm_destroy(c);
    if (r) return r;
    if (e != cudaSuccess) return cuda_fail(e, "layout tuner");
    ms[q] /= (float)steps;
  }
  const bool aos_applies = lay[0] == 2 || lay[0] == 3;
  const bool aos = aos_applies && ms[0] < ms[1];
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_layout[LayoutKey(dims->nx, dims->ny, dims->nz, storage, flags)] = aos;
  }
  *layout = aos ? lay[0] : lay[1];
  if (ms_aos) *ms_aos = aos_applies ? ms[0] : -1.f;
  if (ms_soa) *ms_soa = ms[1];
  return LBM_OK;
}

int lbm_set_block(lbm_ctx* c, int block_x) {
  if (!c) return fail(LBM_EINVAL, "null context");
  if (block_x < 0 || block_x > 128 || (block_x % 32) != 0) return fail(LBM_EINVAL, "block_x must be 0 or a multiple of 32 up to 128");
  c->block_x = block_x;
  c->block_y = 1;
  return LBM_OK;
}

}  // extern "C"

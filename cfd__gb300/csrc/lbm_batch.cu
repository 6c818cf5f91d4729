// lbm_batch.cu — batched tunnels (include/lbm_batch.h).
//
// Every tunnel keeps the single-tunnel data layout (its own in-place
// population set, link words and types).  A device array of descriptors
// (grid, pointers, parameters, tile shape, first tile) lets one kernel
// step all tunnels: CTA b of G walks global tiles b, b + G, b + 2G, ...;
// each tile is 128 threads covering tx cells along x and 128/tx rows along y
// of one z-plane of one tunnel, located by a binary search over the
// tunnels' first-tile prefix.  The per-cell work is step_cell(), the same
// code as the single-tunnel kernel, so results are bit-identical to lbm_step.
//
// Tile width per tunnel (32, 64 or 128) is chosen to leave the fewest idle
// threads for that tunnel's nx and ny, or set by lbm_batch_set_tile.
// The descriptors of up to 64 tunnels travel by value in the launch's
// parameter space (read through the constant cache, as single-tunnel
// parameters are); larger batches take one launch per 64 tunnels per step.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/lbm.h"
#include "../../include/lbm_batch.h"
#include "lbm_kernels.cuh"

extern "C" int lbm_internal_fail(int code, const char* msg);

namespace lbm {
cudaError_t launch_links(const uint8_t* tipo, uint32_t* link, int nx, int ny, int nz, cudaStream_t s);
cudaError_t launch_reduce3(const double* part, int64_t n, double* out, cudaStream_t s);
bool bl_table(float bl, int nz, bool f64, std::vector<unsigned char>& out);
}  // namespace lbm

using namespace lbm;

namespace {

struct TunnelDesc {
  Dev d;
  Params P;
  Uni<float> U;
  int tx, ty, gx, gy;   // tile shape, tiles along x and y
};

constexpr int kTile = 128;
static_assert(sizeof(TunnelDesc) % 4 == 0, "descriptor copied as 32-bit words");
constexpr int kPerLaunch = 64;   // tunnels whose descriptors ride in one launch's parameters

// One launch's share of the batch, passed by value: the descriptors sit in
// the kernel parameter space (constant bank), like a single tunnel's Params.
struct BatchArgs {
  int ntun;
  int ntiles;
  int aos;                     // every tunnel of this launch keeps its set in the AoSoA layout (else SoA)
  int first[kPerLaunch + 1];   // first tile of each tunnel (prefix), local to this launch
  const int4* tiles;           // per tile: {tunnel | log2(tile width) << 8, x0, y0, z}, device
  TunnelDesc t[kPerLaunch];
};
static_assert(sizeof(BatchArgs) < 32000, "kernel parameter space");

// AB: the launch's AoSoA block width (0: its tunnels are SoA).
template <class St, int PAR, bool FAST, int MINB, int AB>
__global__ void __launch_bounds__(kTile, MINB) k_batch_step(const __grid_constant__ BatchArgs A) {
  // A tile's tunnel is found by a search over the launch's first-tile
  // prefix: the index is the same for the whole CTA, so the search and the
  // descriptor reads (straight from the parameter bank) stay on the uniform
  // datapath.  Its origin comes from its word in the launch's tile table (one
  // 16-byte load, the same address for the whole CTA), which spares the
  // divisions by the tile counts.
  for (int t = blockIdx.x; t < A.ntiles; t += gridDim.x) {
    const int4 w = __ldg(A.tiles + t);
    int lo = 0, hi = A.ntun;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (A.first[mid] <= t) lo = mid;
      else hi = mid;
    }
    const TunnelDesc& D = A.t[lo];
    const int lg = w.x >> 8;
    const int x = w.y + (int)(threadIdx.x & ((1u << lg) - 1u));
    const int y = w.z + (int)(threadIdx.x >> lg);
    const int z = w.w;
    if (x < D.d.nx && y < D.d.ny) {
      const int32_t cell = (z * D.d.ny + y) * D.d.nx + x;
      if constexpr (AB != 0 && FAST)
        step_cell_at<St, PAR, false, false, false, FAST>(D.d, D.P, D.U, x, y, z, cell,
                                                         AddrAos<St, PAR, int32_t, true, AB>(D.d, cell, x, y, z));
      else
        step_cell<St, PAR, false, false, false, FAST>(D.d, D.P, D.U, x, y, z);
    }
  }
}

// The device copy of the batch's step count advances with the steps (stream
// order, so a captured graph advances it on every replay).
__global__ void k_steps_add(uint32_t* c, uint32_t n) { *c += n; }
__global__ void k_steps_set(uint32_t* c, uint32_t v) { *c = v; }

int bfail(int code, const std::string& m) { return lbm_internal_fail(code, m.c_str()); }

// Cells per population slot of a tunnel's set, the AoSoA rows' padding included.
size_t set_cells(const Dev& d) { return (size_t)d.nxp * d.ny * d.nz; }

#define BCK(call, what)                                                                  \
  do {                                                                                   \
    cudaError_t _e = (call);                                                             \
    if (_e != cudaSuccess) {                                                             \
      cudaGetLastError();                                                                \
      return bfail(_e == cudaErrorMemoryAllocation ? LBM_ENOMEM : LBM_ECUDA,             \
                   std::string(what) + ": " + cudaGetErrorString(_e));                   \
    }                                                                                    \
  } while (0)

Ops ops_for_batch(int storage) {
  switch (storage) {
    case LBM_F16S: return ops_f16s();
    case LBM_BF16S: return ops_bf16s();
    case LBM_F16SR: return ops_f16sr();
    case LBM_BF16SR: return ops_bf16sr();
    default: return ops_f32();
  }
}

}  // namespace

struct lbm_batch {
  int storage = LBM_F32;
  bool fast = true;
  std::vector<lbm_dims> dims;
  std::vector<TunnelDesc> host;
  std::vector<int> tile_req;         // requested tile width (0 = cost model)
  std::vector<bool> configured, typed;
  std::vector<void*> allocs;
  std::vector<BatchArgs> args;       // one per launch of a step (64 tunnels each)
  long long ntiles = 0;
  int sms = 1;                       // multiprocessors of the device
  int minb = 8;                      // resident CTAs per SM the mode-1 kernel is built for (8 or 6)
  Ops ops{};
  double* partials = nullptr;
  int64_t npart = 0;
  double* red = nullptr;
  double* stage = nullptr;
  int64_t stage_n = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int64_t steps = 0;
  int64_t cells = 0;
  int64_t bytes = 0;
  bool desc_dirty = true;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};   // by start parity
  int graph_steps = 32;
  int mode = 0;                      // 0: graph of per-tunnel chains, 1: one launch over all tiles
  std::vector<cudaStream_t> lanes;   // capture-time streams, one per tunnel (mode 0)
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> joins;
  std::vector<void*> blf;            // per tunnel: nz inlet boundary-layer factors
  uint32_t* steps_dev = nullptr;     // the step count on the device: the SR forms' rounding seeds
  int4* tiles = nullptr;             // tile table of the mode-1 launches
  size_t tiles_cap = 0;              // its capacity in tiles
};

namespace {

int balloc(lbm_batch* b, void** p, size_t bytes, const char* what) {
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    char buf[200];
    snprintf(buf, sizeof buf, "device allocation of %.3f GB for %s failed: %s", bytes / 1e9, what,
             cudaGetErrorString(e));
    *p = nullptr;
    return bfail(LBM_ENOMEM, buf);
  }
  b->allocs.push_back(*p);
  b->bytes += (int64_t)bytes;
  return LBM_OK;
}

// Fewest idle threads for (nx, ny); ties go to the wider tile.
int pick_tile(int nx, int ny) {
  int best = 128;
  double best_w = 1e30;
  for (int tx : {128, 64, 32}) {
    const int ty = kTile / tx;
    const double used = (double)nx * ny;
    const double launched = (double)((nx + tx - 1) / tx) * tx * ((ny + ty - 1) / ty) * ty;
    const double w = launched / used;
    if (w < best_w - 1e-12) { best_w = w; best = tx; }
  }
  return best;
}

void drop_graphs(lbm_batch* b) {
  for (auto& g : b->graph)
    if (g) { cudaGraphExecDestroy(g); g = nullptr; }
}

int sync_desc(lbm_batch* b) {
  if (!b->desc_dirty) return LBM_OK;
  // Launch arguments change: graphs hold them by value, so drop them.
  drop_graphs(b);
  b->args.clear();
  long long total = 0;
  // One launch (or more, 64 tunnels each) per layout class, so that each
  // kernel instance carries a single addressing path.  Within a launch, tiles
  // of the largest tunnels come first: the last CTAs then finish with the
  // small ones, which evens out the tail.
  std::vector<size_t> order(b->host.size());
  for (size_t k = 0; k < order.size(); ++k) order[k] = k;
  std::stable_sort(order.begin(), order.end(), [&](size_t p, size_t q) {
    if (b->host[p].d.aos != b->host[q].d.aos) return b->host[p].d.aos > b->host[q].d.aos;
    return b->host[p].d.N > b->host[q].d.N;
  });
  std::vector<std::pair<size_t, size_t>> runs;   // [k0, k1) of `order`, one layout, <= 64 tunnels
  for (size_t k0 = 0; k0 < order.size();) {
    size_t k1 = k0;
    while (k1 < order.size() && k1 - k0 < (size_t)kPerLaunch && b->host[order[k1]].d.aos == b->host[order[k0]].d.aos)
      ++k1;
    runs.push_back({k0, k1});
    k0 = k1;
  }
  std::vector<int4> table;           // every launch's tile words, one after the other
  std::vector<size_t> table_at;      // where each launch's words start
  for (const auto& run : runs) {
    BatchArgs A;
    memset(&A, 0, sizeof A);
    const size_t k0 = run.first, k1 = run.second;
    A.aos = b->host[order[k0]].d.aos;
    table_at.push_back(table.size());
    long long t = 0;
    for (size_t kk = k0; kk < k1; ++kk) {
      const size_t k = order[kk];
      TunnelDesc& D = b->host[k];
      const int tx = b->tile_req[k] ? b->tile_req[k] : pick_tile(D.d.nx, D.d.ny);
      const int lg = tx == 32 ? 5 : (tx == 64 ? 6 : 7);
      D.tx = tx;
      D.ty = kTile / tx;
      D.gx = (D.d.nx + tx - 1) / tx;
      D.gy = (D.d.ny + D.ty - 1) / D.ty;
      A.first[kk - k0] = (int)t;
      A.t[kk - k0] = D;
      t += (long long)D.gx * D.gy * D.d.nz;
      if (t >= INT32_MAX) return bfail(LBM_EINVAL, "too many tiles in one launch (keep a batch under 2^31 tiles)");
      for (int z = 0; z < D.d.nz; ++z)
        for (int by = 0; by < D.gy; ++by)
          for (int bx = 0; bx < D.gx; ++bx)
            table.push_back(make_int4((int)(kk - k0) | (lg << 8), bx * tx, by * D.ty, z));
    }
    A.ntun = (int)(k1 - k0);
    A.first[A.ntun] = (int)t;
    A.ntiles = (int)t;
    b->args.push_back(A);
    total += t;
  }
  // the table goes to the device once per change of the descriptors (no
  // launch of the old table is in flight: the stream is drained first)
  BCK(cudaStreamSynchronize(b->stream), "stream sync");
  if (table.size() > b->tiles_cap) {
    if (b->tiles) cudaFree(b->tiles);
    b->tiles = nullptr;
    b->tiles_cap = 0;
    BCK(cudaMalloc(&b->tiles, table.size() * sizeof(int4)), "tile table");
    b->tiles_cap = table.size();
  }
  if (!table.empty())
    BCK(cudaMemcpy(b->tiles, table.data(), table.size() * sizeof(int4), cudaMemcpyHostToDevice), "tile table upload");
  for (size_t q = 0; q < b->args.size(); ++q) b->args[q].tiles = b->tiles + table_at[q];
  b->ntiles = total;
  b->desc_dirty = false;
  return LBM_OK;
}

template <class St, bool FAST, int MINB>
void launch_batch_m(lbm_batch* b, const BatchArgs& A0, int parity, int grid, uint32_t off) {
  // the SR forms: each tunnel's seed is the device step count + off
  BatchArgs A1;
  if constexpr (St::kSR) {
    A1 = A0;
    for (int i = 0; i < A1.ntun; ++i) A1.t[i].d.seed = off;
  }
  const BatchArgs& A = St::kSR ? A1 : A0;
  if constexpr (sizeof(typename St::store_t) == 2) {   // blocks of 64 cells: 16-bit forms only
    if (A.aos == 64) {
      if (parity == 0) k_batch_step<St, 0, FAST, MINB, 64><<<grid, kTile, 0, b->stream>>>(A);
      else k_batch_step<St, 1, FAST, MINB, 64><<<grid, kTile, 0, b->stream>>>(A);
      return;
    }
  }
  if (A.aos) {
    if (parity == 0) k_batch_step<St, 0, FAST, MINB, 32><<<grid, kTile, 0, b->stream>>>(A);
    else k_batch_step<St, 1, FAST, MINB, 32><<<grid, kTile, 0, b->stream>>>(A);
  } else {
    if (parity == 0) k_batch_step<St, 0, FAST, MINB, 0><<<grid, kTile, 0, b->stream>>>(A);
    else k_batch_step<St, 1, FAST, MINB, 0><<<grid, kTile, 0, b->stream>>>(A);
  }
}

template <class St>
void launch_batch(lbm_batch* b, int parity, uint32_t off) {
  for (const BatchArgs& A : b->args) {
    const int per_sm = b->minb;
    // 16 times the CTAs the SMs hold at once, each walking every G-th tile:
    // the block scheduler refills an SM as its CTAs finish, instead of one
    // wave of CTAs that walk their shares in step (64 uneven tunnels: 0.85x
    // of running them one after another with one wave, 0.93x with sixteen).
    const int grid = std::min(b->sms * per_sm * 16, std::max(1, A.ntiles));
    if (b->fast) {
      if (per_sm == 6) launch_batch_m<St, true, 6>(b, A, parity, grid, off);
      else launch_batch_m<St, true, 8>(b, A, parity, grid, off);
    } else {
      if (per_sm == 6) launch_batch_m<St, false, 6>(b, A, parity, grid, off);
      else launch_batch_m<St, false, 8>(b, A, parity, grid, off);
    }
  }
}

// One mode-1 step; off: its place after the device step count.
void launch_one(lbm_batch* b, int parity, uint32_t off) {
  switch (b->storage) {
    case LBM_F16S: launch_batch<StF16S>(b, parity, off); break;
    case LBM_BF16S: launch_batch<StBF16S>(b, parity, off); break;
    case LBM_F16SR: launch_batch<StF16SR>(b, parity, off); break;
    case LBM_BF16SR: launch_batch<StBF16SR>(b, parity, off); break;
    default: launch_batch<StF32>(b, parity, off); break;
  }
}

Launch tunnel_launch(const lbm_dims& d);

// Mode 0: tunnel k's steps go to lane k; lanes fork from and join back into
// the batch stream, so a captured graph holds T independent chains that the
// GPU runs concurrently, each launch with its own constant-bank parameters.
cudaError_t launch_chains(lbm_batch* b, int parity, int nsteps) {
  cudaError_t e = cudaEventRecord(b->fork, b->stream);
  if (e != cudaSuccess) return e;
  for (size_t k = 0; k < b->host.size(); ++k) {
    cudaStream_t L = b->lanes[k];
    if ((e = cudaStreamWaitEvent(L, b->fork, 0)) != cudaSuccess) return e;
    const TunnelDesc& D = b->host[k];
    Dev dd = D.d;
    for (int s = 0; s < nsteps; ++s) {
      dd.seed = (uint32_t)s;   // the SR forms' seed: the device step count + s
      e = b->ops.step(dd, D.P, (parity + s) & 1, true, false, false, b->fast, tunnel_launch(b->dims[k]), L);
      if (e != cudaSuccess) return e;
    }
    if ((e = cudaEventRecord(b->joins[k], L)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(b->stream, b->joins[k], 0)) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

int check_ready(lbm_batch* b) {
  if (!b) return bfail(LBM_EINVAL, "null batch");
  for (size_t k = 0; k < b->host.size(); ++k) {
    if (!b->typed[k]) return bfail(LBM_ESTATE, "tunnel " + std::to_string(k) + ": cell types not set");
    if (!b->configured[k]) return bfail(LBM_ESTATE, "tunnel " + std::to_string(k) + ": parameters not set");
  }
  return LBM_OK;
}

Launch tunnel_launch(const lbm_dims& d) {
  Launch L;
  L.occ = 8;
  L.pipe = 0;
  const int bx = d.nx < 64 ? ((d.nx + 31) / 32) * 32 : 64;
  L.block = dim3(bx, 1, 1);
  L.grid = dim3((d.nx + bx - 1) / bx, d.ny, d.nz);
  return L;
}

}  // namespace

extern "C" {

int lbm_batch_create(const lbm_dims* dims, int ntunnels, int storage, int flags, lbm_batch** out) {
  if (!dims || !out || ntunnels < 1) return bfail(LBM_EINVAL, "need at least one tunnel and an output handle");
  *out = nullptr;
  if (storage != LBM_F32 && storage != LBM_F16S && storage != LBM_BF16S && storage != LBM_F16SR &&
      storage != LBM_BF16SR)
    return bfail(LBM_ENOTSUP, "batched tunnels support LBM_F32 and the 16-bit forms");
  if (flags & ~LBM_FLAG_STRICT) return bfail(LBM_EINVAL, "batched tunnels accept LBM_FLAG_STRICT only");
  lbm_batch* b = new lbm_batch();
  b->storage = storage;
  b->fast = !(flags & LBM_FLAG_STRICT);
  b->ops = ops_for_batch(storage);
  b->dims.assign(dims, dims + ntunnels);
  b->host.resize(ntunnels);
  b->tile_req.assign(ntunnels, 0);
  b->configured.assign(ntunnels, false);
  b->typed.assign(ntunnels, false);
  int r = LBM_OK;
  for (int k = 0; k < ntunnels && !r; ++k) {
    const lbm_dims& d = dims[k];
    if (d.nx < 1 || d.ny < 1 || d.nz < 1) { r = bfail(LBM_EINVAL, "grid dimensions must be >= 1"); break; }
    const int64_t N = (int64_t)d.nx * d.ny * d.nz;
    if ((int64_t)Q * N >= (int64_t)INT32_MAX) { r = bfail(LBM_EINVAL, "a batched tunnel must hold under 113 M cells"); break; }
    TunnelDesc& D = b->host[k];
    memset(&D, 0, sizeof D);
    D.d.nx = d.nx; D.d.ny = d.ny; D.d.nz = d.nz; D.d.N = N;
    // the AoSoA layout where the FAST step can use it: blocks of 64 cells for
    // the 16-bit forms, 32 for fp32, rows padded to a multiple of the block
    const int ab = storage != LBM_F32 ? 64 : kAosB;
    const int nxp = (d.nx + ab - 1) / ab * ab;
    const bool aos = b->fast && (int64_t)Q * nxp * d.ny * d.nz < (int64_t)INT32_MAX;
    D.d.aos = aos ? ab : 0;
    D.d.nxp = aos ? nxp : d.nx;
    void* p = nullptr;
    const size_t sb = set_cells(D.d) * Q * b->ops.elem_bytes;
    if ((r = balloc(b, &p, sb, "populations"))) break;
    D.d.pop = p;
    if ((r = balloc(b, &p, (size_t)N, "cell types"))) break;
    D.d.tipo = static_cast<uint8_t*>(p);
    if ((r = balloc(b, &p, sizeof(uint32_t) * (size_t)N, "link words"))) break;
    D.d.link = static_cast<uint32_t*>(p);
    if ((r = balloc(b, &p, sizeof(float) * (size_t)d.nz, "inlet boundary-layer factors"))) break;
    b->blf.push_back(p);
    b->cells += N;
  }
  void* p = nullptr;
  if (!r) r = balloc(b, &p, 3 * sizeof(double), "reduction result");
  b->red = static_cast<double*>(p);
  if (!r) r = balloc(b, &p, sizeof(uint32_t), "step count");
  b->steps_dev = static_cast<uint32_t*>(p);
  if (r) { lbm_batch_destroy(b); return r; }
  for (auto& D : b->host) D.d.seed_base = b->steps_dev;
  cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { lbm_batch_destroy(b); return bfail(LBM_ECUDA, "stream creation failed"); }
  b->own_stream = true;
  for (int k = 0; k < ntunnels; ++k) {
    TunnelDesc& D = b->host[k];
    cudaMemsetAsync(D.d.pop, 0, set_cells(D.d) * Q * b->ops.elem_bytes, b->stream);
    cudaMemsetAsync((void*)D.d.tipo, 0, (size_t)D.d.N, b->stream);
  }
  cudaMemsetAsync(b->steps_dev, 0, sizeof(uint32_t), b->stream);
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  b->sms = std::max(1, sms);   // mode 1: minb resident 128-thread CTAs per SM, sixteen waves
  e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) { lbm_batch_destroy(b); return bfail(LBM_ECUDA, "initial clear failed"); }
  *out = b;
  return LBM_OK;
}

int lbm_batch_destroy(lbm_batch* b) {
  if (!b) return bfail(LBM_EINVAL, "null batch");
  if (b->stream) cudaStreamSynchronize(b->stream);
  drop_graphs(b);
  for (cudaStream_t L : b->lanes) cudaStreamDestroy(L);
  for (cudaEvent_t e : b->joins) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  for (void* p : b->allocs) cudaFree(p);
  if (b->partials) cudaFree(b->partials);
  if (b->stage) cudaFree(b->stage);
  if (b->tiles) cudaFree(b->tiles);
  if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return LBM_OK;
}

int lbm_batch_set_stream(lbm_batch* b, void* s) {
  if (!b) return bfail(LBM_EINVAL, "null batch");
  BCK(cudaStreamSynchronize(b->stream), "stream sync");
  if (b->own_stream) cudaStreamDestroy(b->stream);
  b->stream = static_cast<cudaStream_t>(s);
  b->own_stream = false;
  drop_graphs(b);
  return LBM_OK;
}

int lbm_batch_configure(lbm_batch* b, int k, const lbm_params* p) {
  if (!b || !p) return bfail(LBM_EINVAL, "null argument");
  if (k < 0 || k >= (int)b->host.size()) return bfail(LBM_EINVAL, "tunnel index out of range");
  if (p->closure != 0) return bfail(LBM_ENOTSUP, "the batched form runs the Smagorinsky closure only");
  Params P;
  P.omega_plus = p->omega_plus; P.magic = p->magic; P.les_cs = p->les_cs;
  for (int a = 0; a < 3; ++a) { P.belt[a] = p->belt_u[a]; P.inlet[a] = p->inlet_u[a]; }
  P.sponge_start = p->sponge_start; P.sponge_len = p->sponge_len; P.bl = p->bl_thickness;
  P.closure = p->closure;
  std::vector<unsigned char> tab;
  const bool on = bl_table(p->bl_thickness, b->host[k].d.nz, false, tab);
  if (on) {
    BCK(cudaMemcpyAsync(b->blf[k], tab.data(), tab.size(), cudaMemcpyHostToDevice, b->stream), "boundary-layer table");
    BCK(cudaStreamSynchronize(b->stream), "boundary-layer table sync");
  }
  b->host[k].d.blf = on ? b->blf[k] : nullptr;
  b->host[k].P = P;
  b->host[k].U = make_uni<float>(P, (b->storage == LBM_F16S || b->storage == LBM_F16SR) ? StF16S::kScale : 1.0f);
  b->configured[k] = true;
  b->desc_dirty = true;
  return LBM_OK;
}

int lbm_batch_set_types(lbm_batch* b, int k, const uint32_t* tipo, size_t n) {
  if (!b || !tipo) return bfail(LBM_EINVAL, "null argument");
  if (k < 0 || k >= (int)b->host.size()) return bfail(LBM_EINVAL, "tunnel index out of range");
  TunnelDesc& D = b->host[k];
  if ((int64_t)n != D.d.N) return bfail(LBM_EINVAL, "cell-type field size differs from the tunnel's N");
  std::vector<uint8_t> t8(n);
  for (size_t i = 0; i < n; ++i) {
    if (tipo[i] > 7u) return bfail(LBM_EINVAL, "cell type is not a CELULA code (0..7)");
    t8[i] = (uint8_t)tipo[i];
  }
  BCK(cudaMemcpyAsync((void*)D.d.tipo, t8.data(), n, cudaMemcpyHostToDevice, b->stream), "types upload");
  BCK(launch_links(D.d.tipo, (uint32_t*)D.d.link, D.d.nx, D.d.ny, D.d.nz, b->stream), "link kernel");
  BCK(cudaStreamSynchronize(b->stream), "types sync");
  b->typed[k] = true;
  return LBM_OK;
}

int lbm_batch_init_equilibrium(lbm_batch* b) {
  int r = check_ready(b);
  if (r) return r;
  for (size_t k = 0; k < b->host.size(); ++k) {
    const TunnelDesc& D = b->host[k];
    BCK(b->ops.init(D.d, D.P, true, tunnel_launch(b->dims[k]), b->stream), "init kernel");
  }
  b->steps = 0;
  k_steps_set<<<1, 1, 0, b->stream>>>(b->steps_dev, 0u);
  BCK(cudaGetLastError(), "step count");
  return LBM_OK;
}

int lbm_batch_set_tile(lbm_batch* b, int k, int tile_x) {
  if (!b) return bfail(LBM_EINVAL, "null batch");
  if (k < 0 || k >= (int)b->host.size()) return bfail(LBM_EINVAL, "tunnel index out of range");
  if (tile_x != 0 && tile_x != 32 && tile_x != 64 && tile_x != 128) return bfail(LBM_EINVAL, "tile_x must be 0, 32, 64 or 128");
  b->tile_req[k] = tile_x;
  b->desc_dirty = true;
  return LBM_OK;
}

int lbm_batch_step(lbm_batch* b, int n) {
  int r = check_ready(b);
  if (r) return r;
  if (n < 0) return bfail(LBM_EINVAL, "negative step count");
  if ((r = sync_desc(b))) return r;
  const int G = b->graph_steps;
  if (b->mode == 0 && b->lanes.empty()) {
    b->lanes.resize(b->host.size());
    b->joins.resize(b->host.size());
    for (size_t k = 0; k < b->host.size(); ++k) {
      BCK(cudaStreamCreateWithFlags(&b->lanes[k], cudaStreamNonBlocking), "lane stream");
      BCK(cudaEventCreateWithFlags(&b->joins[k], cudaEventDisableTiming), "lane event");
    }
    BCK(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming), "fork event");
  }
  while (n >= G) {
    const int par = (int)(b->steps & 1);
    if (!b->graph[par]) {
      cudaGraph_t g;
      BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "graph capture begin");
      cudaError_t ce = cudaSuccess;
      if (b->mode == 0) ce = launch_chains(b, par, G);
      else for (int s = 0; s < G; ++s) launch_one(b, (par + s) & 1, (uint32_t)s);
      k_steps_add<<<1, 1, 0, b->stream>>>(b->steps_dev, (uint32_t)G);
      cudaError_t e = cudaStreamEndCapture(b->stream, &g);
      if (ce != cudaSuccess) e = ce;
      if (e != cudaSuccess) return bfail(LBM_ECUDA, std::string("graph capture: ") + cudaGetErrorString(e));
      e = cudaGraphInstantiate(&b->graph[par], g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) return bfail(LBM_ECUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    }
    BCK(cudaGraphLaunch(b->graph[par], b->stream), "graph launch");
    b->steps += G;
    n -= G;
  }
  if (n > 0 && b->mode == 0) {
    BCK(launch_chains(b, (int)(b->steps & 1), n), "batch step launch");
    k_steps_add<<<1, 1, 0, b->stream>>>(b->steps_dev, (uint32_t)n);
    BCK(cudaGetLastError(), "step count");
    b->steps += n;
    n = 0;
  }
  for (int s = 0; s < n; ++s) {
    launch_one(b, (int)((b->steps + s) & 1), (uint32_t)s);
    BCK(cudaGetLastError(), "batch step launch");
  }
  if (n > 0) {
    k_steps_add<<<1, 1, 0, b->stream>>>(b->steps_dev, (uint32_t)n);
    BCK(cudaGetLastError(), "step count");
    b->steps += n;
  }
  return LBM_OK;
}

int lbm_batch_get_populations(lbm_batch* b, int k, double* g, size_t n) {
  if (!b || !g) return bfail(LBM_EINVAL, "null argument");
  if (k < 0 || k >= (int)b->host.size()) return bfail(LBM_EINVAL, "tunnel index out of range");
  const TunnelDesc& D = b->host[k];
  if ((int64_t)n != Q * D.d.N) return bfail(LBM_EINVAL, "population array must hold 19*N_k values");
  if (b->stage_n < D.d.N) {
    if (b->stage) cudaFree(b->stage);
    b->stage = nullptr;
    BCK(cudaMalloc(&b->stage, sizeof(double) * (size_t)D.d.N), "state staging");
    b->stage_n = D.d.N;
  }
  const Launch L = tunnel_launch(b->dims[k]);
  for (int q = 0; q < Q; ++q) {
    BCK(b->ops.get_dir(D.d, b->stage, q, (int)(b->steps & 1), true, L, b->stream), "population gather");
    BCK(cudaMemcpyAsync(g + (size_t)q * D.d.N, b->stage, sizeof(double) * D.d.N, cudaMemcpyDeviceToHost, b->stream),
        "population download");
    BCK(cudaStreamSynchronize(b->stream), "population sync");
  }
  return LBM_OK;
}

int lbm_batch_forces(lbm_batch* b, double* f) {
  if (!b || !f) return bfail(LBM_EINVAL, "null argument");
  for (size_t k = 0; k < b->host.size(); ++k) {
    const TunnelDesc& D = b->host[k];
    const Launch L = tunnel_launch(b->dims[k]);
    const int64_t nb = (int64_t)L.grid.x * L.grid.y * L.grid.z;
    if (b->npart < nb) {
      if (b->partials) cudaFree(b->partials);
      b->partials = nullptr;
      BCK(cudaMalloc(&b->partials, 3 * sizeof(double) * (size_t)nb), "reduction partials");
      b->npart = nb;
    }
    BCK(b->ops.forces(D.d, (int)(b->steps & 1), true, b->partials, L, b->stream), "force kernel");
    BCK(launch_reduce3(b->partials, nb, b->red, b->stream), "reduce kernel");
    BCK(cudaMemcpyAsync(f + 3 * k, b->red, 3 * sizeof(double), cudaMemcpyDeviceToHost, b->stream), "force download");
  }
  BCK(cudaStreamSynchronize(b->stream), "force sync");
  return LBM_OK;
}

int lbm_batch_set_mode(lbm_batch* b, int mode) {
  if (!b) return bfail(LBM_EINVAL, "null batch");
  if (mode != 0 && mode != 1) return bfail(LBM_EINVAL, "mode must be 0 (graph of tunnel chains) or 1 (one launch over all tiles)");
  BCK(cudaStreamSynchronize(b->stream), "stream sync");
  if (mode != b->mode) drop_graphs(b);
  b->desc_dirty = true;
  b->mode = mode;
  return LBM_OK;
}

int lbm_batch_get_tile(lbm_batch* b, int k, int* tile_x) {
  if (!b || !tile_x) return bfail(LBM_EINVAL, "null argument");
  if (k < 0 || k >= (int)b->host.size()) return bfail(LBM_EINVAL, "tunnel index out of range");
  int r = sync_desc(b);
  if (r) return r;
  *tile_x = b->host[k].tx;
  return LBM_OK;
}

int lbm_batch_autotune(lbm_batch* b, int steps, int* mode_out, int* minb_out, float* ms_out) {
  int r = check_ready(b);
  if (r) return r;
  if (steps < 1 || steps > 100000) return bfail(LBM_EINVAL, "steps must be in [1, 100000]");
  const int G = b->graph_steps;
  const int n = ((steps + G - 1) / G) * G;   // whole graph replays
  // every tunnel's set is saved and put back: the trials advance copies
  std::vector<void*> keep(b->host.size(), nullptr);
  for (size_t k = 0; k < b->host.size(); ++k) {
    const size_t bytes = set_cells(b->host[k].d) * Q * b->ops.elem_bytes;
    if (cudaMalloc(&keep[k], bytes) != cudaSuccess) {
      cudaGetLastError();
      for (void* p : keep) if (p) cudaFree(p);
      return bfail(LBM_ENOMEM, "no device memory for the tuner's copies of the tunnels' states");
    }
    cudaMemcpyAsync(keep[k], b->host[k].d.pop, bytes, cudaMemcpyDeviceToDevice, b->stream);
  }
  const int64_t steps0 = b->steps;
  const int mode0 = b->mode, minb0 = b->minb;
  const std::vector<int> tiles0 = b->tile_req;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  auto trial = [&](float* ms) -> int {
    b->desc_dirty = true;
    int q = lbm_batch_step(b, G);   // builds the graphs for this choice
    if (q) return q;
    if (cudaEventRecord(e0, b->stream) != cudaSuccess) return bfail(LBM_ECUDA, "tuner event");
    if ((q = lbm_batch_step(b, n))) return q;
    cudaEventRecord(e1, b->stream);
    if (cudaEventSynchronize(e1) != cudaSuccess) return bfail(LBM_ECUDA, "tuner event");
    cudaEventElapsedTime(ms, e0, e1);
    *ms /= (float)n;
    return LBM_OK;
  };
  // mode 0 (graph of per-tunnel chains), then mode 1 at both register caps
  float best = 1e30f, ms = 0.f;
  int best_mode = 0, best_minb = 8;
  std::vector<int> best_tiles = tiles0;
  b->mode = 0;
  if (!(r = trial(&ms)) && ms < best) { best = ms; best_mode = 0; }
  float best1 = 1e30f;
  int minb1 = 8;
  for (int mb : {8, 6}) {
    if (r) break;
    b->mode = 1;
    b->minb = mb;
    if (!(r = trial(&ms)) && ms < best1) { best1 = ms; minb1 = mb; }
  }
  // mode 1: tile width per size class (tunnels of equal nx), coordinate descent
  std::vector<int> classes;
  for (const auto& D : b->host) classes.push_back(D.d.nx);
  std::sort(classes.begin(), classes.end());
  classes.erase(std::unique(classes.begin(), classes.end()), classes.end());
  b->minb = minb1;
  for (int cls : classes) {
    int keep_tx = 0;
    for (int tx : {32, 64, 128}) {
      if (r) break;
      std::vector<int> save = b->tile_req;
      for (size_t k = 0; k < b->host.size(); ++k)
        if (b->host[k].d.nx == cls) b->tile_req[k] = tx;
      if (!(r = trial(&ms)) && ms < best1) { best1 = ms; keep_tx = tx; }
      b->tile_req = save;
    }
    if (keep_tx)
      for (size_t k = 0; k < b->host.size(); ++k)
        if (b->host[k].d.nx == cls) b->tile_req[k] = keep_tx;
  }
  if (!r && best1 < best) { best = best1; best_mode = 1; best_minb = minb1; best_tiles = b->tile_req; }
  // put the states back
  for (size_t k = 0; k < b->host.size(); ++k) {
    const size_t bytes = set_cells(b->host[k].d) * Q * b->ops.elem_bytes;
    cudaMemcpyAsync(b->host[k].d.pop, keep[k], bytes, cudaMemcpyDeviceToDevice, b->stream);
  }
  cudaError_t e = cudaStreamSynchronize(b->stream);
  for (void* p : keep) cudaFree(p);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  b->steps = steps0;
  k_steps_set<<<1, 1, 0, b->stream>>>(b->steps_dev, (uint32_t)steps0);
  drop_graphs(b);
  b->desc_dirty = true;
  if (r) { b->mode = mode0; b->minb = minb0; b->tile_req = tiles0; return r; }
  if (e != cudaSuccess) return bfail(LBM_ECUDA, std::string("tuner state restore: ") + cudaGetErrorString(e));
  b->mode = best_mode;
  b->minb = best_minb;
  b->tile_req = best_mode == 1 ? best_tiles : tiles0;
  if (mode_out) *mode_out = best_mode;
  if (minb_out) *minb_out = best_minb;
  if (ms_out) *ms_out = best;
  return LBM_OK;
}

int lbm_batch_info(lbm_batch* b, int64_t* total_cells, int64_t* device_bytes) {
  if (!b) return bfail(LBM_EINVAL, "null batch");
  if (total_cells) *total_cells = b->cells;
  if (device_bytes) *device_bytes = b->bytes;
  return LBM_OK;
}

}  // extern "C"

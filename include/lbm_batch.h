/*
 * lbm_batch.h — many wind tunnels of uneven sizes stepped together.
 *
 * The reference runs one tunnel per solver object and one compute dispatch
 * per tunnel step (src/backend/webgpu/solver.js:395-415).  A batch holds T
 * independent tunnels (each with its own grid, cell types and parameters —
 * the same data as one lbm_ctx) and advances all of them together.
 * lbm_batch_step captures 32 steps of every tunnel into a CUDA graph and
 * replays it: by default one independent chain of single-tunnel launches per
 * tunnel (the GPU overlaps the chains), or (lbm_batch_set_mode 1) one
 * launch per step and layout class whose CTAs (sixteen times as many as the
 * GPU holds at once) each walk every G-th tile of those tunnels.  Arithmetic
 * is identical to lbm_step (same per-cell code), so each tunnel's state
 * equals the state a separate lbm_ctx would reach.
 * Storage forms: LBM_F32 and the 16-bit forms, LBM_F16SR / LBM_BF16SR
 * included (in-place layout only; every tunnel keeps its set in the AoSoA
 * layout of lbm.h's LBM_FLAG_AOS note, blocks of 64 cells for the 16-bit
 * forms and 32 for fp32, rows padded, unless the batch is LBM_FLAG_STRICT).
 * The SR forms round each tunnel's stores with the same seeds as a separate
 * context: the batch keeps its step count on the device as well, advanced in
 * stream order by the captured graphs.
 */
#ifndef CFD_GB300_LBM_BATCH_H
#define CFD_GB300_LBM_BATCH_H

#include "lbm.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct lbm_batch lbm_batch;

/* T tunnels, dims[k] each; flags: LBM_FLAG_STRICT only. */
int lbm_batch_create(const lbm_dims* dims, int ntunnels, int storage, int flags, lbm_batch** out);
int lbm_batch_destroy(lbm_batch* b);
int lbm_batch_set_stream(lbm_batch* b, void* cuda_stream);
/* per-tunnel lbm_configure / lbm_set_types */
int lbm_batch_configure(lbm_batch* b, int k, const lbm_params* p);
int lbm_batch_set_types(lbm_batch* b, int k, const uint32_t* tipo, size_t n);
/* shaderInit in every tunnel; step counter to 0 */
int lbm_batch_init_equilibrium(lbm_batch* b);
/* n steps of every tunnel (CUDA-graph replay of the mode's launches) */
int lbm_batch_step(lbm_batch* b, int n);
/* tunnel k's state, 19*N_k doubles, natural layout (as lbm_get_populations) */
int lbm_batch_get_populations(lbm_batch* b, int k, double* g, size_t n);
/* raw momentum-exchange force of every tunnel: 3*T doubles (as lbm_forces) */
int lbm_batch_forces(lbm_batch* b, double* f);
/* tile width along x of tunnel k (32, 64 or 128 threads; the tile is 128
 * threads); 0 = the cost model (least idle threads) */
int lbm_batch_set_tile(lbm_batch* b, int k, int tile_x);
/* 0 (default): each step of each tunnel is its own launch of the
 * single-tunnel kernel; the captured graph holds one chain per tunnel and
 * the GPU runs the chains concurrently.  1: one launch per step and layout
 * class whose CTAs walk the tiles of those tunnels (descriptors in the
 * launch parameters, tile origins in a device table of 16 bytes per tile
 * that the batch allocates when it first needs it). */
int lbm_batch_set_mode(lbm_batch* b, int mode);
int lbm_batch_info(lbm_batch* b, int64_t* total_cells, int64_t* device_bytes);
/* The tile width along x tunnel k's tiles use in the mode-1 launch. */
int lbm_batch_get_tile(lbm_batch* b, int k, int* tile_x);
/* Measured choice of how the batch steps: mode 0; mode 1 with the kernel
 * built for 8 or 6 resident 128-thread CTAs per SM; then, for mode 1, the
 * tile width (32, 64, 128) of each size class (tunnels of equal nx), one
 * class at a time.  Each candidate runs `steps` steps (rounded up to whole
 * 32-step graph replays) timed with CUDA events on copies of the tunnels'
 * states; states and step count are put back, the fastest choice is kept.
 * The copies take one population set per tunnel of device memory for the
 * duration.  Outputs (nullable): mode, resident CTAs per SM, ms per step. */
int lbm_batch_autotune(lbm_batch* b, int steps, int* mode, int* min_blocks, float* ms_per_step);

#ifdef __cplusplus
}
#endif
#endif /* CFD_GB300_LBM_BATCH_H */

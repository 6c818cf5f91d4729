/*
 * lbm.h — C ABI of the GB300 (sm_103a) D3Q19 wind-tunnel solver.
 *
 * This is the drop-in boundary: every entry point replaces one member of the
 * solver class API that the reference's two browser backends share
 * (src/backend/webgpu/solver.js:36-528, src/backend/webgl2/solver.js:46-573;
 * the webgl2 file states the API is the same, src/backend/webgl2/solver.js:7-10).
 * A JavaScript host binds it through an N-API addon; the Python host in
 * cfd__gb300/solver.py binds it through ctypes.  Plain pointers and sizes only.
 *
 * Conventions
 *   - every call returns int: 0 = LBM_OK, < 0 = an LBM_E* code;
 *     lbm_last_error() returns the calling thread's last message;
 *   - a context owns all device memory it allocates; the caller owns host
 *     buffers passed in;
 *   - one CUDA stream per context (the legacy default stream unless the caller
 *     hands one in with lbm_set_stream); enqueue calls are asynchronous,
 *     lbm_read_*, lbm_get_*, lbm_forces, lbm_mass and lbm_sync synchronise;
 *   - calls on one context are not thread-safe;
 *   - no call traps or hangs the GPU: device-side loops are bounded and report
 *     LBM_ETIMEDOUT.
 *
 * Data contract (identical to the reference)
 *   - population index order, velocities and weights: src/core/lattice.js:57-89
 *     (opposite pairs adjacent: (0),(1,2),...,(17,18));
 *   - stored value is the shifted population g_i = f_i - w_i
 *     (src/core/lattice.js:6-46); rest state = all zeros;
 *   - linear cell index cell = (z*ny + y)*nx + x (src/core/emit/wgsl.js:15);
 *   - population arrays crossing this ABI are direction-major SoA,
 *     g[i*N + cell] (src/core/emit/wgsl.js:13-26), holding the post-collision
 *     state the next step streams from;
 *   - cell classes are the CELULA codes (src/core/emit/ir.js:71-80).
 */
#ifndef CFD_GB300_LBM_H
#define CFD_GB300_LBM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LBM_Q 19

/* status codes */
#define LBM_OK          0
#define LBM_EINVAL     (-1)   /* bad argument, size mismatch, null handle */
#define LBM_ENOMEM     (-2)   /* device allocation refused (message gives GB) */
#define LBM_ECUDA      (-3)   /* CUDA runtime error (message gives the call) */
#define LBM_ETIMEDOUT  (-4)   /* a bounded device or host loop gave up */
#define LBM_ESTATE     (-5)   /* call out of order (e.g. step before set_types) */
#define LBM_ENOTSUP    (-6)   /* feature not available for this storage/layout */

/* cell classes, src/core/emit/ir.js:71-80 */
#define LBM_FLUIDO        0
#define LBM_SOLIDO        1
#define LBM_ENTRADA       2
#define LBM_SAIDA         3
#define LBM_SOLIDO_MOVEL  4
#define LBM_ESPELHO_Y     5
#define LBM_ESPELHO_Z     6
#define LBM_PAREDE        7

/* population storage forms */
#define LBM_F32    0   /* fp32 g_i (152 B/cell/step) */
#define LBM_F16S   1   /* fp16 of g_i * 2^10, fp32 arithmetic (76 B/cell/step) */
#define LBM_BF16S  2   /* bf16 of g_i, fp32 arithmetic (76 B/cell/step) */
#define LBM_F64    3   /* fp64 g_i and fp64 arithmetic: the accuracy reference */
#define LBM_F16SR  4   /* as LBM_F16S, the step's stores rounded stochastically:
                          the 13 bits fp16 drops from the fp32 value decide the
                          rounding direction against a per-cell, per-step,
                          per-direction hash (unbiased; reproducible: the hash
                          depends on the cell, the step count and the
                          direction only; the learned closure's steps and
                          batched tunnels round the same way).  In-place set
                          only. */
#define LBM_BF16SR 5   /* as LBM_BF16S, stores rounded stochastically (16
                          dropped bits), same limits as LBM_F16SR */

/* lbm_create flags */
#define LBM_FLAG_WRITE_MACROS  1  /* the last step of each lbm_step writes (u, delta) */
#define LBM_FLAG_PINGPONG      2  /* two population sets, natural layout, the
                                     reference's A/B pull exactly
                                     (src/backend/webgpu/solver.js:10-24);
                                     default is one in-place set (esoteric pull) */
#define LBM_FLAG_STRICT        4  /* the shader's arithmetic read literally: one
                                     IEEE operation per written operator, no
                                     fused multiply-add (src/core/emit/ir.js);
                                     default is the FAST restatement (fixed
                                     fused multiply-adds, u = m (1/rho)); both
                                     are reproduced bit for bit by the oracle */
#define LBM_FLAG_SOA           8  /* keep the in-place set in the SoA layout
                                     (slot k of cell c at k N + c) */
#define LBM_FLAG_AOS          16  /* keep it in the AoSoA layout (blocks of
                                     cells along x, their 19 slots one after
                                     the other: 64 cells for the 16-bit
                                     forms, 32 for fp32; rows padded to a
                                     multiple of the block) where that
                                     applies: the FAST in-place step, fp32
                                     arithmetic, 19 x (padded cells) < 2^31.
                                     Without either flag: the layout
                                     lbm_autotune_layout measured faster for
                                     this grid, storage and flags earlier in
                                     the process, else AoSoA where it applies
                                     (the faster one on GB300).  The layout
                                     is internal: populations in and out are
                                     always the natural layout. */

typedef struct lbm_ctx lbm_ctx;

typedef struct { int32_t nx, ny, nz; } lbm_dims;

/* Fields of the 80-byte Params uniform (src/core/emit/wgsl.js:123-135) as the
 * reference packs them (src/backend/webgpu/solver.js:285-291).  All fp32, as
 * the uniform is.  `closure` selects the eddy-viscosity model: 0 = Smagorinsky
 * (src/core/emit/ir.js:262-301), 1 = the learned MLP set by lbm_set_closure
 * evaluated every step, k > 1 = evaluated every k-th step (lbm_closure.h). */
typedef struct {
  float omega_plus;      /* P.omegaPlus */
  float magic;           /* P.magic (TRT Lambda), default 3/16 */
  float les_cs;          /* P.lesCs, 0 disables LES exactly */
  float belt_u[3];       /* P.beltU.xyz */
  float inlet_u[3];      /* P.inletU.xyz */
  float sponge_start;    /* P.sponge.x */
  float sponge_len;      /* P.sponge.y */
  float bl_thickness;    /* P.sponge.z (espessuraCL) */
  int32_t closure;       /* 0 Smagorinsky, k >= 1 learned closure every k-th step */
} lbm_params;

typedef struct {
  int64_t n_cells;
  int64_t device_bytes;    /* everything this context allocated */
  int32_t storage;         /* LBM_F32 ... */
  int32_t flags;
  int64_t steps;           /* steps done since init / set_populations */
  int32_t parity;          /* steps & 1 — the in-place layout's phase */
  int32_t block_x;         /* chosen launch shape of the step kernel */
  int32_t layout;          /* population set: 0 in-place SoA, 1 ping-pong, 2 in-place AoSoA
                              in blocks of 32 cells, 3 in blocks of 64 */
} lbm_info;

/* SolverWebGPU.criar (src/backend/webgpu/solver.js:93-124): allocates; fails
 * with LBM_ENOMEM and a size message (GB) when the device refuses. */
int lbm_create(const lbm_dims* dims, int storage, int flags, lbm_ctx** out);

/* SolverWebGPU.destruir (src/backend/webgpu/solver.js:523-527). */
int lbm_destroy(lbm_ctx* ctx);

/* Optional: run this context's work on the caller's cudaStream_t. */
int lbm_set_stream(lbm_ctx* ctx, void* cuda_stream);

/* SolverWebGPU.configurar (src/backend/webgpu/solver.js:277-293). */
int lbm_configure(lbm_ctx* ctx, const lbm_params* p);

/* SolverWebGPU.definirTipos (src/backend/webgpu/solver.js:296-301): LBM_EINVAL
 * when n != N or a code is > 7. */
int lbm_set_types(lbm_ctx* ctx, const uint32_t* tipo, size_t n);

/* SolverWebGPU.inicializar (src/backend/webgpu/solver.js:338-349) with the
 * init kernel shaderInit (src/core/emit/wgsl.js:269-302); resets steps to 0. */
int lbm_init_equilibrium(lbm_ctx* ctx);

/* SolverWebGPU.definirCampo upload half (src/backend/webgpu/solver.js:363-389):
 * g is 19*N doubles, SoA, rounded to the storage type on upload.  Resets steps. */
int lbm_set_populations(lbm_ctx* ctx, const double* g, size_t n);

/* Reads the current state back as 19*N doubles, SoA, natural layout.  No
 * counterpart in the reference (it never reads populations back); needed for
 * state parity and checkpointing. */
int lbm_get_populations(lbm_ctx* ctx, double* g, size_t n);

/* SolverWebGPU.passo (src/backend/webgpu/solver.js:395-415): n steps enqueued
 * back to back, no sync.  With LBM_FLAG_WRITE_MACROS the last step writes the
 * pulled (pre-collision) macros (src/core/emit/wgsl.js:244-256). */
int lbm_step(lbm_ctx* ctx, int n);

/* n steps that also record, for every step, the momentum-exchange force of the
 * state the step streams from (the value medirForcas would return just before
 * that step, without the rest offset) as 3 doubles per step into out_f
 * (3*n doubles, host).  One device->host copy at the end. */
int lbm_step_forces(lbm_ctx* ctx, int n, double* out_f);

/* The same, enqueued: returns at once with a ticket (> 0) in *ticket; out_f
 * must stay valid until lbm_forces_done reports the ticket finished (with
 * page-locked memory the copy overlaps the host and the next steps).  The
 * asynchronous counterpart of medirForcas (an async method in the reference,
 * src/backend/webgpu/solver.js:486-508).  Up to 16 calls may be in flight. */
int lbm_step_forces_async(lbm_ctx* ctx, int n, double* out_f, int64_t* ticket);

/* *done = 1 when the call that returned `ticket` has landed in its out_f;
 * wait != 0 blocks until it has. */
int lbm_forces_done(lbm_ctx* ctx, int64_t ticket, int wait, int* done);

/* SolverWebGPU.atualizarMacros (src/backend/webgpu/solver.js:511-520) with
 * shaderMacros (src/core/emit/wgsl.js:442-476); solid cells report 0. */
int lbm_update_macros(lbm_ctx* ctx);

/* SolverWebGPU.lerMacros (src/backend/webgpu/solver.js:427-442): out is 4*N
 * floats (ux, uy, uz, delta) per cell. */
int lbm_read_macros(lbm_ctx* ctx, float* out, size_t n);

/* SolverWebGPU.medirForcas device half (src/backend/webgpu/solver.js:486-508,
 * kernels src/core/emit/wgsl.js:332-435): raw momentum-exchange force on the
 * SOLIDO cells, fp64 accumulation.  The caller subtracts the rest offset
 * (calibrarRepouso, src/backend/webgpu/solver.js:480-484). */
int lbm_forces(lbm_ctx* ctx, double f[3]);

/* Sum of delta over all non-solid cells of the current state, fp64.  The
 * reference computes it on the host from lerMacros (tests/nucleo.html:209-216). */
int lbm_mass(lbm_ctx* ctx, double* sum_delta);

/* Wait for all work on the context's stream. */
int lbm_sync(lbm_ctx* ctx);

int lbm_get_info(lbm_ctx* ctx, lbm_info* info);

/* Thread-local message of the last failing call ("" if none). */
const char* lbm_last_error(void);

/* Launch-shape override of the step kernel (threads along x per block; 0 =
 * the shape lbm_autotune measured for this grid, storage, flags and layout
 * earlier in the process, else 64). */
int lbm_set_block(lbm_ctx* ctx, int block_x);

/* Measured choice of the step kernel's launch: every candidate shape
 * (threads along x and y of the block, the register-cap variant, and for the
 * SoA layout the pipelined step) runs `steps` steps timed with CUDA events
 * on a copy of the current state; the state and the step count are put
 * back, the fastest shape is applied and remembered for contexts of the
 * same grid, storage, flags and layout created later in the process.  The
 * copy takes one population set of device memory for the duration.
 * Outputs (nullable): the chosen block shape, the variant code of
 * lbm_set_launch, and the measured milliseconds per step.  No counterpart
 * in the reference (its workgroup is fixed at 64 x 1 x 1,
 * src/core/emit/wgsl.js:186). */
int lbm_autotune(lbm_ctx* ctx, int steps, int* block_x, int* block_y, int* variant, float* ms_per_step);

/* Measured choice of the in-place set's layout for a grid: a free stream in
 * an all-fluid box of these dimensions runs `steps` steps in each layout
 * (timed with CUDA events; two contexts created and destroyed in turn); the
 * faster layout becomes the default of lbm_create for this grid, storage and
 * flags in this process.  layout: 2 or 3 AoSoA (blocks of 32 / 64 cells), 0 SoA (1 if flags ask for the
 * ping-pong set); ms_*: milliseconds per step (-1 where AoSoA does not
 * apply; nullable).  No counterpart in the reference. */
int lbm_autotune_layout(const lbm_dims* dims, int storage, int flags, int steps, int* layout, float* ms_aos,
                        float* ms_soa);

/* Launch shape plus register-cap variant of the plain step kernel:
 * min_blocks = 8 (64 registers/thread), 6 (80) or 0 (default 8); with the
 * AoSoA layout 8 forms the store addresses again after the collide and 9
 * keeps them in registers from the loads; with the SoA layout 8 addresses
 * each slot from its own base pointer, 20 from one base and the slots'
 * 32-bit offsets, 21 from one base and slot x N (20 and 21 need 19 N < 2^31
 * and apply to the plain step with fp32 arithmetic); 100 + k (k = 4, 8, 16)
 * selects the pipelined SoA step with k cells per thread along z. */
int lbm_set_launch(lbm_ctx* ctx, int block_x, int min_blocks);

/* Momentum-exchange force for callers that cannot allocate device memory when
 * they need it: real-time loops that must not take cudaMalloc's implicit
 * device synchronisation, and hosts that own every device buffer through
 * their own pool or allocator (a JavaScript/N-API host, a framework's
 * caching allocator).  No counterpart in the reference.  Same value as
 * lbm_forces (raw, before the rest offset), computed from buffers the caller
 * owns: pop = 19*N fp32 populations on the device, direction-major, natural
 * layout g[i*N + cell]; tipo = N cell classes on the device, ONE BYTE each
 * (uint8; lbm_set_types takes uint32 on the host, so narrow that array
 * before passing it here); f_out = 3 doubles on the device, written when the
 * work on `stream` (a cudaStream_t, NULL = legacy default stream) completes.
 * Enqueues only; no synchronisation.  Allocates nothing: its per-row partial
 * sums live in a 1.5 MiB array built into the library, so ny*nz may be at
 * most 65536 (LBM_EINVAL beyond).  The first call on a device looks up that
 * array's device address with the device current.  The address is kept per
 * device ordinal, so only the device's
 * primary context (the CUDA runtime's default) is supported.  Every call
 * shares the one array: calls that overlap on the GPU (other streams, other
 * host threads) race, so callers must order them. */
int lbm_forces_noalloc(const float* pop, const uint8_t* tipo, const lbm_dims* dims, double* f_out, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* CFD_GB300_LBM_H */

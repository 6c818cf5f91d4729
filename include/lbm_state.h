/*
 * lbm_state.h — state I/O for a solver context: checkpoint / restore of the
 * raw population storage, and a macros read-back that does not block.
 *
 * No counterpart in the reference: its populations are written
 * (definirCampo, src/backend/webgpu/solver.js:363-389) but never read back,
 * and its macros read-back (lerMacros, :427-442) waits for the copy.
 *
 * A checkpoint is a 48-byte lbm_state_header followed by the population set
 * exactly as it sits in device memory (in-place layout with its step parity,
 * or the current set of the ping-pong layout; AoSoA rows with their padding
 * cells, which stay zero), so a context restored from it
 * continues bit for bit as the saved one would have.  The learned closure's
 * held output is not part of it: after a restore the network is evaluated
 * again on the first step.
 */
#ifndef CFD_GB300_LBM_STATE_H
#define CFD_GB300_LBM_STATE_H

#include <stddef.h>
#include <stdint.h>

#include "lbm.h"

#ifdef __cplusplus
extern "C" {
#endif

#define LBM_STATE_MAGIC 0x33424743u   /* "CGB3" little-endian */
#define LBM_STATE_VERSION 1u

typedef struct {
  uint32_t magic, version;
  int32_t nx, ny, nz;
  int32_t storage;        /* LBM_F32 / LBM_F16S / LBM_BF16S / LBM_F64 */
  int32_t layout;         /* 0 in-place SoA, 1 ping-pong, 2 in-place AoSoA in blocks of 32 cells, 3 of 64 */
  int32_t parity;         /* in-place: step parity of the stored set */
  int64_t steps;          /* steps taken when saved */
  uint64_t payload_bytes; /* 19 * cells (AoSoA: rows padded) * bytes per stored value */
} lbm_state_header;

/* Bytes a checkpoint of ctx takes (header + payload). */
int lbm_state_bytes(lbm_ctx* ctx, size_t* bytes);

/* Checkpoint into dst (at least lbm_state_bytes); synchronises. */
int lbm_save_state(lbm_ctx* ctx, void* dst, size_t bytes);

/* Restore a checkpoint; LBM_EINVAL when the header does not match the
 * context (grid, storage form or layout) or the size is wrong. */
int lbm_load_state(lbm_ctx* ctx, const void* src, size_t bytes);

/* Macros of the current state (as lbm_update_macros + lbm_read_macros) into
 * out (4*N floats), enqueued on the context's stream; returns at once.  out
 * must stay valid until lbm_macros_ready reports 1 (page-locked memory lets
 * the copy overlap the host). */
int lbm_read_macros_async(lbm_ctx* ctx, float* out, size_t n);

/* *ready = 1 when the last lbm_read_macros_async has landed, else 0. */
int lbm_macros_ready(lbm_ctx* ctx, int* ready);

#ifdef __cplusplus
}
#endif
#endif /* CFD_GB300_LBM_STATE_H */

/*
 * vox.h — C ABI of the GB300 triangle-mesh voxelizer.
 *
 * Replaces voxelizar() of the reference (src/geom/voxel.js:376-433), which the
 * app calls on the CPU before building the tunnel (index.html:612-650):
 *   1. shell: every voxel whose box the surface overlaps (exact triangle-box
 *      separating-axis test, src/geom/voxel.js:61-98, gated by the squared
 *      point-triangle distance <= 0.75, :105-151, :169-228);
 *   2. seal: the shell dilated over the 26-neighbourhood (:244-267);
 *   3. flood: 6-connected fill of the exterior from the six domain faces
 *      through non-barrier voxels (:278-327);
 *   4. skin: one non-cascading growth of the exterior into non-shell voxels
 *      (:333-355);
 *   5. classes FLUIDO 0 / CASCA 1 / DENTRO 2 and the narrow-band signed
 *      distance (:401-415).
 * The output classes equal the reference's bit for bit: predicates are
 * evaluated in fp32 with a certified error bound, and the few (triangle,
 * voxel) pairs whose margin lies inside the bound are re-evaluated in fp64
 * with the reference's operation order.
 *
 * Errors are reported as LBM_E* codes with the message in lbm_last_error().
 */
#ifndef CFD_GB300_VOX_H
#define CFD_GB300_VOX_H

#include <stddef.h>
#include <stdint.h>

#include "lbm.h"

#ifdef __cplusplus
extern "C" {
#endif

#define VOX_FLUIDO 0
#define VOX_CASCA 1
#define VOX_DENTRO 2

/* The reference's stats object (src/geom/voxel.js:417-430) plus GPU counters. */
typedef struct {
  int64_t n_cells, n_casca, n_dentro, n_solido;
  int64_t triangulo_fora;   /* triangles whose banded box misses the grid */
  int32_t oco_suspeito;     /* nDentro < 0.25 nCasca and nCasca > 500 */
  int32_t flood_iterations;
  int64_t n_pairs;          /* (triangle, voxel) pairs tested */
  int64_t n_deferred;       /* pairs re-evaluated in fp64 */
  float ms_raster, ms_flood, ms_total, _pad;
} vox_stats;

/* voxelizar (src/geom/voxel.js:376-433).
 *   pos      nvert*3 float32 vertex coordinates, lattice units (cell = 1)
 *   idx      ntri*3 vertex indices (each < nvert, else LBM_EINVAL)
 *   band     distance band in cells (reference default 1.5)
 *   seal     selarFrestas (reference default 1)
 *   tipo_out N bytes: VOX_* per cell, cell = (z*ny + y)*nx + x
 *   sdf_out  N floats or NULL: signed distance, negative inside, band + 1
 *            outside the band
 *   stats    may be NULL */
int vox_voxelize(const float* pos, size_t nvert, const uint32_t* idx, size_t ntri, const lbm_dims* dims,
                 float band, int seal, uint8_t* tipo_out, float* sdf_out, vox_stats* stats);

#ifdef __cplusplus
}
#endif
#endif /* CFD_GB300_VOX_H */

/*
 * lbm_vis.h — the visualisation compute of the wind tunnel as CUDA kernels on
 * headless device buffers, reading a solver context's macros field
 * (ux, uy, uz, delta per cell) and cell types.
 *
 * The reference runs these as WebGPU compute passes inside its renderer; the
 * arithmetic is restated here without a graphics API:
 *
 *  - smoke: a passive density field advected by the flow, one step =
 *    semi-Lagrangian back-trace (pass `recuar`, src/render/fumaca.js:147-160)
 *    then the MacCormack correction with the eight-corner limiter, the
 *    dissipation, the domain cut-off and the rake emission (pass `corrigir`,
 *    src/render/fumaca.js:186-218; rake src/render/fumaca.js:96-132).  The
 *    density is stored as fp16, as the reference's rgba16float volume is;
 *    density samples are trilinear with clamp-to-edge, evaluated exactly in
 *    fp32 (the reference leaves that to the texture unit).
 *  - streak particles: Euler sub-steps through the nearest-cell velocity,
 *    ageing and the hashed respawn (src/render/renderer.js:50-117).
 *
 * Both read ctx's macros buffer as it is: it is current after a step with
 * LBM_FLAG_WRITE_MACROS or after lbm_update_macros.
 */
#ifndef CFD_GB300_LBM_VIS_H
#define CFD_GB300_LBM_VIS_H

#include <stddef.h>
#include <stdint.h>

#include "lbm.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Rake (src/render/fumaca.js:62-67, :583-590): the emission plane x, the
 * filament spacing along y and z, the filament radius, and the y / z extent. */
typedef struct {
  float x, passo_y, passo_z, raio;
  float y0, y1, z0, z1;
} vis_rake;

/* One advection step's parameters (src/render/fumaca.js:603-615): dt in
 * lattice steps, dissipation per step, injected density, and the advance in
 * cells this step stands for (dt * 0.05 in the reference). */
typedef struct {
  float dt, dissipacao, taxa, avanco;
} vis_fumo;

typedef struct vis_fumaca vis_fumaca;

/* Three fp16 volumes of the context's grid (current, next, intermediate),
 * zeroed. */
int vis_fumaca_create(lbm_ctx* ctx, vis_fumaca** out);
int vis_fumaca_destroy(vis_fumaca* f);
int vis_fumaca_limpar(vis_fumaca* f);

/* One smoke step on the context's stream. */
int vis_fumaca_passo(vis_fumaca* f, const vis_rake* rake, const vis_fumo* params);

/* Current density as fp16 bit patterns (n = N), read or written; both
 * synchronise. */
int vis_fumaca_ler(vis_fumaca* f, uint16_t* out, size_t n);
int vis_fumaca_definir(vis_fumaca* f, const uint16_t* in, size_t n);

/* Streak particles (src/render/renderer.js:51): pos = (x, y, z, life),
 * ant = (previous x, y, z, 1 when a trace is drawn / 0 on respawn). */
typedef struct {
  float pos[4];
  float ant[4];
} vis_part;

typedef struct vis_esteiras vis_esteiras;

int vis_esteiras_create(lbm_ctx* ctx, size_t n, vis_esteiras** out);
int vis_esteiras_destroy(vis_esteiras* e);
int vis_esteiras_definir(vis_esteiras* e, const vis_part* in, size_t n);
int vis_esteiras_ler(vis_esteiras* e, vis_part* out, size_t n);

/* One frame: nsub Euler sub-steps of dt_quadro / nsub each through the
 * nearest-cell velocity; `quadro` seeds the respawn hash. */
int vis_esteiras_passo(vis_esteiras* e, float dt_quadro, int nsub, uint32_t quadro);

/* The same frame for the ground streaks (src/render/rasante.js:95-149): they
 * leave below z = 0.4 and respawn just after the inlet, biased to the floor
 * (z = 0.6 + h^3 * altura). */
int vis_rasantes_passo(vis_esteiras* e, float dt_quadro, int nsub, uint32_t quadro, float altura);

/* Camera of the smoke render (the reference's scene uniform,
 * src/render/comum.js:31-47, and smoke light, src/render/fumaca.js:62-67). */
typedef struct {
  float inv_view_proj[16];   /* column-major, clip space -> world (depth 0..1) */
  float olho[3];             /* camera position, world */
  float densidade;           /* extinction per unit density */
  float g;                   /* Henyey-Greenstein anisotropy */
  int32_t passos, passos_luz;
  float luz[4];              /* light direction (normalised inside), intensity */
  float quadro;              /* frame number for the per-pixel jitter */
  int32_t largura, altura;   /* image in pixels */
} vis_camera;

/* Ray-march of the current smoke volume (src/render/fumaca.js:218-349) into
 * rgba (largura * altura * 4 floats, row 0 at the top, premultiplied
 * radiance and 1 - transmittance); no opaque depth buffer, rays that miss the
 * domain give 0.  Synchronises. */
int vis_fumaca_render(vis_fumaca* f, const vis_camera* cam, float* rgba, size_t n);

/* Surface pressure coefficient of a triangle mesh (lattice coordinates), one
 * value per triangle at its centroid, as the body shader samples it per
 * fragment (src/render/renderer.js:168-180): the face normal
 * n = normalize(cross(v1 - v0, v2 - v0)), the sample point c + 1.8 n (or
 * c - 1.8 n when that cell is solid), Cp = delta / max(1.5 u_ref^2, 1e-12)
 * from the nearest cell's macros.  Synchronises. */
int vis_cp_triangulos(lbm_ctx* ctx, const float* pos, size_t nv, const uint32_t* idx, size_t nt, float u_ref,
                      float* cp_out);

#ifdef __cplusplus
}
#endif
#endif /* CFD_GB300_LBM_VIS_H */

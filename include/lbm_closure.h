/*
 * lbm_closure.h — learned eddy-viscosity closure for the D3Q19 TRT step.
 *
 * No counterpart in the reference, whose only sub-grid model is the
 * closed-form Smagorinsky relaxation time (src/core/emit/ir.js:262-301).  A
 * 6 -> 32 -> 32 -> 1 MLP (ReLU hidden layers, softplus output) maps six
 * per-cell features of the non-equilibrium stress to an eddy viscosity
 * nu_t >= 0; the step then relaxes with tau = tau0 + 3 nu_t and the TRT
 * omega- that keeps Lambda fixed.  Smagorinsky is the per-cell fallback when
 * the network's output is not finite or exceeds nu_max.
 *
 * Features (fp32, from the pulled populations of a FLUIDO cell):
 *   x0 = ln(qs/rho + 1e-9)     qs = sqrt(2 Pi:Pi)  (|S| up to 2 rho cs^2 tau)
 *   x1 = tr(Pi) / (qs + 1e-12)
 *   x2 = det(Pi) / (qs^3 + 1e-30)
 *   x3 = (Pxy^2 + Pxz^2 + Pyz^2) / (Pi:Pi/2 + 1e-30)
 *   x4 = omega0 = 1 / tau0     (the local molecular relaxation rate)
 *   x5 = 100 delta             (density deviation)
 * checked against the trained range [lo, hi] (outside: Smagorinsky for that
 * cell), normalised as (x - mean) / std, rounded to bf16 for the tensor cores;
 * weights bf16, accumulation fp32 (tensor cores).  Training runs in fp32
 * with hand-written forward / backward / Adam kernels.  A feature can be
 * switched off by giving it a huge std (its normalised value is then 0).
 */
#ifndef CFD_GB300_LBM_CLOSURE_H
#define CFD_GB300_LBM_CLOSURE_H

#include <stddef.h>
#include <stdint.h>

#include "lbm.h"

#ifdef __cplusplus
extern "C" {
#endif

#define CLOSURE_IN 6
#define CLOSURE_H 32

typedef struct {
  float w1[CLOSURE_H * CLOSURE_IN];   /* row-major [out][in] */
  float b1[CLOSURE_H];
  float w2[CLOSURE_H * CLOSURE_H];
  float b2[CLOSURE_H];
  float w3[CLOSURE_H];
  float b3;
  float mean[CLOSURE_IN], std[CLOSURE_IN];
  float nu_scale;                      /* nu_t = nu_scale * softplus(y) */
  float nu_max;                        /* above this the cell falls back to Smagorinsky */
  float lo[CLOSURE_IN], hi[CLOSURE_IN];   /* raw-feature range the network was trained on:
                                             a cell outside it falls back to Smagorinsky
                                             (-inf / +inf: no bound) */
  int32_t coef;                        /* 0: the output is nu_t (tau = tau0 + 3 nu_t);
                                          1: the output is a per-cell Smagorinsky Cs^2,
                                          relaxed as src/core/emit/ir.js:284-299 does
                                          with 18 Cs^2 from the network */
} closure_weights;

typedef struct {
  int32_t steps;          /* Adam steps */
  int32_t batch;          /* samples per step (e.g. 65536) */
  float lr, beta1, beta2, eps;
  uint64_t seed;          /* minibatch draw and (when init != 0) weight init */
  int32_t init;           /* 1: draw initial weights from seed; 0: start from *w */
  int32_t _pad;
} closure_cfg;

/* Trains w on m samples (feats m*6 fp32 raw features, target m fp32 nu_t)
 * with the normalisation and nu_scale already set in *w.  Loss history (one
 * value per step, normalised MSE) into loss_out (may be NULL). */
int closure_train(const float* feats, const float* target, size_t m, const closure_cfg* cfg, closure_weights* w,
                  float* loss_out);

/* Loss and gradient of the current weights on a fixed set of samples, fp32
 * kernels (for checking the backward pass): grad has the layout of the
 * weight fields w1, b1, w2, b2, w3, b3 (1313 floats). */
int closure_grad(const float* feats, const float* target, size_t m, const closure_weights* w, float* loss,
                 float* grad);

/* nu_t of m feature rows through a tensor-core engine of the step (bf16
 * features and weights, fp32 accumulation); fallback rows get NaN.
 *   engine 0: warp-level mma.sync.m16n8k16, 32 cells per warp, biases added
 *             in fp32 (the accumulators start at the bias);
 *   engine 1: CTA-level tcgen05.mma, 128 cells per CTA, accumulators in
 *             tensor memory, biases in bf16 as an extra K column. */
int closure_eval(const closure_weights* w, const float* feats, size_t m, int engine, float* nu_out);

/* Training samples from a fine run held by ctx (grid nx x ny x nz; the
 * coarse grid is (nx/2, ny/2, nz/2), an odd last fine layer is dropped).
 * The fine macros are box-filtered over 2x2x2 blocks; S is the strain rate
 * of the filtered velocity by central differences on the coarse grid;
 * tau_ab = <u_a u_b> - <u_a><u_b> the resolved residual stress; the target
 * is the least-squares eddy viscosity nu_t = max(0, -tau^d:S / (2 S:S)) in
 * coarse lattice units, 0 where |S| = sqrt(2 S:S) < s_min (the ratio is
 * ill-conditioned there), and the features are those of the coarse
 * non-equilibrium stress
 * Pi = -(2/3) rho (tau0_coarse + 3 nu_t) S.  One row per coarse cell with
 * x0 <= X < x1 (X fastest, then Y, then Z): rows = (x1-x0)(ny/2)(nz/2),
 * feats 6 floats per row, target NaN where the coarse cell or one of its six
 * face neighbours has a fine cell that is not FLUIDO. */
int closure_samples(lbm_ctx* ctx, float tau0_coarse, float s_min, int x0, int x1, float* feats, float* target,
                    size_t rows);

/* Network for a solver context.  lbm_params.closure = 1 then evaluates it in
 * every step; closure = k > 1 evaluates it every k-th step and relaxes the
 * steps in between with the nu_t it gave (held per cell, 4 bytes a cell).
 * LBM_ENOTSUP for the fp64 reference form, STRICT arithmetic and ping-pong;
 * a step with the closure on a set of 19 N >= 2^31 elements (N > 113 M cells)
 * returns LBM_ENOTSUP too (the closure steps index with 32 bits). */
int lbm_set_closure(lbm_ctx* ctx, const closure_weights* w);

/* Engine of the fused step's network (see closure_eval); default 0. */
int lbm_closure_engine(lbm_ctx* ctx, int engine);

/* Network evaluations that fell back to Smagorinsky and FLUIDO cells the
 * network was evaluated for, since the last call; resets both counters.
 * LBM_ETIMEDOUT (counts still returned) if a tensor-core wait gave up. */
int lbm_closure_stats(lbm_ctx* ctx, int64_t* fallback_cells, int64_t* fluid_cells);

#ifdef __cplusplus
}
#endif
#endif /* CFD_GB300_LBM_CLOSURE_H */

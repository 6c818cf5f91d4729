/*
 * lbm_oracle.c — CPU oracle for the D3Q19 wind-tunnel step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, on the CPU, what the
 * reference's generated WGSL step computes (the reference has no CPU step of
 * its own: src/core/lattice.js:143-147).  Only tests/, the smoke check and the
 * CPU baseline leg of bench.py load it, and only to check or to time against;
 * the product library never links it.
 *
 * Built with -ffp-contract=off and without -ffast-math so every fp32 operation
 * is one IEEE operation in the order the shader text writes it.
 *
 * Tables (src/core/lattice.js:57-89):
 *   C    velocity set, opposite pairs adjacent
 *   W    1/3, 1/18 x6, 1/36 x12 — as the 9-significant-digit literals the
 *        emitter prints (num(), src/core/emit/ir.js:99-106)
 *   OPP  opp(0)=0, opp(i)=((i-1)^1)+1 (src/core/lattice.js:89)
 *   MIRROR[axis][i]  specular reflection index (espelharIdx,
 *        src/core/emit/ir.js:86-93)
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_Q 19
#define ORC_UNROLL _Pragma("GCC unroll 32")
#define ORC_FLUIDO 0u
#define ORC_SOLIDO 1u
#define ORC_ENTRADA 2u
#define ORC_SAIDA 3u
#define ORC_SOLIDO_MOVEL 4u
#define ORC_ESPELHO_Y 5u
#define ORC_ESPELHO_Z 6u
#define ORC_PAREDE 7u

#define ORC_F32 0
#define ORC_F16S 1
#define ORC_BF16S 2
#define ORC_F16SR 4
#define ORC_BF16SR 5

/* Same field layout as lbm_params in include/lbm.h. */
typedef struct {
  float omega_plus, magic, les_cs;
  float belt_u[3], inlet_u[3];
  float sponge_start, sponge_len, bl_thickness;
  int32_t closure;
} orc_params;

static const int ORC_C[ORC_Q][3] = {
    {0, 0, 0},
    {1, 0, 0},  {-1, 0, 0}, {0, 1, 0},  {0, -1, 0}, {0, 0, 1},  {0, 0, -1},
    {1, 1, 0},  {-1, -1, 0}, {1, -1, 0}, {-1, 1, 0}, {1, 0, 1},  {-1, 0, -1},
    {1, 0, -1}, {-1, 0, 1}, {0, 1, 1},  {0, -1, -1}, {0, 1, -1}, {0, -1, 1},
};
static int ORC_OPP[ORC_Q];
static int ORC_MIRROR[3][ORC_Q];

static const float W_f[ORC_Q] = {
    0.333333333f,
    0.0555555556f, 0.0555555556f, 0.0555555556f, 0.0555555556f, 0.0555555556f, 0.0555555556f,
    0.0277777778f, 0.0277777778f, 0.0277777778f, 0.0277777778f, 0.0277777778f, 0.0277777778f,
    0.0277777778f, 0.0277777778f, 0.0277777778f, 0.0277777778f, 0.0277777778f, 0.0277777778f,
};
/* 2 w_i / c_s^2 = 6 w_i, as num() prints it (src/core/emit/ir.js:185) */
static const float SIXW_f[ORC_Q] = {
    0.0f,
    0.333333333f, 0.333333333f, 0.333333333f, 0.333333333f, 0.333333333f, 0.333333333f,
    0.166666667f, 0.166666667f, 0.166666667f, 0.166666667f, 0.166666667f, 0.166666667f,
    0.166666667f, 0.166666667f, 0.166666667f, 0.166666667f, 0.166666667f, 0.166666667f,
};
/* fp64 reference form: the exact rationals rounded once to double */
static double W_d[ORC_Q];
static double SIXW_d[ORC_Q];

static void orc_tables(void) {
  static int done = 0;
  if (done) return;
  for (int i = 0; i < ORC_Q; ++i) {
    ORC_OPP[i] = i == 0 ? 0 : (((i - 1) ^ 1) + 1);
    W_d[i] = i == 0 ? 1.0 / 3.0 : (i <= 6 ? 1.0 / 18.0 : 1.0 / 36.0);
    SIXW_d[i] = i == 0 ? 0.0 : 2.0 * W_d[i] * 3.0;
  }
  for (int ax = 0; ax < 3; ++ax)
    for (int i = 0; i < ORC_Q; ++i) {
      int c[3] = {ORC_C[i][0], ORC_C[i][1], ORC_C[i][2]};
      c[ax] = -c[ax];
      ORC_MIRROR[ax][i] = -1;
      for (int j = 0; j < ORC_Q; ++j)
        if (ORC_C[j][0] == c[0] && ORC_C[j][1] == c[1] && ORC_C[j][2] == c[2]) ORC_MIRROR[ax][i] = j;
    }
  done = 1;
}

/* IEEE 754 binary16 and bfloat16 round-to-nearest-even conversions, written
 * from the format definitions. */
static uint16_t orc_f32_to_f16(float f) {
  uint32_t x;
  memcpy(&x, &f, 4);
  const uint32_t sign = (x >> 16) & 0x8000u;
  const uint32_t ex = (x >> 23) & 0xffu;
  uint32_t mant = x & 0x7fffffu;
  if (ex == 0xffu) return (uint16_t)(sign | (mant ? 0x7e00u : 0x7c00u));
  const int e = (int)ex - 127 + 15;
  if (e >= 31) return (uint16_t)(sign | 0x7c00u);
  if (e <= 0) {
    if (e < -10) return (uint16_t)sign;
    mant |= 0x800000u;
    const int shift = 14 - e;
    uint32_t hm = mant >> shift;
    const uint32_t rem = mant & ((1u << shift) - 1u);
    const uint32_t half = 1u << (shift - 1);
    if (rem > half || (rem == half && (hm & 1u))) hm++;
    return (uint16_t)(sign | hm);
  }
  uint32_t h = sign | ((uint32_t)e << 10) | (mant >> 13);
  const uint32_t rem = mant & 0x1fffu;
  if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h++;
  return (uint16_t)h;
}

static float orc_f16_to_f32(uint16_t h) {
  const uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
  const uint32_t ex = (h >> 10) & 0x1fu;
  const uint32_t mant = h & 0x3ffu;
  float f;
  if (ex == 0) {
    f = ldexpf((float)mant, -24);
    if (sign) f = -f;
    return f;
  }
  uint32_t x;
  if (ex == 31) x = sign | 0x7f800000u | (mant << 13);
  else x = sign | ((ex - 15u + 127u) << 23) | (mant << 13);
  memcpy(&f, &x, 4);
  return f;
}

static uint16_t orc_f32_to_bf16(float f) {
  uint32_t x;
  memcpy(&x, &f, 4);
  if ((x & 0x7f800000u) == 0x7f800000u && (x & 0x7fffffu)) return (uint16_t)((x >> 16) | 0x40u);
  const uint32_t lsb = (x >> 16) & 1u;
  x += 0x7fffu + lsb;
  return (uint16_t)(x >> 16);
}

static float orc_bf16_to_f32(uint16_t b) {
  const uint32_t x = (uint32_t)b << 16;
  float f;
  memcpy(&f, &x, 4);
  return f;
}

/* Round toward zero (truncation) into binary16 and bfloat16: the last step
 * of the stochastic rounding of the SR storage forms. */
static uint16_t orc_f32_to_f16_rz(float f) {
  uint32_t x;
  memcpy(&x, &f, 4);
  const uint32_t sign = (x >> 16) & 0x8000u;
  const uint32_t ex = (x >> 23) & 0xffu;
  uint32_t mant = x & 0x7fffffu;
  if (ex == 0xffu) return (uint16_t)(sign | (mant ? 0x7e00u : 0x7c00u));
  const int e = (int)ex - 127 + 15;
  if (e >= 31) return (uint16_t)(sign | 0x7bffu);   /* toward zero: the largest finite value */
  if (e <= 0) {
    if (e < -10) return (uint16_t)sign;
    mant |= 0x800000u;
    return (uint16_t)(sign | (mant >> (14 - e)));
  }
  return (uint16_t)(sign | ((uint32_t)e << 10) | (mant >> 13));
}

/* Stochastic rounding of a store (the SR storage forms, cfd__gb300/csrc/lbm_core.cuh
 * sr_seed / sr_cell_hash / sr_mult): r, the top `bits` bits of
 * hash(cell, step) * (odd multiplier of direction i), is added to the fp32
 * bit pattern of the value in the stored scale, which is then truncated. */
static inline uint32_t orc_sr_seed(int64_t step) { return (uint32_t)((uint64_t)step * 0x632BE5ABull); }
static inline uint32_t orc_sr_hash(uint32_t cell, uint32_t seed) {
  uint32_t h = cell * 0x9E3779B1u + seed;
  h ^= h >> 16;
  h *= 0x7FEB352Du;
  h ^= h >> 15;
  h *= 0x846CA68Bu;
  h ^= h >> 16;
  return h;
}
static inline uint32_t orc_sr_bits(uint32_t h, int i, int bits) {
  return (h * (0x9E3779B1u * (2u * (uint32_t)i + 1u))) >> (32 - bits);
}

static inline int orc_is_solid(uint32_t t) {
  return t == ORC_SOLIDO || t == ORC_SOLIDO_MOVEL || t == ORC_PAREDE;
}

/* ---- fp32 instantiation ---- */
#define REAL float
#define SFX _f32
#define ORC_IS_FLOAT 1
#define LIT(x) x##f
#define W__f32 W_f
#define SIXW__f32 SIXW_f
#define ORC_SQRT sqrtf
#define ORC_POW powf
#define ORC_FMA fmaf
#include "lbm_oracle_impl.h"
#undef REAL
#undef SFX
#undef ORC_IS_FLOAT
#undef LIT
#undef ORC_SQRT
#undef ORC_POW
#undef ORC_FMA

/* ---- fp64 instantiation (the accuracy reference) ---- */
#define REAL double
#define SFX _f64
#define ORC_IS_FLOAT 0
#define LIT(x) x
#define W__f64 W_d
#define SIXW__f64 SIXW_d
#define ORC_SQRT sqrt
#define ORC_POW pow
#define ORC_FMA fma
#include "lbm_oracle_impl.h"
#undef REAL
#undef SFX
#undef ORC_IS_FLOAT
#undef LIT
#undef ORC_SQRT
#undef ORC_POW
#undef ORC_FMA

/* ---- exported entry points (ctypes) ---- */
__attribute__((constructor)) static void orc_ctor(void) { orc_tables(); }
void orc_setup(void) { orc_tables(); }

void orc_tables_out(int* c57, int* opp19, int* mirror57, float* w19, float* sixw19, double* wd19) {
  orc_tables();
  for (int i = 0; i < ORC_Q; ++i) {
    for (int a = 0; a < 3; ++a) {
      c57[3 * i + a] = ORC_C[i][a];
      mirror57[a * ORC_Q + i] = ORC_MIRROR[a][i];
    }
    opp19[i] = ORC_OPP[i];
    w19[i] = W_f[i];
    sixw19[i] = SIXW_f[i];
    wd19[i] = W_d[i];
  }
}

void orc_quantize_f32(float* v, int64_t n, int storage) {
  for (int64_t i = 0; i < n; ++i) v[i] = orc_q_f32(v[i], storage);
}

uint16_t orc_f16_bits(float f) { return orc_f32_to_f16(f); }
/* One stochastically rounded store of value v (unscaled) for direction i of a
 * cell with rounding hash hsr (tests). */
float orc_sr_store_f32(float v, int storage, uint32_t hsr, int i) { return orc_qs_f32(v, storage, hsr, i); }
uint32_t orc_sr_cell_hash(uint32_t cell, int64_t step) { return orc_sr_hash(cell, orc_sr_seed(step)); }
float orc_f16_value(uint16_t h) { return orc_f16_to_f32(h); }
uint16_t orc_bf16_bits(float f) { return orc_f32_to_bf16(f); }

/*
 * lbm_oracle_impl.h — CPU restatement of the reference's D3Q19 step, init,
 * macros and momentum-exchange kernels.  TEST INFRASTRUCTURE ONLY: included
 * twice by lbm_oracle.c (REAL = float, REAL = double).  Nothing in the
 * product links this.
 *
 * Every expression keeps the operand order of the generated shader, so that a
 * build with -ffp-contract=off evaluates each fp32 operation exactly as
 * written:
 *   step body       src/core/emit/ir.js:493-533 (blocks :166-478)
 *   kernel header   src/core/emit/wgsl.js:184-222 (wrap :159-182)
 *   macros write    src/core/emit/wgsl.js:244-256
 *   init            src/core/emit/wgsl.js:269-302
 *   forces          src/core/emit/wgsl.js:332-396, reduce :407-435
 *   macros kernel   src/core/emit/wgsl.js:442-476
 *
 * Required macros: REAL, SFX (function suffix), the constant tables
 * W_SFX / SIXW_SFX (weights and 6 w_i as the shader literals), LIT(x).
 */

#define CAT2(a, b) a##b
#define CAT(a, b) CAT2(a, b)
#define FN(name) CAT(name, SFX)

/* Quantisation of stored populations (16-bit forms); identity for plain. */
static inline REAL FN(orc_q)(REAL v, int storage) {
#if ORC_IS_FLOAT
  if (storage == ORC_F16S || storage == ORC_F16SR) return orc_f16_to_f32(orc_f32_to_f16(v * 1024.0f)) * (1.0f / 1024.0f);
  if (storage == ORC_BF16S || storage == ORC_BF16SR) return orc_bf16_to_f32(orc_f32_to_bf16(v));
#else
  (void)storage;
#endif
  return v;
}

/* Quantisation of a step's output population i of a cell whose rounding hash
 * is hsr: stochastic for the SR forms, else orc_q. */
static inline REAL FN(orc_qs)(REAL v, int storage, uint32_t hsr, int i) {
#if ORC_IS_FLOAT
  if (storage == ORC_F16SR || storage == ORC_BF16SR) {
    const int f16 = storage == ORC_F16SR;
    float s = f16 ? v * 1024.0f : v;
    uint32_t x;
    memcpy(&x, &s, 4);
    x += orc_sr_bits(hsr, i, f16 ? 13 : 16);
    memcpy(&s, &x, 4);
    if (f16) return orc_f16_to_f32(orc_f32_to_f16_rz(s)) * (1.0f / 1024.0f);
    return orc_bf16_to_f32((uint16_t)(x >> 16));
  }
#else
  (void)hsr; (void)i;
#endif
  return FN(orc_q)(v, storage);
}

/* c_i . v in the order dotC (src/core/emit/ir.js:116-126) emits it. */
static inline REAL FN(orc_dotc)(int i, REAL vx, REAL vy, REAL vz) {
  const REAL v[3] = {vx, vy, vz};
  int first = 1;
  REAL acc = LIT(0.0);
  ORC_UNROLL
  for (int a = 0; a < 3; ++a) {
    const int c = ORC_C[i][a];
    if (c == 0) continue;
    if (first) { acc = c > 0 ? v[a] : -v[a]; first = 0; }
    else acc = c > 0 ? acc + v[a] : acc - v[a];
  }
  return acc;   /* 0.0 literal when c_i = 0 */
}

/* w_i (delta + rho (3 cu + 4.5 cu^2 - 1.5 uu)) ; e0 = w0 (delta - 1.5 rho uu)
 * src/core/emit/ir.js:216-232 */
static inline void FN(orc_equilibrium)(REAL delta, REAL rho, REAL ux, REAL uy, REAL uz,
                                       REAL uu, REAL* e) {
  e[0] = FN(W_)[0] * (delta - LIT(1.5) * rho * uu);
  ORC_UNROLL
  for (int i = 1; i < ORC_Q; ++i) {
    const REAL cu = FN(orc_dotc)(i, ux, uy, uz);
    e[i] = FN(W_)[i] * (delta + rho * (LIT(3.0) * cu + LIT(4.5) * cu * cu - LIT(1.5) * uu));
  }
}


/* FAST restatement of the equilibrium: w (rho a + delta) with
 * a = cu (4.5 cu + 3) - 1.5 uu, both by fused multiply-add. */
static inline void FN(orc_equilibrium_fast)(REAL delta, REAL rho, REAL ux, REAL uy, REAL uz, REAL uu15, REAL* e) {
  e[0] = FN(W_)[0] * ORC_FMA(-rho, uu15, delta);
  ORC_UNROLL
  for (int i = 1; i < ORC_Q; ++i) {
    const REAL cu = FN(orc_dotc)(i, ux, uy, uz);
    const REAL a = ORC_FMA(cu, ORC_FMA(LIT(4.5), cu, LIT(3.0)), -uu15);
    e[i] = FN(W_)[i] * ORC_FMA(rho, a, delta);
  }
}

/*
 * One reference step over every cell, A/B ping-pong, natural SoA layout.
 * src -> dst; macros (4 per cell) written when non-null.  Solid cells leave
 * dst untouched (src/core/emit/wgsl.js:201-204).
 */
void FN(orc_step)(const orc_params* P, int nx, int ny, int nz, const uint32_t* tipo,
                  const REAL* src, REAL* dst, float* macros, int storage, int nthreads, int fast_in,
                  int64_t step) {
  const uint32_t sr_seed = orc_sr_seed(step);   /* SR storage forms: the step's rounding seed */
  /* FAST restatement: fixed fused multiply-adds (ORC_FMA), u = m (1/rho),
   * omega- = (tau - 1/2) / (Lambda + (tau - 1/2)/2).  The fp64 reference form is
   * always STRICT. */
  const int fast = ORC_IS_FLOAT ? fast_in : 0;
  const int64_t N = (int64_t)nx * ny * nz;
  const REAL omegaPlus = (REAL)P->omega_plus, magic = (REAL)P->magic, lesCs = (REAL)P->les_cs;
  const REAL spStart = (REAL)P->sponge_start, spLen = (REAL)P->sponge_len;
  const REAL bl = (REAL)P->bl_thickness;
  const REAL inx = (REAL)P->inlet_u[0], iny = (REAL)P->inlet_u[1], inz = (REAL)P->inlet_u[2];
  const REAL bx = (REAL)P->belt_u[0], by = (REAL)P->belt_u[1], bz = (REAL)P->belt_u[2];
  (void)nthreads;
#if defined(_OPENMP)
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
#endif
  for (int z = 0; z < nz; ++z) {
    for (int y = 0; y < ny; ++y) {
      for (int x = 0; x < nx; ++x) {
        const int64_t cell = ((int64_t)z * ny + y) * nx + x;
        const uint32_t hsr = orc_sr_hash((uint32_t)cell, sr_seed);
        const uint32_t ct = tipo[cell];
        if (orc_is_solid(ct)) {
          if (macros) { macros[4 * cell] = 0; macros[4 * cell + 1] = 0; macros[4 * cell + 2] = 0; macros[4 * cell + 3] = 0; }
          continue;
        }
        /* periodic neighbour coordinates (src/core/emit/wgsl.js:176-180) */
        const int xs[3] = {x == 0 ? nx - 1 : x - 1, x, x == nx - 1 ? 0 : x + 1};
        const int ys[3] = {y == 0 ? ny - 1 : y - 1, y, y == ny - 1 ? 0 : y + 1};
        const int zs[3] = {z == 0 ? nz - 1 : z - 1, z, z == nz - 1 ? 0 : z + 1};

        /* inlet boundary-layer factor (src/core/emit/wgsl.js:217-220) */
        const REAL uInletBL = bl > LIT(1.0) ? bl : LIT(1.0);
        const REAL zc = (REAL)z + LIT(0.5);
        const REAL blf = zc < bl ? ORC_POW(zc / uInletBL, LIT(0.1428571429)) : LIT(1.0);
        const REAL uex = inx * blf, uey = iny * blf, uez = inz * blf;

        /* blocoPull (src/core/emit/ir.js:166-189) */
        REAL g[ORC_Q];
        g[0] = src[cell];
        ORC_UNROLL
        for (int i = 1; i < ORC_Q; ++i) {
          const int sx = xs[1 - ORC_C[i][0]], sy = ys[1 - ORC_C[i][1]], sz = zs[1 - ORC_C[i][2]];
          const int64_t s = ((int64_t)sz * ny + sy) * nx + sx;
          const uint32_t t = tipo[s];
          if (orc_is_solid(t)) {
            const REAL wx = t == ORC_SOLIDO_MOVEL ? bx : LIT(0.0);
            const REAL wy = t == ORC_SOLIDO_MOVEL ? by : LIT(0.0);
            const REAL wz = t == ORC_SOLIDO_MOVEL ? bz : LIT(0.0);
            g[i] = src[(int64_t)ORC_OPP[i] * N + cell] + FN(SIXW_)[i] * (FN(orc_dotc)(i, wx, wy, wz));
          } else {
            g[i] = src[(int64_t)i * N + s];
          }
        }

        /* blocoMomentos (src/core/emit/ir.js:192-213).  FAST: from the pair
         * sums s_k = g_i + g_j and differences d_k = g_i - g_j (j = opp i). */
        REAL sp[9], dp[9];
        REAL delta, rho, ux, uy, uz, uu, rinv = LIT(0.0);
        if (fast) {
          ORC_UNROLL
          for (int k = 0; k < 9; ++k) { sp[k] = g[2 * k + 1] + g[2 * k + 2]; dp[k] = g[2 * k + 1] - g[2 * k + 2]; }
          delta = g[0];
          ORC_UNROLL
          for (int k = 0; k < 9; ++k) delta = delta + sp[k];
          rho = LIT(1.0) + delta;
          REAL m[3];
          ORC_UNROLL
          for (int a = 0; a < 3; ++a) {
            int first = 1;
            REAL acc = LIT(0.0);
            ORC_UNROLL
            for (int k = 0; k < 9; ++k) {
              const int c = ORC_C[2 * k + 1][a];
              if (c == 0) continue;
              if (first) { acc = c > 0 ? dp[k] : -dp[k]; first = 0; }
              else acc = c > 0 ? acc + dp[k] : acc - dp[k];
            }
            m[a] = acc;
          }
          rinv = LIT(1.0) / rho;
          ux = m[0] * rinv; uy = m[1] * rinv; uz = m[2] * rinv;
          uu = ORC_FMA(uz, uz, ORC_FMA(uy, uy, ux * ux));
        } else {
          delta = g[0];
          ORC_UNROLL
          for (int i = 1; i < ORC_Q; ++i) delta = delta + g[i];
          rho = LIT(1.0) + delta;
          REAL m[3];
          ORC_UNROLL
          for (int a = 0; a < 3; ++a) {
            int first = 1;
            REAL acc = LIT(0.0);
            ORC_UNROLL
            for (int i = 0; i < ORC_Q; ++i) {
              const int c = ORC_C[i][a];
              if (c == 0) continue;
              if (first) { acc = c > 0 ? g[i] : -g[i]; first = 0; }
              else acc = c > 0 ? acc + g[i] : acc - g[i];
            }
            m[a] = acc;
          }
          ux = m[0] / rho; uy = m[1] / rho; uz = m[2] / rho;
          uu = ux * ux + uy * uy + uz * uz;
        }
        const REAL uu15 = LIT(1.5) * uu;

        REAL* out[ORC_Q];
        ORC_UNROLL
        for (int i = 0; i < ORC_Q; ++i) out[i] = dst + (int64_t)i * N + cell;

        if (ct == ORC_ESPELHO_Y || ct == ORC_ESPELHO_Z) {
          /* blocoEspelho (src/core/emit/ir.js:383-390) */
          const int ax = ct == ORC_ESPELHO_Y ? 1 : 2;
          ORC_UNROLL
          for (int i = 0; i < ORC_Q; ++i) *out[i] = FN(orc_qs)(g[ORC_MIRROR[ax][i]], storage, hsr, i);
        } else if (ct == ORC_ENTRADA && fast) {
          const REAL uuIn = ORC_FMA(uez, uez, ORC_FMA(uey, uey, uex * uex));
          const REAL uuIn15 = LIT(1.5) * uuIn;
          REAL e[ORC_Q];
          FN(orc_equilibrium_fast)(LIT(0.0), LIT(1.0), uex, uey, uez, uuIn15, e);
          for (int i = 0; i < ORC_Q; ++i) *out[i] = FN(orc_qs)(e[i], storage, hsr, i);
        } else if (ct == ORC_ENTRADA) {
          /* blocoEntrada (src/core/emit/ir.js:405-422) */
          const REAL deltaIn = LIT(0.0), rhoIn = LIT(1.0);
          const REAL uuIn = uex * uex + uey * uey + uez * uez;
          *out[0] = FN(orc_qs)(FN(W_)[0] * (deltaIn - LIT(1.5) * rhoIn * uuIn), storage, hsr, 0);
          ORC_UNROLL
          for (int i = 1; i < ORC_Q; ++i) {
            const REAL ci = FN(orc_dotc)(i, uex, uey, uez);
            *out[i] = FN(orc_qs)(FN(W_)[i] * (deltaIn + rhoIn * (LIT(3.0) * ci + LIT(4.5) * ci * ci - LIT(1.5) * uuIn)), storage, hsr, i);
          }
        } else if (ct == ORC_SAIDA && fast) {
          *out[0] = FN(orc_qs)(FN(W_)[0] * (-uu15), storage, hsr, 0);
          ORC_UNROLL
          for (int i = 1; i < ORC_Q; ++i) {
            const REAL cu = FN(orc_dotc)(i, ux, uy, uz);
            *out[i] = FN(orc_qs)(FN(W_)[i] * ORC_FMA(cu, ORC_FMA(LIT(4.5), cu, LIT(3.0)), -uu15), storage, hsr, i);
          }
        } else if (ct == ORC_SAIDA) {
          /* blocoSaida with the pulled u (src/core/emit/ir.js:432-444, :512-515) */
          *out[0] = FN(orc_qs)(FN(W_)[0] * (LIT(-1.5) * uu), storage, hsr, 0);
          ORC_UNROLL
          for (int i = 1; i < ORC_Q; ++i) {
            const REAL cu = FN(orc_dotc)(i, ux, uy, uz);
            *out[i] = FN(orc_qs)(FN(W_)[i] * (LIT(3.0) * cu + LIT(4.5) * cu * cu - LIT(1.5) * uu), storage, hsr, i);
          }
        } else if (fast) {
          /* FLUIDO, FAST pair form: e_i + e_j = 2w (delta + rho (4.5 cu^2 - 1.5 uu)),
           * e_i - e_j = 6 w rho cu, fused as B = fma(-rho, 1.5 uu, delta),
           * E = fma(4.5 rho cu, cu, B), ns = fma(-2w, E, s), nd = fma(-6 w rho, cu, d);
           * Pi from the pair sums; TRT on the pairs. */
          const REAL B = ORC_FMA(-rho, uu15, delta);
          const REAL e0 = FN(W_)[0] * B;
          const REAL a45 = LIT(4.5) * rho;
          const REAL r6a = (LIT(6.0) * FN(W_)[1]) * rho, r6d = (LIT(6.0) * FN(W_)[7]) * rho;
          REAL ns[9], nd[9];
          ORC_UNROLL
          for (int k = 0; k < 9; ++k) {
            const int i = 2 * k + 1;
            const REAL cu = FN(orc_dotc)(i, ux, uy, uz);
            const REAL E = ORC_FMA(a45 * cu, cu, B);
            ns[k] = ORC_FMA(-(LIT(2.0) * FN(W_)[i]), E, sp[k]);
            nd[k] = ORC_FMA(-(i <= 6 ? r6a : r6d), cu, dp[k]);
          }
          const REAL tau0 = LIT(1.0) / omegaPlus;
          REAL omegaP, omegaM;
          {
            static const int PA[6] = {0, 1, 2, 0, 0, 1}, PB[6] = {0, 1, 2, 1, 2, 2};
            REAL pi[6];
            ORC_UNROLL
            for (int q = 0; q < 6; ++q) {
              int first = 1;
              REAL acc = LIT(0.0);
              ORC_UNROLL
              for (int k = 0; k < 9; ++k) {
                const int coef = ORC_C[2 * k + 1][PA[q]] * ORC_C[2 * k + 1][PB[q]];
                if (coef == 0) continue;
                if (first) { acc = coef > 0 ? ns[k] : -ns[k]; first = 0; }
                else acc = coef > 0 ? acc + ns[k] : acc - ns[k];
              }
              pi[q] = acc;
            }
            const REAL pd = ORC_FMA(pi[2], pi[2], ORC_FMA(pi[1], pi[1], pi[0] * pi[0]));
            const REAL po = ORC_FMA(pi[5], pi[5], ORC_FMA(pi[4], pi[4], pi[3] * pi[3]));
            const REAL pp = ORC_FMA(LIT(2.0), po, pd);
            const REAL qs = ORC_SQRT(LIT(2.0) * pp);
            const REAL c18 = LIT(18.0) * lesCs * lesCs;
            const REAL tauT = LIT(0.5) * (tau0 + ORC_SQRT(ORC_FMA(c18 * qs, rinv, tau0 * tau0)));
            omegaP = LIT(1.0) / tauT;
            const REAL tm = tauT - LIT(0.5);
            omegaM = tm / ORC_FMA(LIT(0.5), tm, magic);
          }
          REAL o[ORC_Q];
          o[0] = ORC_FMA(-omegaP, g[0] - e0, g[0]);
          const REAL hP = LIT(0.5) * omegaP, hM = LIT(0.5) * omegaM;
          ORC_UNROLL
          for (int k = 0; k < 9; ++k) {
            const int i = 2 * k + 1, j = i + 1;
            o[i] = ORC_FMA(-hM, nd[k], ORC_FMA(-hP, ns[k], g[i]));
            o[j] = ORC_FMA(hM, nd[k], ORC_FMA(-hP, ns[k], g[j]));
          }
          const REAL sxs = ((REAL)x - spStart) / (spLen > LIT(1.0) ? spLen : LIT(1.0));
          REAL sigma = sxs > LIT(0.0) ? sxs : LIT(0.0);
          sigma = sigma < LIT(1.0) ? sigma : LIT(1.0);
          const REAL sig2 = sigma * sigma;
          if (sig2 != LIT(0.0)) {
            const REAL uuInf = ORC_FMA(inz, inz, ORC_FMA(iny, iny, inx * inx));
            const REAL uuInf15 = LIT(1.5) * uuInf;
            const REAL oms = LIT(1.0) - sig2;
            ORC_UNROLL
            for (int i = 0; i < ORC_Q; ++i) {
              const REAL si = i == 0 ? LIT(0.0) : FN(orc_dotc)(i, inx, iny, inz);
              const REAL t = i == 0 ? FN(W_)[0] * (-uuInf15)
                                    : FN(W_)[i] * ORC_FMA(si, ORC_FMA(LIT(4.5), si, LIT(3.0)), -uuInf15);
              o[i] = ORC_FMA(t, sig2, o[i] * oms);
            }
          }
          ORC_UNROLL
          for (int i = 0; i < ORC_Q; ++i) *out[i] = FN(orc_qs)(o[i], storage, hsr, i);
        } else {
          /* FLUIDO: blocoEquilibrio, blocoLES, blocoColisao, blocoEsponja */
          REAL e[ORC_Q];
          if (fast) FN(orc_equilibrium_fast)(delta, rho, ux, uy, uz, uu15, e);
          else FN(orc_equilibrium)(delta, rho, ux, uy, uz, uu, e);
          REAL n[ORC_Q];
          ORC_UNROLL
          for (int i = 0; i < ORC_Q; ++i) n[i] = g[i] - e[i];
          /* Pi_ab = sum c_ia c_ib n_i, terms in index order (src/core/emit/ir.js:269-282) */
          static const int PA[6] = {0, 1, 2, 0, 0, 1}, PB[6] = {0, 1, 2, 1, 2, 2};
          REAL pi[6];
          ORC_UNROLL
          for (int k = 0; k < 6; ++k) {
            int first = 1;
            REAL acc = LIT(0.0);
            ORC_UNROLL
            for (int i = 0; i < ORC_Q; ++i) {
              const int coef = ORC_C[i][PA[k]] * ORC_C[i][PB[k]];
              if (coef == 0) continue;
              if (first) { acc = coef > 0 ? n[i] : -n[i]; first = 0; }
              else acc = coef > 0 ? acc + n[i] : acc - n[i];
            }
            pi[k] = acc;
          }
          const REAL tau0 = LIT(1.0) / omegaPlus;
          REAL omegaP, omegaM;
          if (fast) {
            const REAL pd = ORC_FMA(pi[2], pi[2], ORC_FMA(pi[1], pi[1], pi[0] * pi[0]));
            const REAL po = ORC_FMA(pi[5], pi[5], ORC_FMA(pi[4], pi[4], pi[3] * pi[3]));
            const REAL pp = ORC_FMA(LIT(2.0), po, pd);
            const REAL qs = ORC_SQRT(LIT(2.0) * pp);
            const REAL c18 = LIT(18.0) * lesCs * lesCs;
            const REAL tauT = LIT(0.5) * (tau0 + ORC_SQRT(ORC_FMA(c18 * qs, rinv, tau0 * tau0)));
            omegaP = LIT(1.0) / tauT;
            const REAL tm = tauT - LIT(0.5);
            omegaM = tm / ORC_FMA(LIT(0.5), tm, magic);
          } else {
            const REAL pp = pi[0] * pi[0] + pi[1] * pi[1] + pi[2] * pi[2] +
                            LIT(2.0) * (pi[3] * pi[3] + pi[4] * pi[4] + pi[5] * pi[5]);
            const REAL qs = ORC_SQRT(LIT(2.0) * pp);
            const REAL tauT = LIT(0.5) * (tau0 + ORC_SQRT(tau0 * tau0 + LIT(18.0) * lesCs * lesCs * qs / rho));
            omegaP = LIT(1.0) / tauT;
            omegaM = LIT(1.0) / (magic / (LIT(1.0) / omegaP - LIT(0.5)) + LIT(0.5));
          }

          /* blocoColisao (src/core/emit/ir.js:304-323) */
          REAL o[ORC_Q];
          if (fast) o[0] = ORC_FMA(-omegaP, g[0] - e[0], g[0]);
          else o[0] = g[0] - omegaP * (g[0] - e[0]);
          ORC_UNROLL
          for (int i = 1; i < ORC_Q; i += 2) {
            const int j = i + 1;
            const REAL p = LIT(0.5) * ((g[i] + g[j]) - (e[i] + e[j]));
            const REAL mm = LIT(0.5) * ((g[i] - g[j]) - (e[i] - e[j]));
            if (fast) {
              o[i] = ORC_FMA(-omegaM, mm, ORC_FMA(-omegaP, p, g[i]));
              o[j] = ORC_FMA(omegaM, mm, ORC_FMA(-omegaP, p, g[j]));
            } else {
              o[i] = g[i] - omegaP * p - omegaM * mm;
              o[j] = g[j] - omegaP * p + omegaM * mm;
            }
          }

          /* blocoEsponja (src/core/emit/ir.js:458-478); mix(a,b,t) = a(1-t) + bt */
          const REAL sxs = ((REAL)x - spStart) / (spLen > LIT(1.0) ? spLen : LIT(1.0));
          REAL sigma = sxs > LIT(0.0) ? sxs : LIT(0.0);
          sigma = sigma < LIT(1.0) ? sigma : LIT(1.0);
          const REAL sig2 = sigma * sigma;
          if (fast) {
            const REAL uuInf = ORC_FMA(inz, inz, ORC_FMA(iny, iny, inx * inx));
            const REAL uuInf15 = LIT(1.5) * uuInf;
            REAL t[ORC_Q];
            t[0] = FN(W_)[0] * (-uuInf15);
            ORC_UNROLL
            for (int i = 1; i < ORC_Q; ++i) {
              const REAL si = FN(orc_dotc)(i, inx, iny, inz);
              t[i] = FN(W_)[i] * ORC_FMA(si, ORC_FMA(LIT(4.5), si, LIT(3.0)), -uuInf15);
            }
            if (sig2 != LIT(0.0)) {
              const REAL oms = LIT(1.0) - sig2;
              ORC_UNROLL
              for (int i = 0; i < ORC_Q; ++i) o[i] = ORC_FMA(t[i], sig2, o[i] * oms);
            }
          } else {
            const REAL uuInf = inx * inx + iny * iny + inz * inz;
            {
              const REAL t0 = FN(W_)[0] * (LIT(-1.5) * uuInf);
              o[0] = o[0] * (LIT(1.0) - sig2) + t0 * sig2;
            }
            ORC_UNROLL
            for (int i = 1; i < ORC_Q; ++i) {
              const REAL si = FN(orc_dotc)(i, inx, iny, inz);
              const REAL ti = FN(W_)[i] * (LIT(3.0) * si + LIT(4.5) * si * si - LIT(1.5) * uuInf);
              o[i] = o[i] * (LIT(1.0) - sig2) + ti * sig2;
            }
          }
          ORC_UNROLL
          for (int i = 0; i < ORC_Q; ++i) *out[i] = FN(orc_qs)(o[i], storage, hsr, i);
        }
        if (macros) {
          macros[4 * cell] = (float)ux; macros[4 * cell + 1] = (float)uy;
          macros[4 * cell + 2] = (float)uz; macros[4 * cell + 3] = (float)delta;
        }
      }
    }
  }
}

/* shaderInit (src/core/emit/wgsl.js:269-302): every cell, including solids. */
void FN(orc_init)(const orc_params* P, int nx, int ny, int nz, const uint32_t* tipo, REAL* dst,
                  int storage) {
  const int64_t N = (int64_t)nx * ny * nz;
  for (int64_t cell = 0; cell < N; ++cell) {
    const uint32_t ct = tipo[cell];
    REAL ux = (REAL)P->inlet_u[0], uy = (REAL)P->inlet_u[1], uz = (REAL)P->inlet_u[2];
    if (ct == ORC_SOLIDO) { ux = LIT(0.0); uy = LIT(0.0); uz = LIT(0.0); }
    if (ct == ORC_SOLIDO_MOVEL) { ux = (REAL)P->belt_u[0]; uy = (REAL)P->belt_u[1]; uz = (REAL)P->belt_u[2]; }
    const REAL delta = LIT(0.0), rho = LIT(1.0);
    const REAL uu = ux * ux + uy * uy + uz * uz;
    REAL e[ORC_Q];
    FN(orc_equilibrium)(delta, rho, ux, uy, uz, uu, e);
    ORC_UNROLL
    for (int i = 0; i < ORC_Q; ++i) dst[(int64_t)i * N + cell] = FN(orc_q)(e[i], storage);
  }
}

/* shaderMacros (src/core/emit/wgsl.js:442-476): moments of the stored state.
 * zero_solids = 1 writes 0 for SOLIDO/SOLIDO_MOVEL/PAREDE cells. */
void FN(orc_macros)(int nx, int ny, int nz, const uint32_t* tipo, const REAL* pop, float* macros,
                    int zero_solids) {
  const int64_t N = (int64_t)nx * ny * nz;
  for (int64_t cell = 0; cell < N; ++cell) {
    if (zero_solids && orc_is_solid(tipo[cell])) {
      macros[4 * cell] = macros[4 * cell + 1] = macros[4 * cell + 2] = macros[4 * cell + 3] = 0;
      continue;
    }
    REAL g[ORC_Q];
    ORC_UNROLL
    for (int i = 0; i < ORC_Q; ++i) g[i] = pop[(int64_t)i * N + cell];
    REAL delta = g[0];
    ORC_UNROLL
    for (int i = 1; i < ORC_Q; ++i) delta = delta + g[i];
    const REAL rho = LIT(1.0) + delta;
    REAL m[3];
    ORC_UNROLL
    for (int a = 0; a < 3; ++a) {
      int first = 1;
      REAL acc = LIT(0.0);
      ORC_UNROLL
      for (int i = 0; i < ORC_Q; ++i) {
        const int c = ORC_C[i][a];
        if (c == 0) continue;
        if (first) { acc = c > 0 ? g[i] : -g[i]; first = 0; }
        else acc = c > 0 ? acc + g[i] : acc - g[i];
      }
      m[a] = acc;
    }
    macros[4 * cell] = (float)(m[0] / rho);
    macros[4 * cell + 1] = (float)(m[1] / rho);
    macros[4 * cell + 2] = (float)(m[2] / rho);
    macros[4 * cell + 3] = (float)delta;
  }
}

/* Per-link momentum exchange of one FLUIDO cell (src/core/emit/wgsl.js:356-379):
 * q = 2 (g_i + w_i) in REAL, added component-wise as the shader's vec3. */
static inline void FN(orc_cell_force)(int nx, int ny, int nz, const uint32_t* tipo, const REAL* pop,
                                      int x, int y, int z, REAL f[3]) {
  const int64_t N = (int64_t)nx * ny * nz;
  const int64_t cell = ((int64_t)z * ny + y) * nx + x;
  f[0] = f[1] = f[2] = LIT(0.0);
  if (tipo[cell] != ORC_FLUIDO) return;
  const int xs[3] = {x == 0 ? nx - 1 : x - 1, x, x == nx - 1 ? 0 : x + 1};
  const int ys[3] = {y == 0 ? ny - 1 : y - 1, y, y == ny - 1 ? 0 : y + 1};
  const int zs[3] = {z == 0 ? nz - 1 : z - 1, z, z == nz - 1 ? 0 : z + 1};
  ORC_UNROLL
  for (int i = 1; i < ORC_Q; ++i) {
    const int64_t nb = ((int64_t)zs[1 + ORC_C[i][2]] * ny + ys[1 + ORC_C[i][1]]) * nx + xs[1 + ORC_C[i][0]];
    if (tipo[nb] != ORC_SOLIDO) continue;
    const REAL q = LIT(2.0) * (pop[(int64_t)i * N + cell] + FN(W_)[i]);
    ORC_UNROLL
    for (int a = 0; a < 3; ++a) {
      const int c = ORC_C[i][a];
      f[a] = f[a] + (c > 0 ? q : (c < 0 ? -q : LIT(0.0)));
    }
  }
}

/* Force, fp64 accumulation of the per-link REAL values (the GPU's method). */
void FN(orc_forces_acc64)(int nx, int ny, int nz, const uint32_t* tipo, const REAL* pop, double out[3]) {
  double s[3] = {0, 0, 0};
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) {
        const int64_t N = (int64_t)nx * ny * nz;
        const int64_t cell = ((int64_t)z * ny + y) * nx + x;
        if (tipo[cell] != ORC_FLUIDO) continue;
        const int xs[3] = {x == 0 ? nx - 1 : x - 1, x, x == nx - 1 ? 0 : x + 1};
        const int ys[3] = {y == 0 ? ny - 1 : y - 1, y, y == ny - 1 ? 0 : y + 1};
        const int zs[3] = {z == 0 ? nz - 1 : z - 1, z, z == nz - 1 ? 0 : z + 1};
        ORC_UNROLL
        for (int i = 1; i < ORC_Q; ++i) {
          const int64_t nb = ((int64_t)zs[1 + ORC_C[i][2]] * ny + ys[1 + ORC_C[i][1]]) * nx + xs[1 + ORC_C[i][0]];
          if (tipo[nb] != ORC_SOLIDO) continue;
          const REAL q = LIT(2.0) * (pop[(int64_t)i * N + cell] + FN(W_)[i]);
          ORC_UNROLL
          for (int a = 0; a < 3; ++a) s[a] += (double)ORC_C[i][a] * (double)q;
        }
      }
  out[0] = s[0]; out[1] = s[1]; out[2] = s[2];
}

/* Force with the reference's own REAL reduction order: per-cell vec3 in
 * direction order, a 64-lane tree per workgroup along x, then one 256-lane
 * workgroup that strides the partials and trees them
 * (src/core/emit/wgsl.js:384-393, :419-432). */
void FN(orc_forces_faithful)(int nx, int ny, int nz, const uint32_t* tipo, const REAL* pop, REAL out[3]) {
  const int gx = (nx + 63) / 64;
  const int64_t nparts = (int64_t)gx * ny * nz;
  REAL* parts = (REAL*)malloc(sizeof(REAL) * 3 * (size_t)nparts);
  REAL sh[64][3];
  for (int wz = 0; wz < nz; ++wz)
    for (int wy = 0; wy < ny; ++wy)
      for (int wx = 0; wx < gx; ++wx) {
        for (int lid = 0; lid < 64; ++lid) {
          const int x = wx * 64 + lid;
          if (x < nx) FN(orc_cell_force)(nx, ny, nz, tipo, pop, x, wy, wz, sh[lid]);
          else sh[lid][0] = sh[lid][1] = sh[lid][2] = LIT(0.0);
        }
        for (int s = 32; s > 0; s >>= 1)
          for (int lid = 0; lid < s; ++lid)
            ORC_UNROLL
            for (int a = 0; a < 3; ++a) sh[lid][a] = sh[lid][a] + sh[lid + s][a];
        const int64_t p = wx + (int64_t)gx * (wy + (int64_t)ny * wz);
        ORC_UNROLL
        for (int a = 0; a < 3; ++a) parts[3 * p + a] = sh[0][a];
      }
  REAL acc[256][3];
  for (int lid = 0; lid < 256; ++lid) {
    acc[lid][0] = acc[lid][1] = acc[lid][2] = LIT(0.0);
    for (int64_t i = lid; i < nparts; i += 256)
      ORC_UNROLL
      for (int a = 0; a < 3; ++a) acc[lid][a] = acc[lid][a] + parts[3 * i + a];
  }
  for (int s = 128; s > 0; s >>= 1)
    for (int lid = 0; lid < s; ++lid)
      ORC_UNROLL
      for (int a = 0; a < 3; ++a) acc[lid][a] = acc[lid][a] + acc[lid + s][a];
  out[0] = acc[0][0]; out[1] = acc[0][1]; out[2] = acc[0][2];
  free(parts);
}

/* Sum of delta over non-solid cells, fp64 accumulation. */
double FN(orc_mass)(int nx, int ny, int nz, const uint32_t* tipo, const REAL* pop) {
  const int64_t N = (int64_t)nx * ny * nz;
  double s = 0.0;
  for (int64_t cell = 0; cell < N; ++cell) {
    if (orc_is_solid(tipo[cell])) continue;
    REAL d = pop[cell];
    ORC_UNROLL
    for (int i = 1; i < ORC_Q; ++i) d = d + pop[(int64_t)i * N + cell];
    s += (double)d;
  }
  return s;
}

/* n steps with ping-pong (numbered from step0: the SR forms' seeds); returns
 * 0 when the state ends in a, 1 in b. */
int FN(orc_run)(const orc_params* P, int nx, int ny, int nz, const uint32_t* tipo, REAL* a, REAL* b,
                int nsteps, int storage, int nthreads, int fast, int64_t step0) {
  REAL* s = a;
  REAL* d = b;
  ORC_UNROLL
  for (int k = 0; k < nsteps; ++k) {
    FN(orc_step)(P, nx, ny, nz, tipo, s, d, NULL, storage, nthreads, fast, step0 + k);
    REAL* t = s; s = d; d = t;
  }
  return s == a ? 0 : 1;
}

#undef FN
#undef CAT
#undef CAT2

/*
 * vox_oracle.c — CPU oracle for the triangle-mesh voxelizer and the tunnel
 * cell-type assembly.
 *
 * TEST INFRASTRUCTURE ONLY (loaded by tests/ and the CPU baseline leg of
 * bench.py; never linked into the product).
 *
 * Restates src/geom/voxel.js:61-433 in fp64 with JavaScript semantics: the
 * mesh positions arrive as float32 (Float32Array) and are promoted; every
 * intermediate is a double; `dist2` is a Float32Array, so each store rounds to
 * float; Math.min/max/floor/ceil/abs/sqrt map to their C double equivalents;
 * Number.isFinite(sum of the nine coordinates) filters bad triangles.
 * Built with -ffp-contract=off so no product is fused into an add.
 *
 * Also restates montarTipos / areaFrontalCorpo / corpoAnalitico
 * (src/core/tunel.js:39-168).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define VOX_FLUIDO 0
#define VOX_CASCA 1
#define VOX_DENTRO 2

typedef struct {
  int64_t n_cells, n_casca, n_dentro, n_solido, triangulo_fora;
  int32_t oco_suspeito;
  int32_t _pad;
  int64_t n_deferred;   /* unused by the oracle (GPU-side statistic) */
} vox_stats_orc;

static inline double dmin3(double a, double b, double c) { double m = a < b ? a : b; return m < c ? m : c; }
static inline double dmax3(double a, double b, double c) { double m = a > b ? a : b; return m > c ? m : c; }

/* trianguloTocaCaixa, src/geom/voxel.js:61-98 (Akenine-Moller SAT). */
static int sat_axis(double a, double b, double fa, double fb, int i, int j, const double* v0,
                    const double* v1, const double* v2, const double* h) {
  const double p0 = a * v0[i] + b * v0[j];
  const double p1 = a * v1[i] + b * v1[j];
  const double p2 = a * v2[i] + b * v2[j];
  const double mn = dmin3(p0, p1, p2), mx = dmax3(p0, p1, p2);
  const double r = fa * h[i] + fb * h[j];
  return !(mn > r || mx < -r);
}

int orc_tri_box(const double* v0, const double* v1, const double* v2, const double* h) {
  const double e0[3] = {v1[0] - v0[0], v1[1] - v0[1], v1[2] - v0[2]};
  const double e1[3] = {v2[0] - v1[0], v2[1] - v1[1], v2[2] - v1[2]};
  const double e2[3] = {v0[0] - v2[0], v0[1] - v2[1], v0[2] - v2[2]};
  const double* es[3] = {e0, e1, e2};
  for (int k = 0; k < 3; ++k) {
    const double* e = es[k];
    const double fx = fabs(e[0]), fy = fabs(e[1]), fz = fabs(e[2]);
    if (!sat_axis(e[2], -e[1], fz, fy, 1, 2, v0, v1, v2, h)) return 0;
    if (!sat_axis(-e[2], e[0], fz, fx, 0, 2, v0, v1, v2, h)) return 0;
    if (!sat_axis(e[1], -e[0], fy, fx, 0, 1, v0, v1, v2, h)) return 0;
  }
  for (int k = 0; k < 3; ++k) {
    if (dmin3(v0[k], v1[k], v2[k]) > h[k]) return 0;
    if (dmax3(v0[k], v1[k], v2[k]) < -h[k]) return 0;
  }
  const double n[3] = {e0[1] * e1[2] - e0[2] * e1[1], e0[2] * e1[0] - e0[0] * e1[2],
                       e0[0] * e1[1] - e0[1] * e1[0]};
  const double d = n[0] * v0[0] + n[1] * v0[1] + n[2] * v0[2];
  const double r = fabs(n[0]) * h[0] + fabs(n[1]) * h[1] + fabs(n[2]) * h[2];
  return fabs(d) <= r;
}

/* distQuadPontoTriangulo, src/geom/voxel.js:105-151 (Ericson 5.1.5). */
double orc_dist2_point_tri(const double* p, const double* a, const double* b, const double* c) {
  const double abx = b[0] - a[0], aby = b[1] - a[1], abz = b[2] - a[2];
  const double acx = c[0] - a[0], acy = c[1] - a[1], acz = c[2] - a[2];
  const double apx = p[0] - a[0], apy = p[1] - a[1], apz = p[2] - a[2];
  const double d1 = abx * apx + aby * apy + abz * apz;
  const double d2 = acx * apx + acy * apy + acz * apz;
  if (d1 <= 0 && d2 <= 0) return apx * apx + apy * apy + apz * apz;
  const double bpx = p[0] - b[0], bpy = p[1] - b[1], bpz = p[2] - b[2];
  const double d3 = abx * bpx + aby * bpy + abz * bpz;
  const double d4 = acx * bpx + acy * bpy + acz * bpz;
  if (d3 >= 0 && d4 <= d3) return bpx * bpx + bpy * bpy + bpz * bpz;
  const double vc = d1 * d4 - d3 * d2;
  if (vc <= 0 && d1 >= 0 && d3 <= 0) {
    const double v = d1 / (d1 - d3);
    const double qx = apx - v * abx, qy = apy - v * aby, qz = apz - v * abz;
    return qx * qx + qy * qy + qz * qz;
  }
  const double cpx = p[0] - c[0], cpy = p[1] - c[1], cpz = p[2] - c[2];
  const double d5 = abx * cpx + aby * cpy + abz * cpz;
  const double d6 = acx * cpx + acy * cpy + acz * cpz;
  if (d6 >= 0 && d5 <= d6) return cpx * cpx + cpy * cpy + cpz * cpz;
  const double vb = d5 * d2 - d1 * d6;
  if (vb <= 0 && d2 >= 0 && d6 <= 0) {
    const double w = d2 / (d2 - d6);
    const double qx = apx - w * acx, qy = apy - w * acy, qz = apz - w * acz;
    return qx * qx + qy * qy + qz * qz;
  }
  const double va = d3 * d6 - d5 * d4;
  if (va <= 0 && (d4 - d3) >= 0 && (d5 - d6) >= 0) {
    const double w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
    const double qx = bpx + w * (cpx - bpx), qy = bpy + w * (cpy - bpy), qz = bpz + w * (cpz - bpz);
    return qx * qx + qy * qy + qz * qz;
  }
  const double den = 1 / (va + vb + vc);
  const double v = vb * den, w = vc * den;
  const double qx = apx - (v * abx + w * acx);
  const double qy = apy - (v * aby + w * acy);
  const double qz = apz - (v * abz + w * acz);
  return qx * qx + qy * qy + qz * qz;
}

/* rasterizar, src/geom/voxel.js:169-228.  flags/dist2 have N entries. */
int64_t orc_rasterize(const float* pos, const uint32_t* idx, int64_t ntri, int nx, int ny, int nz,
                      double banda, uint8_t* flags, float* dist2) {
  const int64_t N = (int64_t)nx * ny * nz;
  for (int64_t i = 0; i < N; ++i) { flags[i] = 0; dist2[i] = INFINITY; }
  const double h[3] = {0.5, 0.5, 0.5};
  int64_t fora = 0;
  for (int64_t t = 0; t < ntri; ++t) {
    const int64_t i0 = (int64_t)idx[3 * t] * 3, i1 = (int64_t)idx[3 * t + 1] * 3, i2 = (int64_t)idx[3 * t + 2] * 3;
    const double a[3] = {pos[i0], pos[i0 + 1], pos[i0 + 2]};
    const double b[3] = {pos[i1], pos[i1 + 1], pos[i1 + 2]};
    const double c[3] = {pos[i2], pos[i2 + 1], pos[i2 + 2]};
    const double sum = a[0] + a[1] + a[2] + b[0] + b[1] + b[2] + c[0] + c[1] + c[2];
    if (!isfinite(sum)) continue;
    double lo[3], hi[3];
    const int n[3] = {nx, ny, nz};
    int r0[3], r1[3];
    for (int k = 0; k < 3; ++k) {
      lo[k] = floor(dmin3(a[k], b[k], c[k]) - banda);
      hi[k] = ceil(dmax3(a[k], b[k], c[k]) + banda);
      const double l = lo[k] > 0 ? lo[k] : 0;
      const double u = hi[k] < n[k] - 1 ? hi[k] : n[k] - 1;
      r0[k] = l > 2147483647.0 ? 2147483647 : (int)l;
      r1[k] = u < -2147483647.0 ? -2147483647 : (int)u;
    }
    if (r1[0] < r0[0] || r1[1] < r0[1] || r1[2] < r0[2]) { fora++; continue; }
    for (int z = r0[2]; z <= r1[2]; ++z)
      for (int y = r0[1]; y <= r1[1]; ++y) {
        const int64_t base = ((int64_t)z * ny + y) * nx;
        for (int x = r0[0]; x <= r1[0]; ++x) {
          const double p[3] = {x + 0.5, y + 0.5, z + 0.5};
          const int64_t cell = base + x;
          const double d2 = orc_dist2_point_tri(p, a, b, c);
          if (d2 < (double)dist2[cell]) dist2[cell] = (float)d2;
          if (d2 <= 0.75 && flags[cell] != VOX_CASCA) {
            const double la[3] = {a[0] - p[0], a[1] - p[1], a[2] - p[2]};
            const double lb[3] = {b[0] - p[0], b[1] - p[1], b[2] - p[2]};
            const double lc[3] = {c[0] - p[0], c[1] - p[1], c[2] - p[2]};
            if (orc_tri_box(la, lb, lc, h)) flags[cell] = VOX_CASCA;
          }
        }
      }
  }
  return fora;
}

/* dilatar, src/geom/voxel.js:244-267 (26-neighbourhood, clamped). */
void orc_dilate(const uint8_t* flags, int nx, int ny, int nz, uint8_t* d) {
  const int64_t N = (int64_t)nx * ny * nz;
  memset(d, 0, (size_t)N);
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) {
        if (flags[((int64_t)z * ny + y) * nx + x] != VOX_CASCA) continue;
        const int z0 = z > 0 ? z - 1 : 0, z1 = z < nz - 1 ? z + 1 : nz - 1;
        const int y0 = y > 0 ? y - 1 : 0, y1 = y < ny - 1 ? y + 1 : ny - 1;
        const int x0 = x > 0 ? x - 1 : 0, x1 = x < nx - 1 ? x + 1 : nx - 1;
        for (int k = z0; k <= z1; ++k)
          for (int j = y0; j <= y1; ++j)
            for (int i = x0; i <= x1; ++i) d[((int64_t)k * ny + j) * nx + i] = 1;
      }
}

/* inundarExterior, src/geom/voxel.js:278-327: 6-connected fill from the six
 * faces through non-barrier cells.  Explicit stack (the visit order does not
 * change the reached set). */
void orc_flood(const uint8_t* barreira, int nx, int ny, int nz, uint8_t* visitado) {
  const int64_t N = (int64_t)nx * ny * nz;
  const int64_t nxny = (int64_t)nx * ny;
  memset(visitado, 0, (size_t)N);
  int64_t* pilha = (int64_t*)malloc(sizeof(int64_t) * (size_t)N);
  int64_t topo = 0;
#define PUSH(c) do { const int64_t _c = (c); if (!visitado[_c] && !barreira[_c]) { visitado[_c] = 1; pilha[topo++] = _c; } } while (0)
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y) { PUSH(((int64_t)z * ny + y) * nx); PUSH(((int64_t)z * ny + y) * nx + nx - 1); }
  for (int z = 0; z < nz; ++z)
    for (int x = 0; x < nx; ++x) { PUSH(((int64_t)z * ny) * nx + x); PUSH(((int64_t)z * ny + ny - 1) * nx + x); }
  for (int y = 0; y < ny; ++y)
    for (int x = 0; x < nx; ++x) { PUSH((int64_t)y * nx + x); PUSH(((int64_t)(nz - 1) * ny + y) * nx + x); }
  while (topo > 0) {
    const int64_t cell = pilha[--topo];
    const int64_t x = cell % nx;
    const int64_t y = (cell / nx) % ny;
    const int64_t z = cell / nxny;
    if (x > 0) PUSH(cell - 1);
    if (x < nx - 1) PUSH(cell + 1);
    if (y > 0) PUSH(cell - nx);
    if (y < ny - 1) PUSH(cell + nx);
    if (z > 0) PUSH(cell - nxny);
    if (z < nz - 1) PUSH(cell + nxny);
  }
#undef PUSH
  free(pilha);
}

/* recuperarPele, src/geom/voxel.js:333-355: one non-cascading growth of the
 * exterior into non-shell cells. */
void orc_skin(uint8_t* exterior, const uint8_t* flags, int nx, int ny, int nz) {
  const int64_t N = (int64_t)nx * ny * nz;
  const int64_t nxny = (int64_t)nx * ny;
  uint8_t* antes = (uint8_t*)malloc((size_t)N);
  memcpy(antes, exterior, (size_t)N);
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) {
        const int64_t c = ((int64_t)z * ny + y) * nx + x;
        if (antes[c] || flags[c] == VOX_CASCA) continue;
        const int viz = (x > 0 && antes[c - 1]) || (x < nx - 1 && antes[c + 1]) ||
                        (y > 0 && antes[c - nx]) || (y < ny - 1 && antes[c + nx]) ||
                        (z > 0 && antes[c - nxny]) || (z < nz - 1 && antes[c + nxny]);
        if (viz) exterior[c] = 1;
      }
  free(antes);
}

/* voxelizar, src/geom/voxel.js:376-433.  tipo_out: N bytes {0,1,2};
 * sdf_out: N floats (nullable). */
int orc_voxelize(const float* pos, int64_t nvert, const uint32_t* idx, int64_t ntri, int nx, int ny,
                 int nz, double banda, int selar, uint8_t* tipo_out, float* sdf_out,
                 vox_stats_orc* st) {
  (void)nvert;
  const int64_t N = (int64_t)nx * ny * nz;
  uint8_t* flags = (uint8_t*)malloc((size_t)N);
  float* dist2 = (float*)malloc(sizeof(float) * (size_t)N);
  uint8_t* barreira = (uint8_t*)malloc((size_t)N);
  uint8_t* exterior = (uint8_t*)malloc((size_t)N);
  const int64_t fora = orc_rasterize(pos, idx, ntri, nx, ny, nz, banda, flags, dist2);
  if (selar) orc_dilate(flags, nx, ny, nz, barreira);
  else memcpy(barreira, flags, (size_t)N);
  orc_flood(barreira, nx, ny, nz, exterior);
  if (selar) orc_skin(exterior, flags, nx, ny, nz);
  int64_t nc = 0, nd = 0;
  for (int64_t i = 0; i < N; ++i) {
    uint8_t t = VOX_FLUIDO;
    if (flags[i] == VOX_CASCA) { t = VOX_CASCA; nc++; }
    else if (!exterior[i]) { t = VOX_DENTRO; nd++; }
    tipo_out[i] = t;
  }
  if (sdf_out) {
    const double fora_banda = banda + 1;
    for (int64_t i = 0; i < N; ++i) {
      const double d = isinf(dist2[i]) ? fora_banda : sqrt((double)dist2[i]);
      sdf_out[i] = (float)(tipo_out[i] == VOX_FLUIDO ? d : -d);
    }
  }
  if (st) {
    memset(st, 0, sizeof(*st));
    st->n_cells = N; st->n_casca = nc; st->n_dentro = nd; st->n_solido = nc + nd;
    st->triangulo_fora = fora;
    st->oco_suspeito = ((double)nd < (double)nc * 0.25) && nc > 500;
  }
  free(flags); free(dist2); free(barreira); free(exterior);
  return 0;
}

/* ---- tunnel assembly, src/core/tunel.js ---- */

/* montarTipos (src/core/tunel.js:39-108); corpo nullable (VOXEL codes). */
void orc_montar_tipos(int nx, int ny, int nz, const uint8_t* corpo, int esteira, double fracao,
                      uint32_t* tipo, double* sponge_start, double* sponge_len) {
  const int64_t N = (int64_t)nx * ny * nz;
  for (int64_t i = 0; i < N; ++i) tipo[i] = (corpo && corpo[i] != VOX_FLUIDO) ? 1u : 0u;
  const uint32_t piso = esteira ? 4u : 7u;
#define IDX(x, y, z) ((((int64_t)(z)) * ny + (y)) * nx + (x))
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y) { tipo[IDX(0, y, z)] = 2u; tipo[IDX(nx - 1, y, z)] = 3u; }
  for (int z = 0; z < nz; ++z)
    for (int x = 0; x < nx; ++x) { tipo[IDX(x, 0, z)] = 5u; tipo[IDX(x, ny - 1, z)] = 5u; }
  for (int y = 0; y < ny; ++y)
    for (int x = 0; x < nx; ++x) { tipo[IDX(x, y, 0)] = piso; tipo[IDX(x, y, nz - 1)] = 6u; }
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y) { tipo[IDX(0, y, z)] = 2u; tipo[IDX(nx - 1, y, z)] = 3u; }
#undef IDX
  /* Math.round(v) = floor(v + 0.5) */
  double comp = floor(nx * fracao + 0.5);
  if (comp < 4) comp = 4;
  *sponge_len = comp;
  *sponge_start = nx - 1 - comp;
}

/* areaFrontalCorpo (src/core/tunel.js:118-133). */
int64_t orc_area_frontal_corpo(const uint8_t* corpo, int nx, int ny, int nz) {
  int64_t n = 0;
  for (int z = 1; z < nz - 1; ++z)
    for (int y = 1; y < ny - 1; ++y) {
      const int64_t base = ((int64_t)z * ny + y) * nx;
      for (int x = 1; x < nx - 1; ++x)
        if (corpo[base + x] != VOX_FLUIDO) { n++; break; }
    }
  return n;
}

/* corpoAnalitico (src/core/tunel.js:144-168): kind 0 sphere, 1 cylinder (axis y). */
void orc_corpo_analitico(int nx, int ny, int nz, int kind, double cx, double cy, double cz, double raio,
                         uint8_t* corpo) {
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) {
        const double dx = x + 0.5 - cx, dy = y + 0.5 - cy, dz = z + 0.5 - cz;
        const int dentro = kind == 0 ? (dx * dx + dy * dy + dz * dz <= raio * raio)
                                     : (dx * dx + dz * dz <= raio * raio);
        corpo[((int64_t)z * ny + y) * nx + x] = dentro ? VOX_DENTRO : VOX_FLUIDO;
      }
}

// lbm_kernels.cuh — the step, init, macros, force and mass kernels, templated
// on the population storage form.  Included by one lbm_inst_<form>.cu per form
// (compiled in parallel, -fmad=false).
//
// Two population layouts:
//
//  * IN-PLACE (default).  One population set; each population crosses HBM once
//    per step (read 19, write 19: 152 B/cell in fp32).  The scheme is the
//    "esoteric pull" of Lehmann (2022, Computation 10(6):92): for each
//    opposite pair (i, i+1), i odd, with nb = x + c_i, a cell reads and writes
//    the same two slots, F[.][x] and F[.][nb], swapping which slot holds which
//    direction with the step parity.  With e = (steps even):
//        pulled g_i     = F[e ? i+1 : i][x]      (= post-collision g_i(x - c_i))
//        pulled g_{i+1} = F[e ? i : i+1][nb]     (= post-collision g_{i+1}(x + c_i))
//        writes g*_i -> F[e ? i : i+1][nb],  g*_{i+1} -> F[e ? i+1 : i][x]
//    The reference's fluid-node bounce-back (src/core/emit/ir.js:166-189) needs
//    the cell's own post-collision g_{opp k} when x - c_k is solid.  That value
//    sits in the other slot of the same location, which in this step belongs
//    to the solid cell and is touched by nobody else, so the bounce-back read
//    is the same load with the slot bit flipped: race-free and exact.
//
//  * A/B PING-PONG (flag LBM_FLAG_PINGPONG).  The reference's own scheme
//    (src/backend/webgpu/solver.js:10-24): natural SoA, pull from the 18
//    neighbours of src into dst, types gathered per direction.  Kept as the
//    faithful debug path; both layouts give bit-identical states.
#pragma once
#include <algorithm>
#include <type_traits>

#include "closure_mlp.cuh"
#include "lbm_core.cuh"

struct lbm_ctx;   // include/lbm.h

namespace lbm {

// Device-side view of one context's buffers.
struct Dev {
  int nx, ny, nz;
  int64_t N;
  void* pop;          // in-place: the set; ping-pong: the current (front) set
  void* pop2;         // ping-pong only: the back set
  const uint8_t* tipo;   // cell classes
  const uint32_t* link;  // link words (in-place layout)
  float4* macros;        // nullable
  double* force;         // nullable: kForceSlots x 3 doubles accumulated by the fused force
  const void* blf;       // nullable: nz inlet boundary-layer factors in the arithmetic type
  int aos;               // 0: the in-place set in SoA; else its AoSoA block width (32 or 64, elem_off)
  int nxp;               // AoSoA: the row length in cells, nx rounded up to the block width
  uint32_t seed;         // the SR storage forms' rounding seed: sr_seed(step count), or with
  const uint32_t* seed_base;   // a device step counter (batches) sr_seed(*seed_base + seed)
};

// The step's rounding seed (the SR storage forms).
__device__ __forceinline__ uint32_t dev_seed(const Dev& d) {
  return d.seed_base ? sr_seed((int64_t)(uint32_t)(*d.seed_base + d.seed)) : d.seed;
}

// The in-place set's two layouts.  SoA: slot k of location c at k N + c.
// AoSoA: each row of nx cells is padded to nxp, a multiple of the block
// width B, and the padded cells are cut into blocks of B along x; a block
// holds its 19 slots one after the other, B elements each, so slot k of the
// location with padded index p = (z ny + y) nxp + x sits at
// (p / B) 19 B + B k + p % B = (p & ~(B-1)) 19 + B k + (p & (B-1)).  A
// warp's access to one slot still covers 32 consecutive elements, and every
// slot of a location is a constant offset (B k elements) from the location's
// slot 0.  B = 32 for fp32 (a slot row is a 128-byte line), 64 for the
// 16-bit forms (again a 128-byte line, read by a CTA's two warps together).
// The padding cells are never read or written.
constexpr int kAosB = 32;
__host__ __device__ __forceinline__ int64_t aos_base(int64_t c, int B = kAosB) {
  return (c & ~(int64_t)(B - 1)) * 19 + (c & (B - 1));
}
// The padded index of cell c (AoSoA).
__device__ __forceinline__ int64_t padded_cell(const Dev& d, int64_t c) {
  return d.nxp == d.nx ? c : c + (c / d.nx) * (int64_t)(d.nxp - d.nx);
}
// d.aos: 0 (SoA) or the AoSoA block width
__device__ __forceinline__ int64_t elem_off(const Dev& d, int k, int64_t c) {
  return d.aos ? aos_base(padded_cell(d, c), d.aos) + (int64_t)d.aos * k : (int64_t)k * d.N + c;
}

struct Wrap {
  int xm, xp, ym, yp, zm, zp;
};

__device__ __forceinline__ Wrap wrap3(int x, int y, int z, int nx, int ny, int nz) {
  Wrap w;
  w.xm = x == 0 ? nx - 1 : x - 1;
  w.xp = x == nx - 1 ? 0 : x + 1;
  w.ym = y == 0 ? ny - 1 : y - 1;
  w.yp = y == ny - 1 ? 0 : y + 1;
  w.zm = z == 0 ? nz - 1 : z - 1;
  w.zp = z == nz - 1 ? 0 : z + 1;
  return w;
}

// Cell index of x + s*c_k (s = +1 downstream, -1 upstream), periodic.
__device__ __forceinline__ int64_t nbr(int k, int s, int x, int y, int z, const Wrap& w, int nx, int ny) {
  const int dx = s * cx(k), dy = s * cy(k), dz = s * cz(k);
  const int xx = dx > 0 ? w.xp : (dx < 0 ? w.xm : x);
  const int yy = dy > 0 ? w.yp : (dy < 0 ? w.ym : y);
  const int zz = dz > 0 ? w.zp : (dz < 0 ? w.zm : z);
  return ((int64_t)zz * ny + yy) * nx + xx;
}

// Where post-collision population k of cell `cell` lives in the in-place
// layout at parity p (0: before an even step).  Returns the element offset.
__device__ __forceinline__ int64_t eso_loc(const Dev& d, int k, int p, int64_t cell, int x, int y, int z,
                                           const Wrap& w) {
  if (k == 0) return elem_off(d, 0, cell);
  if (k & 1) {  // + member of the pair, stored at the downstream neighbour
    const int64_t nb = nbr(k, +1, x, y, z, w, d.nx, d.ny);
    return elem_off(d, p == 0 ? k + 1 : k, nb);
  }
  return elem_off(d, p == 0 ? k - 1 : k, cell);  // - member, stored locally
}

// Warp-level fp64 sum of three values; lane 0 adds them to dst atomically.
// The fused force of one step accumulates into kForceSlots copies of
// (fx, fy, fz), the block row picking the copy, so that the cells next to the
// body do not all serialise on the same three addresses; the host (or
// k_sum_slots) sums the copies.  Each such cell adds its own contribution
// where it is computed: no value stays live through the collide and no warp
// has to reconverge for a reduction.
constexpr int kForceSlots = 32;

__device__ __forceinline__ void add_force(double* dst, double a, double b, double c) {
  double* slot = dst + 3 * ((blockIdx.y + blockIdx.z * gridDim.y) & (kForceSlots - 1));
  atomicAdd(slot + 0, a);
  atomicAdd(slot + 1, b);
  atomicAdd(slot + 2, c);
}

// ------------------------------------------------------------------ step
// Offsets are 32-bit when every element index of a population set fits
// (19 N < 2^31, up to 113 M cells), else 64-bit.
template <bool W64> struct OffT { using type = int32_t; };
template <> struct OffT<true> { using type = int64_t; };

// Periodic neighbour displacements of one cell (src/core/emit/wgsl.js:176-180).
template <typename Off>
struct Deltas {
  Off xp, yp, ym, zp, zm;
  __device__ __forceinline__ Deltas(int x, int y, int z, int nx, int ny, int nz) {
    const Off nxny = (Off)nx * ny;
    xp = x == nx - 1 ? (Off)(1 - nx) : (Off)1;
    yp = y == ny - 1 ? (Off)nx - nxny : (Off)nx;
    ym = y == 0 ? nxny - (Off)nx : -(Off)nx;
    zp = z == nz - 1 ? -nxny * (Off)(nz - 1) : nxny;
    zm = z == 0 ? nxny * (Off)(nz - 1) : -nxny;
  }
  // x + c_i for the odd (first) member of each pair
  __device__ __forceinline__ Off odd(int i) const {
    switch (i) {
      case 1: return xp;
      case 3: return yp;
      case 5: return zp;
      case 7: return xp + yp;
      case 9: return xp + ym;
      case 11: return xp + zp;
      case 13: return xp + zm;
      case 15: return yp + zp;
      default: return yp + zm;   // 17
    }
  }
};

// An integer the compiler must treat as changed here (an empty asm): values
// derived from it are formed again afterwards instead of being kept live.
__device__ __forceinline__ void opaque(int32_t& v) { asm volatile("" : "+r"(v)); }
__device__ __forceinline__ void opaque(uint32_t& v) { asm volatile("" : "+r"(v)); }
__device__ __forceinline__ void opaque(int64_t& v) { asm volatile("" : "+l"(v)); }
template <class T>
__device__ __forceinline__ void opaque(T*& p) { asm volatile("" : "+l"(p)); }

// Where the in-place step of parity PAR finds the two slots of pair k
// (i = 2k + 1): slot A = (E ? i + 1 : i) holds, at the cell itself, the
// pulled g_i and receives g*_{i+1}; slot B = (E ? i : i + 1) holds, at the
// neighbour x + c_i, the pulled g_{i+1} and receives g*_i.  A bounce-back
// link re-reads the other slot of the same location (B at the cell, A at
// the neighbour).
__host__ __device__ constexpr int slot_a(int k, int par) { return par == 0 ? 2 * k + 2 : 2 * k + 1; }
__host__ __device__ constexpr int slot_b(int k, int par) { return par == 0 ? 2 * k + 1 : 2 * k + 2; }

// Base pointers of the population slots for one launch of the in-place step
// (parity-dependent), passed by value in the kernel parameters: an access is
// then base + element index, formed in one multiply-add with the base read
// from the constant bank.
struct SlotPtrs {
  void* a[9];
  void* b[9];
  void* rest;
  int32_t oa[9];    // the same slots as element offsets from the set's base
  int32_t ob[9];    // (filled when 19 N < 2^31)
};

template <class St>
inline SlotPtrs make_slots(const Dev& d, int par) {
  using S = typename St::store_t;
  SlotPtrs t;
  S* F = static_cast<S*>(d.pop);
  for (int k = 0; k < 9; ++k) {
    t.a[k] = F + (int64_t)slot_a(k, par) * d.N;
    t.b[k] = F + (int64_t)slot_b(k, par) * d.N;
    const bool fits = (int64_t)Q * d.N < (int64_t)INT32_MAX;
    t.oa[k] = fits ? (int32_t)((int64_t)slot_a(k, par) * d.N) : 0;
    t.ob[k] = fits ? (int32_t)((int64_t)slot_b(k, par) * d.N) : 0;
  }
  t.rest = F;
  return t;
}

// Addressing of one cell's accesses: from the set's base, the slot offset
// and the neighbour displacement (AddrSet), or from the launch's slot
// pointers and the cell / neighbour element indices (AddrSlots).
template <class St, int PAR, class Off>
struct AddrSet {
  using S = typename St::store_t;
  S* Fc;
  Off N;
  Deltas<Off> D;
  __device__ __forceinline__ AddrSet(const Dev& d, Off cell, int x, int y, int z)
      : Fc(static_cast<S*>(d.pop) + cell), N((Off)d.N), D(x, y, z, d.nx, d.ny, d.nz) {}
  // the slot and neighbour addresses are formed again for the stores
  // (the batched kernel, whose descriptors leave fewer registers free)
  __device__ __forceinline__ void refresh() {
    opaque(Fc); opaque(N); opaque(D.xp); opaque(D.yp); opaque(D.ym); opaque(D.zp); opaque(D.zm);
  }
  __device__ __forceinline__ S* rest() const { return Fc; }
  __device__ __forceinline__ S* a(int k, bool nb) const {
    return Fc + (nb ? D.odd(2 * k + 1) : (Off)0) + (Off)slot_a(k, PAR) * N;
  }
  __device__ __forceinline__ S* b(int k, bool nb) const {
    return Fc + (nb ? D.odd(2 * k + 1) : (Off)0) + (Off)slot_b(k, PAR) * N;
  }
};

template <class St, int PAR, class Off>
struct AddrSlots {
  using S = typename St::store_t;
  const SlotPtrs& T;
  Off cell;
  Deltas<Off> D;
  __device__ __forceinline__ AddrSlots(const Dev& d, const SlotPtrs& t, Off c, int x, int y, int z)
      : T(t), cell(c), D(x, y, z, d.nx, d.ny, d.nz) {}
  __device__ __forceinline__ void refresh() {}
  __device__ __forceinline__ S* rest() const { return static_cast<S*>(T.rest) + cell; }
  __device__ __forceinline__ S* a(int k, bool nb) const {
    return static_cast<S*>(T.a[k]) + (nb ? cell + D.odd(2 * k + 1) : cell);
  }
  __device__ __forceinline__ S* b(int k, bool nb) const {
    return static_cast<S*>(T.b[k]) + (nb ? cell + D.odd(2 * k + 1) : cell);
  }
};

// SoA addressing from one base pointer and the slots' 32-bit element
// offsets in the launch parameters (19 N < 2^31): slot offset + cell +
// displacement is one 32-bit add with a constant-bank operand.  The index
// state is made opaque before the collide, so the store addresses are formed
// again rather than kept live.
template <class St, int PAR>
struct AddrOffs {
  using S = typename St::store_t;
  S* F;
  const SlotPtrs& T;
  int32_t cell;
  Deltas<int32_t> D;
  __device__ __forceinline__ AddrOffs(const Dev& d, const SlotPtrs& t, int32_t c, int x, int y, int z)
      : F(static_cast<S*>(d.pop)), T(t), cell(c), D(x, y, z, d.nx, d.ny, d.nz) {}
  __device__ __forceinline__ void refresh() {
    opaque(cell); opaque(D.xp); opaque(D.yp); opaque(D.ym); opaque(D.zp); opaque(D.zm);
  }
  __device__ __forceinline__ S* rest() const { return F + cell; }
  __device__ __forceinline__ S* a(int k, bool nb) const { return F + (T.oa[k] + (nb ? cell + D.odd(2 * k + 1) : cell)); }
  __device__ __forceinline__ S* b(int k, bool nb) const { return F + (T.ob[k] + (nb ? cell + D.odd(2 * k + 1) : cell)); }
};

// Neighbour displacements in AoSoA elements (aos_base(c + d) - aos_base(c)):
// a y or z displacement is a whole number of blocks, so it is 19 times the
// cell displacement; +1 in x is +1 inside a block, the next block's lane 0
// (19 * 32 - 31) from lane 31, and the row's first block from x = nx - 1.
template <class Off, int B = kAosB>
struct DeltasAos {
  Off xp, yp, ym, zp, zm;
  // bw: the block width when B = 0 (chosen at run time); nxp: the padded
  // row length.  +1 in x from the row's last cell wraps to its first.
  __device__ __forceinline__ DeltasAos(int x, int y, int z, int nx, int nxp, int ny, int nz, int bw = B) {
    const Deltas<Off> D(x, y, z, nxp, ny, nz);   // y and z strides of the padded rows
    const int W = B ? B : bw;
    const Off next = (Off)(19 * W - (W - 1));
    const int l = nx - 1;
    xp = x == l ? -((Off)(l & ~(W - 1)) * 19 + (Off)(l & (W - 1))) : ((x & (W - 1)) != W - 1 ? (Off)1 : next);
    yp = (Off)19 * D.yp;
    ym = (Off)19 * D.ym;
    zp = (Off)19 * D.zp;
    zm = (Off)19 * D.zm;
  }
  __device__ __forceinline__ Off odd(int i) const {
    switch (i) {
      case 1: return xp;
      case 3: return yp;
      case 5: return zp;
      case 7: return xp + yp;
      case 9: return xp + ym;
      case 11: return xp + zp;
      case 13: return xp + zm;
      case 15: return yp + zp;
      default: return yp + zm;   // 17
    }
  }
};

// AoSoA addressing: the location's slot-0 element (own cell, or a
// neighbour's) plus the slot as a constant 32 k elements.  RF: make the index
// state opaque to the compiler before the collide, so that the store
// addresses are formed again instead of being kept in registers since the
// loads (fewer live registers, more instructions); the tuner picks.  PAD:
// the rows may be padded (nxp > nx); without it the padded index is the cell
// index, one term less for the register allocation of the tightest kernels.
template <class St, int PAR, class Off, bool RF = true, int B = kAosB, bool PAD = true>
struct AddrAos {
  using S = typename St::store_t;
  S* F;
  Off ob;
  DeltasAos<Off, B> D;
  __device__ __forceinline__ AddrAos(const Dev& d, Off cell, int x, int y, int z)
      : F(static_cast<S*>(d.pop)),
        ob((Off)aos_base(PAD ? cell + ((Off)z * d.ny + y) * (Off)(d.nxp - d.nx) : cell, B)),
        D(x, y, z, d.nx, d.nxp, d.ny, d.nz) {}
  __device__ __forceinline__ void refresh() {
    if constexpr (RF) { opaque(ob); opaque(D.xp); opaque(D.yp); opaque(D.ym); opaque(D.zp); opaque(D.zm); }
  }
  __device__ __forceinline__ S* rest() const { return F + ob; }
  __device__ __forceinline__ S* a(int k, bool nb) const {
    return (F + (nb ? ob + D.odd(2 * k + 1) : ob)) + B * slot_a(k, PAR);
  }
  __device__ __forceinline__ S* b(int k, bool nb) const {
    return (F + (nb ? ob + D.odd(2 * k + 1) : ob)) + B * slot_b(k, PAR);
  }
};

// Either layout, chosen per context at run time (d.aos is the same for every
// thread): the closure steps, whose time goes to the network, not to
// addressing.
template <class St, int PAR, class Off>
struct AddrRt {
  using S = typename St::store_t;
  S* F;
  Off N, own;
  int bw;   // AoSoA block width, 0 for SoA
  Deltas<Off> D;
  DeltasAos<Off, 0> DA;
  __device__ __forceinline__ AddrRt(const Dev& d, Off cell, int x, int y, int z)
      : F(static_cast<S*>(d.pop)), N((Off)d.N),
        own(d.aos ? (Off)aos_base(cell + ((Off)z * d.ny + y) * (Off)(d.nxp - d.nx), d.aos) : cell), bw(d.aos),
        D(x, y, z, d.nx, d.ny, d.nz), DA(x, y, z, d.nx, d.nxp, d.ny, d.nz, d.aos ? d.aos : kAosB) {}
  __device__ __forceinline__ Off at(int slot, int k, bool nb) const {
    if (bw) return (nb ? own + DA.odd(2 * k + 1) : own) + (Off)(bw * slot);
    return (nb ? own + D.odd(2 * k + 1) : own) + (Off)slot * N;
  }
  __device__ __forceinline__ S* rest() const { return F + own; }
  __device__ __forceinline__ S* a(int k, bool nb) const { return F + at(slot_a(k, PAR), k, nb); }
  __device__ __forceinline__ S* b(int k, bool nb) const { return F + at(slot_b(k, PAR), k, nb); }
};

// A store of an unscaled population value: rounded to nearest, or for the SR
// storage forms stochastically with the cell's hash (the offset is formed
// when the value exists: the empty asm ties the hash to it).
template <class St>
struct PopStore {
  uint32_t h;
  __device__ __forceinline__ PopStore(const Dev& d, uint32_t cell) : h(0u) {
    if constexpr (St::kSR) h = sr_cell_hash(cell, dev_seed(d));
  }
  template <class S, class R>
  __device__ __forceinline__ void operator()(S* p, R v, int i) const {
    if constexpr (St::kSR) {
      uint32_t hh = h;
      const R vs = v * R(St::kScale);
      asm volatile("" : "+r"(hh) : "f"(vs));
      St::st_sr(p, vs, (hh * sr_mult(i)) >> (32 - St::kSRBits));
    } else {
      St::st(p, v);
    }
  }
};

// In-place step.  Grid: (ceil(nx/bx), ceil(ny/by), nz), block (bx, by).
// PAR: step parity (0 even).  MAC: write (u, delta).  FRC: accumulate the
// momentum-exchange force of the state being streamed.
// One cell of the in-place step (everything the step does for cell x, y, z).
// Shared by the single-tunnel kernel and the batched kernel, so both run
// the identical arithmetic.
// FRC: the cell's momentum-exchange force goes to d.force (add_force).
template <class St, int PAR, bool MAC, bool FRC, bool W64, bool FAST, class Addr, class Rates = SmagRates>
__device__ __forceinline__ void step_cell_at(const Dev& d, const Params& P, const Uni<typename St::real>& U, int x,
                                             int y, int z, typename OffT<W64>::type cell, Addr ad,
                                             Rates rates = Rates()) {
  double fx = 0.0, fy = 0.0, fz = 0.0;
  using R = typename St::real;
  using S = typename St::store_t;
  // SC: a form stored times a power-of-two scale (fp16) runs the FAST collide
  // on the stored values themselves (moments_fast_scaled): bit-identical
  // results without a multiply per loaded and per stored population.
  constexpr bool SC = FAST && St::kScaled;
  const R scale = R(St::kScale), inv_scale = R(1.0) / R(St::kScale);
  auto ld = [](const S* p) -> R { return SC ? St::ld_raw(p) : St::ld(p); };
  auto st = [](S* p, R v) { if (SC) St::st_raw(p, v); else St::st(p, v); };
  const int nx = d.nx, ny = d.ny;
  // The normal-slot loads do not wait for the link word: they are issued
  // together with it, and the rare bounce-back links are re-read below.
  const uint32_t lw = __ldg(d.link + cell);
  R g[Q];
  g[0] = ld(ad.rest());
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    g[2 * k + 1] = ld(ad.a(k, false));
    g[2 * k + 2] = ld(ad.b(k, true));
  }
  const uint32_t ct = (lw >> LINK_CLASS_SHIFT) & 7u;
  if (is_solid(ct)) {
    if (MAC) d.macros[cell] = make_float4(0.f, 0.f, 0.f, 0.f);
    return;
  }
  const uint32_t bbmask = lw & 0x3ffffu;
  if (bbmask) {
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      if ((bbmask >> (2 * k)) & 1u) g[2 * k + 1] = ld(ad.b(k, false));
      if ((bbmask >> (2 * k + 1)) & 1u) g[2 * k + 2] = ld(ad.a(k, true));
    }
    // Bounce-back links: moving-wall term and the fused force (the force
    // uses the unscaled g: fma(S g, 1/S, w) = RN(g + w)).
    auto link_q = [&](int k) -> R {
      return R(2.0) * (SC ? fma_r<R>(g[k], inv_scale, Lit<R>::w(k)) : g[k] + Lit<R>::w(k));
    };
    if (lw & LINK_SLOW) {
      const Wrap w = wrap3(x, y, z, nx, ny, d.nz);
#pragma unroll
      for (int k = 1; k < Q; ++k) {
        if (!((bbmask >> (k - 1)) & 1u)) continue;
        const uint32_t t = d.tipo[nbr(k, -1, x, y, z, w, nx, ny)];
        if (t == SOLIDO_MOVEL) {
          const R mw = Lit<R>::sixw(k) * (dotc<R>(k, R(P.belt[0]), R(P.belt[1]), R(P.belt[2])));
          g[k] = g[k] + (SC ? mw * scale : mw);
        }
        if (FRC && ct == FLUIDO && t == SOLIDO) {
          const R q = link_q(k);
          fx -= (double)(cx(k) * q); fy -= (double)(cy(k) * q); fz -= (double)(cz(k) * q);
        }
      }
    } else if (FRC && ct == FLUIDO && (lw & LINK_BODY)) {
#pragma unroll
      for (int k = 1; k < Q; ++k) {
        if (!((bbmask >> (k - 1)) & 1u)) continue;
        const R q = link_q(k);
        fx -= (double)(cx(k) * q); fy -= (double)(cy(k) * q); fz -= (double)(cz(k) * q);
      }
    }
    if (FRC && (fx != 0.0 || fy != 0.0 || fz != 0.0)) add_force(d.force, fx, fy, fz);
  }
  R delta, rho, ux, uy, uz, uu, rinv = R(0.0);
  R sp[9], dp[9];
  if (SC) moments_fast_scaled<R>(g, inv_scale, sp, dp, delta, rho, ux, uy, uz, uu, rinv);
  else if (FAST) moments_fast<R>(g, sp, dp, delta, rho, ux, uy, uz, uu, rinv);
  else moments_strict<R>(g, delta, rho, ux, uy, uz, uu);
  if (MAC) d.macros[cell] = make_float4((float)ux, (float)uy, (float)uz, (float)(SC ? delta * inv_scale : delta));
  // g*_i of an odd i goes to the neighbour's slot B; g*_{i+1} stays local in
  // slot A; the rest population stays put.
  ad.refresh();
  // the SR storage forms round each store stochastically (sr_cell_hash)
  uint32_t hsr = 0;
  if constexpr (St::kSR) hsr = sr_cell_hash((uint32_t)cell, dev_seed(d));
  auto put = [&](S* p, R v, int i) {
    if constexpr (St::kSR) {
      // the hash passes through an empty asm that also reads the stored
      // value, so each rounding offset is formed when its value exists, not
      // all 19 at the start (which would keep them live through the collide)
      uint32_t h = hsr;
      const R vs = SC ? v : v * R(St::kScale);
      asm volatile("" : "+r"(h) : "f"(vs));
      St::st_sr(p, vs, (h * sr_mult(i)) >> (32 - St::kSRBits));
    } else {
      st(p, v);
    }
  };
  collide<R, FAST, SC>(P, U, ct, x, z, g, sp, dp, delta, rho, ux, uy, uz, uu, rinv, static_cast<const R*>(d.blf),
                       [&](int i, R v) {
    if (i == 0) put(ad.rest(), v, 0);
    else if (i & 1) put(ad.b((i - 1) >> 1, true), v, i);
    else put(ad.a((i - 2) >> 1, false), v, i);
  }, scale, rates);
}

// One cell of the in-place step (everything the step does for cell x, y, z),
// addressing from the set's base.  Shared by the batched kernel, so it runs
// the identical arithmetic.  FRC: the cell's momentum-exchange force goes to
// d.force (add_force).
template <class St, int PAR, bool MAC, bool FRC, bool W64, bool FAST>
__device__ __forceinline__ void step_cell(const Dev& d, const Params& P, const Uni<typename St::real>& U, int x, int y,
                                          int z) {
  using Off = typename OffT<W64>::type;
  const Off cell = ((Off)z * d.ny + y) * d.nx + x;
  step_cell_at<St, PAR, MAC, FRC, W64, FAST>(d, P, U, x, y, z, cell, AddrSet<St, PAR, Off>(d, cell, x, y, z));
}

// MINB: minimum resident 128-thread blocks per SM the register allocation
// must allow (8 -> 64 registers, 6 -> 80); the autotuner picks per form.  The
// fused force is added where it is computed, so the force variant fits 64 too.
// SOAV (SoA set): 0 slot pointers (AddrSlots), 1 one base and 32-bit slot
// offsets (AddrOffs), 2 one base and slot x N (AddrSet); 1 and 2 need
// 19 N < 2^31.
// PAD (AoSoA): rows padded to the block width (false: nx is a multiple of it).
template <class St, int PAR, bool MAC, bool FRC, bool W64, bool FAST, int MINB, bool AOS = false, bool RF = true,
          int SOAV = 0, int AB = kAosB, bool PAD = true>
__global__ void __launch_bounds__(128, MINB)
k_step_inplace(Dev d, Params P, Uni<typename St::real> U, SlotPtrs T) {
  using Off = typename OffT<W64>::type;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x < d.nx && y < d.ny) {
    const Off cell = ((Off)z * d.ny + y) * d.nx + x;
    if constexpr (AOS)
      step_cell_at<St, PAR, MAC, FRC, W64, FAST>(d, P, U, x, y, z, cell,
                                                 AddrAos<St, PAR, Off, RF, AB, PAD>(d, cell, x, y, z));
    else if constexpr (SOAV == 1 && !W64)
      step_cell_at<St, PAR, MAC, FRC, W64, FAST>(d, P, U, x, y, z, cell, AddrOffs<St, PAR>(d, T, cell, x, y, z));
    else if constexpr (SOAV == 2 && !W64)
      step_cell_at<St, PAR, MAC, FRC, W64, FAST>(d, P, U, x, y, z, cell, AddrSet<St, PAR, Off>(d, cell, x, y, z));
    else
      step_cell_at<St, PAR, MAC, FRC, W64, FAST>(d, P, U, x, y, z, cell,
                                                 AddrSlots<St, PAR, Off>(d, T, cell, x, y, z));
  }
}

// Arguments of the closure step.
struct CloArgs {
  const MlpFrag* F;             // the network
  unsigned long long* nfb;      // fallback counter (cells whose output was not usable)
  unsigned* err;                // set when a tensor-core wait gave up (engine 1)
  float* nu;                    // per-cell output: written by mode 1, read by mode 2
  float omega0;                 // feature x4 = 1 / tau0
  int coef;                     // 1: the output is a Smagorinsky Cs^2, 0: nu_t
  CloConst K;                   // feature range, normalisation, output bounds
};

// Shared memory of the warp engine: it parks a fluid cell's pulled g and
// moments (a column per thread) while the network runs, so that the
// registers of the pull and of the network are not live at the same time.
struct CloShared {
  float stash[Q + 7][128];
};

// In-place step with the learned eddy-viscosity closure (fp32 arithmetic,
// FAST form).  The same pull, bounce-back and fused force as step_cell.
// MODE 0: for FLUIDO cells the six features of the pulled non-equilibrium
//   stress feed the network, which gives nu_t and tau = tau0 + 3 nu_t,
//   omega- keeping Lambda fixed (or, in the coefficient form, a per-cell
//   Cs^2 for the Smagorinsky relaxation); a cell whose features are outside the
//   trained range or whose output is not usable relaxes with the Smagorinsky
//   rates (src/core/emit/ir.js:284-299) and is counted.
// MODE 1: the same, and nu_t (NaN for a fallback cell) is stored per cell.
// MODE 2: no network: the rates come from the stored nu_t (Smagorinsky where
//   it is NaN) -- the steps between two network evaluations of a closure
//   that is evaluated every k-th step.  Not instantiated: those steps run
//   k_step_held, the plain step's cell code with the same rate rule.
// This kernel is the warp engine (closure_mlp.cuh, mma.sync per 32 cells);
// the CTA engine is k_step_closure_tc below.  Every other class goes through
// collide() unchanged, before the network.  Modes 0 and 1 run 64 x 2 threads
// per block; mode 2 any shape.
template <class St, int PAR, bool MAC, bool FRC, bool W64, int ENG, int MODE>
__global__ void __launch_bounds__(128, MODE == 2 ? 8 : 6)
k_step_closure(Dev d, Params P, Uni<float> U, CloArgs A) {
  using R = float;
  using S = typename St::store_t;
  using Off = typename OffT<W64>::type;
  static_assert(sizeof(typename St::real) == 4, "closure step is fp32 arithmetic");
  static_assert(ENG == 0, "the CTA engine is k_step_closure_tc");
  constexpr bool NET = MODE != 2;
  __shared__ CloShared SH;
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  const int nx = d.nx, ny = d.ny;
  const bool inr = x < nx && y < ny;
  const Off cell = ((Off)z * ny + y) * nx + x;
  const AddrRt<St, PAR, Off> ad(d, cell, x, y, z);
  double fx = 0.0, fy = 0.0, fz = 0.0;
  const PopStore<St> put(d, (uint32_t)cell);
  auto emit = [&](int i, R v) {
    if (i == 0) put(ad.rest(), v, 0);
    else if (i & 1) put(ad.b((i - 1) >> 1, true), v, i);
    else put(ad.a((i - 2) >> 1, false), v, i);
  };
  R g[Q];
  R delta = R(0.0), rho = R(1.0), ux = R(0.0), uy = R(0.0), uz = R(0.0), uu = R(0.0), rinv = R(1.0);
  float feat[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  bool fluid = false, inside = false;
  if (inr) {
    const uint32_t lw = __ldg(d.link + cell);
    g[0] = St::ld(ad.rest());
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      g[2 * k + 1] = St::ld(ad.a(k, false));
      g[2 * k + 2] = St::ld(ad.b(k, true));
    }
    const uint32_t ct = (lw >> LINK_CLASS_SHIFT) & 7u;
    if (is_solid(ct)) {
      if (MAC) d.macros[cell] = make_float4(0.f, 0.f, 0.f, 0.f);
    } else {
      const uint32_t bb = lw & 0x3ffffu;
      if (bb) {
#pragma unroll
        for (int k = 0; k < 9; ++k) {
          if ((bb >> (2 * k)) & 1u) g[2 * k + 1] = St::ld(ad.b(k, false));
          if ((bb >> (2 * k + 1)) & 1u) g[2 * k + 2] = St::ld(ad.a(k, true));
        }
        if (lw & LINK_SLOW) {
          const Wrap w = wrap3(x, y, z, nx, ny, d.nz);
#pragma unroll
          for (int k = 1; k < Q; ++k) {
            if (!((bb >> (k - 1)) & 1u)) continue;
            const uint32_t t = d.tipo[nbr(k, -1, x, y, z, w, nx, ny)];
            if (t == SOLIDO_MOVEL) g[k] = g[k] + Lit<R>::sixw(k) * (dotc<R>(k, R(P.belt[0]), R(P.belt[1]), R(P.belt[2])));
            if (FRC && ct == FLUIDO && t == SOLIDO) {
              const R q = R(2.0) * (g[k] + Lit<R>::w(k));
              fx -= (double)(cx(k) * q); fy -= (double)(cy(k) * q); fz -= (double)(cz(k) * q);
            }
          }
        } else if (FRC && ct == FLUIDO && (lw & LINK_BODY)) {
#pragma unroll
          for (int k = 1; k < Q; ++k) {
            if (!((bb >> (k - 1)) & 1u)) continue;
            const R q = R(2.0) * (g[k] + Lit<R>::w(k));
            fx -= (double)(cx(k) * q); fy -= (double)(cy(k) * q); fz -= (double)(cz(k) * q);
          }
        }
      }
      if (FRC && (fx != 0.0 || fy != 0.0 || fz != 0.0)) add_force(d.force, fx, fy, fz);
      R sp[9], dp[9];
      moments_fast<R>(g, sp, dp, delta, rho, ux, uy, uz, uu, rinv);
      if (MAC) d.macros[cell] = make_float4(ux, uy, uz, delta);
      if (ct == FLUIDO) {
        fluid = true;
        if constexpr (NET) {
          // Pi_ab = sum_i c_ia c_ib g_i - (delta / 3) delta_ab - rho u_a u_b
          // (minus the shifted equilibrium's second moment), for the features
          const PiT<R> m = pi_fast<R>(sp);
          const R d3 = delta * R(1.0 / 3.0);
          const R rux = rho * ux, ruy = rho * uy, ruz = rho * uz;
          closure_features(m.xx - d3 - rux * ux, m.yy - d3 - ruy * uy, m.zz - d3 - ruz * uz, m.xy - rux * uy,
                           m.xz - rux * uz, m.yz - ruy * uz, rinv, delta, feat);
          feat[4] = A.omega0;
          inside = closure_in_range(A.K, feat);
#pragma unroll
          for (int a = 0; a < 6; ++a) feat[a] = (feat[a] - A.K.mean[a]) * A.K.inv_std[a];
#pragma unroll
          for (int i = 0; i < Q; ++i) SH.stash[i][tid] = g[i];
          SH.stash[Q + 0][tid] = delta; SH.stash[Q + 1][tid] = rho; SH.stash[Q + 2][tid] = ux;
          SH.stash[Q + 3][tid] = uy; SH.stash[Q + 4][tid] = uz; SH.stash[Q + 5][tid] = uu;
          SH.stash[Q + 6][tid] = rinv;
        }
      } else {
        collide<R, true>(P, U, ct, x, z, g, sp, dp, delta, rho, ux, uy, uz, uu, rinv, static_cast<const R*>(d.blf),
                         emit);
      }
    }
  }
  float nu = 0.0f;
  if constexpr (NET) {
    __syncwarp();
    const float yv = warp_mlp(*A.F, feat);
    if (fluid) {
#pragma unroll
      for (int i = 0; i < Q; ++i) g[i] = SH.stash[i][tid];
      delta = SH.stash[Q + 0][tid]; rho = SH.stash[Q + 1][tid]; ux = SH.stash[Q + 2][tid];
      uy = SH.stash[Q + 3][tid]; uz = SH.stash[Q + 4][tid]; uu = SH.stash[Q + 5][tid];
      rinv = SH.stash[Q + 6][tid];
      nu = inside ? closure_nu(A.K, yv) : __int_as_float(0x7fc00000);
      if (MODE == 1) A.nu[cell] = nu;
    }
  } else {
    if (fluid) nu = __ldg(A.nu + cell);
  }
  bool fell_back = false;
  if (fluid) {
    R sp[9], dp[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      sp[k] = g[2 * k + 1] + g[2 * k + 2];
      dp[k] = g[2 * k + 1] - g[2 * k + 2];
    }
    R e0, ns[9], nd[9];
    fluid_neq_fast<R>(sp, dp, delta, rho, ux, uy, uz, uu, e0, ns, nd);
    R omegaP, omegaM;
    if (nu == nu) {
      if (A.coef) {
        // coefficient form: the output is Cs^2 of the Smagorinsky relaxation
        smag_rates_c18<R>(P, U, ns, rinv, 18.0f * nu, omegaP, omegaM);
      } else {
        const float tauT = U.tau0 + 3.0f * nu, tm = tauT - 0.5f;
        omegaP = __frcp_rn(tauT);
        omegaM = __fdividef(tm, fmaf(0.5f, tm, P.magic));
      }
    } else {
      fell_back = true;
      smag_rates_fast<R>(P, U, ns, rinv, omegaP, omegaM);
    }
    trt_emit_fast<R>(U, x, g, e0, ns, nd, omegaP, omegaM, U.sp_tf, emit);
  }
  if constexpr (NET) {
    const unsigned fb = __ballot_sync(0xffffffffu, fell_back);
    if (fb && (threadIdx.x & 31) == 0 && A.nfb) atomicAdd(A.nfb, (unsigned long long)__popc(fb));
  }
}

// The learned-closure step on the CTA engine (closure_tc.cuh): persistent
// CTAs of 128 threads walk tiles of 64 x 2 cells (x, y) of one z plane; a CTA
// sets up its tensor memory, mbarrier and B operands once.  Per tile every
// thread pulls its cell exactly as k_step_closure does, collides the
// boundary classes at once, and for a FLUIDO cell keeps the pulled g and its
// moments in registers while the network runs (one CTA barrier and one
// tcgen05.mma round trip per hidden layer, the output layer on the CUDA
// cores); then the rates and TRT as in
// k_step_closure.  MODE 0 or 1 (mode 2 has no network: k_step_closure).
// Rates of the closure's held steps (evaluated every k-th step): from the
// eddy viscosity stored per cell by the last network step, the Smagorinsky
// rates where it is NaN (a fallback cell) -- the same rules as the network
// step uses with a fresh output.
struct HeldRates {
  float v;     // the cell's stored eddy viscosity (or Cs^2), loaded with the populations
  int coef;
  template <typename R>
  __device__ __forceinline__ void operator()(const Params& P, const Uni<R>& U, const R* ns, R rinv, R& omegaP,
                                             R& omegaM) const {
    if (v == v) {
      if (coef) {
        smag_rates_c18<R>(P, U, ns, rinv, 18.0f * v, omegaP, omegaM);
      } else {
        const float tauT = U.tau0 + 3.0f * v, tm = tauT - 0.5f;
        omegaP = __frcp_rn(tauT);
        omegaM = __fdividef(tm, fmaf(0.5f, tm, P.magic));
      }
    } else {
      smag_rates_fast<R>(P, U, ns, rinv, omegaP, omegaM);
    }
  }
};

// A held closure step: the plain in-place step's cell code and addressing
// (either layout), with HeldRates for FLUIDO cells.
// AB: the AoSoA block width, 0 for the SoA layout.
template <class St, int PAR, bool MAC, bool FRC, int AB>
__global__ void __launch_bounds__(128, 8) k_step_held(Dev d, Params P, Uni<typename St::real> U, SlotPtrs T,
                                                      const float* __restrict__ nu, int coef) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x < d.nx && y < d.ny) {
    const int32_t cell = (z * d.ny + y) * d.nx + x;
    const HeldRates rates{__ldg(nu + cell), coef};
    if constexpr (AB != 0)
      step_cell_at<St, PAR, MAC, FRC, false, true>(d, P, U, x, y, z, cell,
                                                   AddrAos<St, PAR, int32_t, true, AB>(d, cell, x, y, z), rates);
    else
      step_cell_at<St, PAR, MAC, FRC, false, true>(d, P, U, x, y, z, cell,
                                                   AddrSlots<St, PAR, int32_t>(d, T, cell, x, y, z), rates);
  }
}

constexpr int kClosureTcPerSm = 6;
template <class St, int PAR, bool MAC, bool FRC, bool W64, int MODE, int AB>
__global__ void __launch_bounds__(128, kClosureTcPerSm)
k_step_closure_tc(Dev d, Params P, Uni<float> U, CloArgs A, SlotPtrs T, int gx, int gy) {
  using R = float;
  using S = typename St::store_t;
  using Off = typename OffT<W64>::type;
  static_assert(sizeof(typename St::real) == 4, "closure step is fp32 arithmetic");
  static_assert(MODE != 2, "held steps have no network");
  __shared__ TcPersist SH;
  const int tid = threadIdx.x;
  const uint32_t tmem = tcp_setup(SH, A.F->tcb, A.F->w3b, tid);
  uint32_t phase = 0;
  bool dead = false;
  unsigned nfb = 0;
  const int nx = d.nx, ny = d.ny;
  // tile t = (z gy + byi) gx + bxi, walked with stride gridDim.x: the
  // decomposition is divided out once and then advanced with carries
  const int G = (int)gridDim.x;
  const int gsx = G % gx, gsy = (G / gx) % gy, gsz = G / (gx * gy);
  int bxi = (int)blockIdx.x % gx, byi = ((int)blockIdx.x / gx) % gy, z = (int)blockIdx.x / (gx * gy);
  for (; z < d.nz;) {
    const int x = bxi * 64 + (tid & 63), y = byi * 2 + (tid >> 6);
    const bool inr = x < nx && y < ny;
    const Off cell = ((Off)z * ny + (inr ? y : 0)) * nx + (inr ? x : 0);
    // addressing of the context's layout (32-bit offsets), or either layout
    // chosen at run time for sets past 2^31 elements
    using Ad = std::conditional_t<W64, AddrRt<St, PAR, Off>,
                                  std::conditional_t<AB != 0, AddrAos<St, PAR, Off, true, AB ? AB : kAosB>,
                                                     AddrSlots<St, PAR, Off>>>;
    const Ad ad = [&]() {
      if constexpr (W64 || AB != 0) return Ad(d, cell, inr ? x : 0, inr ? y : 0, z);
      else return Ad(d, T, cell, inr ? x : 0, inr ? y : 0, z);
    }();
    const PopStore<St> put(d, (uint32_t)cell);
    auto emit = [&](int i, R v) {
      if (i == 0) put(ad.rest(), v, 0);
      else if (i & 1) put(ad.b((i - 1) >> 1, true), v, i);
      else put(ad.a((i - 2) >> 1, false), v, i);
    };
    R g[Q];
    R delta = R(0.0), rho = R(1.0), ux = R(0.0), uy = R(0.0), uz = R(0.0), uu = R(0.0), rinv = R(1.0);
    float feat[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    bool fluid = false, inside = false;
    if (inr) {
      double fx = 0.0, fy = 0.0, fz = 0.0;
      const uint32_t lw = __ldg(d.link + cell);
      g[0] = St::ld(ad.rest());
#pragma unroll
      for (int k = 0; k < 9; ++k) {
        g[2 * k + 1] = St::ld(ad.a(k, false));
        g[2 * k + 2] = St::ld(ad.b(k, true));
      }
      const uint32_t ct = (lw >> LINK_CLASS_SHIFT) & 7u;
      if (is_solid(ct)) {
        if (MAC) d.macros[cell] = make_float4(0.f, 0.f, 0.f, 0.f);
      } else {
        const uint32_t bb = lw & 0x3ffffu;
        if (bb) {
#pragma unroll
          for (int k = 0; k < 9; ++k) {
            if ((bb >> (2 * k)) & 1u) g[2 * k + 1] = St::ld(ad.b(k, false));
            if ((bb >> (2 * k + 1)) & 1u) g[2 * k + 2] = St::ld(ad.a(k, true));
          }
          if (lw & LINK_SLOW) {
            const Wrap w = wrap3(x, y, z, nx, ny, d.nz);
#pragma unroll
            for (int k = 1; k < Q; ++k) {
              if (!((bb >> (k - 1)) & 1u)) continue;
              const uint32_t tk = d.tipo[nbr(k, -1, x, y, z, w, nx, ny)];
              if (tk == SOLIDO_MOVEL)
                g[k] = g[k] + Lit<R>::sixw(k) * (dotc<R>(k, R(P.belt[0]), R(P.belt[1]), R(P.belt[2])));
              if (FRC && ct == FLUIDO && tk == SOLIDO) {
                const R q = R(2.0) * (g[k] + Lit<R>::w(k));
                fx -= (double)(cx(k) * q); fy -= (double)(cy(k) * q); fz -= (double)(cz(k) * q);
              }
            }
          } else if (FRC && ct == FLUIDO && (lw & LINK_BODY)) {
#pragma unroll
            for (int k = 1; k < Q; ++k) {
              if (!((bb >> (k - 1)) & 1u)) continue;
              const R q = R(2.0) * (g[k] + Lit<R>::w(k));
              fx -= (double)(cx(k) * q); fy -= (double)(cy(k) * q); fz -= (double)(cz(k) * q);
            }
          }
        }
        if (FRC && (fx != 0.0 || fy != 0.0 || fz != 0.0)) add_force(d.force, fx, fy, fz);
        R sp[9], dp[9];
        moments_fast<R>(g, sp, dp, delta, rho, ux, uy, uz, uu, rinv);
        if (MAC) d.macros[cell] = make_float4(ux, uy, uz, delta);
        if (ct == FLUIDO) {
          fluid = true;
          const PiT<R> m = pi_fast<R>(sp);
          const R d3 = delta * R(1.0 / 3.0);
          const R rux = rho * ux, ruy = rho * uy, ruz = rho * uz;
          closure_features(m.xx - d3 - rux * ux, m.yy - d3 - ruy * uy, m.zz - d3 - ruz * uz, m.xy - rux * uy,
                           m.xz - rux * uz, m.yz - ruy * uz, rinv, delta, feat);
          feat[4] = A.omega0;
          inside = closure_in_range(A.K, feat);
#pragma unroll
          for (int a = 0; a < 6; ++a) feat[a] = (feat[a] - A.K.mean[a]) * A.K.inv_std[a];
        } else {
          collide<R, true>(P, U, ct, x, z, g, sp, dp, delta, rho, ux, uy, uz, uu, rinv,
                           static_cast<const R*>(d.blf), emit);
        }
      }
    }
    const float yv = tcp_mlp(SH, tmem, tid, feat, phase, dead);
    if (fluid) {
      const float nu = inside ? closure_nu(A.K, yv) : __int_as_float(0x7fc00000);
      if (MODE == 1) A.nu[cell] = nu;
      R sp[9], dp[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) {
        sp[k] = g[2 * k + 1] + g[2 * k + 2];
        dp[k] = g[2 * k + 1] - g[2 * k + 2];
      }
      R e0, ns[9], nd[9];
      fluid_neq_fast<R>(sp, dp, delta, rho, ux, uy, uz, uu, e0, ns, nd);
      R omegaP, omegaM;
      if (nu == nu) {
        if (A.coef) {
          smag_rates_c18<R>(P, U, ns, rinv, 18.0f * nu, omegaP, omegaM);
        } else {
          const float tauT = U.tau0 + 3.0f * nu, tm = tauT - 0.5f;
          omegaP = __frcp_rn(tauT);
          omegaM = __fdividef(tm, fmaf(0.5f, tm, P.magic));
        }
      } else {
        ++nfb;
        smag_rates_fast<R>(P, U, ns, rinv, omegaP, omegaM);
      }
      trt_emit_fast<R>(U, x, g, e0, ns, nd, omegaP, omegaM, U.sp_tf, emit);
    }
    bxi += gsx;
    const int cx_ = bxi >= gx;
    bxi -= cx_ ? gx : 0;
    byi += gsy + cx_;
    const int cy_ = byi >= gy;
    byi -= cy_ ? gy : 0;
    z += gsz + cy_;
  }
  tcp_teardown(SH, tmem, tid, phase, dead);
  // fallback count: one atomic per warp for the whole kernel
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) nfb += __shfl_down_sync(0xffffffffu, nfb, o);
  if ((tid & 31) == 0 && nfb && A.nfb) atomicAdd(A.nfb, (unsigned long long)nfb);
  if (tid == 0 && SH.err && A.err) atomicOr(A.err, 1u);
}

// A/B ping-pong step: the reference's pull verbatim (tipo gathered per link).
template <class St, bool MAC, bool FRC, bool FAST>
__global__ void __launch_bounds__(128) k_step_ab(Dev d, Params P, Uni<typename St::real> U) {
  using R = typename St::real;
  using S = typename St::store_t;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  const int nx = d.nx, ny = d.ny;
  double fx = 0.0, fy = 0.0, fz = 0.0;
  if (x < nx && y < ny) {
    const int64_t N = d.N;
    const int64_t cell = ((int64_t)z * ny + y) * nx + x;
    const uint32_t ct = d.tipo[cell];
    if (is_solid(ct)) {
      if (MAC) d.macros[cell] = make_float4(0.f, 0.f, 0.f, 0.f);
    } else {
      const S* src = static_cast<const S*>(d.pop);
      S* dst = static_cast<S*>(d.pop2);
      const Wrap w = wrap3(x, y, z, nx, ny, d.nz);
      R g[Q];
      g[0] = St::ld(src + cell);
#pragma unroll
      for (int i = 1; i < Q; ++i) {
        const int64_t s = nbr(i, -1, x, y, z, w, nx, ny);
        const uint32_t t = d.tipo[s];
        if (is_solid(t)) {
          const R bx = t == SOLIDO_MOVEL ? R(P.belt[0]) : R(0.0);
          const R by = t == SOLIDO_MOVEL ? R(P.belt[1]) : R(0.0);
          const R bz = t == SOLIDO_MOVEL ? R(P.belt[2]) : R(0.0);
          const R gb = St::ld(src + (int64_t)opp(i) * N + cell);
          g[i] = gb + Lit<R>::sixw(i) * (dotc<R>(i, bx, by, bz));
          if (FRC && ct == FLUIDO && t == SOLIDO) {
            const R q = R(2.0) * (gb + Lit<R>::w(i));
            fx -= (double)(cx(i) * q); fy -= (double)(cy(i) * q); fz -= (double)(cz(i) * q);
          }
        } else {
          g[i] = St::ld(src + (int64_t)i * N + s);
        }
      }
      R delta, rho, ux, uy, uz, uu, rinv = R(0.0);
      R sp[9], dp[9];
      if (FAST) moments_fast<R>(g, sp, dp, delta, rho, ux, uy, uz, uu, rinv);
      else moments_strict<R>(g, delta, rho, ux, uy, uz, uu);
      if (MAC) d.macros[cell] = make_float4((float)ux, (float)uy, (float)uz, (float)delta);
      collide<R, FAST>(P, U, ct, x, z, g, sp, dp, delta, rho, ux, uy, uz, uu, rinv, static_cast<const R*>(d.blf),
                       [&](int i, R v) { St::st(dst + (int64_t)i * N + cell, v); });
    }
  }
  if (FRC && (fx != 0.0 || fy != 0.0 || fz != 0.0)) add_force(d.force, fx, fy, fz);
}

// ------------------------------------------------------------------ init
// shaderInit (src/core/emit/wgsl.js:269-302): free-stream equilibrium in every
// cell; SOLIDO at rest, SOLIDO_MOVEL at the belt velocity.  Writes the
// parity-0 in-place layout, or the natural layout of `pop` for ping-pong.
template <class St, bool INPLACE>
__global__ void k_init(Dev d, Params P) {
  using R = typename St::real;
  using S = typename St::store_t;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= d.nx || y >= d.ny) return;
  const int64_t N = d.N;
  const int64_t cell = ((int64_t)z * d.ny + y) * d.nx + x;
  const uint32_t ct = d.tipo[cell];
  R ux = R(P.inlet[0]), uy = R(P.inlet[1]), uz = R(P.inlet[2]);
  if (ct == SOLIDO) { ux = R(0.0); uy = R(0.0); uz = R(0.0); }
  if (ct == SOLIDO_MOVEL) { ux = R(P.belt[0]); uy = R(P.belt[1]); uz = R(P.belt[2]); }
  const R delta = R(0.0), rho = R(1.0);
  const R uu = ux * ux + uy * uy + uz * uz;
  S* F = static_cast<S*>(d.pop);
  const Wrap w = wrap3(x, y, z, d.nx, d.ny, d.nz);
#pragma unroll
  for (int k = 0; k < Q; ++k) {
    const R e = equilibrium<R, false>(k, delta, rho, ux, uy, uz, uu, R(0.0));  // init is STRICT in both modes
    const int64_t off = INPLACE ? eso_loc(d, k, 0, cell, x, y, z, w) : (int64_t)k * N + cell;
    St::st(F + off, e);
  }
}

// ------------------------------------------------- state upload/download
// One direction k of a natural-layout array <-> storage.
template <class St, bool INPLACE>
__global__ void k_put_dir(Dev d, const double* __restrict__ v, int k, int parity) {
  using S = typename St::store_t;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= d.nx || y >= d.ny) return;
  const int64_t cell = ((int64_t)z * d.ny + y) * d.nx + x;
  const Wrap w = wrap3(x, y, z, d.nx, d.ny, d.nz);
  const int64_t off = INPLACE ? eso_loc(d, k, parity, cell, x, y, z, w) : (int64_t)k * d.N + cell;
  St::st(static_cast<S*>(d.pop) + off, St::from_double(v[cell]));
}

template <class St, bool INPLACE>
__global__ void k_get_dir(Dev d, double* __restrict__ v, int k, int parity) {
  using S = typename St::store_t;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= d.nx || y >= d.ny) return;
  const int64_t cell = ((int64_t)z * d.ny + y) * d.nx + x;
  const Wrap w = wrap3(x, y, z, d.nx, d.ny, d.nz);
  const int64_t off = INPLACE ? eso_loc(d, k, parity, cell, x, y, z, w) : (int64_t)k * d.N + cell;
  v[cell] = (double)St::ld(static_cast<const S*>(d.pop) + off);
}

// Gather the 19 post-collision populations of one cell from the current state.
template <class St, bool INPLACE>
__device__ __forceinline__ void gather_state(const Dev& d, int parity, int64_t cell, int x, int y, int z,
                                             typename St::real* g) {
  using S = typename St::store_t;
  const S* F = static_cast<const S*>(d.pop);
  const Wrap w = wrap3(x, y, z, d.nx, d.ny, d.nz);
#pragma unroll
  for (int k = 0; k < Q; ++k) {
    const int64_t off = INPLACE ? eso_loc(d, k, parity, cell, x, y, z, w) : (int64_t)k * d.N + cell;
    g[k] = St::ld(F + off);
  }
}

// shaderMacros (src/core/emit/wgsl.js:442-476): moments of the stored state,
// no streaming.  Solid cells report zero.
template <class St, bool INPLACE>
__global__ void k_macros(Dev d, int parity) {
  using R = typename St::real;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= d.nx || y >= d.ny) return;
  const int64_t cell = ((int64_t)z * d.ny + y) * d.nx + x;
  if (is_solid(d.tipo[cell])) { d.macros[cell] = make_float4(0.f, 0.f, 0.f, 0.f); return; }
  R g[Q];
  gather_state<St, INPLACE>(d, parity, cell, x, y, z, g);
  R delta = g[0];
#pragma unroll
  for (int i = 1; i < Q; ++i) delta = delta + g[i];
  const R rho = R(1.0) + delta;
  const R mx = signed_sum<R>(g, [](int i) { return cx(i); });
  const R my = signed_sum<R>(g, [](int i) { return cy(i); });
  const R mz = signed_sum<R>(g, [](int i) { return cz(i); });
  d.macros[cell] = make_float4((float)(mx / rho), (float)(my / rho), (float)(mz / rho), (float)delta);
}

// Block sum of three doubles into out[3*blockLinear + c] (deterministic order).
__device__ __forceinline__ void block_partials3(double a, double b, double c, double* out) {
  __shared__ double sh[3][32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
    c += __shfl_down_sync(0xffffffffu, c, o);
  }
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  const int nw = (blockDim.x * blockDim.y + 31) >> 5;
  if ((tid & 31) == 0) { sh[0][tid >> 5] = a; sh[1][tid >> 5] = b; sh[2][tid >> 5] = c; }
  __syncthreads();
  if (tid == 0) {
    double s0 = 0, s1 = 0, s2 = 0;
    for (int k = 0; k < nw; ++k) { s0 += sh[0][k]; s1 += sh[1][k]; s2 += sh[2][k]; }
    const int64_t b_lin = blockIdx.x + (int64_t)gridDim.x * (blockIdx.y + (int64_t)gridDim.y * blockIdx.z);
    out[3 * b_lin + 0] = s0;
    out[3 * b_lin + 1] = s1;
    out[3 * b_lin + 2] = s2;
  }
}

// Momentum exchange of the current state (src/core/emit/wgsl.js:356-379):
// FLUIDO cells, links whose downstream neighbour is SOLIDO, per-link value
// 2 (g_i + w_i) in the storage's arithmetic, fp64 accumulation.
template <class St, bool INPLACE>
__global__ void k_forces(Dev d, int parity, double* partials) {
  using R = typename St::real;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  double fx = 0, fy = 0, fz = 0;
  if (x < d.nx && y < d.ny) {
    const int64_t cell = ((int64_t)z * d.ny + y) * d.nx + x;
    if (d.tipo[cell] == FLUIDO) {
      using S = typename St::store_t;
      const S* F = static_cast<const S*>(d.pop);
      const Wrap w = wrap3(x, y, z, d.nx, d.ny, d.nz);
#pragma unroll
      for (int i = 1; i < Q; ++i) {
        if (d.tipo[nbr(i, +1, x, y, z, w, d.nx, d.ny)] != SOLIDO) continue;
        const int64_t off = INPLACE ? eso_loc(d, i, parity, cell, x, y, z, w) : (int64_t)i * d.N + cell;
        const R q = R(2.0) * (St::ld(F + off) + Lit<R>::w(i));
        fx += (double)(cx(i) * q); fy += (double)(cy(i) * q); fz += (double)(cz(i) * q);
      }
    }
  }
  block_partials3(fx, fy, fz, partials);
}

// Sum of delta over non-solid cells (delta summed in storage arithmetic in
// index order, as shaderMacros does; fp64 across cells).
template <class St, bool INPLACE>
__global__ void k_mass(Dev d, int parity, double* partials) {
  using R = typename St::real;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  double m = 0;
  if (x < d.nx && y < d.ny) {
    const int64_t cell = ((int64_t)z * d.ny + y) * d.nx + x;
    if (!is_solid(d.tipo[cell])) {
      R g[Q];
      gather_state<St, INPLACE>(d, parity, cell, x, y, z, g);
      R delta = g[0];
#pragma unroll
      for (int i = 1; i < Q; ++i) delta = delta + g[i];
      m = (double)delta;
    }
  }
  block_partials3(m, 0.0, 0.0, partials);
}

// ------------------------------------------------- pipelined in-place step
// The same step as k_step_inplace, with load latency hidden by software
// pipelining: each thread walks KZ cells along z; while it collides cell k,
// the 19 populations of cell k+1 are already in flight into its own shared
// memory slots (cp.async, one 4-byte copy per population, so no registers
// are held by the outstanding loads).  The prefetch takes the normal slots of
// the parity; a link whose upstream cell is solid (bounce-back, rare) is
// re-read directly from its bounce-back slot at collide time.  Every
// (slot, location) a cell touches belongs to that cell alone in this step, so
// prefetching cell k+1 before cell k's stores is race-free.
// 16-bit forms copy the aligned 32-bit word holding the element.
__device__ __forceinline__ void cp_async4(uint32_t saddr, const void* g) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(saddr), "l"(g) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

template <class St, int PAR, bool FAST, int KZ, int BX>
__global__ void __launch_bounds__(BX, 768 / BX) k_step_pipe(Dev d, Params P, Uni<typename St::real> U) {
  using R = typename St::real;
  using S = typename St::store_t;
  using Off = int32_t;
  static_assert(sizeof(S) <= 4, "pipelined step: 32-bit or 16-bit storage");
  __shared__ uint32_t buf[2][Q][BX];
  const int tid = threadIdx.x;
  const int x = blockIdx.x * BX + tid;
  const int y = blockIdx.y;
  const int z0 = blockIdx.z * KZ;
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const bool xin = x < nx;
  const int zend = min(z0 + KZ, nz);
  const Off N = (Off)d.N;
  const Off nxny = (Off)nx * ny;
  S* const F = static_cast<S*>(d.pop);
  constexpr bool E = (PAR == 0);

  // issue the normal-slot copies of cell (x, y, z) into stage st
  auto prefetch = [&](int z, int st) {
    const Off cell = (Off)z * nxny + (Off)y * nx + x;
    const Deltas<Off> D(x, y, z, nx, ny, nz);
    const uint32_t base = (uint32_t)__cvta_generic_to_shared(&buf[st][0][tid]);
    auto copy = [&](int k, Off e) {
      const S* p = F + e;
      const char* a = reinterpret_cast<const char*>(p);
      if (sizeof(S) == 2) a -= (reinterpret_cast<uintptr_t>(a) & 2u);
      cp_async4(base + (uint32_t)(k * BX * 4), a);
    };
    copy(0, cell);
#pragma unroll
    for (int i = 1; i < Q; i += 2) {
      copy(i, cell + (Off)(E ? i + 1 : i) * N);
      copy(i + 1, cell + D.odd(i) + (Off)(E ? i : i + 1) * N);
    }
  };
  auto word_shift = [&](Off e) -> uint32_t {
    return sizeof(S) == 2 ? (uint32_t)((reinterpret_cast<uintptr_t>(F + e) & 2u) << 3) : 0u;
  };

  if (!xin) return;
  // prefetches never wait on a link word (solid cells' slots are read and
  // ignored); the link word of the next cell is loaded one cell ahead
  uint32_t lw_next = __ldg(d.link + (Off)z0 * nxny + (Off)y * nx + x);
  prefetch(z0, 0);
  cp_async_commit();
  for (int z = z0; z < zend; ++z) {
    const int st = (z - z0) & 1;
    const uint32_t lw = lw_next;
    if (z + 1 < zend) {
      lw_next = __ldg(d.link + (Off)(z + 1) * nxny + (Off)y * nx + x);
      prefetch(z + 1, st ^ 1);
    }
    cp_async_commit();
    cp_async_wait<1>();          // this cell's copies have landed
    const uint32_t ct = (lw >> LINK_CLASS_SHIFT) & 7u;
    if (is_solid(ct)) continue;  // solid: nothing to do (macros are not written here)
    const Off cell = (Off)z * nxny + (Off)y * nx + x;
    const Deltas<Off> D(x, y, z, nx, ny, nz);
    R g[Q];
    g[0] = St::from_word(buf[st][0][tid], word_shift(cell));
#pragma unroll
    for (int i = 1; i < Q; i += 2) {
      const Off ei = cell + (Off)(E ? i + 1 : i) * N;
      const Off ej = cell + D.odd(i) + (Off)(E ? i : i + 1) * N;
      g[i] = St::from_word(buf[st][i][tid], word_shift(ei));
      g[i + 1] = St::from_word(buf[st][i + 1][tid], word_shift(ej));
    }
    const uint32_t bbmask = lw & 0x3ffffu;
    if (bbmask) {
      // bounce-back links: the other slot of the same location
#pragma unroll
      for (int i = 1; i < Q; i += 2) {
        if ((bbmask >> (i - 1)) & 1u) g[i] = St::ld(F + cell + (Off)(E ? i : i + 1) * N);
        if ((bbmask >> i) & 1u) g[i + 1] = St::ld(F + cell + D.odd(i) + (Off)(E ? i + 1 : i) * N);
      }
      if (lw & LINK_SLOW) {
        const Wrap w = wrap3(x, y, z, nx, ny, nz);
#pragma unroll
        for (int k = 1; k < Q; ++k) {
          if (!((bbmask >> (k - 1)) & 1u)) continue;
          if (d.tipo[nbr(k, -1, x, y, z, w, nx, ny)] == SOLIDO_MOVEL)
            g[k] = g[k] + Lit<R>::sixw(k) * (dotc<R>(k, R(P.belt[0]), R(P.belt[1]), R(P.belt[2])));
        }
      }
    }
    R delta, rho, ux, uy, uz, uu, rinv = R(0.0);
    R sp[9], dp[9];
    if (FAST) moments_fast<R>(g, sp, dp, delta, rho, ux, uy, uz, uu, rinv);
    else moments_strict<R>(g, delta, rho, ux, uy, uz, uu);
    S* const Fc = F + cell;
    collide<R, FAST>(P, U, ct, x, z, g, sp, dp, delta, rho, ux, uy, uz, uu, rinv, static_cast<const R*>(d.blf),
                     [&](int i, R v) {
      if (i == 0) {
        St::st(Fc, v);
      } else if (i & 1) {
        St::st(Fc + D.odd(i) + (Off)(E ? i : i + 1) * N, v);
      } else {
        St::st(Fc + (Off)(E ? i : i - 1) * N, v);
      }
    });
  }
  cp_async_wait<0>();
}

// ---------------------------------------------------------------- launchers
struct Launch {
  dim3 grid, block;
  int occ = 8;   // register-cap variant of the plain in-place step (8 or 6)
  int pipe = 0;  // > 0: pipelined step, cells per thread along z (4, 8, 16)
};

using StepClosureFn = cudaError_t (*)(const Dev&, const Params&, int parity, bool mac, bool frc, int engine,
                                      int mode, const CloArgs&, Launch, cudaStream_t);

struct Ops {
  cudaError_t (*step)(const Dev&, const Params&, int parity, bool inplace, bool mac, bool frc, bool fast, Launch,
                      cudaStream_t);
  cudaError_t (*init)(const Dev&, const Params&, bool inplace, Launch, cudaStream_t);
  cudaError_t (*put_dir)(const Dev&, const double*, int k, int parity, bool inplace, Launch, cudaStream_t);
  cudaError_t (*get_dir)(const Dev&, double*, int k, int parity, bool inplace, Launch, cudaStream_t);
  cudaError_t (*macros)(const Dev&, int parity, bool inplace, Launch, cudaStream_t);
  cudaError_t (*forces)(const Dev&, int parity, bool inplace, double* partials, Launch, cudaStream_t);
  cudaError_t (*mass)(const Dev&, int parity, bool inplace, double* partials, Launch, cudaStream_t);
  // in-place FAST step with the learned closure (engine 0/1, mode 0/1/2 of
  // k_step_closure); null for the fp64 reference form
  StepClosureFn step_closure;
  int elem_bytes;
};

template <class St>
struct OpsImpl {
  using R = typename St::real;
  // The fp64 reference form is always STRICT.
  static constexpr bool kFastOK = sizeof(R) == 4;
  template <int PAR, bool MAC, bool FRC, bool FAST, bool PAD>
  static void go_aos(const Dev& d, const Params& P, const Uni<R>& U, Launch L, cudaStream_t s, const SlotPtrs& T) {
    static_assert(sizeof(R) == 4, "the AoSoA step runs fp32 arithmetic");
    constexpr int kDefault = MAC ? 6 : 8;
    // variant 9: store addresses kept in registers from the loads
    // blocks of 64 cells: the 16-bit forms only (lbm_create)
    if constexpr (sizeof(typename St::store_t) == 2) {
      if (d.aos == 64) {
        if (!MAC && !FRC && L.occ == 9)
          k_step_inplace<St, PAR, MAC, FRC, false, FAST, kDefault, true, false, 0, 64, PAD><<<L.grid, L.block, 0, s>>>(d, P, U, T);
        else
          k_step_inplace<St, PAR, MAC, FRC, false, FAST, kDefault, true, true, 0, 64, PAD><<<L.grid, L.block, 0, s>>>(d, P, U, T);
        return;
      }
    }
    if (!MAC && !FRC && L.occ == 9)
      k_step_inplace<St, PAR, MAC, FRC, false, FAST, kDefault, true, false, 0, kAosB, PAD><<<L.grid, L.block, 0, s>>>(d, P, U, T);
    else
      k_step_inplace<St, PAR, MAC, FRC, false, FAST, kDefault, true, true, 0, kAosB, PAD><<<L.grid, L.block, 0, s>>>(d, P, U, T);
  }
  template <int PAR, bool MAC, bool FRC, bool FAST>
  static void go_inplace(const Dev& d, const Params& P, const Uni<R>& U, Launch L, cudaStream_t s) {
    constexpr int kDefault = sizeof(R) == 8 ? 4 : (MAC ? 6 : 8);
    const bool w64 = (int64_t)Q * d.N >= (int64_t)INT32_MAX;
    if constexpr (!MAC && !FRC && sizeof(typename St::store_t) <= 4 && !St::kSR) {
      if (L.pipe > 0 && !w64 && !d.aos) {
        const dim3 grid((d.nx + 63) / 64, d.ny, (d.nz + L.pipe - 1) / L.pipe);
        if (L.pipe == 4) k_step_pipe<St, PAR, FAST, 4, 64><<<grid, 64, 0, s>>>(d, P, U);
        else if (L.pipe == 8) k_step_pipe<St, PAR, FAST, 8, 64><<<grid, 64, 0, s>>>(d, P, U);
        else k_step_pipe<St, PAR, FAST, 16, 64><<<grid, 64, 0, s>>>(d, P, U);
        return;
      }
    }
    const SlotPtrs T = make_slots<St>(d, PAR);
    if (d.aos) {
      if constexpr (FAST && sizeof(R) == 4) {
        if (d.nxp == d.nx) go_aos<PAR, MAC, FRC, FAST, false>(d, P, U, L, s, T);
        else go_aos<PAR, MAC, FRC, FAST, true>(d, P, U, L, s, T);
      }
      return;
    }
    // SoA addressing variants of the plain step (20: 32-bit slot offsets,
    // 21: base + slot x N), both with the store addresses formed again
    if constexpr (!MAC && !FRC && sizeof(R) == 4) {
      if (!w64 && L.occ == 20) {
        k_step_inplace<St, PAR, MAC, FRC, false, FAST, kDefault, false, true, 1><<<L.grid, L.block, 0, s>>>(d, P, U, T);
        return;
      }
      if (!w64 && L.occ == 21) {
        k_step_inplace<St, PAR, MAC, FRC, false, FAST, kDefault, false, true, 2><<<L.grid, L.block, 0, s>>>(d, P, U, T);
        return;
      }
    }
    // the plain hot-loop variant also exists with a looser register cap
    if (!MAC && !FRC && sizeof(R) == 4 && L.occ == 6) {
      if (w64) k_step_inplace<St, PAR, MAC, FRC, true, FAST, 6><<<L.grid, L.block, 0, s>>>(d, P, U, T);
      else k_step_inplace<St, PAR, MAC, FRC, false, FAST, 6><<<L.grid, L.block, 0, s>>>(d, P, U, T);
      return;
    }
    if (w64) k_step_inplace<St, PAR, MAC, FRC, true, FAST, kDefault><<<L.grid, L.block, 0, s>>>(d, P, U, T);
    else k_step_inplace<St, PAR, MAC, FRC, false, FAST, kDefault><<<L.grid, L.block, 0, s>>>(d, P, U, T);
  }
  template <bool FAST>
  static void go(const Dev& d, const Params& P, const Uni<R>& U, int parity, bool inplace, bool mac, bool frc,
                 Launch L, cudaStream_t s) {
    if (inplace) {
      if (parity == 0) {
        if (mac) { frc ? go_inplace<0, true, true, FAST>(d, P, U, L, s) : go_inplace<0, true, false, FAST>(d, P, U, L, s); }
        else { frc ? go_inplace<0, false, true, FAST>(d, P, U, L, s) : go_inplace<0, false, false, FAST>(d, P, U, L, s); }
      } else {
        if (mac) { frc ? go_inplace<1, true, true, FAST>(d, P, U, L, s) : go_inplace<1, true, false, FAST>(d, P, U, L, s); }
        else { frc ? go_inplace<1, false, true, FAST>(d, P, U, L, s) : go_inplace<1, false, false, FAST>(d, P, U, L, s); }
      }
    } else {
      if (mac) { if (frc) k_step_ab<St, true, true, FAST><<<L.grid, L.block, 0, s>>>(d, P, U); else k_step_ab<St, true, false, FAST><<<L.grid, L.block, 0, s>>>(d, P, U); }
      else { if (frc) k_step_ab<St, false, true, FAST><<<L.grid, L.block, 0, s>>>(d, P, U); else k_step_ab<St, false, false, FAST><<<L.grid, L.block, 0, s>>>(d, P, U); }
    }
  }
  static cudaError_t step(const Dev& d, const Params& P, int parity, bool inplace, bool mac, bool frc, bool fast,
                          Launch L, cudaStream_t s) {
    if (d.aos && !(fast && kFastOK && inplace)) return cudaErrorNotSupported;   // AoSoA: FAST, in-place only
    if (St::kSR && !inplace) return cudaErrorNotSupported;                      // SR forms: in-place only
    const Uni<R> U = make_uni<R>(P, R(St::kScale));
    if (fast && kFastOK) go<kFastOK>(d, P, U, parity, inplace, mac, frc, L, s);
    else go<false>(d, P, U, parity, inplace, mac, frc, L, s);
    return cudaGetLastError();
  }
  static cudaError_t init(const Dev& d, const Params& P, bool inplace, Launch L, cudaStream_t s) {
    if (inplace) k_init<St, true><<<L.grid, L.block, 0, s>>>(d, P);
    else k_init<St, false><<<L.grid, L.block, 0, s>>>(d, P);
    return cudaGetLastError();
  }
  static cudaError_t put_dir(const Dev& d, const double* v, int k, int parity, bool inplace, Launch L, cudaStream_t s) {
    if (inplace) k_put_dir<St, true><<<L.grid, L.block, 0, s>>>(d, v, k, parity);
    else k_put_dir<St, false><<<L.grid, L.block, 0, s>>>(d, v, k, parity);
    return cudaGetLastError();
  }
  static cudaError_t get_dir(const Dev& d, double* v, int k, int parity, bool inplace, Launch L, cudaStream_t s) {
    if (inplace) k_get_dir<St, true><<<L.grid, L.block, 0, s>>>(d, v, k, parity);
    else k_get_dir<St, false><<<L.grid, L.block, 0, s>>>(d, v, k, parity);
    return cudaGetLastError();
  }
  static cudaError_t macros(const Dev& d, int parity, bool inplace, Launch L, cudaStream_t s) {
    if (inplace) k_macros<St, true><<<L.grid, L.block, 0, s>>>(d, parity);
    else k_macros<St, false><<<L.grid, L.block, 0, s>>>(d, parity);
    return cudaGetLastError();
  }
  static cudaError_t forces(const Dev& d, int parity, bool inplace, double* part, Launch L, cudaStream_t s) {
    if (inplace) k_forces<St, true><<<L.grid, L.block, 0, s>>>(d, parity, part);
    else k_forces<St, false><<<L.grid, L.block, 0, s>>>(d, parity, part);
    return cudaGetLastError();
  }
  static cudaError_t mass(const Dev& d, int parity, bool inplace, double* part, Launch L, cudaStream_t s) {
    if (inplace) k_mass<St, true><<<L.grid, L.block, 0, s>>>(d, parity, part);
    else k_mass<St, false><<<L.grid, L.block, 0, s>>>(d, parity, part);
    return cudaGetLastError();
  }
  // Persistent CTA engine: as many CTAs as fit at once, at most one per tile.
  template <int PAR, bool MAC, bool FRC, bool W64, int MODE>
  static void go_closure_tc(const Dev& d, const Params& P, const Uni<float>& U, const CloArgs& A, cudaStream_t s) {
    if constexpr (sizeof(R) == 4) {
      const SlotPtrs T = make_slots<St>(d, PAR);
      constexpr bool k16 = sizeof(typename St::store_t) == 2;   // blocks of 64 cells: 16-bit forms only
      auto* k = (!W64 && d.aos) ? &k_step_closure_tc<St, PAR, MAC, FRC, W64, MODE, 32>
                                : &k_step_closure_tc<St, PAR, MAC, FRC, W64, MODE, 0>;
      if constexpr (k16)
        if (!W64 && d.aos == 64) k = &k_step_closure_tc<St, PAR, MAC, FRC, W64, MODE, k16 ? 64 : 32>;
      // the kernel is built for kClosureTcPerSm resident CTAs per SM
      // (launch bounds), each holding 32 of the SM's 512 TMEM columns
      int dev = 0, sms = 1;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      const int per_sm = kClosureTcPerSm;
      const int gx = (d.nx + 63) / 64, gy = (d.ny + 1) / 2;
      const long long ntiles = (long long)gx * gy * d.nz;
      const unsigned grid = (unsigned)std::max<long long>(1, std::min<long long>(ntiles, (long long)per_sm * sms));
      k<<<grid, 128, 0, s>>>(d, P, U, A, T, gx, gy);
    }
  }
  // The closure steps index the set with 32 bits (the caller refuses
  // 19 N >= 2^31).
  template <int PAR, bool MAC, bool FRC, int ENG, int MODE>
  static void go_closure(const Dev& d, const Params& P, const Uni<float>& U, const CloArgs& A, Launch L,
                         cudaStream_t s) {
    static_assert(MODE != 2, "held steps run k_step_held");
    if constexpr (ENG == 1) {
      go_closure_tc<PAR, MAC, FRC, false, MODE>(d, P, U, A, s);
      return;
    }
    if constexpr (sizeof(R) == 4 && ENG == 0) {
      // network steps: 64 x 2 threads, four warps
      const dim3 block(64, 2), grid((d.nx + 63) / 64, (d.ny + 1) / 2, d.nz);
      k_step_closure<St, PAR, MAC, FRC, false, ENG, MODE><<<grid, block, 0, s>>>(d, P, U, A);
    }
  }
  template <int PAR, bool MAC, bool FRC>
  static void go_closure_m(const Dev& d, const Params& P, const Uni<float>& U, int engine, int mode,
                           const CloArgs& A, Launch L, cudaStream_t s) {
    if constexpr (sizeof(R) == 4) {
      if (mode == 2) {
        const Uni<R> Us = make_uni<R>(P, R(St::kScale));
        const SlotPtrs T = make_slots<St>(d, PAR);
        if constexpr (sizeof(typename St::store_t) == 2) {   // blocks of 64 cells: 16-bit forms only
          if (d.aos == 64) {
            k_step_held<St, PAR, MAC, FRC, 64><<<L.grid, L.block, 0, s>>>(d, P, Us, T, A.nu, A.coef);
            return;
          }
        }
        if (d.aos) k_step_held<St, PAR, MAC, FRC, 32><<<L.grid, L.block, 0, s>>>(d, P, Us, T, A.nu, A.coef);
        else k_step_held<St, PAR, MAC, FRC, 0><<<L.grid, L.block, 0, s>>>(d, P, Us, T, A.nu, A.coef);
        return;
      }
    }
    if (engine == 0) { mode == 1 ? go_closure<PAR, MAC, FRC, 0, 1>(d, P, U, A, L, s) : go_closure<PAR, MAC, FRC, 0, 0>(d, P, U, A, L, s); }
    else { mode == 1 ? go_closure<PAR, MAC, FRC, 1, 1>(d, P, U, A, L, s) : go_closure<PAR, MAC, FRC, 1, 0>(d, P, U, A, L, s); }
  }
  static cudaError_t step_closure(const Dev& d, const Params& P, int parity, bool mac, bool frc, int engine,
                                  int mode, const CloArgs& A, Launch L, cudaStream_t s) {
    if constexpr (sizeof(R) == 4) {
      const Uni<float> U = make_uni<float>(P);
      if (parity == 0) {
        if (mac) { frc ? go_closure_m<0, true, true>(d, P, U, engine, mode, A, L, s) : go_closure_m<0, true, false>(d, P, U, engine, mode, A, L, s); }
        else { frc ? go_closure_m<0, false, true>(d, P, U, engine, mode, A, L, s) : go_closure_m<0, false, false>(d, P, U, engine, mode, A, L, s); }
      } else {
        if (mac) { frc ? go_closure_m<1, true, true>(d, P, U, engine, mode, A, L, s) : go_closure_m<1, true, false>(d, P, U, engine, mode, A, L, s); }
        else { frc ? go_closure_m<1, false, true>(d, P, U, engine, mode, A, L, s) : go_closure_m<1, false, false>(d, P, U, engine, mode, A, L, s); }
      }
      return cudaGetLastError();
    }
    return cudaErrorNotSupported;
  }
  // Everything but the closure steps, whose kernels are instantiated in a
  // unit of their own (lbm_inst_*_clo.cu) so that the two compile in parallel.
  static Ops make() {
    Ops o;
    o.step = &step; o.init = &init; o.put_dir = &put_dir; o.get_dir = &get_dir;
    o.macros = &macros; o.forces = &forces; o.mass = &mass;
    o.step_closure = nullptr;
    o.elem_bytes = (int)sizeof(typename St::store_t);
    return o;
  }
  static StepClosureFn closure_entry() { return &step_closure; }
};

// What other units of the library see of a context.
struct CtxView {
  int nx, ny, nz;
  int64_t N;
  float4* macros;
  const uint8_t* tipo;
  cudaStream_t stream;
};
int ctx_view(::lbm_ctx* c, CtxView* v);   // lbm_api.cu; makes sure the macros buffer exists

Ops ops_f32();
Ops ops_f64();
Ops ops_f16s();
Ops ops_bf16s();
StepClosureFn closure_f32();
StepClosureFn closure_f16s();
StepClosureFn closure_bf16s();
StepClosureFn closure_f16sr();
StepClosureFn closure_bf16sr();
Ops ops_f16sr();
Ops ops_bf16sr();

}  // namespace lbm

// closure_tc.cuh — the learned closure's 6 -> 32 -> 32 -> 1 MLP for one CTA
// of 128 cells on the 5th-generation tensor cores (tcgen05.mma, kind::f16,
// bf16 operands from shared memory, fp32 accumulators in tensor memory).
//
// One tile = a CTA's 128 cells (thread tid <-> MMA row tid <-> TMEM lane
// tid).  Per layer: every thread writes its row of the A operand to shared
// memory, one thread issues the MMA(s) and commits them to an mbarrier, every
// thread waits on it and reads its row of the accumulator back with
// tcgen05.ld.  A CTA sets up once and then walks many tiles (persistent).
// The two hidden layers run on the tensor cores; the 32 -> 1 output layer
// runs on the CUDA cores from the second layer's accumulators (one dot
// product per thread), which spares a third barrier and MMA round trip.
// Biases ride in the K dimension: A carries a constant 1 in column kb and B
// holds the bias there (layer 1: K = 16 = 6 features + 1 + 9 zeros; layer 2:
// K = 48 = 32 hidden + 1 + 15 zeros), so the accumulators start at zero and
// no bias add is needed.
//
// Operand layout in shared memory: K-major, no swizzle, the canonical
// "core matrix" arrangement: a core matrix is 8 rows x 16 bytes (8 bf16 along
// K) stored contiguously; core matrices adjacent in K are LBO = 128 bytes
// apart, 8-row groups are SBO = (K / 8) * 128 bytes apart.  Byte offset of
// (row r, element k):  (r / 8) * SBO + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2.
//
// Descriptors (PTX ISA, tcgen05 "shared memory descriptor" and "instruction
// descriptor"):
//   smem desc: [0,14) addr >> 4, [16,30) LBO >> 4, [32,46) SBO >> 4,
//              [46,48) = 1, [49,52) base offset 0, [52] LBO mode 0,
//              [61,64) swizzle 0 (none)
//   idesc (kind::f16): [4,6) D format 1 (f32), [7,10) A format 1 (bf16),
//              [10,13) B format 1 (bf16), [15] A K-major 0, [16] B K-major 0,
//              [17,23) N >> 3, [24,29) M >> 4
#pragma once
#include <cstdint>

namespace lbm {

constexpr int TC_ROWS = 128;        // cells per tile (M)
constexpr int TC_K1 = 16, TC_K2 = 48;
constexpr int TC_B1_BYTES = 32 * TC_K1 * 2;      // 1024
constexpr int TC_B2_BYTES = 32 * TC_K2 * 2;      // 3072
constexpr int TC_B_BYTES = TC_B1_BYTES + TC_B2_BYTES;   // 4096 (the output layer runs on the CUDA cores)
constexpr uint32_t TC_TMEM_COLS = 32;
constexpr uint32_t TC_WAIT_LIMIT = 1u << 20;     // suspended mbarrier tries (<= ~1 us each) before giving up

// Byte offset of (row r, element k) in a K-major no-swizzle operand with K
// elements per row.
__host__ __device__ constexpr uint32_t tc_off(int r, int k, int K) {
  return (uint32_t)((r >> 3) * (K / 8) * 128 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, int K) {
  const uint64_t lbo = 128, sbo = (uint64_t)(K / 8) * 128;
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((lbo >> 4) << 16) | ((sbo >> 4) << 32) | (1ull << 46);
}

__host__ __device__ constexpr uint32_t tc_idesc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t dtmem, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
      :
      : "r"(dtmem), "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(smem_addr(bar))
               : "memory");
}

// One wait on the phase of the given parity: the hardware suspends the
// thread until the phase completes or about `hint_ns` nanoseconds pass.
__device__ __forceinline__ bool mbar_try(uint64_t* bar, uint32_t parity, uint32_t hint_ns) {
  uint32_t ok;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\nselp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity), "r"(hint_ns)
      : "memory");
  return ok != 0;
}

// Bounded wait for the phase of the given parity; false when it gave up
// (after TC_WAIT_LIMIT suspended tries of up to a microsecond each).  A
// suspended warp leaves the issue slots to the CTAs that are streaming
// populations.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  for (uint32_t i = 0; i < TC_WAIT_LIMIT; ++i)
    if (mbar_try(bar, parity, 1000u)) return true;
  return false;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void proxy_fence() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

// 16 consecutive fp32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float tc_ld1(uint32_t taddr) {
  uint32_t r;
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x1.b32 {%0}, [%1];\n" : "=r"(r) : "r"(taddr) : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
  return __uint_as_float(r);
}

__device__ __forceinline__ uint32_t tc_relu_pack(float a, float b) {
  uint32_t r;
  asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;\n" : "=r"(r) : "f"(b), "f"(a));
  return r;
}

__device__ __forceinline__ uint32_t tc_pack(float a, float b) {
  uint32_t r;
  asm("cvt.rn.bf16x2.f32 %0, %1, %2;\n" : "=r"(r) : "f"(b), "f"(a));
  return r;
}

__device__ __forceinline__ void sts128(uint8_t* base, uint32_t off, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
  *reinterpret_cast<uint4*>(base + off) = make_uint4(a, b, c, d);
}

// ------------------------------------------------------------------ persistent
// The engine of the persistent closure step (k_step_closure_tc): a CTA sets
// up once (TMEM columns, the mbarrier, the B operands, the constant columns
// of the A operands) and then walks many 128-cell tiles; per tile it pays one
// CTA barrier and one MMA round trip per hidden layer.
//
// A operands live in two buffers so that the constant columns never need
// rewriting: a1 (K = 16: features 0..5, the bias 1 at element 6, zeros to
// 15 -- elements 8..15 are a separate core matrix, written once) and a2
// (K = 48: 32 hidden values, the bias 1 at element 32, zeros to 47 -- the
// core matrices of elements 32..47 are written once).
struct TcPersist {
  alignas(128) uint8_t a1[TC_ROWS * TC_K1 * 2];
  alignas(128) uint8_t a2[TC_ROWS * TC_K2 * 2];
  alignas(128) uint8_t b[TC_B_BYTES];
  float w3[32];      // output layer on the CUDA cores: weights and bias,
  float b3;          // bf16-rounded (the values the MMA form would use)
  alignas(8) uint64_t mbar;
  uint32_t tmem;
  uint32_t err;      // a wait gave up: no further MMA is issued
};

__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

// Set-up of a persistent CTA (128 threads, every thread calls it).  w3b:
// the output layer's 32 weights and its bias, bf16-rounded, as fp32.
__device__ __forceinline__ uint32_t tcp_setup(TcPersist& S, const uint4* __restrict__ bw,
                                              const float* __restrict__ w3b, int tid) {
  if (tid < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_addr(&S.tmem)),
                 "r"(TC_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_addr(&S.mbar)) : "memory");
    mbar_init_fence();
    S.err = 0;
  }
  uint4* bd = reinterpret_cast<uint4*>(S.b);
  for (int i = tid; i < TC_B_BYTES / 16; i += TC_ROWS) bd[i] = __ldg(bw + i);
  if (tid < 32) S.w3[tid] = __ldg(w3b + tid);
  if (tid == 32) S.b3 = __ldg(w3b + 32);
  // constant columns of this thread's rows
  sts128(S.a1, tc_off(tid, 8, TC_K1), 0u, 0u, 0u, 0u);
  sts128(S.a2, tc_off(tid, 32, TC_K2), 0x3F80u, 0u, 0u, 0u);   // bf16 1.0 at element 32
  sts128(S.a2, tc_off(tid, 40, TC_K2), 0u, 0u, 0u, 0u);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  return S.tmem;
}

// Make this thread's A row visible to the tensor core, meet the CTA, and let
// thread 0 issue `nk` K-steps of 16 from `a` (K elements per row) against the
// B operand at b_off into TMEM columns [0, N), committed to the mbarrier.
// `dead`: this thread has seen a wait give up.  The barrier ORs it over the
// CTA, so every thread takes the same decision: once any wait has given up,
// no further MMA is issued.  Returns whether the MMA was issued.
__device__ __forceinline__ bool tcp_issue(TcPersist& S, const uint8_t* a, uint32_t tmem, int tid, int K, int N,
                                          int nk, uint32_t b_off, bool& dead) {
  proxy_fence();
  tc_fence_before();
  dead = __syncthreads_or(dead ? 1 : 0) != 0;
  const bool go = !dead;
  if (go && tid == 0) {
    tc_fence_after();
    const uint32_t a0 = smem_addr(a), b0 = smem_addr(S.b) + b_off;
    const uint32_t idesc = tc_idesc(TC_ROWS, N);
    for (int k = 0; k < nk; ++k)
      tc_mma(tmem, tc_desc(a0 + (uint32_t)k * 256u, K), tc_desc(b0 + (uint32_t)k * 256u, K), idesc, k > 0);
    tc_commit(&S.mbar);
  }
  return go;
}

// Bounded wait for the committed MMAs of the phase with parity `par`; a
// thread that gives up sets `dead` and records it in S.err for the report.
__device__ __forceinline__ bool tcp_wait(TcPersist& S, uint32_t par, bool& dead) {
  const bool ok = mbar_wait(&S.mbar, par);
  if (!ok) { dead = true; S.err = 1; }
  tc_fence_after();
  return ok;
}

// Layer epilogue of a hidden layer: this thread's 32 accumulator columns ->
// ReLU -> bf16 -> elements 0..31 of its row of a2.
__device__ __forceinline__ void tcp_hidden_to_a2(TcPersist& S, uint32_t tmem, int tid) {
  const uint32_t lane_addr = tmem + ((uint32_t)(tid & ~31) << 16);
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    float v[16];
    tc_ld16(lane_addr + 16u * h, v);
    uint32_t q[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) q[i] = tc_relu_pack(v[2 * i], v[2 * i + 1]);
    sts128(S.a2, tc_off(tid, 16 * h, TC_K2), q[0], q[1], q[2], q[3]);
    sts128(S.a2, tc_off(tid, 16 * h + 8, TC_K2), q[4], q[5], q[6], q[7]);
  }
}

// Output layer (32 -> 1) of this thread's row on the CUDA cores, from the
// second hidden layer's accumulators in TMEM: ReLU, bf16 rounding (the
// operand the MMA form would read), then a fixed-order fp32 dot product.
__device__ __forceinline__ float tcp_output(const TcPersist& S, uint32_t tmem, int tid) {
  const uint32_t lane_addr = tmem + ((uint32_t)(tid & ~31) << 16);
  float y = S.b3;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    float v[16];
    tc_ld16(lane_addr + 16u * h, v);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const uint32_t q = tc_relu_pack(v[2 * i], v[2 * i + 1]);
      y = fmaf(__uint_as_float(q << 16), S.w3[16 * h + 2 * i], y);
      y = fmaf(__uint_as_float(q & 0xffff0000u), S.w3[16 * h + 2 * i + 1], y);
    }
  }
  return y;
}

// The network for the CTA's current tile: x = this thread's normalised
// features (zeros for threads without a fluid cell).  All 128 threads call
// it.  `phase` is the parity of the mbarrier's next phase (two phases per
// tile: the hidden layers on the tensor cores, the output layer on the CUDA
// cores), `dead` the give-up state (tcp_issue).  NaN when the network was
// not run or a wait gave up.
__device__ __forceinline__ float tcp_mlp(TcPersist& S, uint32_t tmem, int tid, const float (&x)[6], uint32_t& phase,
                                         bool& dead) {
  const float nan = __int_as_float(0x7fc00000);
  sts128(S.a1, tc_off(tid, 0, TC_K1), tc_pack(x[0], x[1]), tc_pack(x[2], x[3]), tc_pack(x[4], x[5]), 0x3F80u);
  bool ok = true;
  if (!tcp_issue(S, S.a1, tmem, tid, TC_K1, 32, 1, 0, dead)) return nan;
  ok = tcp_wait(S, phase, dead) && ok;
  phase ^= 1u;
  tcp_hidden_to_a2(S, tmem, tid);
  if (!tcp_issue(S, S.a2, tmem, tid, TC_K2, 32, 3, TC_B1_BYTES, dead)) return nan;
  ok = tcp_wait(S, phase, dead) && ok;
  phase ^= 1u;
  const float y = tcp_output(S, tmem, tid);
  return ok ? y : nan;
}

// End of a persistent CTA.  If a wait gave up (in any thread: ORed over the
// CTA), the last committed MMAs may still be running: wait for that phase
// once more (bounded) before the TMEM columns are released.  `phase` is the
// parity of the next phase, so the last committed one has parity phase ^ 1.
__device__ __forceinline__ void tcp_teardown(TcPersist& S, uint32_t tmem, int tid, uint32_t phase, bool dead) {
  tc_fence_before();
  dead = __syncthreads_or(dead ? 1 : 0) != 0;
  if (dead) (void)mbar_wait(&S.mbar, phase ^ 1u);
  tc_fence_before();
  __syncthreads();
  if (tid < 32) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TC_TMEM_COLS) : "memory");
  }
}

}  // namespace lbm

// closure_tc.cuh — the learned closure's 6 -> 32 -> 32 -> 1 MLP for one CTA
// of 128 cells on the 5th-generation tensor cores (tcgen05.mma, kind::f16,
// bf16 operands from shared memory, fp32 accumulators in tensor memory).
//
// One tile = the CTA's 128 cells (thread tid <-> MMA row tid <-> TMEM lane
// tid).  Per layer: every thread writes its row of the A operand to shared
// memory, one thread issues the MMA(s) and commits them to an mbarrier, every
// thread waits on it and reads its row of the accumulator back with
// tcgen05.ld.  Biases ride in the K dimension: A carries a constant 1 in
// column kb and B holds the bias there (layer 1: K = 16 = 6 features + 1 +
// 9 zeros; layers 2, 3: K = 48 = 32 hidden + 1 + 15 zeros), so the
// accumulators start at zero and no bias add is needed.
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
constexpr int TC_B3_BYTES = 16 * TC_K2 * 2;      // 1536
constexpr int TC_B_BYTES = TC_B1_BYTES + TC_B2_BYTES + TC_B3_BYTES;   // 5632
constexpr int TC_A_BYTES = TC_ROWS * TC_K2 * 2;  // 12288 (layer-1 A uses the first 4096)
constexpr uint32_t TC_TMEM_COLS = 32;
constexpr uint32_t TC_WAIT_LIMIT = 1u << 20;     // mbarrier polls (~0.5 us apart) before giving up

// Byte offset of (row r, element k) in a K-major no-swizzle operand with K
// elements per row.
__host__ __device__ constexpr uint32_t tc_off(int r, int k, int K) {
  return (uint32_t)((r >> 3) * (K / 8) * 128 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

struct TcShared {
  alignas(128) uint8_t a[TC_A_BYTES];
  alignas(128) uint8_t b[TC_B_BYTES];
  alignas(8) uint64_t mbar;
  uint32_t tmem;
  uint32_t err;
};

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

__device__ __forceinline__ bool mbar_try(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for the phase of the given parity; false when it gave up.
// Between polls the warp sleeps, leaving the issue slots to the CTAs that
// are streaming populations.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  for (uint32_t i = 0; i < TC_WAIT_LIMIT; ++i) {
    if (mbar_try(bar, parity)) return true;
    __nanosleep(i < 4 ? 128u : 512u);
  }
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

// Start of a tile: warp 0 allocates TC_TMEM_COLS columns of tensor memory,
// thread 0 initialises the mbarrier, all threads copy the packed B operands
// (bw: TC_B_BYTES, 16-byte aligned).  Every thread of the 128-thread CTA
// calls it; returns the TMEM base address.
__device__ __forceinline__ uint32_t tc_begin(TcShared& S, const uint4* __restrict__ bw, int tid) {
  if (tid < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_addr(&S.tmem)),
                 "r"(TC_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_addr(&S.mbar)) : "memory");
    S.err = 0;
  }
  uint4* bd = reinterpret_cast<uint4*>(S.b);
  for (int i = tid; i < TC_B_BYTES / 16; i += TC_ROWS) bd[i] = __ldg(bw + i);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  return S.tmem;
}

// End of a tile: every thread calls it after its last tcgen05.ld.
__device__ __forceinline__ void tc_end(TcShared& S, uint32_t tmem, int tid) {
  tc_fence_before();
  __syncthreads();
  if (tid < 32) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TC_TMEM_COLS) : "memory");
  }
}

// Make this thread's shared-memory operand row visible to the tensor core,
// wait for every row, and let thread 0 issue `nk` K-steps of 16 into
// columns [0, N) and commit them.
__device__ __forceinline__ void tc_issue(TcShared& S, uint32_t tmem, int tid, int K, int N, int nk,
                                         uint32_t b_off) {
  proxy_fence();
  tc_fence_before();
  __syncthreads();
  if (tid == 0) {
    tc_fence_after();
    const uint32_t a0 = smem_addr(S.a), b0 = smem_addr(S.b) + b_off;
    const uint32_t idesc = tc_idesc(TC_ROWS, N);
    for (int k = 0; k < nk; ++k)   // K-step k covers elements 16k..16k+15: two core matrices
      tc_mma(tmem, tc_desc(a0 + (uint32_t)k * 256u, K), tc_desc(b0 + (uint32_t)k * 256u, K), idesc, k > 0);
    tc_commit(&S.mbar);
  }
}

// Wait for the committed MMAs; on a timeout record it and return false.
__device__ __forceinline__ bool tc_wait(TcShared& S, uint32_t parity) {
  const bool ok = mbar_wait(&S.mbar, parity);
  if (!ok) S.err = 1;
  tc_fence_after();
  return ok;
}

// Hidden layer epilogue: this thread's 32 accumulator columns -> ReLU ->
// bf16 -> its row of the next A operand (K = 48, constant 1 at element 32).
__device__ __forceinline__ void tc_hidden_to_a(TcShared& S, uint32_t tmem, int tid) {
  const uint32_t lane_addr = tmem + ((uint32_t)(tid & ~31) << 16);
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    float v[16];
    tc_ld16(lane_addr + 16u * h, v);
    uint32_t p[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) p[i] = tc_relu_pack(v[2 * i], v[2 * i + 1]);
    sts128(S.a, tc_off(tid, 16 * h, TC_K2), p[0], p[1], p[2], p[3]);
    sts128(S.a, tc_off(tid, 16 * h + 8, TC_K2), p[4], p[5], p[6], p[7]);
  }
  const uint32_t one = 0x3F80u;   // bf16 1.0 in the low half
  sts128(S.a, tc_off(tid, 32, TC_K2), one, 0u, 0u, 0u);
  sts128(S.a, tc_off(tid, 40, TC_K2), 0u, 0u, 0u, 0u);
}

// y (pre-softplus) of this thread's cell; x: normalised features (zeros for
// threads without a cell).  All 128 threads of the CTA must call it, between
// tc_begin and tc_end.  NaN when a wait gave up.
__device__ __forceinline__ float tc_mlp(TcShared& S, uint32_t tmem, int tid, const float (&x)[6]) {
  // layer 1: A row = [x0..x5, 1, 0 x 9]
  sts128(S.a, tc_off(tid, 0, TC_K1), tc_pack(x[0], x[1]), tc_pack(x[2], x[3]), tc_pack(x[4], x[5]), 0x3F80u);
  sts128(S.a, tc_off(tid, 8, TC_K1), 0u, 0u, 0u, 0u);
  tc_issue(S, tmem, tid, TC_K1, 32, 1, 0);
  bool ok = tc_wait(S, 0);
  tc_hidden_to_a(S, tmem, tid);
  // layer 2
  tc_issue(S, tmem, tid, TC_K2, 32, 3, TC_B1_BYTES);
  ok = tc_wait(S, 1) && ok;
  tc_hidden_to_a(S, tmem, tid);
  // layer 3 (N = 16, output in column 0)
  tc_issue(S, tmem, tid, TC_K2, 16, 3, TC_B1_BYTES + TC_B2_BYTES);
  ok = tc_wait(S, 0) && ok;
  const float y = tc_ld1(tmem + ((uint32_t)(tid & ~31) << 16));
  return ok ? y : __int_as_float(0x7fc00000);
}

}  // namespace lbm

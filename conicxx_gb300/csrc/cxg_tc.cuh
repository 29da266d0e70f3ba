// Blackwell tensor-core helpers (sm_103a): tcgen05 MMA with operands in shared memory and the
// accumulator in tensor memory (TMEM), written as inline PTX, on which the whole-GPU root
// factor's FP32 (kind::tf32) and double-float (kind::f16 with BF16 slices) trailing updates are
// built.
//
// Operand layout: the "K-major, no swizzle" canonical layout of the tcgen05 shared-memory matrix
// descriptor. A 128-row x 32-column TF32 panel is stored as core matrices of 8 rows x 16 bytes
// (8 x 4 values, 128 contiguous bytes); element (m, k) sits at byte
//     (k / 4) * 2048 + (m / 8) * 128 + (m % 8) * 16 + (k % 4) * 4,
// so core matrices adjacent in K are 2048 bytes apart (the descriptor's leading-dimension byte
// offset) and adjacent 8-row groups 128 bytes apart (its stride-dimension byte offset). One
// kind::tf32 MMA consumes K = 8 (two core-matrix columns): the MMA over columns 8s .. 8s+7
// starts at byte 4096 s of the panel. A panel is 16 KB.
//
// The same byte layout holds a 128 x 32 BF16 panel as 8 x 8-value core matrices: element (m, k) at
//     (k / 8) * 2048 + (m / 8) * 128 + (m % 8) * 16 + (k % 8) * 2,
// 8 KB per panel, one kind::f16 MMA (K = 16) per 4096 bytes.
//
// D[128 x 128] (+)= A[128 x 8] B[128 x 8]^T accumulates in FP32 in 128 TMEM columns: row i of D in
// TMEM lane i, column j in column base + j. A warp reads only the 32 lanes of its quarter
// (warp index % 4).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace cxg {
namespace tc {

constexpr int kRows = 128;                     // M = N of one MMA
constexpr int kPanelK = 32;                    // columns of one staged panel (one root tile column)
constexpr int kPanelBytes = kRows * kPanelK * 4;  // 16 KB
constexpr uint32_t kLbo = 2048;                // K-direction core-matrix step (bytes)
constexpr uint32_t kSbo = 128;                 // M/N-direction 8-row group step (bytes)
constexpr uint32_t kTmemCols = 128;            // accumulator columns (power of two >= 32)

__device__ __forceinline__ uint32_t smemAddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// byte offset of element (m, k) of a 128 x 32 panel in the layout above
__host__ __device__ __forceinline__ uint32_t panelOffset(int m, int k) {
  return (uint32_t)((k >> 2) * 2048 + (m >> 3) * 128 + (m & 7) * 16 + (k & 3) * 4);
}

// Shared-memory matrix descriptor (64 bits): start address >> 4 in bits 0-13, leading-dimension
// byte offset >> 4 in bits 16-29, stride-dimension byte offset >> 4 in bits 32-45, the fixed
// value 0b001 in bits 46-48, base offset 0, relative offsets, no swizzle (bits 61-63 = 0).
__device__ __forceinline__ uint64_t smemDesc(uint32_t addr) {
  uint64_t d = (uint64_t)((addr >> 4) & 0x3FFFu);
  d |= (uint64_t)((kLbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((kSbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor of kind::tf32: D in FP32 (bits 4-5 = 1), A and B TF32 (bits 7-9 and
// 10-12 = 2), both K-major (bits 15, 16 = 0), N >> 3 in bits 17-22, M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t idescTf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// Instruction descriptor of kind::f16 with BF16 A and B: D in FP32 (bits 4-5 = 1), A and B BF16
// (bits 7-9 and 10-12 = 1), both K-major, N >> 3 in bits 17-22, M >> 4 in bits 24-28. One MMA
// consumes K = 16 (two core-matrix columns of 8 BF16 values each).
__host__ __device__ constexpr uint32_t idescBf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// round to TF32 (nearest, ties away from zero), kept as an FP32 bit pattern
__device__ __forceinline__ float toTf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// D[tmem] (+)= A B^T; issued by one thread
__device__ __forceinline__ void mmaTf32(uint32_t dTmem, uint64_t aDesc, uint64_t bDesc, uint32_t idesc, bool accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dTmem),
      "l"(aDesc), "l"(bDesc), "r"(idesc), "r"(accumulate ? 1u : 0u)
      : "memory");
}

// D[tmem] (+)= A B^T with BF16 operands, FP32 accumulation; issued by one thread
__device__ __forceinline__ void mmaBf16(uint32_t dTmem, uint64_t aDesc, uint64_t bDesc, uint32_t idesc, bool accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dTmem),
      "l"(aDesc), "l"(bDesc), "r"(idesc), "r"(accumulate ? 1u : 0u)
      : "memory");
}

// the MMAs issued so far by this thread arrive on the mbarrier once they complete
__device__ __forceinline__ void commitTo(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

__device__ __forceinline__ void mbarInit(uint32_t mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbarInval(uint32_t mbar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(mbar) : "memory");
}

__device__ __forceinline__ bool mbarTryWait(uint32_t mbar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(mbar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Waits for the phase `parity` of the mbarrier to complete, at most `limitNs` nanoseconds.
__device__ __forceinline__ bool mbarWait(uint32_t mbar, uint32_t parity, unsigned long long limitNs) {
  if (mbarTryWait(mbar, parity)) return true;
  unsigned long long t0;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
  for (;;) {
    if (mbarTryWait(mbar, parity)) return true;
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    if (t - t0 > limitNs) return false;
  }
}

// TMEM allocation by one whole warp: the base address is written to shared memory at `slot`
__device__ __forceinline__ void tmemAlloc(uint32_t slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tmemDealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fenceBeforeSync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fenceAfterSync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes made visible to the tensor core (async proxy)
__device__ __forceinline__ void fenceProxyAsyncShared() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// ---- bulk copies (TMA, non-tensor form) between global and shared memory --------------------
// The expected transaction bytes of the current phase, with the issuing thread's arrival.
__device__ __forceinline__ void mbarArriveExpectTx(uint32_t mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}
// global -> shared, completing `bytes` on the mbarrier (addresses 16-byte aligned, bytes % 16 == 0)
__device__ __forceinline__ void bulkLoad(uint32_t dstSmem, const void* src, uint32_t bytes, uint32_t mbar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dstSmem),
               "l"(src), "r"(bytes), "r"(mbar)
               : "memory");
}
// shared -> global, in the issuing thread's current bulk group
__device__ __forceinline__ void bulkStore(void* dst, uint32_t srcSmem, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(srcSmem), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulkCommit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// the issuing thread's bulk stores have finished reading shared memory
__device__ __forceinline__ void bulkWaitRead0() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// ... and are complete in global memory
__device__ __forceinline__ void bulkWait0() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void fenceProxyAsyncGlobal() { asm volatile("fence.proxy.async.global;" ::: "memory"); }

// 8 consecutive TMEM columns of this thread's lane (warp quarter) into registers
__device__ __forceinline__ void tmemLoad8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr)
               : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

// 8 consecutive TMEM columns of this thread's lane at each of four column offsets (accumulators),
// with one wait for all four loads
__device__ __forceinline__ void tmemLoad8x4(uint32_t taddr, uint32_t accStride, float (&v)[4][8]) {
  uint32_t r[4][8];
#pragma unroll
  for (int a = 0; a < 4; ++a)
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(r[a][0]), "=r"(r[a][1]), "=r"(r[a][2]), "=r"(r[a][3]), "=r"(r[a][4]), "=r"(r[a][5]),
                   "=r"(r[a][6]), "=r"(r[a][7])
                 : "r"(taddr + (uint32_t)a * accStride)
                 : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int i = 0; i < 8; ++i) v[a][i] = __uint_as_float(r[a][i]);
}

// 16 consecutive TMEM columns of this thread's lane (warp quarter) into registers
__device__ __forceinline__ void tmemLoad16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace tc
}  // namespace cxg

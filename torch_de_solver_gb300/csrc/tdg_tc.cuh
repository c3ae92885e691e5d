// Inline-PTX helpers for the tensor-core (tcgen05) path on sm_103a: TMEM allocation, MMA issue and
// commit, TMEM loads, mbarriers with bounded waits, bulk (TMA) copies and the shared-memory
// operand layout the MMAs read.
//
// Operand layout ("K-major interleaved", no swizzle): an R x K operand is tiled into core matrices
// of 8 rows x 16 bytes. Core matrix (i/8, k/EPC) starts at (i/8)*SBO + (k/EPC)*128 bytes, with
// SBO = (K/EPC)*128, and inside it element (i%8, k%EPC) sits at (i%8)*16 + (k%EPC)*ES, where ES is
// the element size and EPC = 16/ES. The MMA descriptor then has LBO = 128 (next core matrix along
// K) and SBO (next 8-row group).
#pragma once
#include <cstdint>
#include <cuda_bf16.h>

namespace tdg {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// byte offset of element (i, k) of an interleaved operand whose rows hold kp elements of es bytes
__device__ __forceinline__ uint32_t ofs(int i, int k, int kp, int es) {
  const int epc = 16 / es;
  return (uint32_t)((i >> 3) * ((kp / epc) * 128) + (k / epc) * 128 + (i & 7) * 16 + (k % epc) * es);
}

__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;     // tcgen05 descriptor version
  return d;                   // base offset 0, no swizzle
}

// instruction descriptor: D = F32, A = B = TF32 (kind::tf32) or BF16 (kind::f16), both K-major
template <bool BF16>
__device__ __forceinline__ uint32_t instr_desc(int m, int n) {
  const uint32_t fmt = BF16 ? 1u : 2u;
  return (1u << 4) | (fmt << 7) | (fmt << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

template <bool BF16>
__device__ __forceinline__ void mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, bool acc) {
  if (BF16)
    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                 " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}"
                 :: "r"(d_tmem), "l"(a), "l"(b), "r"(idesc), "r"((uint32_t)acc));
  else
    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                 " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}"
                 :: "r"(d_tmem), "l"(a), "l"(b), "r"(idesc), "r"((uint32_t)acc));
}

// D += A . B^T with A read from tensor memory (columns = K) and B from shared memory (kind::tf32)
__device__ __forceinline__ void mma_ts_tf32(uint32_t d_tmem, uint32_t a_tmem, uint64_t b, uint32_t idesc, bool acc) {
  asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
               " tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n}"
               :: "r"(d_tmem), "r"(a_tmem), "l"(b), "r"(idesc), "r"((uint32_t)acc));
}

__device__ __forceinline__ void commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
               :: "r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
// generic-proxy writes (shared and global) ordered before later async-proxy accesses
__device__ __forceinline__ void fence_async_all() { asm volatile("fence.proxy.async;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t* dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
               :: "r"(smem_u32(dst_smem)), "r"(ncols));
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(taddr), "r"(ncols));
}

// 8 consecutive 32-bit columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

// two loads of 8 consecutive 32-bit columns (at a0 and a1) behind one wait: the loads and the
// wait are one asm statement, so no use of the registers can be scheduled before the wait
__device__ __forceinline__ void tmem_ld8x2(uint32_t a0, uint32_t a1, float (&v0)[8], float (&v1)[8]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%16];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%8,%9,%10,%11,%12,%13,%14,%15}, [%17];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(a0), "r"(a1)
      : "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    v0[i] = __uint_as_float(r[i]);
    v1[i] = __uint_as_float(r[8 + i]);
  }
}

// store 8 / 4 consecutive 32-bit columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_st8(uint32_t taddr, const float (&v)[8]) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};"
               :: "r"(taddr), "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])),
                  "r"(__float_as_uint(v[2])), "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])),
                  "r"(__float_as_uint(v[5])), "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7]))
               : "memory");
}
__device__ __forceinline__ void tmem_st4(uint32_t taddr, float a, float b, float c, float d) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1,%2,%3,%4};"
               :: "r"(taddr), "r"(__float_as_uint(a)), "r"(__float_as_uint(b)),
                  "r"(__float_as_uint(c)), "r"(__float_as_uint(d)) : "memory");
}
__device__ __forceinline__ void tmem_st_wait() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
               :: "r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// Wait for the phase with the given parity; gives up after a bounded number of polls and
// returns false (the caller records the timeout) instead of spinning forever.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int max_polls = 1 << 24) {
  uint32_t done = 0;
  for (int it = 0; it < max_polls && !done; ++it) {
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                 " selp.u32 %0, 1, 0, p;\n}"
                 : "=r"(done) : "r"(smem_u32(bar)), "r"(parity) : "memory");
  }
  return done != 0;
}

// one-dimensional bulk copy global -> shared, completion counted on `bar` in bytes
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               :: "r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}

// invalidate one 128-byte line of global memory in L2 without writing it back (its contents
// become unspecified): for scratch that nothing reads again
__device__ __forceinline__ void discard_l2(const void* line) {
  asm volatile("discard.global.L2 [%0], 128;" :: "l"(line) : "memory");
}

__device__ __forceinline__ void prefetch_l2(const void* src, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" :: "l"(src), "r"(bytes) : "memory");
}

__device__ __forceinline__ float to_tf32(float x) {
  // round to the nearest TF32 value (10 explicit mantissa bits), ties away from zero: add half a
  // TF32 unit in the last place to the magnitude bits, then clear the 13 low mantissa bits
  return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xffffe000u);
}

// store a value into an operand buffer as TF32 (rounded) or BF16
template <bool BF16>
__device__ __forceinline__ void put(unsigned char* buf, uint32_t off, float v) {
  if (BF16) *reinterpret_cast<__nv_bfloat16*>(buf + off) = __float2bfloat16_rn(v);
  else *reinterpret_cast<float*>(buf + off) = to_tf32(v);
}

template <bool BF16>
__device__ __forceinline__ float get(const unsigned char* buf, uint32_t off) {
  if (BF16) return __bfloat162float(*reinterpret_cast<const __nv_bfloat16*>(buf + off));
  return *reinterpret_cast<const float*>(buf + off);
}

}  // namespace tc
}  // namespace tdg

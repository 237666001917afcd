// Inline-PTX helpers shared by the tensor-core blur passes: tcgen05 MMA
// descriptors and issue, TMEM loads, mbarrier waits with an iteration cap,
// named-barrier reductions and TMA (cp.async.bulk.tensor) copies.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace pxg {
namespace tc {

constexpr long long kWaitCap = 1 << 22;  // mbarrier polls before giving up (far above a tile's MMA time)

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// tcgen05 shared-memory matrix descriptor: K-major, no swizzle.
__device__ __forceinline__ uint64_t mat_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: f16 A and B (K-major), f32 D, M x N.
__host__ __device__ constexpr uint32_t instr_desc(int M, int N) {
  return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// Byte offset of element (row, k) in a K-major no-swizzle operand with K
// columns.
__device__ __forceinline__ uint32_t canon_off(int row, int k, int K) {
  return (uint32_t)((row >> 3) * (K >> 3) * 128 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ void mma_f16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                        uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar)
               : "memory");
}

// Waits for the mbarrier to complete the phase with the given parity;
// returns false if it did not within kWaitCap polls.  A non-blocking test
// first (a phase that has already completed answers in a few cycles), then
// try_wait, which suspends the thread until the phase completes or a
// hardware time limit passes.
__device__ __forceinline__ bool mbar_test(uint32_t mbar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(done)
      : "r"(mbar), "r"(parity)
      : "memory");
  return done != 0;
}
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
  if (mbar_test(mbar, parity)) return true;
  for (long long i = 0; i < kWaitCap; i++) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// 32 lanes x 32 columns of f32 from TMEM (this warp's lane quarter).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ uint16_t f16_bits(uint32_t v) {  // an integer 0..255 as f16
  return __half_as_ushort(__uint2half_rn(v));
}

// Channel c of two RGBX pixels as an f16 pair (x's in the low half): the
// bytes are placed under the f16 exponent of 1024 (0x64), where the mantissa
// step is 1, giving 1024 + v exactly; subtracting 1024 leaves v.
__device__ __forceinline__ uint32_t f16_pair(uint32_t x, uint32_t y, int c) {
  const uint32_t p = __byte_perm(x, y, (uint32_t)c | ((uint32_t)(c + 4) << 4));  // [x_c, y_c, ., .]
  const uint32_t q = __byte_perm(p, 0x64646464u, 0x5140u);                      // [x_c, 64, y_c, 64]
  const __half2 h = __hsub2(*reinterpret_cast<const __half2*>(&q), __halves2half2(__ushort_as_half(0x6400),
                                                                                  __ushort_as_half(0x6400)));
  return *reinterpret_cast<const uint32_t*>(&h);
}

__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(mbar), "r"(count) : "memory");
}
// bar.red.or over the 128 threads of epilogue group g (named barrier 1 + g):
// every thread gets the same answer, so the group leaves a loop together.
__device__ __forceinline__ bool epi_bar_or(int g, bool v) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 p, %1, 0;\n\t"
      "bar.red.or.pred q, %2, 128, p;\n\t"
      "selp.u32 %0, 1, 0, q;\n\t}\n"
      : "=r"(r)
      : "r"((uint32_t)v), "r"(1 + g)
      : "memory");
  return r != 0;
}
__device__ __forceinline__ void epi_bar(int g) {
  asm volatile("bar.sync %0, 128;\n" ::"r"(1 + g) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t mbar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(mbar) : "memory");
}

// 2-D TMA load of one box into shared memory; completion is signalled on the
// mbarrier as transaction bytes.
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const void* tmap, int x, int y, uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(tmap)), "r"(x), "r"(y), "r"(mbar)
      : "memory");
}
// 2-D TMA store of one box from shared memory (bulk async-group).
__device__ __forceinline__ void tma_store_2d(const void* tmap, int x, int y, uint32_t src) {
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];\n" ::"l"(
                   reinterpret_cast<uint64_t>(tmap)),
               "r"(x), "r"(y), "r"(src)
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;\n" ::: "memory"); }
// Waits until at most N of this thread's bulk groups still read shared memory.
template <int N>
__device__ __forceinline__ void bulk_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read %0;\n" ::"n"(N) : "memory");
}
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint32_t mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(mbar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void tmap_prefetch(const void* tmap) {
  asm volatile("prefetch.tensormap [%0];\n" ::"l"(reinterpret_cast<uint64_t>(tmap)) : "memory");
}

// tcgen05 shared-memory matrix descriptor: K-major, 128-byte swizzle.  The
// operand is stored as 1024-byte atoms of 8 rows x 128 bytes (64 f16 along
// K), the 16-byte chunk c of row r at chunk c ^ (r % 8); atoms of successive
// 8-row groups lie SBO bytes apart.  A K step inside an atom advances the
// start address by its byte offset along the row.
__device__ __forceinline__ uint64_t mat_desc_sw128(uint32_t saddr, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)1u << 16) | ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) |
         (1ull << 46) | (2ull << 61);
}
// Byte offset of element (row, k) in a K-major 128-byte-swizzled operand
// whose K extent is split into blocks of 64 (blockBytes apart).
__host__ __device__ __forceinline__ uint32_t sw128_off(int row, int k, uint32_t blockBytes) {
  return (uint32_t)(k >> 6) * blockBytes + (uint32_t)((row >> 3) * 1024 + (row & 7) * 128) +
         (uint32_t)((((k >> 3) & 7) ^ (row & 7)) << 4) + (uint32_t)((k & 7) * 2);
}

// Issue forms for warp-uniform code: the whole warp executes the call with
// the same operands (so they stay in uniform registers) and one lane, chosen
// by elect.sync, issues the operation.
__device__ __forceinline__ void mma_f16_elect(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                              uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred e, p;\n\t"
      "elect.sync _|e, 0xffffffff;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "@e tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}
__device__ __forceinline__ void mma_commit_elect(uint32_t mbar) {
  asm volatile(
      "{\n\t.reg .pred e;\n\t"
      "elect.sync _|e, 0xffffffff;\n\t"
      "@e tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n\t}\n" ::"r"(mbar)
      : "memory");
}
// expect_tx of the box's bytes on the mbarrier, then the 2-D TMA load.
__device__ __forceinline__ void tma_load_2d_elect(uint32_t dst, const void* tmap, int x, int y, uint32_t mbar,
                                                  uint32_t bytes) {
  asm volatile(
      "{\n\t.reg .pred e;\n\t"
      "elect.sync _|e, 0xffffffff;\n\t"
      "@e mbarrier.arrive.expect_tx.shared::cta.b64 _, [%4], %5;\n\t"
      "@e cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n\t}\n" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(tmap)), "r"(x), "r"(y), "r"(mbar), "r"(bytes)
      : "memory");
}

// Shared-memory accesses by 32-bit shared address (no generic addressing).
__device__ __forceinline__ uint4 lds128(uint32_t a) {
  uint4 v;
  asm volatile("ld.shared.v4.u32 {%0, %1, %2, %3}, [%4];\n" : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "r"(a));
  return v;
}
__device__ __forceinline__ uint32_t lds32(uint32_t a) {
  uint32_t v;
  asm volatile("ld.shared.u32 %0, [%1];\n" : "=r"(v) : "r"(a));
  return v;
}
__device__ __forceinline__ void sts128(uint32_t a, uint4 v) {
  asm volatile("st.shared.v4.u32 [%0], {%1, %2, %3, %4};\n" ::"r"(a), "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w)
               : "memory");
}
__device__ __forceinline__ void sts8(uint32_t a, uint32_t v) {
  asm volatile("st.shared.u8 [%0], %1;\n" ::"r"(a), "r"(v) : "memory");
}
__device__ __forceinline__ uint64_t f32x2_splat(float v) {
  return ((uint64_t)__float_as_uint(v) << 32) | __float_as_uint(v);
}
// Two lanes of floor(S / 65280) for accumulators holding S * 2^-24, S < 2^24
// an integer: one packed FMA rounding toward minus infinity, q * C24 + M,
// with C24 = RU(1/65280) * 2^24 and M = 1.5 * 2^23, leaves each quotient in
// the low byte of its result.  With SPLIT the accumulator pair (hi, lo) holds
// S = 256 * S_hi + S_lo and is combined first (exactly: multiples of 2^-24
// below 1).
template <bool SPLIT>
__device__ __forceinline__ void quot2(float h0, float h1, float l0, float l1, uint64_t k256, uint64_t kq,
                                      uint64_t km, uint32_t& q0, uint32_t& q1) {
  if (SPLIT)
    asm("{\n\t.reg .b64 h, l, v, d;\n\t"
        "mov.b64 h, {%2, %3};\n\t"
        "mov.b64 l, {%4, %5};\n\t"
        "fma.rn.f32x2 v, h, %6, l;\n\t"
        "fma.rm.f32x2 d, v, %7, %8;\n\t"
        "mov.b64 {%0, %1}, d;\n\t}\n"
        : "=r"(q0), "=r"(q1)
        : "f"(h0), "f"(h1), "f"(l0), "f"(l1), "l"(k256), "l"(kq), "l"(km));
  else
    asm("{\n\t.reg .b64 h, d;\n\t"
        "mov.b64 h, {%2, %3};\n\t"
        "fma.rm.f32x2 d, h, %4, %5;\n\t"
        "mov.b64 {%0, %1}, d;\n\t}\n"
        : "=r"(q0), "=r"(q1)
        : "f"(h0), "f"(h1), "l"(kq), "l"(km));
}

}  // namespace tc
}  // namespace pxg

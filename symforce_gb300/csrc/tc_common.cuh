// tcgen05 (5th-generation tensor core) helpers shared by the TF32 GEMMs: the canonical K-major
// shared-memory operand layout without swizzle, its matrix descriptor, the kind::tf32 instruction
// descriptor, the three-pass TF32 split, capped mbarrier waits, MMA issue and commit.
#pragma once

#include <cstdint>

namespace sfg {
namespace tc {

constexpr int kTcRows = 128;   // M of the MMA (TMEM lanes)
constexpr int kTcKc = 32;      // K per staged chunk (four MMAs of K = 8)
constexpr unsigned kTcSpin = 1u << 24;


__device__ __forceinline__ uint32_t SmemAddr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Byte offset of element (row, k) of a [rows x kTcKc] K-major operand chunk: core matrices of
// 8 rows x 4 FP32, 128 bytes each, consecutive along K (LBO = 128 B), 8-row groups kTcKc / 4 core
// matrices apart (SBO = 1024 B).
__device__ __forceinline__ uint32_t ChunkOffset(int row, int k) {
  return uint32_t((row >> 3) * 1024 + (k >> 2) * 128 + (row & 7) * 16 + (k & 3) * 4);
}

// Shared-memory matrix descriptor: start address, LBO and SBO in 16-byte units, descriptor version 1,
// no swizzle.
__device__ __forceinline__ uint64_t SmemDesc(uint32_t addr) {
  constexpr uint64_t kLbo = 128 >> 4, kSbo = 1024 >> 4;
  return uint64_t((addr & 0x3FFFF) >> 4) | (kLbo << 16) | (kSbo << 32) | (uint64_t(1) << 46);
}

// Instruction descriptor of kind::tf32: FP32 accumulator, TF32 A and B, both K-major, N and M.
__device__ __forceinline__ uint32_t InstrDesc(int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | (uint32_t(n >> 3) << 17) | (uint32_t(kTcRows >> 4) << 24);
}

__device__ __forceinline__ float TfHi(float x) { return __uint_as_float(__float_as_uint(x) & 0xFFFFE000u); }

__device__ __forceinline__ void MbarInit(uint64_t* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(SmemAddr(bar)) : "memory");
}

// Waits for the completion of the given phase; false if the cap was hit.
__device__ __forceinline__ bool MbarWait(uint64_t* bar, uint32_t phase) {
  const uint32_t addr = SmemAddr(bar);
  for (unsigned it = 0; it < kTcSpin; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(addr), "r"(phase)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void MmaTf32(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                        uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void MmaCommit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(SmemAddr(bar))
               : "memory");
}

// TMEM: allocate / free ncols columns (a power of two >= 32) for this CTA; warp-wide calls.
__device__ __forceinline__ void TmemAlloc(uint32_t* slot, int ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(SmemAddr(slot)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void TmemFree(uint32_t base, int ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(base), "r"(ncols) : "memory");
}
// 16 consecutive FP32 columns of this warp's 32 TMEM lanes (lane = row) into v
__device__ __forceinline__ void TmemLoad16(uint32_t taddr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
      "%14, %15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
        "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

}  // namespace tc
}  // namespace sfg

// Device pieces shared by the split-precision GEMM kernels (lgb_gemm_tc.cu,
// lgb_gemm_persist.cu): the interleaved complex row orders, the 2D TMA load,
// the 64-byte-swizzle K-major shared-memory descriptor and the hi/lo splits.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>

#include "lgb_umma.cuh"

namespace lgb {
namespace splitk {

using namespace umma;

constexpr int kRowBytes = 64;  // K bytes per row and pipeline stage (one 64-byte swizzle atom)

// Poll bound of the pipeline waits: far above a tile's main loop (< 1 ms), far
// below a stuck GPU.
constexpr long long kGemmSpin = 1LL << 22;

// M-side row of component c of complex row i; N-side row of component p of
// complex column j (the two lanes of one complex row sit 16 TMEM lanes apart).
__device__ __forceinline__ int mrow(int c, int i) { return ((i >> 4) << 5) + (c << 4) + (i & 15); }
__device__ __forceinline__ int ncol(int p, int j) { return ((j >> 4) << 5) + ((1 - p) << 4) + (j & 15); }

__device__ __forceinline__ void mbar_expect_tx(uint64_t* m, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(m)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y,
                                            uint64_t* mbar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(mbar))
      : "memory");
}

// K-major shared-memory descriptor with the 64-byte swizzle: rows 64 B apart,
// 8-row groups SBO = 512 B apart, layout type 4 (bits 61-63), version 1.
__device__ __forceinline__ uint64_t sdesc_sw64(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1 << 16;            // leading byte offset (unused within one atom)
  d |= (uint64_t)(512 >> 4) << 32;   // stride byte offset
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)4 << 61;
  return d;
}

// The same with the 128-byte swizzle: rows 128 B apart, SBO = 1024 B, layout
// type 2.  The K-steps of a stage advance the start address by 32 B inside
// the 1 KB-aligned atom, as with the 64-byte form.
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

template <bool BF16>
__device__ __forceinline__ void mma_k(uint32_t d, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
  if constexpr (BF16) {
    mma_f16(d, a, b, id, acc);
  } else {
    mma_tf32(d, a, b, id, acc);
  }
}

// x = hi + lo with hi, lo in the operand format (TF32 bit patterns in FP32
// words, or BF16)
template <bool BF16> struct SElem;
template <> struct SElem<false> {
  using T = float;
  __device__ static void split(float x, T& h, T& l) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    const float hf = __uint_as_float(r);
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x - hf));
    h = hf;
    l = __uint_as_float(r);
  }
};
template <> struct SElem<true> {
  using T = __nv_bfloat16;
  __device__ static void split(float x, T& h, T& l) {
    h = __float2bfloat16_rn(x);
    l = __float2bfloat16_rn(x - __bfloat162float(h));
  }
};

}  // namespace splitk
}  // namespace lgb

// digits.cuh -- balanced base-256 digits of FP64 values as FP16 MMA operands, shared by the split
// precision kernels (split.cu, split_tsmm.cu).
//
// An FP64 value x of a row or column with shared exponent field E is the 62-bit fixed-point
// integer F = |x| * 2^(1084 - E) (sign kept apart); G = F + 0x8080...80 holds F's balanced digits
// as bytes (byte i = digit i + 128, most significant first).  A digit d in [-128, 127] is exact in
// FP16, and so is every product of two digits and every FP32 sum of up to 2^10 of them.
#pragma once
#include <cuda_fp16.h>
#include <stdint.h>

namespace skinny {

constexpr int NDIGITS = 8;

// G = F + 0x8080...80 for the 62-bit fixed-point magnitude F of x relative to exponent field E:
// byte i of G (most significant first) is digit i + 128, so the digits are balanced
__device__ __forceinline__ void g_words(double x, uint32_t E, uint32_t& gh, uint32_t& gl, bool& neg) {
  const uint32_t hi = (uint32_t)__double2hiint(x), lo = (uint32_t)__double2loint(x);
  const uint32_t ef = (hi >> 20) & 0x7FF;
  neg = (hi >> 31) != 0;
  const uint32_t eff = ef ? ef : 1u;
  const uint64_t mant = ((uint64_t)((hi & 0xFFFFFu) | (ef ? 0x100000u : 0u)) << 32) | lo;
  const uint32_t sh = E - eff;
  const uint64_t F = sh < 64 ? ((mant << 9) >> sh) : 0ull;
  const uint64_t G = F + 0x8080808080808080ull;
  gh = (uint32_t)(G >> 32);
  gl = (uint32_t)G;
}

// The eight FP16 digit pairs of elements a, b (a in the low halves), digit i in out[i].  A byte g
// of G becomes the half 1024 + g by pairing it with the byte 0x64 (two byte permutes), and one
// HFMA2 subtracts 1152 and applies each element's sign: (1024 + g - 1152) * s = (g - 128) * s,
// exact in FP16.  About 1.25 instructions per digit.
__device__ __forceinline__ void digit_pairs(uint32_t gha, uint32_t gla, bool na, uint32_t ghb, uint32_t glb, bool nb,
                                            uint32_t (&out)[NDIGITS]) {
  const __half2 s = __halves2half2(na ? __float2half(-1.0f) : __float2half(1.0f),
                                   nb ? __float2half(-1.0f) : __float2half(1.0f));
  const __half2 c = __hmul2(s, __float2half2_rn(-1152.0f));
  auto dig = [&](uint32_t pair, uint32_t sel) {
    const uint32_t u = __byte_perm(pair, 0x64646464u, sel);
    __half2 h = *reinterpret_cast<const __half2*>(&u);
    h = __hfma2(h, s, c);
    return *reinterpret_cast<const uint32_t*>(&h);
  };
#pragma unroll
  for (int w = 0; w < 2; w++) {
    const uint32_t ga = w ? gla : gha, gb = w ? glb : ghb;
    const uint32_t x01 = __byte_perm(ga, gb, 0x6273);  // [a.b3, b.b3, a.b2, b.b2]
    const uint32_t x23 = __byte_perm(ga, gb, 0x4051);  // [a.b1, b.b1, a.b0, b.b0]
    out[4 * w + 0] = dig(x01, 0x4140);
    out[4 * w + 1] = dig(x01, 0x4342);
    out[4 * w + 2] = dig(x23, 0x4140);
    out[4 * w + 3] = dig(x23, 0x4342);
  }
}

}  // namespace skinny

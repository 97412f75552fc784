// Split of complex64 values into BF16 hi and lo parts (x = hi + lo), packed (re, im) per
// 32-bit word: the operand layout of the tensor-core sphere contraction (sphere_tc.cu).
#pragma once

#include <cuda_bf16.h>
#include <cstdint>

namespace pawpy {

__device__ __forceinline__ void split_bf16x2(float2 v, uint32_t &hi, uint32_t &lo) {
  const __nv_bfloat16 hr = __float2bfloat16_rn(v.x), hm = __float2bfloat16_rn(v.y);
  const __nv_bfloat16 lr = __float2bfloat16_rn(v.x - __bfloat162float(hr));
  const __nv_bfloat16 lm = __float2bfloat16_rn(v.y - __bfloat162float(hm));
  hi = (uint32_t)__bfloat16_as_ushort(hr) | ((uint32_t)__bfloat16_as_ushort(hm) << 16);
  lo = (uint32_t)__bfloat16_as_ushort(lr) | ((uint32_t)__bfloat16_as_ushort(lm) << 16);
}

// Picked-point rows: complex64 X[row][xstride] (lo_words == 0), or the split form in K blocks
// of 16 points: BF16 (re, im) words hi[point / 16][row][point % 16], xstride words from one
// block to the next, lo at hi + lo_words.
__device__ __forceinline__ void put_picked(float2 *X, long long row, long long xstride, long long lo_words, int pos,
                                           float2 v) {
  if (lo_words == 0) {
    X[row * xstride + pos] = v;
  } else {
    uint32_t h, l;
    split_bf16x2(v, h, l);
    uint32_t *w = reinterpret_cast<uint32_t *>(X) + (long long)(pos >> 4) * xstride + row * 16 + (pos & 15);
    w[0] = h;
    w[lo_words] = l;
  }
}

}  // namespace pawpy

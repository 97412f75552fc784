// Split of complex64 values into BF16 hi and lo parts (x = hi + lo), packed (re, im) per
// 32-bit word: the operand layout of the tensor-core sphere contraction (sphere_tc.cu).
#pragma once

#include <cuda_bf16.h>
#include <cstdint>

namespace pawpy {

__device__ __forceinline__ void split_bf16x2(float2 v, uint32_t &hi, uint32_t &lo) {
  // packed conversions: (re, im) to two BF16 in one instruction, each rounded to nearest
  const __nv_bfloat162 h = __floats2bfloat162_rn(v.x, v.y);
  const float2 hf = __bfloat1622float2(h);
  const __nv_bfloat162 l = __floats2bfloat162_rn(v.x - hf.x, v.y - hf.y);
  hi = *reinterpret_cast<const uint32_t *>(&h);
  lo = *reinterpret_cast<const uint32_t *>(&l);
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

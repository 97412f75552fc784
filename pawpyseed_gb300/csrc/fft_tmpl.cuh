// Shared-memory FFT of many short lines with the line length N fixed at
// compile time (Stockham autosort, radix 4 first, then 2, 3, 5, 7...; the
// same formulation as block_fft in fft_block.cuh, with every index, radix and
// twiddle stride a compile-time constant and the butterflies in registers).
//
// Two thread mappings, both conflict-free in shared memory:
//  * rows    (elements of a line contiguous, lines ls apart): lanes walk along
//             a line, warps over lines;
//  * columns (lines adjacent, elements es apart): lanes walk across 32
//             adjacent lines, warps over butterflies.
#pragma once

#include "fft_block.cuh"

namespace pawpy {

constexpr int fft_factor(int n, int idx) {
  int cnt = 0;
  while (n % 4 == 0) {
    if (cnt == idx) return 4;
    cnt++;
    n /= 4;
  }
  for (int p = 2; p <= n; p++)
    while (n % p == 0) {
      if (cnt == idx) return p;
      cnt++;
      n /= p;
    }
  return 0;
}

constexpr bool fft_supported(int n) {
  int m = n;
  for (int p = 2; p <= 7; p++)
    while (m % p == 0) m /= p;
  return m == 1 && n >= 2;
}

template <int R, int N, int S>
__host__ __device__ __forceinline__ void dft_t(float2 (&v)[R], float2 (&o)[R], const float2 *tw) {
  constexpr float s = (float)S;
  if constexpr (R == 2) {
    o[0] = cadd(v[0], v[1]);
    o[1] = csub(v[0], v[1]);
  } else if constexpr (R == 4) {
    float2 a = cadd(v[0], v[2]), b = csub(v[0], v[2]);
    float2 c = cadd(v[1], v[3]), d = rot(csub(v[1], v[3]), s);
    o[0] = cadd(a, c);
    o[2] = csub(a, c);
    o[1] = cadd(b, d);
    o[3] = csub(b, d);
  } else if constexpr (R == 3) {
    const float h = 0.86602540378443864676f;  // sqrt(3)/2
    float2 t = cadd(v[1], v[2]);
    float2 m = make_float2(v[0].x - 0.5f * t.x, v[0].y - 0.5f * t.y);
    float2 d = rot(csub(v[1], v[2]), s);
    o[0] = cadd(v[0], t);
    o[1] = make_float2(m.x + h * d.x, m.y + h * d.y);
    o[2] = make_float2(m.x - h * d.x, m.y - h * d.y);
  } else if constexpr (R == 5) {
    const float c1 = 0.30901699437494742410f, c2 = -0.80901699437494742410f;
    const float s1 = 0.95105651629515357212f, s2 = 0.58778525229247312917f;
    float2 a1 = cadd(v[1], v[4]), b1 = csub(v[1], v[4]);
    float2 a2 = cadd(v[2], v[3]), b2 = csub(v[2], v[3]);
    o[0] = cadd(v[0], cadd(a1, a2));
    float2 m1 = make_float2(v[0].x + c1 * a1.x + c2 * a2.x, v[0].y + c1 * a1.y + c2 * a2.y);
    float2 m2 = make_float2(v[0].x + c2 * a1.x + c1 * a2.x, v[0].y + c2 * a1.y + c1 * a2.y);
    float2 n1 = rot(make_float2(s1 * b1.x + s2 * b2.x, s1 * b1.y + s2 * b2.y), s);
    float2 n2 = rot(make_float2(s2 * b1.x - s1 * b2.x, s2 * b1.y - s1 * b2.y), s);
    o[1] = cadd(m1, n1);
    o[4] = csub(m1, n1);
    o[2] = cadd(m2, n2);
    o[3] = csub(m2, n2);
  } else {
    constexpr int step = N / R;
#pragma unroll
    for (int q = 0; q < R; q++) {
      float2 acc = v[0];
#pragma unroll
      for (int r = 1; r < R; r++) {
        float2 w = tw[((r * q) % R) * step];
        if (S < 0) w.y = -w.y;
        acc = cadd(acc, cmul(v[r], w));
      }
      o[q] = acc;
    }
  }
}

template <int N, int R, int SPAN, int S>
__device__ __forceinline__ void fft_butterfly(const float2 *in, float2 *out, int j, int es, const float2 *tw) {
  constexpr int M = N / R;
  constexpr int TSTEP = N / (SPAN * R);
  const int k = j % SPAN;
  float2 v[R], o[R];
#pragma unroll
  for (int r = 0; r < R; r++) {
    float2 x = in[(j + r * M) * es];
    if (r > 0 && SPAN > 1) {
      float2 w = tw[k * r * TSTEP];
      if (S < 0) w.y = -w.y;
      x = cmul(x, w);
    }
    v[r] = x;
  }
  dft_t<R, N, S>(v, o, tw);
  const int base = (j / SPAN) * SPAN * R + k;
#pragma unroll
  for (int q = 0; q < R; q++) out[(base + q * SPAN) * es] = o[q];
}

// One stage over `count` lines.
template <int N, int R, int SPAN, int S, bool ROWS>
__device__ __forceinline__ void fft_stage(const float2 *src, float2 *dst, int count, int ls, int es,
                                          const float2 *tw) {
  constexpr int M = N / R;
  if (ROWS) {
    // flat over (line, butterfly): consecutive threads take consecutive butterflies of a line
    const int total = count * M;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
      int c = t / M, j = t - c * M;
      fft_butterfly<N, R, SPAN, S>(src + c * ls, dst + c * ls, j, 1, tw);
    }
  } else {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int c0 = 0; c0 < count; c0 += 32) {
      int c = c0 + lane;
      if (c < count)
        for (int j = warp; j < M; j += nw) fft_butterfly<N, R, SPAN, S>(src + c, dst + c, j, es, tw);
    }
  }
}

template <int N, int IDX, int SPAN, int S, bool ROWS>
__device__ __forceinline__ float2 *fft_chain(float2 *src, float2 *dst, int count, int ls, int es, const float2 *tw) {
  constexpr int R = fft_factor(N, IDX);
  if constexpr (R == 0) {
    return src;
  } else {
    fft_stage<N, R, SPAN, S, ROWS>(src, dst, count, ls, es, tw);
    __syncthreads();
    return fft_chain<N, IDX + 1, SPAN * R, S, ROWS>(dst, src, count, ls, es, tw);
  }
}

// Transform `count` lines of length N (rows: es == 1; columns: ls == 1).
// Returns the buffer holding the result. All threads of the block must call it.
template <int N, int S, bool ROWS>
__device__ __forceinline__ float2 *block_fft_n(float2 *a, float2 *b, int count, int ls, int es, const float2 *tw) {
  return fft_chain<N, 0, 1, S, ROWS>(a, b, count, ls, es, tw);
}

// Runtime dispatch over the compile-time sizes (2,3,5-smooth N <= 128); other
// lengths take the generic transform.
template <int S, bool ROWS>
__device__ float2 *block_fft_any(float2 *a, float2 *b, const Radices &rx, int count, int ls, int es,
                                 const float2 *tw) {
#define PAWPY_FFT_CASE(n) \
  case n:                 \
    return block_fft_n<n, S, ROWS>(a, b, count, ls, es, tw);
  switch (rx.n) {
    PAWPY_FFT_CASE(8)
    PAWPY_FFT_CASE(9)
    PAWPY_FFT_CASE(10)
    PAWPY_FFT_CASE(12)
    PAWPY_FFT_CASE(15)
    PAWPY_FFT_CASE(16)
    PAWPY_FFT_CASE(18)
    PAWPY_FFT_CASE(20)
    PAWPY_FFT_CASE(24)
    PAWPY_FFT_CASE(25)
    PAWPY_FFT_CASE(27)
    PAWPY_FFT_CASE(30)
    PAWPY_FFT_CASE(32)
    PAWPY_FFT_CASE(36)
    PAWPY_FFT_CASE(40)
    PAWPY_FFT_CASE(45)
    PAWPY_FFT_CASE(48)
    PAWPY_FFT_CASE(50)
    PAWPY_FFT_CASE(54)
    PAWPY_FFT_CASE(60)
    PAWPY_FFT_CASE(64)
    PAWPY_FFT_CASE(72)
    PAWPY_FFT_CASE(75)
    PAWPY_FFT_CASE(80)
    PAWPY_FFT_CASE(81)
    PAWPY_FFT_CASE(90)
    PAWPY_FFT_CASE(96)
    PAWPY_FFT_CASE(100)
    PAWPY_FFT_CASE(108)
    PAWPY_FFT_CASE(120)
    PAWPY_FFT_CASE(125)
    PAWPY_FFT_CASE(128)
    default:
      return block_fft<S>(a, b, rx, count, ls, es, tw);
  }
#undef PAWPY_FFT_CASE
}

}  // namespace pawpy

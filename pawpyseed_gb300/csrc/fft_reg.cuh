// Line FFTs held in registers: a line of compile-time length N is shared by
// T = 1, 2 or 4 lanes of a warp. Lane h of the group holds x[h + T m],
// m < L = N / T, transforms that subsequence with a mixed-radix (4, 2, 3, 5)
// decimation-in-time DFT whose twiddles are compile-time constants, and the
// T subsequences are combined by log2(T) radix-2 steps across lanes (warp
// shuffles). Lane h ends with the L outputs X[L pos(h) + k], k < L, where pos
// reverses the bits of h.
//
// Lanes of a warp are grouped as h = lane / (32 / T), slot c = lane % (32 / T),
// so that 32 / T lines are transformed by a warp at once and lanes of equal h
// touch consecutive elements of shared memory.
//
// Sign convention: X[k] = sum_n x[n] exp(S 2 pi i n k / N) (S = +1: the
// backward transform of the reference).
#pragma once

#include <utility>

#include "fft_tmpl.cuh"

namespace pawpy {
namespace reg {

// ---- compile-time cos / sin of 2 pi m / n (Taylor series on [0, pi/4])
constexpr double kTwoPi = 6.283185307179586476925286766559;

constexpr double sin_series(double x) {
  double x2 = x * x, t = x, s = x;
  for (int n = 1; n <= 11; n++) {
    t *= -x2 / ((2.0 * n) * (2.0 * n + 1.0));
    s += t;
  }
  return s;
}

constexpr double cos_series(double x) {
  double x2 = x * x, t = 1.0, s = 1.0;
  for (int n = 1; n <= 11; n++) {
    t *= -x2 / ((2.0 * n - 1.0) * (2.0 * n));
    s += t;
  }
  return s;
}

struct CS {
  double c, s;
};

constexpr CS cs2pi(long m, long n) {
  m %= n;
  if (m < 0) m += n;
  double sgn_s = 1.0, sgn_c = 1.0;
  if (2 * m > n) {  // theta in (pi, 2 pi): reflect through the x axis
    m = n - m;
    sgn_s = -1.0;
  }
  double th = kTwoPi * (double)m / (double)n;  // [0, pi]
  if (4 * m > n) {                              // (pi/2, pi]: reflect through the y axis
    th = kTwoPi / 2 - th;
    sgn_c = -1.0;
  }
  double c = 0, s = 0;
  if (8 * m > n && 8 * m < 3 * n) {  // (pi/4, 3pi/4) folded to (pi/4, pi/2]
    double u = kTwoPi / 4 - th;
    c = sin_series(u);
    s = cos_series(u);
  } else {
    c = cos_series(th);
    s = sin_series(th);
  }
  return CS{sgn_c * c, sgn_s * s};
}

// ---- compile-time loops
template <typename F, int... I>
__host__ __device__ __forceinline__ void sfor_impl(F &&f, std::integer_sequence<int, I...>) {
  (f(std::integral_constant<int, I>{}), ...);
}
template <int N, typename F>
__host__ __device__ __forceinline__ void sfor(F &&f) {
  sfor_impl(f, std::make_integer_sequence<int, N>{});
}

// x * exp(S 2 pi i M / L)
template <int L, int S, int M>
__host__ __device__ __forceinline__ float2 twiddle(float2 x) {
  constexpr int m = ((M % L) + L) % L;
  if constexpr (m == 0) {
    return x;
  } else if constexpr (4 * m == L) {
    return rot(x, (float)S);
  } else if constexpr (2 * m == L) {
    return make_float2(-x.x, -x.y);
  } else if constexpr (4 * m == 3 * L) {
    return rot(x, (float)-S);
  } else {
    constexpr CS w = cs2pi(m, L);
    constexpr float wr = (float)w.c, wi = (float)(S * w.s);
    return make_float2(x.x * wr - x.y * wi, x.x * wi + x.y * wr);
  }
}

constexpr int radix_of(int L) {
  if (L % 4 == 0 && L != 8) return 4;
  if (L % 2 == 0) return 2;
  if (L % 3 == 0) return 3;
  if (L % 5 == 0) return 5;
  return 0;
}

constexpr bool smooth235(int n) {
  if (n < 1) return false;
  while (n % 2 == 0) n /= 2;
  while (n % 3 == 0) n /= 3;
  while (n % 5 == 0) n /= 5;
  return n == 1;
}

// In-place DFT of a register array (natural order in and out).
template <int L, int S>
__host__ __device__ __forceinline__ void dft(float2 (&x)[L]) {
  static_assert(smooth235(L), "register DFT needs a 2,3,5-smooth length");
  if constexpr (L == 1) {
  } else if constexpr (L == 2 || L == 3 || L == 4 || L == 5) {
    float2 o[L];
    dft_t<L, L, S>(x, o, nullptr);
#pragma unroll
    for (int i = 0; i < L; i++) x[i] = o[i];
  } else {
    constexpr int R = radix_of(L), Q = L / R;
    float2 sub[R][Q];
#pragma unroll
    for (int r = 0; r < R; r++)
#pragma unroll
      for (int q = 0; q < Q; q++) sub[r][q] = x[r + R * q];
#pragma unroll
    for (int r = 0; r < R; r++) dft<Q, S>(sub[r]);
    sfor<Q>([&](auto kk) {
      constexpr int k = decltype(kk)::value;
      float2 v[R], o[R];
      sfor<R>([&](auto rr) {
        constexpr int r = decltype(rr)::value;
        v[r] = twiddle<L, S, r * k>(sub[r][k]);
      });
      dft_t<R, R, S>(v, o, nullptr);
#pragma unroll
      for (int s = 0; s < R; s++) x[k + Q * s] = o[s];
    });
  }
}

constexpr int bitrev(int h, int T) { return T == 4 ? (((h & 1) << 1) | (h >> 1)) : h; }

__device__ __forceinline__ float2 shfl_xor2(float2 v, int mask) {
  return make_float2(__shfl_xor_sync(0xffffffffu, v.x, mask), __shfl_xor_sync(0xffffffffu, v.y, mask));
}

// Whole-line transform: x holds x[h + T m] on entry, X[L bitrev(h) + k] on exit.
// All 32 lanes of the warp must call it together.
template <int N, int T, int S>
__device__ __forceinline__ void line_fft(float2 (&x)[N / T], int h) {
  constexpr int L = N / T;
  static_assert(N % T == 0 && (T == 1 || T == 2 || T == 4), "bad lane split");
  dft<L, S>(x);
  if constexpr (T == 2) {
    // X[k] = Y0[k] + w^k Y1[k], X[k + L] = Y0[k] - w^k Y1[k]
    sfor<L>([&](auto kk) {
      constexpr int k = decltype(kk)::value;
      float2 t = twiddle<N, S, k>(x[k]);
      float2 mine = h ? t : x[k];
      float2 oth = shfl_xor2(mine, 16);
      x[k] = h ? csub(oth, mine) : cadd(mine, oth);
    });
  } else if constexpr (T == 4) {
    // subsequences h and h + 2 first (length 2L), then the two halves (length N)
    sfor<L>([&](auto kk) {
      constexpr int k = decltype(kk)::value;
      float2 t = twiddle<2 * L, S, k>(x[k]);
      float2 mine = (h & 2) ? t : x[k];
      float2 oth = shfl_xor2(mine, 16);
      x[k] = (h & 2) ? csub(oth, mine) : cadd(mine, oth);
    });
    sfor<L>([&](auto kk) {
      constexpr int k = decltype(kk)::value;
      float2 t = (h & 2) ? twiddle<N, S, k + L>(x[k]) : twiddle<N, S, k>(x[k]);
      float2 mine = (h & 1) ? t : x[k];
      float2 oth = shfl_xor2(mine, 8);
      x[k] = (h & 1) ? csub(oth, mine) : cadd(mine, oth);
    });
  }
}

// Lanes per line for a length: the subsequence held by one lane stays short.
constexpr int lanes_for(int n) {
  if (n <= 32) return 1;
  if (n % 4 == 0 && n / 4 >= 12) return n / 2 <= 32 ? 2 : 4;
  if (n % 2 == 0) return 2;
  return 1;
}

}  // namespace reg
}  // namespace pawpy

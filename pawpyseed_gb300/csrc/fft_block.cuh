// Shared-memory mixed-radix FFT of many short lines, one CTA.
//
// Stockham autosort formulation: for a stage of radix R after span Ns,
// butterfly j (0 <= j < n/R) reads x[j + r*n/R], multiplies by
// w^(r * (j mod Ns) * n/(Ns R)), does an R-point DFT and writes
// y[(j/Ns)*Ns*R + (j mod Ns) + q*Ns]. After all stages the line is in natural
// order. Every thread of the block takes butterflies of every line in turn, so
// all lines of a plane advance one stage per __syncthreads().
// Sign +1 is the exp(+i) (backward) transform used by fft3d.
#pragma once

#include <cuda_runtime.h>

namespace pawpy {

struct Radices {
  int n;      // line length
  int ns;     // number of stages
  int r[12];  // radix of each stage (4 preferred, then 2,3,5,7,...)
};

__host__ __device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
// i*a for s=+1, -i*a for s=-1
__host__ __device__ __forceinline__ float2 rot(float2 a, float s) { return make_float2(-s * a.y, s * a.x); }

// y = DFT_R(v) with exp(s*2*pi*i*r*q/R); tw holds exp(+2 pi i m/n), n = line length
template <int S>
__device__ __forceinline__ void small_dft(int R, float2 *v, float2 *o, const float2 *tw, int n) {
  const float s = (float)S;
  if (R == 2) {
    o[0] = cadd(v[0], v[1]);
    o[1] = csub(v[0], v[1]);
  } else if (R == 4) {
    float2 a = cadd(v[0], v[2]), b = csub(v[0], v[2]);
    float2 c = cadd(v[1], v[3]), d = rot(csub(v[1], v[3]), s);
    o[0] = cadd(a, c);
    o[2] = csub(a, c);
    o[1] = cadd(b, d);
    o[3] = csub(b, d);
  } else if (R == 3) {
    const float h = 0.86602540378443864676f;  // sqrt(3)/2
    float2 t = cadd(v[1], v[2]);
    float2 m = make_float2(v[0].x - 0.5f * t.x, v[0].y - 0.5f * t.y);
    float2 d = rot(csub(v[1], v[2]), s);
    o[0] = cadd(v[0], t);
    o[1] = make_float2(m.x + h * d.x, m.y + h * d.y);
    o[2] = make_float2(m.x - h * d.x, m.y - h * d.y);
  } else if (R == 5) {
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
    int step = n / R;
    for (int q = 0; q < R; q++) {
      float2 acc = v[0];
      for (int r = 1; r < R; r++) {
        float2 w = tw[((r * q) % R) * step];
        if (S < 0) w.y = -w.y;
        acc = cadd(acc, cmul(v[r], w));
      }
      o[q] = acc;
    }
  }
}

// Transform `count` lines; element i of line c sits at base[c*ls + i*es].
// Ping-pongs between a and b; returns the buffer that holds the result.
// Requires every radix <= 16. Must be called by all threads of the block.
template <int S>
__device__ float2 *block_fft(float2 *a, float2 *b, const Radices &rx, int count, int ls, int es,
                             const float2 *tw) {
  const int n = rx.n;
  int span = 1;
  float2 *src = a, *dst = b;
  for (int st = 0; st < rx.ns; st++) {
    const int R = rx.r[st];
    const int m = n / R;
    const int tstep = n / (span * R);
    const int total = count * m;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
      int c = t / m, j = t - c * m;
      int k = j % span;
      const float2 *in = src + c * ls;
      float2 v[16], o[16];
      for (int r = 0; r < R; r++) {
        float2 x = in[(j + r * m) * es];
        if (r > 0 && k > 0) {
          float2 w = tw[(k * r * tstep) % n];
          if (S < 0) w.y = -w.y;
          x = cmul(x, w);
        }
        v[r] = x;
      }
      small_dft<S>(R, v, o, tw, n);
      int base = (j / span) * span * R + k;
      float2 *out = dst + c * ls;
      for (int q = 0; q < R; q++) out[(base + q * span) * es] = o[q];
    }
    __syncthreads();
    float2 *tmp = src;
    src = dst;
    dst = tmp;
    span *= R;
  }
  return src;
}

// Host: factor n into radix-4 stages first, then the remaining primes.
inline Radices make_radices(int n) {
  Radices rx{};
  rx.n = n;
  int m = n;
  while (m % 4 == 0 && rx.ns < 12) {
    rx.r[rx.ns++] = 4;
    m /= 4;
  }
  for (int q = 2; m > 1 && rx.ns < 12; q++)
    while (m % q == 0 && rx.ns < 12) {
      rx.r[rx.ns++] = q;
      m /= q;
    }
  if (m != 1) rx.ns = -1;
  for (int i = 0; i < rx.ns; i++)
    if (rx.r[i] > 16) rx.ns = -1;
  return rx;
}

}  // namespace pawpy

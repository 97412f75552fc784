// The two passes of the band FFT (fft3d, linalg.c:14-45, batched over bands)
// with register-resident line transforms (fft_reg.cuh) for grid lengths known
// at compile time; other lengths use the shared-memory kernels of kernels.cu
// and sphere.cu.
//
// Pass A: a CTA owns one plane g1 and loops over bands; per band it scatters
// the plane's coefficients into a padded shared tile, transforms the occupied
// rows along the third axis, then every column along the second axis straight
// from registers to H. Pass B: a CTA owns one plane of the second axis and
// loops over bands; per band it transforms the first axis from H into a
// shared tile and picks the sphere points of the plane (value times Bloch
// phase) into X. Both prefetch the next band's input with cp.async while the
// current one is transformed. Rows and columns outside the plane-wave sphere
// are known to be zero and are neither read nor written. The number of band
// groups (CTAs per plane) is chosen per grid by timing the candidates on the
// first batch (the results do not depend on it).
#pragma once

#include "bf16split.cuh"

#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "fft_reg.cuh"
#include "kernels.h"

namespace pawpy {

namespace {

constexpr int FT = 128;  // threads per CTA

__host__ __device__ constexpr int padded(int n) { return n + 1 + (n & 1); }

// index in [0, N) of the occupied range {(s + i) mod N, i < n}?
__device__ __forceinline__ bool occupied(int idx, int s, int n, int N) {
  int d = idx - s;
  d += d < 0 ? N : 0;
  return d < n;
}

// one lane per line while the line's registers stay moderate
constexpr int direct_lanes(int n) { return n <= 64 ? 1 : reg::lanes_for(n); }

__device__ __forceinline__ int wrapi(int v, int N) {
  v %= N;
  return v < 0 ? v + N : v;
}

}  // namespace

__device__ __forceinline__ void cp_async8(void *dst, const void *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(static_cast<uint32_t>(__cvta_generic_to_shared(dst))),
               "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Pass A. grid (n1 planes, G band groups), FT threads: CTA (p, g) transforms
// plane p of bands g, g + G, ... of the batch. Shared memory: ta [n2][LD] holds
// the plane's coefficients on the occupied rows (its other cells are zeroed
// once: the coefficient positions of a plane are the same for every band), tb
// [n2][LD] the rows after the third-axis transform, stage [2][maxcnt] the
// coefficients of the current and the next band (cp.async), pos [maxcnt] the
// cell of each coefficient.
template <int N2, int N3>
__global__ void __launch_bounds__(FT) k_planes_pipe(const float2 *__restrict__ C, int Wpad, int nb,
                                                    const int *__restrict__ pstart, const int *__restrict__ poff,
                                                    PlaneGeom g, float2 *__restrict__ H) {
  constexpr int LD = padded(N3);
  constexpr int T3 = reg::lanes_for(N3), L3 = N3 / T3;
  constexpr int T2 = reg::lanes_for(N2), L2 = N2 / T2;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int n2 = g.n2, maxcnt = g.maxcnt;
  float2 *ta = reinterpret_cast<float2 *>(smraw);
  float2 *tb = ta + n2 * LD;
  float2 *stage = tb + n2 * LD;
  int *pos = reinterpret_cast<int *>(stage + 2 * maxcnt);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const int p = blockIdx.x, G = gridDim.y;
  const int t0 = pstart[p], cnt = pstart[p + 1] - t0;
  const int s2 = wrapi(g.g2min, N2), s3 = wrapi(g.g3min, N3);
  for (int e = threadIdx.x; e < n2 * LD; e += blockDim.x) ta[e] = make_float2(0.f, 0.f);
  for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
    const int o = poff[t0 + t], row = o / N3, col = o - row * N3;
    int i = row - s2;
    i += i < 0 ? N2 : 0;
    pos[t] = i * LD + col;
  }
  auto prefetch = [&](int b, int buf) {
    const float2 *src = C + (long long)b * Wpad + t0;
    float2 *dst = stage + buf * maxcnt;
    for (int t = threadIdx.x; t < cnt; t += blockDim.x) cp_async8(dst + t, src + t);
    cp_async_commit();
  };
  int b = blockIdx.y;
  if (b < nb) prefetch(b, 0);
  for (int it = 0; b < nb; it++, b += G) {
    if (b + G < nb) {
      prefetch(b + G, (it + 1) & 1);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();  // this band's coefficients landed; the previous band is done with ta and tb
    const float2 *sv = stage + (it & 1) * maxcnt;
    for (int t = threadIdx.x; t < cnt; t += blockDim.x) ta[pos[t]] = sv[t];
    __syncthreads();
    {  // third axis, occupied rows
      constexpr int LPW = 32 / T3;
      const int h = lane / LPW, c = lane % LPW;
      for (int g0 = warp * LPW; g0 < n2; g0 += nw * LPW) {
        const int i = g0 + c;
        const bool ok = i < n2;
        const float2 *rp = ta + (ok ? i : 0) * LD;
        float2 x[L3];
#pragma unroll
        for (int m = 0; m < L3; m++) {
          const int col = h + T3 * m;
          x[m] = ok && occupied(col, s3, g.n3, N3) ? rp[col] : make_float2(0.f, 0.f);
        }
        reg::line_fft<N3, T3, 1>(x, h);
        if (ok) {
          float2 *wp = tb + i * LD + L3 * reg::bitrev(h, T3);
#pragma unroll
          for (int k = 0; k < L3; k++) wp[k] = x[k];
        }
      }
    }
    __syncthreads();
    {  // second axis, every column, to H
      constexpr int LPW = 32 / T2;
      const int h = lane / LPW, c = lane % LPW;
      float2 *out = H + ((long long)b * g.n1 + p) * (N2 * N3);
      for (int g0 = warp * LPW; g0 < N3; g0 += nw * LPW) {
        const int col = g0 + c;
        const bool ok = col < N3;
        float2 x[L2];
#pragma unroll
        for (int m = 0; m < L2; m++) {
          int i = h + T2 * m - s2;
          i += i < 0 ? N2 : 0;
          x[m] = ok && i < n2 ? tb[i * LD + col] : make_float2(0.f, 0.f);
        }
        reg::line_fft<N2, T2, 1>(x, h);
        if (ok) {
          const int o = L2 * reg::bitrev(h, T2);
#pragma unroll
          for (int k = 0; k < L2; k++) out[(o + k) * N3 + col] = x[k];
        }
      }
    }
  }
}

// Pass A without the band loop, for occupancy: grid (n1 planes, ceil(nb /
// BPC) band groups), FT threads split into BPC groups of TPB threads, one band
// each. A group zeroes the occupied cells of its tile [n2][LD], scatters the
// plane's coefficients, transforms the occupied rows in place (a lane owns a
// whole row when T3 = 1, otherwise through a second tile) and then every
// column straight to H.
template <int N2, int N3, int T2, int T3>
__global__ void __launch_bounds__(FT) k_planes_direct(const float2 *__restrict__ C, int Wpad, int nb,
                                                      const int *__restrict__ pstart, const int *__restrict__ poff,
                                                      PlaneGeom g, float2 *__restrict__ H) {
  constexpr int LD = padded(N3), L2 = N2 / T2, L3 = N3 / T3;
  constexpr int NEED = (N2 * T3 > N3 * T2 ? N2 * T3 : N3 * T2);
  constexpr int TPB = 32 * ((NEED + 31) / 32) < FT ? 32 * ((NEED + 31) / 32) : FT;
  constexpr int BPC = FT / TPB;
  constexpr bool INPLACE = T3 == 1;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int n2 = g.n2;
  const int grp = threadIdx.x / TPB, gt = threadIdx.x - grp * TPB;
  float2 *ta = reinterpret_cast<float2 *>(smraw) + grp * (INPLACE ? 1 : 2) * n2 * LD;
  float2 *tb = INPLACE ? ta : ta + n2 * LD;
  const int warp = gt >> 5, lane = threadIdx.x & 31, nwg = TPB / 32;
  const int p = blockIdx.x, b = blockIdx.y * BPC + grp;
  const bool band_ok = grp < BPC && b < nb;
  const int s2 = wrapi(g.g2min, N2), s3 = wrapi(g.g3min, N3);
  const int t0 = pstart[p], cnt = pstart[p + 1] - t0;
  if (band_ok) {
    const int occ = n2 * g.n3;
    for (int e = gt; e < occ; e += TPB) {
      const int i = e / g.n3, c = e - i * g.n3;
      ta[i * LD + (s3 + c >= N3 ? s3 + c - N3 : s3 + c)] = make_float2(0.f, 0.f);
    }
  }
  __syncthreads();
  if (band_ok) {
    const float2 *cb = C + (long long)b * Wpad + t0;
    for (int t = gt; t < cnt; t += TPB) {
      const int o = poff[t0 + t], row = o / N3, col = o - row * N3;
      int i = row - s2;
      i += i < 0 ? N2 : 0;
      ta[i * LD + col] = cb[t];
    }
  }
  __syncthreads();
  if (band_ok) {  // third axis, occupied rows
    constexpr int LPW = 32 / T3;
    const int h = lane / LPW, c = lane % LPW;
    for (int g0 = warp * LPW; g0 < n2; g0 += nwg * LPW) {
      const int i = g0 + c;
      const bool ok = i < n2;
      const float2 *rp = ta + (ok ? i : 0) * LD;
      float2 x[L3];
#pragma unroll
      for (int m = 0; m < L3; m++) {
        const int col = h + T3 * m;
        x[m] = ok && occupied(col, s3, g.n3, N3) ? rp[col] : make_float2(0.f, 0.f);
      }
      reg::line_fft<N3, T3, 1>(x, h);
      if (ok) {
        float2 *wp = tb + i * LD + L3 * reg::bitrev(h, T3);
#pragma unroll
        for (int k = 0; k < L3; k++) wp[k] = x[k];
      }
    }
  }
  __syncthreads();
  if (band_ok) {  // second axis, every column, to H
    constexpr int LPW = 32 / T2;
    const int h = lane / LPW, c = lane % LPW;
    float2 *out = H + ((long long)b * g.n1 + p) * (N2 * N3);
    for (int g0 = warp * LPW; g0 < N3; g0 += nwg * LPW) {
      const int col = g0 + c;
      const bool ok = col < N3;
      float2 x[L2];
#pragma unroll
      for (int m = 0; m < L2; m++) {
        int i = h + T2 * m - s2;
        i += i < 0 ? N2 : 0;
        x[m] = ok && i < n2 ? tb[i * LD + col] : make_float2(0.f, 0.f);
      }
      reg::line_fft<N2, T2, 1>(x, h);
      if (ok) {
        const int o = L2 * reg::bitrev(h, T2);
#pragma unroll
        for (int k = 0; k < L2; k++) out[(o + k) * N3 + col] = x[k];
      }
    }
  }
}

// Pass B. grid (N2 planes j, G band groups), FT threads: CTA (j, g) transforms
// the first axis of plane j of bands g, g + G, ... and picks its sphere
// points. The pick list of plane j is points [plane_first[j],
// plane_first[j + 1]) of cell (i N3 + k within the plane), xo (position in X)
// and phase (Bloch phase at this k-point). Shared memory: stage [2][n1][N3]
// the plane's H rows of the current and the next band (cp.async), tile
// [N1][LD] the transformed plane and, when the plane has at most pts_cap
// points, a copy of its pick list (the same for every band).
// The pick of one plane from a tile of transformed values: the value at tile offset e.x
// (row * LD + column of the plane) times the point's Bloch phase (phase == nullptr: the k-point
// is Gamma, the phase is 1), to offset e.y of the band's picked row Xrow: complex64 values
// (lo_words == 0), or BF16 (re, im) words of the split form, the lo word lo_words after the hi
// word (the entries carry the K-block offsets, bf16split.cuh). The entries are read from global
// memory (L2) U at a time per thread, all loads in flight before the stores.
template <int U>
__device__ __forceinline__ void pick_plane(const float2 *tile, const uint2 *__restrict__ ent,
                                           const float2 *__restrict__ phase, int npj, int t0, int nt, void *Xrow,
                                           long long lo_words) {
  for (int q0 = t0; q0 < npj; q0 += nt * U) {
    uint2 e[U];
    float2 f[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int q = q0 + u * nt;
      if (q < npj) {
        e[u] = __ldg(ent + q);
        if (phase) f[u] = __ldg(phase + q);
      }
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int q = q0 + u * nt;
      if (q < npj) {
        const float2 v = phase ? cmul(tile[e[u].x], f[u]) : tile[e[u].x];
        if (lo_words) {
          uint32_t h, l;
          split_bf16x2(v, h, l);
          uint32_t *w = static_cast<uint32_t *>(Xrow) + e[u].y;
          w[0] = h;
          w[lo_words] = l;
        } else {
          static_cast<float2 *>(Xrow)[e[u].y] = v;
        }
      }
    }
  }
}

// The same from a tile held already split (thi, tlo: the hi and lo words of the transformed
// values; Gamma point, split rows): two words copied per point.
template <int U>
__device__ __forceinline__ void pick_plane_split(const uint32_t *thi, const uint32_t *tlo, const uint2 *__restrict__ ent,
                                                 int npj, int t0, int nt, uint32_t *Xrow, long long lo_words) {
  for (int q0 = t0; q0 < npj; q0 += nt * U) {
    uint2 e[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int q = q0 + u * nt;
      if (q < npj) e[u] = __ldg(ent + q);
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int q = q0 + u * nt;
      if (q < npj) {
        uint32_t *w = Xrow + e[u].y;
        w[0] = thi[e[u].x];
        w[lo_words] = tlo[e[u].x];
      }
    }
  }
}

// the band's picked row: 16 words per row within a K block (split form), xstride values otherwise
__device__ __forceinline__ void *picked_row(float2 *X, long long b, long long xstride, long long lo_words) {
  return lo_words ? static_cast<void *>(reinterpret_cast<uint32_t *>(X) + b * 16)
                  : static_cast<void *>(X + b * xstride);
}

template <int N1, int N3>
__global__ void __launch_bounds__(FT) k_xpick_pipe(const float2 *__restrict__ H, int nb, PlaneGeom g,
                                                   const int *__restrict__ plane_first,
                                                   const uint2 *__restrict__ ent,
                                                   const float2 *__restrict__ phase, int pts_cap,
                                                   float2 *__restrict__ X, long long xstride, long long lo_words) {
  constexpr int LD = padded(N3);
  constexpr int T1 = reg::lanes_for(N1), L1 = N1 / T1;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int n1 = g.n1, per = n1 * N3;
  float2 *stage = reinterpret_cast<float2 *>(smraw);
  float2 *tile = stage + 2 * per;
  float2 *pph = tile + N1 * LD;
  uint2 *pent = reinterpret_cast<uint2 *>(pph + pts_cap);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const int j = blockIdx.x, G = gridDim.y;
  const int s1 = wrapi(g.g1min, N1);
  const long long pstride = (long long)g.N2 * N3;
  auto prefetch = [&](int b, int buf) {
    const float2 *src = H + ((long long)b * n1 * g.N2 + j) * N3;
    float2 *dst = stage + buf * per;
    for (int e = threadIdx.x; e < per; e += blockDim.x) {
      const int p = e / N3, z = e - p * N3;
      cp_async8(dst + e, src + p * pstride + z);
    }
    cp_async_commit();
  };
  const int pf = plane_first[j], npj = plane_first[j + 1] - pf;
  const bool staged = npj <= pts_cap;
  int b = blockIdx.y;
  if (b < nb) prefetch(b, 0);
  if (staged)
    for (int q = threadIdx.x; q < npj; q += blockDim.x) {
      pent[q] = ent[pf + q];
      pph[q] = phase ? phase[pf + q] : make_float2(1.f, 0.f);
    }
  for (int it = 0; b < nb; it++, b += G) {
    if (b + G < nb) {
      prefetch(b + G, (it + 1) & 1);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();  // this band's rows landed; the previous band's pick is done with the tile
    {
      constexpr int LPW = 32 / T1;
      const int h = lane / LPW, c = lane % LPW;
      const float2 *sv = stage + (it & 1) * per;
      for (int g0 = warp * LPW; g0 < N3; g0 += nw * LPW) {
        const int z = g0 + c;
        const bool ok = z < N3;
        float2 x[L1];
#pragma unroll
        for (int m = 0; m < L1; m++) {
          int pp = h + T1 * m - s1;
          pp += pp < 0 ? N1 : 0;
          x[m] = ok && pp < n1 ? sv[pp * N3 + z] : make_float2(0.f, 0.f);
        }
        reg::line_fft<N1, T1, 1>(x, h);
        if (ok) {
          float2 *tp = tile + (L1 * reg::bitrev(h, T1)) * LD + z;
#pragma unroll
          for (int k = 0; k < L1; k++) tp[k * LD] = x[k];
        }
      }
    }
    __syncthreads();
    void *xr = picked_row(X, b, xstride, lo_words);
    if (staged) {
      for (int q = threadIdx.x; q < npj; q += blockDim.x) {
        const float2 v = cmul(tile[pent[q].x], pph[q]);
        if (lo_words) {
          uint32_t h, l;
          split_bf16x2(v, h, l);
          uint32_t *w = static_cast<uint32_t *>(xr) + pent[q].y;
          w[0] = h;
          w[lo_words] = l;
        } else {
          static_cast<float2 *>(xr)[pent[q].y] = v;
        }
      }
    } else {
      pick_plane<8>(tile, ent + pf, phase ? phase + pf : nullptr, npj, threadIdx.x, blockDim.x, xr, lo_words);
    }
  }
}

// Pass B without staging, for occupancy: grid (ceil(nb / BPC) band groups,
// N2 planes j), FT threads split into BPC groups of TPB = 32 ceil(N3 T1 / 32)
// threads, one band each; a group loads plane j of its band from H straight
// into registers (all loads of a lane in flight at once), transforms the
// first axis into its shared tile [N1][LD] and picks from the flat list
// through L1 (consecutive CTAs share a plane). STILE (Gamma point, split rows):
// the transform's outputs are split into BF16 hi and lo words as they enter the
// tile (two planes of [N1][LD] words, the same bytes), once per grid point
// instead of once per picked point, and the pick copies words.
// (three CTAs per SM: the 90^3 tile allows three in shared memory, and the register cap that
// gives them costs a few spilled values of the line transform)
template <int N1, int N3, int T1, bool STILE>
__global__ void __launch_bounds__(FT, 3) k_xpick_direct(const float2 *__restrict__ H, int nb, PlaneGeom g,
                                                     const int *__restrict__ plane_first,
                                                     const uint2 *__restrict__ ent,
                                                     const float2 *__restrict__ phase, float2 *__restrict__ X,
                                                     long long xstride, long long lo_words) {
  constexpr int LD = padded(N3), L1 = N1 / T1;
  constexpr int TPB = 32 * ((N3 * T1 + 31) / 32) < FT ? 32 * ((N3 * T1 + 31) / 32) : FT;  // threads per band
  constexpr int BPC = FT / TPB;
  constexpr int LPW = 32 / T1;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int grp = threadIdx.x / TPB, gt = threadIdx.x - grp * TPB;
  float2 *tile = reinterpret_cast<float2 *>(smraw) + grp * (N1 * LD);
  uint32_t *thi = reinterpret_cast<uint32_t *>(tile), *tlo = thi + N1 * LD;
  const int warp = gt >> 5, lane = threadIdx.x & 31;
  const int b = blockIdx.x * BPC + grp, j = blockIdx.y;
  const int n1 = g.n1, s1 = wrapi(g.g1min, N1);
  const int pstride = g.N2 * N3;  // n1 * N2 * N3 < 2^31
  const bool band_ok = grp < BPC && b < nb;
  if (band_ok) {
    const int h = lane / LPW, c = lane % LPW;
    const float2 *hb = H + ((long long)b * n1 * g.N2 + j) * N3;
    for (int g0 = warp * LPW; g0 < N3; g0 += (TPB / 32) * LPW) {
      const int z = g0 + c;
      const bool ok = z < N3;
      float2 x[L1];
#pragma unroll
      for (int m = 0; m < L1; m++) {
        int pp = h + T1 * m - s1;
        pp += pp < 0 ? N1 : 0;
        x[m] = ok && pp < n1 ? hb[pp * pstride + z] : make_float2(0.f, 0.f);
      }
      reg::line_fft<N1, T1, 1>(x, h);
      if (ok) {
        const int t0 = (L1 * reg::bitrev(h, T1)) * LD + z;
        if constexpr (STILE) {
#pragma unroll
          for (int k = 0; k < L1; k++) split_bf16x2(x[k], thi[t0 + k * LD], tlo[t0 + k * LD]);
        } else {
#pragma unroll
          for (int k = 0; k < L1; k++) tile[t0 + k * LD] = x[k];
        }
      }
    }
  }
  __syncthreads();
  if (!band_ok) return;
  const int pf = plane_first[j], npj = plane_first[j + 1] - pf;
  if constexpr (STILE)
    pick_plane_split<16>(thi, tlo, ent + pf, npj, gt, TPB, reinterpret_cast<uint32_t *>(X) + (long long)b * 16,
                         lo_words);
  else
    pick_plane<16>(tile, ent + pf, phase ? phase + pf : nullptr, npj, gt, TPB, picked_row(X, b, xstride, lo_words),
                   lo_words);
}

// Pass B writing whole grids (resident real-space wavefunctions): grid
// (ceil(nb / BPC) band groups, N2 planes j), FT threads in BPC groups of TPB,
// one band each; the first-axis transform of plane j goes straight from
// registers to the grid of band bb = b0 + b in tiles of 16 bands:
// grid[((bb / 16) N1 N2 N3 + (x N2 + j) N3 + z) 16 + bb % 16] (grid_value_index).
template <int N1, int N3, int T1>
__global__ void __launch_bounds__(FT) k_xgrid(const float2 *__restrict__ H, int nb, PlaneGeom g,
                                              float2 *__restrict__ grid, int b0) {
  constexpr int L1 = N1 / T1;
  constexpr int TPB = 32 * ((N3 * T1 + 31) / 32) < FT ? 32 * ((N3 * T1 + 31) / 32) : FT;
  constexpr int BPC = FT / TPB;
  constexpr int LPW = 32 / T1;
  const int grp = threadIdx.x / TPB, gt = threadIdx.x - grp * TPB;
  const int warp = gt >> 5, lane = threadIdx.x & 31;
  const int b = blockIdx.x * BPC + grp, j = blockIdx.y;
  if (grp >= BPC || b >= nb) return;
  const int n1 = g.n1, s1 = wrapi(g.g1min, N1);
  const int pstride = g.N2 * N3;
  const int h = lane / LPW, c = lane % LPW;
  const float2 *hb = H + ((long long)b * n1 * g.N2 + j) * N3;
  const int bb = b0 + b;
  float2 *gb = grid + ((long long)(bb >> 4) * N1 * g.N2 * N3 + (long long)j * N3) * 16 + (bb & 15);
  for (int g0 = warp * LPW; g0 < N3; g0 += (TPB / 32) * LPW) {
    const int z = g0 + c;
    const bool ok = z < N3;
    float2 x[L1];
#pragma unroll
    for (int m = 0; m < L1; m++) {
      int pp = h + T1 * m - s1;
      pp += pp < 0 ? N1 : 0;
      x[m] = ok && pp < n1 ? hb[pp * pstride + z] : make_float2(0.f, 0.f);
    }
    reg::line_fft<N1, T1, 1>(x, h);
    if (ok) {
      const int o = L1 * reg::bitrev(h, T1);
#pragma unroll
      for (int k = 0; k < L1; k++) gb[((long long)(o + k) * pstride + z) * 16] = x[k];
    }
  }
}

constexpr int direct_bands(int n1, int n3) {
  return 32 * ((n3 * direct_lanes(n1) + 31) / 32) < FT ? FT / (32 * ((n3 * direct_lanes(n1) + 31) / 32)) : 1;
}
constexpr int planes_direct_bands(int n2, int n3) {
  return 32 * (((n2 * direct_lanes(n3) > n3 * direct_lanes(n2) ? n2 * direct_lanes(n3) : n3 * direct_lanes(n2)) + 31) /
               32) < FT
             ? FT / (32 * (((n2 * direct_lanes(n3) > n3 * direct_lanes(n2) ? n2 * direct_lanes(n3)
                                                                            : n3 * direct_lanes(n2)) +
                           31) /
                          32))
             : 1;
}

// ------------------------------------------------------------------ host helpers

namespace fftfast {

constexpr size_t kSmemCap = 200 * 1024;

inline size_t planes_smem(const PlaneGeom &g) {
  return sizeof(float2) * (2 * (size_t)g.n2 * padded(g.N3) + 2 * (size_t)g.maxcnt) + sizeof(int) * (size_t)g.maxcnt;
}
inline size_t planes_direct_smem(const PlaneGeom &g, int bpc, bool inplace) {
  return sizeof(float2) * (size_t)bpc * (inplace ? 1 : 2) * g.n2 * padded(g.N3);
}
inline size_t xpick_direct_smem(const PlaneGeom &g, int bpc) {
  return sizeof(float2) * (size_t)bpc * g.N1 * padded(g.N3);
}
inline size_t xpick_smem(const PlaneGeom &g, int pts_cap = 0) {
  return sizeof(float2) * (2 * (size_t)g.n1 * g.N3 + (size_t)g.N1 * padded(g.N3)) + 16 * (size_t)pts_cap;
}

// guards the attribute and tuning caches (host threads may launch concurrently)
inline std::mutex &cache_mutex() {
  static std::mutex m;
  return m;
}

inline void allow_smem(const void *fn, size_t bytes) {
  static std::map<const void *, size_t> done;
  std::lock_guard<std::mutex> lk(cache_mutex());
  auto &d = done[fn];
  if (bytes > 48 * 1024 && bytes > d) {
    PAWPY_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    d = bytes;
  }
}

// CTAs of fn resident on the whole device at once (FT threads, smem bytes)
inline int resident_ctas(const void *fn, size_t smem) {
  int per_sm = 0, nsm = 0;
  PAWPY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, FT, smem));
  PAWPY_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device()));
  return std::max(1, per_sm) * nsm;
}

// tuned choices per (pass, N1, N2, N3)
inline std::map<std::tuple<int, int, int, int>, int> &tuned() {
  static std::map<std::tuple<int, int, int, int>, int> t;
  return t;
}

inline std::mutex &tune_mutex() {
  static std::mutex m;
  return m;
}

// The choice for a key is made once per process (concurrent first callers wait
// for it), so results never depend on which thread tuned.
template <typename Launch>
inline int tune(const std::tuple<int, int, int, int> &key, const std::vector<int> &cands, Launch launch) {
  {
    std::lock_guard<std::mutex> lk(cache_mutex());
    auto it = tuned().find(key);
    if (it != tuned().end()) return it->second;
  }
  std::lock_guard<std::mutex> tlk(tune_mutex());
  {
    std::lock_guard<std::mutex> lk(cache_mutex());
    auto it = tuned().find(key);
    if (it != tuned().end()) return it->second;
  }
  std::vector<cudaEvent_t> ev(cands.size() + 1);
  for (auto &e : ev) PAWPY_CUDA(cudaEventCreate(&e));
  PAWPY_CUDA(cudaEventRecord(ev[0], stream()));
  for (size_t i = 0; i < cands.size(); i++) {
    launch(cands[i]);
    PAWPY_CUDA(cudaEventRecord(ev[i + 1], stream()));
  }
  PAWPY_CUDA(cudaEventSynchronize(ev.back()));
  int best = cands[0];
  float bms = 1e30f;
  for (size_t i = 0; i < cands.size(); i++) {
    float ms = 0;
    PAWPY_CUDA(cudaEventElapsedTime(&ms, ev[i], ev[i + 1]));
    if (ms < bms) {
      bms = ms;
      best = cands[i];
    }
  }
  {
    std::lock_guard<std::mutex> lk(cache_mutex());
    tuned()[key] = best;
  }
  if (getenv("PAWPY_GPU_TUNE_VERBOSE")) {
    fprintf(stderr, "pawpy tune pass %d grid %dx%dx%d:", std::get<0>(key), std::get<1>(key), std::get<2>(key),
            std::get<3>(key));
    for (size_t i = 0; i < cands.size(); i++) {
      float ms = 0;
      cudaEventElapsedTime(&ms, ev[i], ev[i + 1]);
      fprintf(stderr, " %d:%.4f", cands[i], ms);
    }
    fprintf(stderr, " -> %d\n", best);
  }
  for (auto &e : ev) cudaEventDestroy(e);
  return best;
}

}  // namespace fftfast

// (second, third) lengths of pass A and (first, third) lengths of pass B with
// compiled kernels
#define PAWPY_FFT_PAIRS(X) \
  X(24, 24)                \
  X(36, 36)                \
  X(45, 45)                \
  X(48, 48)                \
  X(50, 50)                \
  X(60, 60)                \
  X(64, 64)                \
  X(72, 72)                \
  X(80, 80)                \
  X(90, 90)                \
  X(96, 96)                \
  X(45, 50)                \
  X(36, 50)

}  // namespace pawpy

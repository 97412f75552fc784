// The two passes of the band FFT (fft3d, linalg.c:14-45, batched over bands)
// with register-resident line transforms (fft_reg.cuh) for grid lengths known
// at compile time; other lengths use the shared-memory kernels of kernels.cu
// and sphere.cu.
//
// Pass A, per (band, PP planes g1): scatter the plane's coefficients into a
// padded shared tile, transform the occupied rows along the third axis, then
// every column along the second axis straight from registers to H.
// Pass B, per (band, JJ planes of the second axis): transform every line along
// the first axis straight from H into a shared tile, then pick the sphere
// points of those planes (value times Bloch phase) into X.
// Rows and columns outside the plane-wave sphere are known to be zero and are
// neither read nor written. PP and JJ are chosen per grid by timing every
// candidate on the first batch (the results do not depend on them).
#pragma once

#include <map>
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

__device__ __forceinline__ int wrapi(int v, int N) {
  v %= N;
  return v < 0 ? v + N : v;
}

}  // namespace

template <int N2, int N3, int PP>
__global__ void __launch_bounds__(FT) k_planes_reg(const float2 *__restrict__ C, int Wpad,
                                                   const int *__restrict__ pstart, const int *__restrict__ poff,
                                                   PlaneGeom g, float2 *__restrict__ H) {
  constexpr int LD = padded(N3);
  constexpr int T3 = reg::lanes_for(N3), L3 = N3 / T3;
  constexpr int T2 = reg::lanes_for(N2), L2 = N2 / T2;
  extern __shared__ float2 tile[];  // [PP][N2][LD]
  const int band = blockIdx.y, p0 = blockIdx.x * PP;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const int np = min(PP, g.n1 - p0);
  const int s2 = wrapi(g.g2min, N2), s3 = wrapi(g.g3min, N3);
  const int occ = g.n2 * g.n3;
  for (int e = threadIdx.x; e < np * occ; e += blockDim.x) {
    const int pl = e / occ, r = e - pl * occ, i = r / g.n3, c = r - i * g.n3;
    const int row = s2 + i >= N2 ? s2 + i - N2 : s2 + i, col = s3 + c >= N3 ? s3 + c - N3 : s3 + c;
    tile[(pl * N2 + row) * LD + col] = make_float2(0.f, 0.f);
  }
  __syncthreads();
  const float2 *cb = C + (long long)band * Wpad;
  for (int pl = 0; pl < np; pl++)
    for (int t = pstart[p0 + pl] + threadIdx.x; t < pstart[p0 + pl + 1]; t += blockDim.x) {
      const int o = poff[t], row = o / N3, col = o - row * N3;
      tile[(pl * N2 + row) * LD + col] = cb[t];
    }
  __syncthreads();
  {  // third axis, occupied rows only
    constexpr int LPW = 32 / T3;
    const int h = lane / LPW, c = lane % LPW;
    const int nlines = np * g.n2;
    for (int g0 = warp * LPW; g0 < nlines; g0 += nw * LPW) {
      const int line = g0 + c;
      const bool ok = line < nlines;
      const int pl = ok ? line / g.n2 : 0, i = ok ? line - pl * g.n2 : 0;
      const int row = s2 + i >= N2 ? s2 + i - N2 : s2 + i;
      float2 *rp = tile + (pl * N2 + row) * LD;
      float2 x[L3];
#pragma unroll
      for (int m = 0; m < L3; m++) {
        const int col = h + T3 * m;
        x[m] = ok && occupied(col, s3, g.n3, N3) ? rp[col] : make_float2(0.f, 0.f);
      }
      reg::line_fft<N3, T3, 1>(x, h);
      if (ok) {
        const int o = L3 * reg::bitrev(h, T3);
#pragma unroll
        for (int k = 0; k < L3; k++) rp[o + k] = x[k];
      }
    }
  }
  __syncthreads();
  {  // second axis, every column, to H
    constexpr int LPW = 32 / T2;
    const int h = lane / LPW, c = lane % LPW;
    const int nlines = np * N3;
    for (int g0 = warp * LPW; g0 < nlines; g0 += nw * LPW) {
      const int line = g0 + c;
      const bool ok = line < nlines;
      const int pl = ok ? line / N3 : 0, col = ok ? line - pl * N3 : 0;
      const float2 *cp = tile + pl * N2 * LD + col;
      float2 x[L2];
#pragma unroll
      for (int m = 0; m < L2; m++) {
        const int row = h + T2 * m;
        x[m] = ok && occupied(row, s2, g.n2, N2) ? cp[row * LD] : make_float2(0.f, 0.f);
      }
      reg::line_fft<N2, T2, 1>(x, h);
      if (ok) {
        float2 *out = H + ((long long)band * g.n1 + p0 + pl) * (N2 * N3) + col;
        const int o = L2 * reg::bitrev(h, T2);
#pragma unroll
        for (int k = 0; k < L2; k++) out[(o + k) * N3] = x[k];
      }
    }
  }
}

template <int N1, int N3, int JJ>
__global__ void __launch_bounds__(FT) k_xpick_reg(const float2 *__restrict__ H, PlaneGeom g,
                                                  const GatherSeg *__restrict__ segs,
                                                  const int *__restrict__ plane_start, int kq,
                                                  float2 *__restrict__ X, long long xstride) {
  constexpr int LD = padded(N3);
  constexpr int T1 = reg::lanes_for(N1), L1 = N1 / T1;
  extern __shared__ float2 tile[];  // [JJ][N1][LD]
  const int band = blockIdx.y, j0 = blockIdx.x * JJ;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const int nj = min(JJ, g.N2 - j0);
  const int s1 = wrapi(g.g1min, N1);
  {
    constexpr int LPW = 32 / T1;
    const int h = lane / LPW, c = lane % LPW;
    const int nlines = nj * N3;
    for (int g0 = warp * LPW; g0 < nlines; g0 += nw * LPW) {
      const int line = g0 + c;
      const bool ok = line < nlines;
      const int jl = ok ? line / N3 : 0, z = ok ? line - jl * N3 : 0;
      const float2 *hp = H + ((long long)band * g.n1 * g.N2 + j0 + jl) * N3 + z;
      const int pstride = g.N2 * N3;  // n1 * N2 * N3 < 2^31
      float2 x[L1];
#pragma unroll
      for (int m = 0; m < L1; m++) {
        int p = h + T1 * m - s1;
        p += p < 0 ? N1 : 0;
        x[m] = ok && p < g.n1 ? hp[p * pstride] : make_float2(0.f, 0.f);
      }
      reg::line_fft<N1, T1, 1>(x, h);
      if (ok) {
        float2 *tp = tile + (jl * N1 + L1 * reg::bitrev(h, T1)) * LD + z;
#pragma unroll
        for (int k = 0; k < L1; k++) tp[k * LD] = x[k];
      }
    }
  }
  __syncthreads();
  float2 *xb = X + (long long)band * xstride;
  for (int jl = 0; jl < nj; jl++) {
    const int j = j0 + jl;
    const float2 *tp = tile + jl * N1 * LD;
    for (int si = plane_start[j] + warp; si < plane_start[j + 1]; si += nw) {
      const GatherSeg sg = segs[si];
      const float2 *ph = sg.phase + (long long)kq * sg.phase_stride;
      for (int p = lane; p < sg.npts; p += 32) {
        const int idx = sg.idx[p], xr = idx / N3, z = idx - xr * N3;
        xb[sg.x_off + p] = cmul(tp[xr * LD + z], ph[p]);
      }
    }
  }
}

// ------------------------------------------------------------------ host helpers

namespace fftfast {

constexpr size_t kSmemCap = 200 * 1024;

inline size_t tile_bytes(int planes, int rows, int cols) { return sizeof(float2) * (size_t)planes * rows * padded(cols); }

inline void allow_smem(const void *fn, size_t bytes) {
  static std::map<const void *, size_t> done;
  auto &d = done[fn];
  if (bytes > 48 * 1024 && bytes > d) {
    PAWPY_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    d = bytes;
  }
}

// tuned tile counts per (pass, N1, N2, N3)
inline std::map<std::tuple<int, int, int, int>, int> &tuned() {
  static std::map<std::tuple<int, int, int, int>, int> t;
  return t;
}

template <typename Launch>
inline int tune(const std::tuple<int, int, int, int> &key, const std::vector<int> &cands, Launch launch) {
  auto it = tuned().find(key);
  if (it != tuned().end()) return it->second;
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
  for (auto &e : ev) cudaEventDestroy(e);
  tuned()[key] = best;
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

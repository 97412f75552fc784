// Device kernels of the band-projection path: coefficient layout, the batched
// backward 3D FFT (fft3d, linalg.c:14-45; the last pass, fused with the sphere
// gather, is in sphere.cu), and the double-precision GEMV of the per-band
// compensation terms (compensation_terms, projector.c:850-963).
#include <algorithm>
#include <cstdlib>
#include <cuda_runtime.h>

#include "fft_tmpl.cuh"
#include "kernels.h"

namespace pawpy {

// ===================================================================== coefficients

__global__ void k_permute(const float2 *__restrict__ Cu, int W, const int *__restrict__ perm,
                          float2 *__restrict__ C, int Wpad) {
  int b = blockIdx.y;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < Wpad; t += gridDim.x * blockDim.x)
    C[(long long)b * Wpad + t] = t < W ? Cu[(long long)b * W + perm[t]] : make_float2(0.f, 0.f);
}

void launch_permute(const float2 *Cu, int W, const int *perm, float2 *C, int Wpad, int nb) {
  if (nb <= 0) return;
  dim3 grid(ceil_div(Wpad, 256 * 4), nb);
  PAWPY_LAUNCH("permute", k_permute<<<grid, 256, 0, stream()>>>(Cu, W, perm, C, Wpad));
}

// Reads each band's coefficients in order (coalesced) from its host array and
// scatters them to their sorted positions. Host reads cross the CPU-GPU link
// with a latency of microseconds, so a thread issues LH independent loads
// before its first store. The kernel is persistent over (band, tile of
// LH x LH_THREADS coefficients) pairs with a few blocks: it runs beside the
// transforms of the k-points already uploaded and leaves them most SM slots.
namespace {
constexpr int LH = 8;
constexpr int LH_THREADS = 128;
constexpr int LH_TILE = LH * LH_THREADS;
}

__global__ void __launch_bounds__(LH_THREADS) k_load_host_bands(const float2 *const *__restrict__ hb, int W,
                                                                const int *__restrict__ inv,
                                                                float2 *__restrict__ C, int Wpad, int nb) {
  const int tiles = (Wpad + LH_TILE - 1) / LH_TILE;
  for (long long t = blockIdx.x; t < (long long)tiles * nb; t += gridDim.x) {
    const int b = (int)(t / tiles), w0 = (int)(t - (long long)b * tiles) * LH_TILE + threadIdx.x;
    const float2 *__restrict__ src = hb[b];
    float2 *__restrict__ dst = C + (long long)b * Wpad;
    float2 v[LH];
#pragma unroll
    for (int i = 0; i < LH; i++) {
      const int w = w0 + i * LH_THREADS;
      v[i] = w < W ? src[w] : make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int i = 0; i < LH; i++) {
      const int w = w0 + i * LH_THREADS;
      if (w < W)
        dst[inv[w]] = v[i];
      else if (w < Wpad)
        dst[w] = v[i];
    }
  }
}

void launch_load_host_bands(const float2 *const *host_bands, int W, const int *invperm, float2 *C, int Wpad,
                            int nb) {
  if (nb <= 0) return;
  static int blocks = [] {
    int sms = 0;
    PAWPY_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device()));
    int per_sm = 1;
    if (const char *e = getenv("PAWPY_GPU_LOAD_BLOCKS_PER_SM")) per_sm = std::max(1, atoi(e));
    return sms * per_sm;
  }();
  const long long work = (long long)ceil_div(Wpad, LH_TILE) * nb;
  const int grid = (int)std::min<long long>(blocks, work);
  PAWPY_LAUNCH("load_host",
               k_load_host_bands<<<grid, LH_THREADS, 0, stream()>>>(host_bands, W, invperm, C, Wpad, nb));
}

// ===================================================================== FFT

// One CTA per (plane p, band b): scatter the plane's coefficients into a zeroed
// N2 x N3 tile, transform rows (length N3, stride 1) then columns (length N2,
// stride N3), store the tile.
__global__ void k_fft_planes(const float2 *__restrict__ C, int Wpad, const int *__restrict__ pstart,
                             const int *__restrict__ poff, PlaneGeom g, Radices r2, Radices r3,
                             const float2 *__restrict__ tw2g, const float2 *__restrict__ tw3g,
                             float2 *__restrict__ H) {
  extern __shared__ float2 sm[];
  const int plane = g.N2 * g.N3;
  float2 *a = sm, *b = sm + plane, *tw2 = sm + 2 * plane, *tw3 = tw2 + g.N2;
  const int p = blockIdx.x, band = blockIdx.y;
  for (int i = threadIdx.x; i < plane; i += blockDim.x) a[i] = make_float2(0.f, 0.f);
  for (int i = threadIdx.x; i < g.N2; i += blockDim.x) tw2[i] = tw2g[i];
  for (int i = threadIdx.x; i < g.N3; i += blockDim.x) tw3[i] = tw3g[i];
  __syncthreads();
  const float2 *cb = C + (long long)band * Wpad;
  for (int t = pstart[p] + threadIdx.x; t < pstart[p + 1]; t += blockDim.x) a[poff[t]] = cb[t];
  __syncthreads();
  float2 *res = block_fft_any<1, true>(a, b, r3, g.N2, g.N3, 1, tw3);
  float2 *oth = res == a ? b : a;
  res = block_fft_any<1, false>(res, oth, r2, g.N3, 1, g.N3, tw2);
  float2 *out = H + ((long long)band * g.n1 + p) * plane;
  for (int i = threadIdx.x; i < plane; i += blockDim.x) out[i] = res[i];
}

void launch_fft_planes(const float2 *C, int Wpad, const int *plane_start, const int *plane_off,
                       const PlaneGeom &g, const Radices &r2, const Radices &r3, const float2 *tw2,
                       const float2 *tw3, float2 *H, int nb) {
  if (nb <= 0 || g.n1 <= 0) return;
  size_t smem = sizeof(float2) * (2 * (size_t)g.N2 * g.N3 + g.N2 + g.N3);
  PAWPY_REQUIRE(smem <= 227 * 1024, "FFT plane does not fit in shared memory");
  allow_dynamic_smem((const void *)k_fft_planes, smem);
  dim3 grid(g.n1, nb);
  PAWPY_LAUNCH("fft_planes", k_fft_planes<<<grid, 256, smem, stream()>>>(C, Wpad, plane_start, plane_off,
                                                                          g, r2, r3, tw2, tw3, H));
  note_work("fft_planes", 8.0 * ((double)Wpad + (double)g.n1 * g.N2 * g.N3) * nb);
}

// Generic: one CTA per (line group along `axis`, band); lines are loaded whole.
__global__ void k_fft_axis(float2 *__restrict__ grid, int N1, int N2, int N3, int axis, Radices r,
                           const float2 *__restrict__ twg) {
  extern __shared__ float2 sm[];
  const int n = r.n;
  float2 *a = sm, *b = sm + n, *tw = sm + 2 * n;
  long long gsz = (long long)N1 * N2 * N3;
  float2 *gb = grid + (long long)blockIdx.y * gsz;
  int line = blockIdx.x;
  long long base, stride;
  if (axis == 2) {
    base = (long long)line * N3;
    stride = 1;
  } else if (axis == 1) {
    int i = line / N3, k = line % N3;
    base = (long long)i * N2 * N3 + k;
    stride = N3;
  } else {
    base = line;
    stride = (long long)N2 * N3;
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    tw[i] = twg[i];
    a[i] = gb[base + i * stride];
  }
  __syncthreads();
  float2 *res = block_fft<1>(a, b, r, 1, n, 1, tw);
  for (int i = threadIdx.x; i < n; i += blockDim.x) gb[base + i * stride] = res[i];
}

void launch_fft_axis(float2 *grid, int nb, int N1, int N2, int N3, int axis, const Radices &r,
                     const float2 *tw) {
  int lines = axis == 2 ? N1 * N2 : axis == 1 ? N1 * N3 : N2 * N3;
  size_t smem = sizeof(float2) * 3 * (size_t)r.n;
  dim3 g(lines, nb);
  PAWPY_LAUNCH("fft_axis", k_fft_axis<<<g, 64, smem, stream()>>>(grid, N1, N2, N3, axis, r, tw));
}

__global__ void k_scatter_grid(const int *__restrict__ Gs, const float2 *__restrict__ Cs, int nw, int N1,
                               int N2, int N3, float2 *__restrict__ grid) {
  for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < nw; w += gridDim.x * blockDim.x) {
    int g1 = ((Gs[3 * w] % N1) + N1) % N1;
    int g2 = ((Gs[3 * w + 1] % N2) + N2) % N2;
    int g3 = ((Gs[3 * w + 2] % N3) + N3) % N3;
    grid[((long long)g1 * N2 + g2) * N3 + g3] = Cs[w];
  }
}

void launch_scatter_grid(const int *Gs, const float2 *Cs, int nw, int N1, int N2, int N3, float2 *grid) {
  PAWPY_CUDA(cudaMemsetAsync(grid, 0, sizeof(float2) * (size_t)N1 * N2 * N3, stream()));
  if (nw > 0)
    PAWPY_LAUNCH("scatter", k_scatter_grid<<<ceil_div(nw, 256), 256, 0, stream()>>>(Gs, Cs, nw, N1, N2, N3, grid));
}

__global__ void k_scale_c128(const float2 *__restrict__ g, long n, double s, double2 *__restrict__ out) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    out[i] = make_double2(g[i].x * s, g[i].y * s);
}

void launch_scale_to_c128(const float2 *grid, long n, double scale, double2 *out) {
  PAWPY_LAUNCH("scale", k_scale_c128<<<ceil_div(n, 256 * 8), 256, 0, stream()>>>(grid, n, scale, out));
}

// ===================================================================== FP64 compensation

__global__ void k_zgemv_f64(const double2 *__restrict__ A, long long lda, int M, int K,
                            const double2 *__restrict__ b, double2 *__restrict__ out) {
  int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  int lane = threadIdx.x & 31;
  if (row >= M) return;
  const double2 *a = A + (long long)row * lda;
  double re = 0, im = 0;
  for (int k = lane; k < K; k += 32) {
    double2 x = a[k], y = b[k];
    re += x.x * y.x + x.y * y.y;
    im += x.x * y.y - x.y * y.x;
  }
  for (int o = 16; o > 0; o >>= 1) {
    re += __shfl_xor_sync(0xffffffffu, re, o);
    im += __shfl_xor_sync(0xffffffffu, im, o);
  }
  if (lane == 0) out[row] = make_double2(out[row].x + re, out[row].y + im);
}

void launch_zgemv_f64(const double2 *A, long long lda, int M, int K, const double2 *b, double2 *out) {
  if (M <= 0) return;
  PAWPY_LAUNCH("comp_f64", k_zgemv_f64<<<ceil_div(M, 8), 256, 0, stream()>>>(A, lda, M, K, b, out));
}

}  // namespace pawpy

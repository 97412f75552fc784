// Augmentation columns of the PAW terms and result layout kernels.
//
// compensation_terms (projector.c:850-963) adds, for every (basis band, k),
//   O_M = sum_{s in M}  conj(P_R,s)^T D_s P_S,s       (D_s = <phi|phi> - <phit|phit>)
//   O_R = sum_{s in N_R} conj(P_R,s)^T W_S,s          (W = <(phi-phit) smooth|psi_S>)
//   O_S = sum_{s in N_S} conj(W_R,s)^T P_S,s
//   O_N = sum_pairs     conj(P_R,s1)^T Q P_S,s2 exp(2 pi i k.d)
// Each term is a dot product between a column gathered from the basis side
// (A) and a column built from the defect side (B). A holds copies of basis
// projector coefficients; B holds D P_S, W_S, P_S and Q P_S e^{i phi} built in
// double precision. Appending A and B to the plane-wave coefficients turns the
// whole PAW overlap into one contraction per k-point.
#include <cuda_runtime.h>

#include "kernels.h"

namespace pawpy {

__global__ void k_aug_a(const float2 *__restrict__ P, int Pt, const float2 *__restrict__ WP, int Pw, int nb,
                        const int *__restrict__ src, int Kc, int Kcpad, double2 *__restrict__ A64,
                        float2 *__restrict__ A32) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  int b = blockIdx.y, k = blockIdx.z;
  if (c >= Kcpad) return;
  float2 v = make_float2(0.f, 0.f);
  if (c < Kc) {
    int s = src[c];
    v = s < Pt ? P[((long long)k * nb + b) * Pt + s] : WP[((long long)k * nb + b) * Pw + (s - Pt)];
    if (A64) A64[((long long)k * nb + b) * Kc + c] = make_double2(v.x, v.y);
  }
  if (A32) A32[((long long)k * nb + b) * Kcpad + c] = v;
}

void launch_aug_a(const float2 *P, int Pt, const float2 *WP, int Pw, int nb, int nk, const int *src, int Kc,
                  int Kcpad, double2 *A64, float2 *A32) {
  if (Kcpad <= 0 || nb <= 0 || nk <= 0) return;
  dim3 g(ceil_div(Kcpad, 128), nb, nk);
  PAWPY_LAUNCH("aug_a", k_aug_a<<<g, 128, 0, stream()>>>(P, Pt, WP, Pw, nb, src, Kc, Kcpad, A64, A32));
}

__global__ void k_aug_b(const float2 *__restrict__ P, int Pt, const float2 *__restrict__ WP, int Pw, int nbtot,
                        int b0, int nb, const int *__restrict__ ptr, const int *__restrict__ col,
                        const double2 *__restrict__ val, const int *__restrict__ pair,
                        const double2 *__restrict__ phase, int npairs, int Kc, int Kcpad,
                        double2 *__restrict__ B64, float2 *__restrict__ B32) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  int b = blockIdx.y, k = blockIdx.z;
  if (c >= Kcpad) return;
  double re = 0, im = 0;
  if (c < Kc) {
    long long row = (long long)k * nbtot + b0 + b;
    for (int e = ptr[c]; e < ptr[c + 1]; e++) {
      int s = col[e];
      float2 x = s < Pt ? P[row * Pt + s] : WP[row * Pw + (s - Pt)];
      double2 w = val[e];
      re += w.x * x.x - w.y * x.y;
      im += w.x * x.y + w.y * x.x;
    }
    int p = pair[c];
    if (p >= 0) {
      double2 f = phase[(long long)k * npairs + p];
      double r2 = re * f.x - im * f.y, i2 = re * f.y + im * f.x;
      re = r2;
      im = i2;
    }
    if (B64) B64[((long long)k * nb + b) * Kc + c] = make_double2(re, im);
  }
  if (B32) B32[((long long)k * nb + b) * Kcpad + c] = make_float2((float)re, (float)im);
}

void launch_aug_b(const float2 *P, int Pt, const float2 *WP, int Pw, int nbtot, int b0, int nb, int nk,
                  const int *ptr, const int *col, const double2 *val, const int *pair, const double2 *phase,
                  int npairs, int Kc, int Kcpad, double2 *B64, float2 *B32) {
  if (Kcpad <= 0 || nb <= 0 || nk <= 0) return;
  dim3 g(ceil_div(Kcpad, 128), nb, nk);
  PAWPY_LAUNCH("aug_b", k_aug_b<<<g, 128, 0, stream()>>>(P, Pt, WP, Pw, nbtot, b0, nb, ptr, col, val, pair, phase,
                                                        npairs, Kc, Kcpad, B64, B32));
}

// The FP32 form of k_aug_b for the batched contraction (its B columns are FP32): val32[k][e]
// holds the entry times the column's pair phase. One thread per column and four bands.
__global__ void k_aug_b32(const float2 *__restrict__ P, int Pt, const float2 *__restrict__ WP, int Pw, int nbtot,
                          int nb, const int *__restrict__ ptr, const int *__restrict__ col,
                          const float2 *__restrict__ val32, int nent, int Kc, int Kcpad,
                          float2 *__restrict__ B32) {
  constexpr int NBT = 4;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int bb = blockIdx.y * NBT, k = blockIdx.z;
  if (c >= Kcpad) return;
  float re[NBT], im[NBT];
#pragma unroll
  for (int u = 0; u < NBT; u++) re[u] = im[u] = 0.f;
  if (c < Kc) {
    const float2 *vk = val32 + (long long)k * nent;
    for (int e = ptr[c]; e < ptr[c + 1]; e++) {
      const int s = col[e];
      const float2 w = vk[e];
#pragma unroll
      for (int u = 0; u < NBT; u++) {
        if (bb + u < nb) {
          const long long row = (long long)k * nbtot + bb + u;
          const float2 x = s < Pt ? P[row * Pt + s] : WP[row * Pw + (s - Pt)];
          re[u] = fmaf(w.x, x.x, fmaf(-w.y, x.y, re[u]));
          im[u] = fmaf(w.x, x.y, fmaf(w.y, x.x, im[u]));
        }
      }
    }
  }
#pragma unroll
  for (int u = 0; u < NBT; u++)
    if (bb + u < nb) B32[((long long)k * nb + bb + u) * Kcpad + c] = make_float2(re[u], im[u]);
}

__global__ void k_aug_val32(const double2 *__restrict__ val, const int *__restrict__ e_pair, int n, int ne,
                            const double2 *__restrict__ phase, int npairs, float2 *__restrict__ val32) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y;
  if (e >= ne) return;
  double2 v = e < n ? val[e] : make_double2(0.0, 0.0);
  if (e < n && e_pair[e] >= 0) {
    const double2 f = phase[(long long)k * npairs + e_pair[e]];
    v = make_double2(v.x * f.x - v.y * f.y, v.x * f.y + v.y * f.x);
  }
  val32[(long long)k * ne + e] = make_float2((float)v.x, (float)v.y);
}

void launch_aug_val32(const double2 *val, const int *e_pair, int n, int ne, const double2 *phase, int npairs, int nk,
                      float2 *val32) {
  if (ne <= 0 || nk <= 0) return;
  dim3 g(ceil_div(ne, 256), nk);
  PAWPY_LAUNCH("aug_setup", k_aug_val32<<<g, 256, 0, stream()>>>(val, e_pair, n, ne, phase, npairs, val32));
}

void launch_aug_b32(const float2 *P, int Pt, const float2 *WP, int Pw, int nbtot, int nb, int nk, const int *ptr,
                    const int *col, const float2 *val32, int nent, int Kc, int Kcpad, float2 *B32) {
  if (Kcpad <= 0 || nb <= 0 || nk <= 0) return;
  dim3 g(ceil_div(Kcpad, 128), ceil_div(nb, 4), nk);
  PAWPY_LAUNCH("aug_b", k_aug_b32<<<g, 128, 0, stream()>>>(P, Pt, WP, Pw, nbtot, nb, ptr, col, val32, nent, Kc,
                                                          Kcpad, B32));
}

__global__ void k_to_host_layout(const float2 *__restrict__ S, int nk, int nbS, int nbR, double2 *__restrict__ out) {
  long long n = (long long)nk * nbS * nbR;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    int k = (int)(e % nk);
    long long r = e / nk;
    int bR = (int)(r % nbR), bS = (int)(r / nbR);
    float2 v = S[((long long)k * nbS + bS) * nbR + bR];
    out[e] = make_double2(v.x, v.y);
  }
}

void launch_to_host_layout(const float2 *S, int nk, int nbS, int nbR, double2 *out) {
  long long n = (long long)nk * nbS * nbR;
  PAWPY_LAUNCH("to_host", k_to_host_layout<<<ceil_div(n, 256 * 4), 256, 0, stream()>>>(S, nk, nbS, nbR, out));
}

__global__ void k_extract_band(const float2 *__restrict__ S, int nk, int nbS, int nbR, int band,
                               double2 *__restrict__ out) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nk * nbR) return;
  int k = e % nk, bR = e / nk;
  float2 v = S[((long long)k * nbS + band) * nbR + bR];
  out[e] = make_double2(v.x, v.y);
}

void launch_extract_band(const float2 *S, int nk, int nbS, int nbR, int band, double2 *out) {
  PAWPY_LAUNCH("extract", k_extract_band<<<ceil_div(nk * nbR, 256), 256, 0, stream()>>>(S, nk, nbS, nbR, band, out));
}

// One block per defect band: the weighted sums of |S|^2 over (basis band, k),
// per channel, reduced in a fixed order (FP64).
namespace {
constexpr int BC_THREADS = 256;
}

__global__ void __launch_bounds__(BC_THREADS)
    k_band_character(const float2 *__restrict__ S, int nk, int nbS, int nbR, const double *__restrict__ wv,
                     const double *__restrict__ wc, int nwk, int nch, double *__restrict__ v,
                     double *__restrict__ c) {
  __shared__ double red[4][BC_THREADS];
  const int bS = blockIdx.x;
  double sv[2] = {0.0, 0.0}, sc[2] = {0.0, 0.0};
  const long long n = (long long)nk * nbR;
  for (long long e = threadIdx.x; e < n; e += BC_THREADS) {
    const int k = (int)(e / nbR), bR = (int)(e - (long long)k * nbR);
    const float2 s = S[((long long)k * nbS + bS) * nbR + bR];
    const double p = (double)s.x * s.x + (double)s.y * s.y;
    const long long w = (long long)bR * nk + k;
    if (nch > 1 && k >= nwk) {
      sv[1] += p * wv[w];
      sc[1] += p * wc[w];
    } else {
      sv[0] += p * wv[w];
      sc[0] += p * wc[w];
    }
  }
  red[0][threadIdx.x] = sv[0];
  red[1][threadIdx.x] = sv[1];
  red[2][threadIdx.x] = sc[0];
  red[3][threadIdx.x] = sc[1];
  __syncthreads();
  for (int h = BC_THREADS / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h)
      for (int q = 0; q < 4; q++) red[q][threadIdx.x] += red[q][threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x < nch) {
    v[(long long)bS * nch + threadIdx.x] = red[threadIdx.x][0];
    c[(long long)bS * nch + threadIdx.x] = red[2 + threadIdx.x][0];
  }
}

void launch_band_character(const float2 *S, int nk, int nbS, int nbR, const double *wv, const double *wc, int nwk,
                           int nch, double *v, double *c) {
  if (nbS <= 0) return;
  if (nch < 1 || nch > 2 || (nch == 2 && nk != 2 * nwk))
    throw Error(ERR_ARG, "band character: one channel, or two spin channels of nwk k-points each");
  PAWPY_LAUNCH("band_character",
               k_band_character<<<nbS, BC_THREADS, 0, stream()>>>(S, nk, nbS, nbR, wv, wc, nwk, nch, v, c));
}

}  // namespace pawpy

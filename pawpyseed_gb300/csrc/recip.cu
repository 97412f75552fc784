// Augmentation coefficients of the aug_recip method (get_aug_freqs,
// projector.c:276-331, 420-453): for every band, the smoothed partial-wave
// differences of a set of sites, weighted by the band's projector coefficients,
// spread onto the real-space grid and transformed forward (fwd_fft3d,
// linalg.c:47-79), then read at the k-point's plane waves:
//
//   CA[G] = sqrt(V)/N^3 sum_r x(r) exp(-i G.r),
//   x(r)  = sum_{s,p} <p_{s,p}|psi> T_{s,p}(r) exp(-i k.path_s(r)).
//
// The sphere tables already hold tab = conj(T) dV V^-1/2 and phase =
// exp(i k.path), so with y(r) = sum_{s,p} conj(<p|psi>) tab(r) phase(r) =
// conj(x(r)) dV V^-1/2 the forward transform is the conjugate of a backward
// one: CA[G] = conj(sum_r y(r) exp(+i G.r)) (dV = V/N^3). Both passes below
// therefore use the backward line transforms of the projection path:
//
//   pass 1, per real-space plane j (second axis) and band: y of the plane's
//     sphere points summed per grid cell in a fixed order (site order), then
//     the transform along the first axis; the occupied planes g1 of the
//     plane-wave sphere go to H[band][g1 plane][j][k];
//   pass 2, per g1 plane and band: the 2D transform of H along the third and
//     second axes, then CA of the plane's coefficients (conjugated), in the
//     sorted plane-wave order of the coefficient arrays; optionally
//     D = C + CA as well.
#include <cuda_runtime.h>

#include "fft_tmpl.cuh"
#include "kernels.h"

namespace pawpy {

__global__ void k_recip_xspread(RecipSpread c, const float2 *__restrict__ P, int Pstride, int nkp, int kq,
                                int N1, int N2, int N3, int g1min, int n1, Radices r1,
                                const float2 *__restrict__ tw1g, float2 *__restrict__ H) {
  extern __shared__ float2 sm[];
  const int plane = N1 * N3;
  float2 *a = sm, *b = sm + plane, *tw = sm + 2 * plane;
  const int j = blockIdx.x, band = blockIdx.y;
  for (int i = threadIdx.x; i < plane; i += blockDim.x) a[i] = make_float2(0.f, 0.f);
  for (int i = threadIdx.x; i < N1; i += blockDim.x) tw[i] = tw1g[i];
  __syncthreads();
  const float2 *pb = P + (long long)band * Pstride;
  const float2 *ph = c.phase + (long long)kq * c.npts;
  for (int u = c.cell_first[j] + threadIdx.x; u < c.cell_first[j + 1]; u += blockDim.x) {
    float2 y = make_float2(0.f, 0.f);
    for (int e = c.ent_first[u]; e < c.ent_first[u + 1]; e++) {
      const int s = c.ent_site[e];
      const long long pt = c.ent_pt[e];
      const int np = c.site_npts[s], T = c.site_total[s];
      const float2 *t = c.tab + c.site_val[s] + (pt - c.site_pt[s]);
      const float2 *pp = pb + c.site_pcol[s];
      float2 v = make_float2(0.f, 0.f);
      for (int q = 0; q < T; q++) {
        const float2 w = __ldg(pp + q), tv = __ldg(t + (long long)q * np);
        // conj(w) * tv
        v.x += w.x * tv.x + w.y * tv.y;
        v.y += w.x * tv.y - w.y * tv.x;
      }
      const float2 f = __ldg(ph + pt);
      y.x += v.x * f.x - v.y * f.y;
      y.y += v.x * f.y + v.y * f.x;
    }
    a[c.ucell[u]] = y;
  }
  (void)nkp;
  __syncthreads();
  // transform along the first axis: N3 lines of length N1, element stride N3
  float2 *res = block_fft_any<1, false>(a, b, r1, N3, 1, N3, tw);
  float2 *out = H + (long long)band * n1 * N2 * N3;
  for (int idx = threadIdx.x; idx < n1 * N3; idx += blockDim.x) {
    const int p = idx / N3, k = idx % N3;
    int g1 = (g1min + p) % N1;
    if (g1 < 0) g1 += N1;
    out[((long long)p * N2 + j) * N3 + k] = res[g1 * N3 + k];
  }
}

__global__ void k_recip_planes_pick(const float2 *__restrict__ H, PlaneGeom g, const int *__restrict__ pstart,
                                    const int *__restrict__ poff, Radices r2, Radices r3,
                                    const float2 *__restrict__ tw2g, const float2 *__restrict__ tw3g,
                                    const float2 *__restrict__ C, int Wpad, float2 *__restrict__ CA,
                                    float2 *__restrict__ D) {
  extern __shared__ float2 sm[];
  const int plane = g.N2 * g.N3;
  float2 *a = sm, *b = sm + plane, *tw2 = sm + 2 * plane, *tw3 = tw2 + g.N2;
  const int p = blockIdx.x, band = blockIdx.y;
  const float2 *src = H + ((long long)band * g.n1 + p) * plane;
  for (int i = threadIdx.x; i < plane; i += blockDim.x) a[i] = src[i];
  for (int i = threadIdx.x; i < g.N2; i += blockDim.x) tw2[i] = tw2g[i];
  for (int i = threadIdx.x; i < g.N3; i += blockDim.x) tw3[i] = tw3g[i];
  __syncthreads();
  float2 *res = block_fft_any<1, true>(a, b, r3, g.N2, g.N3, 1, tw3);
  float2 *oth = res == a ? b : a;
  res = block_fft_any<1, false>(res, oth, r2, g.N3, 1, g.N3, tw2);
  const long long row = (long long)band * Wpad;
  for (int t = pstart[p] + threadIdx.x; t < pstart[p + 1]; t += blockDim.x) {
    const float2 z = res[poff[t]];
    const float2 v = make_float2(z.x, -z.y);
    CA[row + t] = v;
    if (D) {
      const float2 cv = C[row + t];
      D[row + t] = make_float2(cv.x + v.x, cv.y + v.y);
    }
  }
}

size_t recip_xspread_smem(int N1, int N3) { return sizeof(float2) * (2 * (size_t)N1 * N3 + N1); }
size_t recip_planes_smem(int N2, int N3) { return sizeof(float2) * (2 * (size_t)N2 * N3 + N2 + N3); }

void launch_recip_xspread(const RecipSpread &c, const float2 *P, int Pstride, int nkp, int kq, const PlaneGeom &g,
                          const Radices &r1, const float2 *tw1, float2 *H, int nb) {
  if (nb <= 0 || g.n1 <= 0) return;
  const size_t smem = recip_xspread_smem(g.N1, g.N3);
  PAWPY_REQUIRE(smem <= 227 * 1024, "aug_recip: an (N1 x N3) grid plane does not fit in shared memory");
  allow_dynamic_smem((const void *)k_recip_xspread, smem);
  dim3 grid(g.N2, nb);
  PAWPY_LAUNCH("recip_spread", k_recip_xspread<<<grid, 256, smem, stream()>>>(c, P, Pstride, nkp, kq, g.N1, g.N2, g.N3,
                                                                               g.g1min, g.n1, r1, tw1, H));
}

void launch_recip_planes_pick(const float2 *H, const PlaneGeom &g, const int *pstart, const int *poff,
                              const Radices &r2, const Radices &r3, const float2 *tw2, const float2 *tw3,
                              const float2 *C, int Wpad, float2 *CA, float2 *D, int nb) {
  if (nb <= 0 || g.n1 <= 0) return;
  const size_t smem = recip_planes_smem(g.N2, g.N3);
  PAWPY_REQUIRE(smem <= 227 * 1024, "aug_recip: an (N2 x N3) grid plane does not fit in shared memory");
  allow_dynamic_smem((const void *)k_recip_planes_pick, smem);
  dim3 grid(g.n1, nb);
  PAWPY_LAUNCH("recip_planes", k_recip_planes_pick<<<grid, 256, smem, stream()>>>(H, g, pstart, poff, r2, r3, tw2,
                                                                                  tw3, C, Wpad, CA, D));
}

}  // namespace pawpy

// Device kernels of the band-projection path: coefficient layout, the batched
// backward 3D FFT (fft3d, linalg.c:14-45), the augmentation-sphere tables
// (setup_site, utils.c:590-696) and gather (onto_projector_helper,
// projector.c:223-274), and the double-precision GEMV of the per-band
// compensation terms (compensation_terms, projector.c:850-963).
#include <cuda_runtime.h>

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
  float2 *res = block_fft<1>(a, b, r3, g.N2, g.N3, 1, tw3);
  float2 *oth = res == a ? b : a;
  res = block_fft<1>(res, oth, r2, g.N3, 1, g.N3, tw2);
  float2 *out = H + ((long long)band * g.n1 + p) * plane;
  for (int i = threadIdx.x; i < plane; i += blockDim.x) out[i] = res[i];
}

void launch_fft_planes(const float2 *C, int Wpad, const int *plane_start, const int *plane_off,
                       const PlaneGeom &g, const Radices &r2, const Radices &r3, const float2 *tw2,
                       const float2 *tw3, float2 *H, int nb) {
  if (nb <= 0 || g.n1 <= 0) return;
  size_t smem = sizeof(float2) * (2 * (size_t)g.N2 * g.N3 + g.N2 + g.N3);
  PAWPY_REQUIRE(smem <= 227 * 1024, "FFT plane does not fit in shared memory");
  static size_t configured = 0;
  if (smem > 48 * 1024 && smem > configured) {
    PAWPY_CUDA(cudaFuncSetAttribute(k_fft_planes, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    configured = smem;
  }
  dim3 grid(g.n1, nb);
  PAWPY_LAUNCH("fft_planes", k_fft_planes<<<grid, 256, smem, stream()>>>(C, Wpad, plane_start, plane_off,
                                                                          g, r2, r3, tw2, tw3, H));
}

// One CTA per (row j, band b): gather the n1 planes' row j into an N1 x N3 tile
// (row (g1min+p) mod N1), transform along the first axis, scale, store u[b][:, j, :].
__global__ void k_fft_x(const float2 *__restrict__ H, PlaneGeom g, Radices r1,
                        const float2 *__restrict__ tw1g, float scale, float2 *__restrict__ u) {
  extern __shared__ float2 sm[];
  const int tile = g.N1 * g.N3;
  float2 *a = sm, *b = sm + tile, *tw1 = sm + 2 * tile;
  const int j = blockIdx.x, band = blockIdx.y;
  for (int i = threadIdx.x; i < g.N1; i += blockDim.x) tw1[i] = tw1g[i];
  for (int i = threadIdx.x; i < tile; i += blockDim.x) {
    int row = i / g.N3, k = i - row * g.N3;
    int p = row - g.g1min;
    p = ((p % g.N1) + g.N1) % g.N1;  // plane whose g1 maps to this row
    float2 v = make_float2(0.f, 0.f);
    if (p < g.n1) v = H[(((long long)band * g.n1 + p) * g.N2 + j) * g.N3 + k];
    a[i] = v;
  }
  __syncthreads();
  float2 *res = block_fft<1>(a, b, r1, g.N3, 1, g.N3, tw1);
  float2 *ub = u + (long long)band * g.N1 * g.N2 * g.N3;
  for (int i = threadIdx.x; i < tile; i += blockDim.x) {
    int row = i / g.N3, k = i - row * g.N3;
    float2 v = res[i];
    ub[((long long)row * g.N2 + j) * g.N3 + k] = make_float2(v.x * scale, v.y * scale);
  }
}

void launch_fft_x(const float2 *H, const PlaneGeom &g, const Radices &r1, const float2 *tw1, float scale,
                  float2 *u, int nb) {
  if (nb <= 0) return;
  size_t smem = sizeof(float2) * (2 * (size_t)g.N1 * g.N3 + g.N1);
  PAWPY_REQUIRE(smem <= 227 * 1024, "FFT tile does not fit in shared memory");
  static size_t configured = 0;
  if (smem > 48 * 1024 && smem > configured) {
    PAWPY_CUDA(cudaFuncSetAttribute(k_fft_x, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    configured = smem;
  }
  dim3 grid(g.N2, nb);
  PAWPY_LAUNCH("fft_x", k_fft_x<<<grid, 256, smem, stream()>>>(H, g, r1, tw1, scale, u));
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

// ===================================================================== sphere tables

__device__ __forceinline__ void d_to_cart(const double *f, const double *L, double *o) {
  double t0 = f[0] * L[0] + f[1] * L[3] + f[2] * L[6];
  double t1 = f[0] * L[1] + f[1] * L[4] + f[2] * L[7];
  double t2 = f[0] * L[2] + f[1] * L[5] + f[2] * L[8];
  o[0] = t0;
  o[1] = t1;
  o[2] = t2;
}

// |v| rounded once, as the reference's pow(x, 0.5) (a correctly rounded square root) gives it
__device__ __forceinline__ double d_norm(const double *v) { return sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }

__device__ __forceinline__ void box_point(const SiteDesc &s, long long lin, int *ijk) {
  int w3 = 2 * s.g[2] + 1, w2 = 2 * s.g[1] + 1;
  int kk = (int)(lin % w3);
  long long r = lin / w3;
  int jj = (int)(r % w2);
  int ii = (int)(r / w2);
  ijk[0] = ii - s.g[0] + s.c[0];
  ijk[1] = jj - s.g[1] + s.c[1];
  ijk[2] = kk - s.g[2] + s.c[2];
}

// unwrapped Cartesian path from the site to grid point ijk, and whether it is inside R0
__device__ __forceinline__ bool inside(const SiteDesc &s, const int *ijk, const double *L, const int *N,
                                       double *path) {
  double fr[3] = {(double)ijk[0] / N[0] - s.coord[0], (double)ijk[1] / N[1] - s.coord[1],
                  (double)ijk[2] / N[2] - s.coord[2]};
  d_to_cart(fr, L, path);
  return d_norm(path) < s.R0;
}

__global__ void k_sphere_count(const SiteDesc *__restrict__ sites, const double *__restrict__ Lg,
                               const int *__restrict__ Ng, int *__restrict__ counts) {
  __shared__ int total;
  const SiteDesc s = sites[blockIdx.x];
  double L[9];
  int N[3] = {Ng[0], Ng[1], Ng[2]};
  for (int i = 0; i < 9; i++) L[i] = Lg[i];
  if (threadIdx.x == 0) total = 0;
  __syncthreads();
  long long box = (long long)(2 * s.g[0] + 1) * (2 * s.g[1] + 1) * (2 * s.g[2] + 1);
  int c = 0;
  for (long long lin = threadIdx.x; lin < box; lin += blockDim.x) {
    int ijk[3];
    double path[3];
    box_point(s, lin, ijk);
    if (inside(s, ijk, L, N, path)) c++;
  }
  atomicAdd(&total, c);
  __syncthreads();
  if (threadIdx.x == 0) counts[blockIdx.x] = total;
}

void launch_sphere_count(const SiteDesc *sites, int nsites, const double *lattice, const int *fftg,
                         int *counts) {
  if (nsites <= 0) return;
  PAWPY_LAUNCH("sphere_count", k_sphere_count<<<nsites, 256, 0, stream()>>>(sites, lattice, fftg, counts));
}

__device__ double d_fact(int n) {
  double t = 1;
  for (int m = 1; m <= n; m++) t *= m;
  return t;
}

// associated Legendre function with the Condon-Shortley phase (explicit sum, utils.c:377-386)
__device__ double d_plm(int l, int m, double x) {
  double pre = 1.0;
  if (m < 0) {
    int am = -m;
    pre = ((am & 1) ? -1.0 : 1.0) * d_fact(l - am) / d_fact(l + am);
    m = am;
  }
  double acc = 0;
  for (int n = l; n >= 0 && 2 * n - l - m >= 0; n--)
    acc += pow(x, (double)(2 * n - l - m)) * d_fact(2 * n) / d_fact(2 * n - l - m) / d_fact(n) /
           d_fact(l - n) * (((l - n) & 1) ? -1.0 : 1.0);
  return pre * acc * ((m & 1) ? -1.0 : 1.0) * pow(1 - x * x, m / 2.0) / pow(2.0, (double)l);
}

// One CTA per site: walk the box in the reference's (i, j, k) order, keep the
// points with |path| < R0 in that order (block scan), and tabulate
// conj(p(r) Y_lm(theta, phi)) dV (lm-major) plus exp(i k.path) per k-point.
__global__ void k_sphere_fill(const SiteDesc *__restrict__ sites, const SpeciesDev *__restrict__ species,
                              const double *__restrict__ Lg, const int *__restrict__ Ng, double dv,
                              const double *__restrict__ kcart, int nkp, long long total_pts,
                              int *__restrict__ idx, float2 *__restrict__ tab, float2 *__restrict__ phase) {
  __shared__ int warp_cnt[32];
  __shared__ int base_s;
  const SiteDesc s = sites[blockIdx.x];
  const SpeciesDev &sp = species[s.species];
  double L[9];
  int N[3] = {Ng[0], Ng[1], Ng[2]};
  for (int i = 0; i < 9; i++) L[i] = Lg[i];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (threadIdx.x == 0) base_s = 0;
  __syncthreads();
  long long box = (long long)(2 * s.g[0] + 1) * (2 * s.g[1] + 1) * (2 * s.g[2] + 1);
  for (long long start = 0; start < box; start += blockDim.x) {
    long long lin = start + threadIdx.x;
    int ijk[3];
    double path[3];
    bool in = false;
    if (lin < box) {
      box_point(s, lin, ijk);
      in = inside(s, ijk, L, N, path);
    }
    unsigned m = __ballot_sync(0xffffffffu, in);
    if (lane == 0) warp_cnt[wid] = __popc(m);
    __syncthreads();
    int before = 0, chunk = 0;
    for (int w = 0; w < nw; w++) {
      if (w < wid) before += warp_cnt[w];
      chunk += warp_cnt[w];
    }
    int pos = base_s + before + __popc(m & ((1u << lane) - 1u));
    if (in && pos < s.npts) {
      int ii = ((ijk[0] % N[0]) + N[0]) % N[0];
      int jj = ((ijk[1] % N[1]) + N[1]) % N[1];
      int kk = ((ijk[2] % N[2]) + N[2]) % N[2];
      idx[s.pt_off + pos] = (ii * N[1] + jj) * N[2] + kk;
      // minimum-image displacement from the site to the wrapped grid point (utils.c:51-73)
      double gp[3] = {(double)ii / N[0], (double)jj / N[1], (double)kk / N[2]};
      double t[3] = {0, 0, 0}, r = INFINITY;
      for (int a = -1; a <= 1; a++)
        for (int b = -1; b <= 1; b++)
          for (int c = -1; c <= 1; c++) {
            double f[3] = {gp[0] + a - s.coord[0], gp[1] + b - s.coord[1], gp[2] + c - s.coord[2]};
            double v[3];
            d_to_cart(f, L, v);
            double dd = d_norm(v);
            if (dd < r) {
              r = dd;
              t[0] = v[0];
              t[1] = v[1];
              t[2] = v[2];
            }
          }
      double theta = 0, phi = 0;
      if (r != 0) {
        theta = acos(t[2] / r);
        if (r - fabs(t[2]) == 0 || t[0] * t[0] + t[1] * t[1] == 0)
          phi = 0;
        else
          phi = acos(t[0] / sqrt(t[0] * t[0] + t[1] * t[1]));
        if (t[1] < 0) phi = 2 * M_PI - phi;
      }
      double ct = cos(theta);
      for (int lm = 0; lm < sp.total; lm++) {
        int l = sp.lm_l[lm], mm = sp.lm_m[lm], fi = sp.lm_f[lm];
        const double *f = sp.f + (long long)fi * sp.size;
        const double *sb = sp.spl + (long long)fi * 3 * sp.size;
        double rad;
        // linear-grid spline interpolation (proj_interpolate, utils.c:461-475)
        double xlast = sp.grid_rmax / sp.size * (sp.size - 1);
        if (r > xlast) {
          rad = 0;
        } else {
          int ind = (int)(r / sp.grid_rmax * sp.size);
          if (ind > sp.size - 2) ind = sp.size - 2;
          double x0 = sp.grid_rmax / sp.size * ind;
          double dd = r - x0;
          rad = f[ind] + dd * (sb[ind] + dd * (sb[sp.size + ind] + dd * sb[2 * sp.size + ind]));
        }
        double nrm = pow((2 * l + 1) / (4 * M_PI) * d_fact(l - mm) / d_fact(l + mm), 0.5);
        double y = nrm * d_plm(l, mm, ct) * rad;
        double sn, cs;
        sincos(mm * phi, &sn, &cs);
        // conj(radial * Y_lm) * dV
        tab[s.val_off + (long long)lm * s.npts + pos] = make_float2((float)(y * cs * dv), (float)(-y * sn * dv));
      }
      for (int q = 0; q < nkp; q++) {
        double kr = kcart[3 * q] * path[0] + kcart[3 * q + 1] * path[1] + kcart[3 * q + 2] * path[2];
        double sn, cs;
        sincos(kr, &sn, &cs);
        phase[(long long)q * total_pts + s.pt_off + pos] = make_float2((float)cs, (float)sn);
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) base_s += chunk;
    __syncthreads();
  }
}

void launch_sphere_fill(const SiteDesc *sites, int nsites, const SpeciesDev *species, const double *lattice,
                        const int *fftg, double dv, const double *kcart, int nkp, long long total_pts,
                        int *idx, float2 *tab, float2 *phase) {
  if (nsites <= 0) return;
  PAWPY_LAUNCH("sphere_fill", k_sphere_fill<<<nsites, 128, 0, stream()>>>(sites, species, lattice, fftg, dv,
                                                                         kcart, nkp, total_pts, idx, tab, phase));
}

// One warp per band, 8 bands per CTA, one CTA column per site. Lanes stride
// over the sphere's points; each lane keeps one accumulator per lm channel and
// the warp reduces them with xor shuffles at the end.
template <int MAXT>
__global__ void __launch_bounds__(256) k_sphere_gather(const SiteDesc *__restrict__ sites,
                                                       const int *__restrict__ idx,
                                                       const float2 *__restrict__ tab,
                                                       const float2 *__restrict__ phase,
                                                       const float2 *__restrict__ u, long long grid,
                                                       float2 *__restrict__ P, int Ptot, int nb) {
  const SiteDesc s = sites[blockIdx.x];
  const int lane = threadIdx.x & 31;
  const int band = blockIdx.y * 8 + (threadIdx.x >> 5);
  if (band >= nb) return;
  const float2 *ub = u + (long long)band * grid;
  const int *ix = idx + s.pt_off;
  const float2 *ph = phase + s.pt_off;
  const float2 *tb = tab + s.val_off;
  float ar[MAXT], ai[MAXT];
#pragma unroll
  for (int t = 0; t < MAXT; t++) ar[t] = ai[t] = 0.f;
  for (int p = lane; p < s.npts; p += 32) {
    float2 x = cmul(ub[ix[p]], ph[p]);
#pragma unroll
    for (int t = 0; t < MAXT; t++) {
      if (t < s.total) {
        float2 v = tb[(long long)t * s.npts + p];
        ar[t] = fmaf(v.x, x.x, fmaf(-v.y, x.y, ar[t]));
        ai[t] = fmaf(v.x, x.y, fmaf(v.y, x.x, ai[t]));
      }
    }
  }
#pragma unroll
  for (int t = 0; t < MAXT; t++) {
    if (t < s.total) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        ar[t] += __shfl_xor_sync(0xffffffffu, ar[t], o);
        ai[t] += __shfl_xor_sync(0xffffffffu, ai[t], o);
      }
    }
  }
  float2 *out = P + (long long)band * Ptot + s.lm_off;
#pragma unroll
  for (int t = 0; t < MAXT; t++)
    if (t < s.total && lane == (t & 31)) out[t] = make_float2(ar[t], ai[t]);
}

void launch_sphere_gather(const SiteDesc *sites, int nsites, const int *idx, const float2 *tab,
                          const float2 *phase, const float2 *u, long long grid, float2 *P, int Ptot, int nb,
                          int max_total) {
  if (nsites <= 0 || nb <= 0) return;
  dim3 g(nsites, ceil_div(nb, 8));
  if (max_total <= 8)
    PAWPY_LAUNCH("sphere_gather", k_sphere_gather<8><<<g, 256, 0, stream()>>>(sites, idx, tab, phase, u, grid, P, Ptot, nb));
  else if (max_total <= 18)
    PAWPY_LAUNCH("sphere_gather", k_sphere_gather<18><<<g, 256, 0, stream()>>>(sites, idx, tab, phase, u, grid, P, Ptot, nb));
  else if (max_total <= 32)
    PAWPY_LAUNCH("sphere_gather", k_sphere_gather<32><<<g, 256, 0, stream()>>>(sites, idx, tab, phase, u, grid, P, Ptot, nb));
  else
    throw Error(ERR_UNSUPPORTED, "more than 32 projector channels on one site");
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

// All-electron wavefunctions on a real-space grid (the 'realspace' method and
// the AE densities of density.c:158-310):
//
//   psi(r) = V^-1/2 sum_G C_G exp(i G.r) exp(2 pi i k.r_frac)
//          + sum_sites sum_{n,l,m} <p_nlm|psi> (phi_nl - phit_nl)(|r - R|)/|r - R| Y_lm(r - R)
//            exp(2 pi i k.(R + T))
//
// at every grid point r within wave_grid[last] of a site R (T the lattice
// vector that wraps the box point onto the grid), as realspace_state
// (density.c:245-310) evaluates it. The sphere tables (points, values of
// (phi - phit)/r Y_lm, phases per k-point) are built once per wavefunction and
// grid, on the device in double precision; the grids of a batch of bands are a
// scatter and three line-transform passes, the Bloch factor, then the sphere
// terms added per grid cell with the sites in order (the reference adds them
// from parallel threads, so its order is not fixed).
#include <cuda_runtime.h>

#include "kernels.h"

namespace pawpy {

namespace {

__device__ __forceinline__ void to_cart(const double *f, const double *L, double *o) {
  o[0] = f[0] * L[0] + f[1] * L[3] + f[2] * L[6];
  o[1] = f[0] * L[1] + f[1] * L[4] + f[2] * L[7];
  o[2] = f[0] * L[2] + f[1] * L[5] + f[2] * L[8];
}

// Box point q of slab jb of site s: grid indices (unwrapped) and the displacement
// r - R from the site (box around round(coord N), density.c:269-287); inside the sphere?
__device__ __forceinline__ bool ae_point(const SiteDesc &s, int jb, int q, const double *L, const int *N, int *ijk,
                                         double *path) {
  const int w2 = 2 * s.g[2] + 1;
  ijk[0] = q / w2 - s.g[0] + s.c[0];
  ijk[1] = jb - s.g[1] + s.c[1];
  ijk[2] = q % w2 - s.g[2] + s.c[2];
  const double fr[3] = {(double)ijk[0] / N[0] - s.coord[0], (double)ijk[1] / N[1] - s.coord[1],
                        (double)ijk[2] / N[2] - s.coord[2]};
  to_cart(fr, L, path);
  return sqrt(path[0] * path[0] + path[1] * path[1] + path[2] * path[2]) < s.R0;
}

}  // namespace

__global__ void k_ae_count(const SiteDesc *__restrict__ sites, const int2 *__restrict__ slabs,
                           const double *__restrict__ Lg, const int *__restrict__ Ng, int *__restrict__ counts) {
  __shared__ int total;
  const int2 sl = slabs[blockIdx.x];
  const SiteDesc s = sites[sl.x];
  double L[9];
  const int N[3] = {Ng[0], Ng[1], Ng[2]};
  for (int i = 0; i < 9; i++) L[i] = Lg[i];
  if (threadIdx.x == 0) total = 0;
  __syncthreads();
  const int n = (2 * s.g[0] + 1) * (2 * s.g[2] + 1);
  int c = 0;
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    int ijk[3];
    double path[3];
    if (ae_point(s, sl.y, q, L, N, ijk, path)) c++;
  }
  atomicAdd(&total, c);
  __syncthreads();
  if (threadIdx.x == 0) counts[blockIdx.x] = total;
}

// One CTA per segment (a non-empty slab): its inside points in (i, k) order, with
// cell = (ii N2 + jj) N3 + kk, the values (phi - phit)(r)/r Y_lm (wave_value2,
// utils.c:522-545: spline on the logarithmic grid, r below the first grid point
// divided by it) and, per k-point, exp(2 pi i k.(R + T)) (density.c:289-300).
__global__ void k_ae_fill(const SiteDesc *__restrict__ sites, const SegFill *__restrict__ segs,
                          const AeSpeciesDev *__restrict__ species, const double *__restrict__ Lg,
                          const int *__restrict__ Ng, const double *__restrict__ kfrac, int nkp, long long npts,
                          int *__restrict__ cell, float2 *__restrict__ val, float2 *__restrict__ phase) {
  __shared__ int warp_cnt[32];
  __shared__ int base_s;
  const SegFill sg = segs[blockIdx.x];
  const SiteDesc s = sites[sg.site];
  const AeSpeciesDev &sp = species[s.species];
  double L[9];
  const int N[3] = {Ng[0], Ng[1], Ng[2]};
  for (int i = 0; i < 9; i++) L[i] = Lg[i];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (threadIdx.x == 0) base_s = 0;
  __syncthreads();
  const int n = (2 * s.g[0] + 1) * (2 * s.g[2] + 1);
  for (int start = 0; start < n; start += blockDim.x) {
    const int q = start + threadIdx.x;
    int ijk[3];
    double t[3];
    const bool in = q < n && ae_point(s, sg.jb, q, L, N, ijk, t);
    const unsigned m = __ballot_sync(0xffffffffu, in);
    if (lane == 0) warp_cnt[wid] = __popc(m);
    __syncthreads();
    int before = 0, chunk = 0;
    for (int w = 0; w < nw; w++) {
      if (w < wid) before += warp_cnt[w];
      chunk += warp_cnt[w];
    }
    const int pos = base_s + before + __popc(m & ((1u << lane) - 1u));
    if (in && pos < sg.npts) {
      int wrapped[3], shift[3];
      for (int a = 0; a < 3; a++) {
        wrapped[a] = ((ijk[a] % N[a]) + N[a]) % N[a];
        shift[a] = (wrapped[a] - ijk[a]) / N[a];  // the lattice vector T (integer division, exact)
      }
      const long long pt = sg.pt_off + pos;
      cell[pt] = (wrapped[0] * N[1] + wrapped[1]) * N[2] + wrapped[2];
      const double r = sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
      // Y_lm of the displacement: cos(theta) = z / r, exp(i phi) = (x + i y) / rho (phi = 0 on
      // the polar axis and at r = 0), associated Legendre functions by recurrence
      double ct = 1.0, cp = 1.0, sn = 0.0;
      if (r != 0) {
        ct = t[2] / r;
        const double rho = sqrt(t[0] * t[0] + t[1] * t[1]);
        if (rho != 0 && r - fabs(t[2]) != 0) {
          cp = t[0] / rho;
          sn = t[1] / rho;
        }
      }
      const double st = sqrt(fmax(0.0, 1.0 - ct * ct));
      double P[4][4];
      P[0][0] = 1.0;
      for (int mm = 1; mm <= 3; mm++) P[mm][mm] = -(2 * mm - 1) * st * P[mm - 1][mm - 1];
      for (int mm = 0; mm < 3; mm++) P[mm + 1][mm] = (2 * mm + 1) * ct * P[mm][mm];
      P[2][0] = (3.0 * ct * P[1][0] - P[0][0]) / 2.0;
      P[3][0] = (5.0 * ct * P[2][0] - 2.0 * P[1][0]) / 3.0;
      P[3][1] = (5.0 * ct * P[2][1] - 3.0 * P[1][1]) / 2.0;
      double er[4] = {1.0, cp, 0, 0}, ei[4] = {0.0, sn, 0, 0};
      for (int mm = 2; mm <= 3; mm++) {
        er[mm] = er[mm - 1] * cp - ei[mm - 1] * sn;
        ei[mm] = er[mm - 1] * sn + ei[mm - 1] * cp;
      }
      // spline on the logarithmic grid x (wave_interpolate, utils.c:477-489)
      const double x0 = sp.x[0], xl = sp.x[sp.size - 1];
      int ind = 0;
      double rem = 0;
      if (r >= x0 && r <= xl) {
        ind = min((int)(log(r / x0) / sp.logstep), sp.size - 2);
        rem = r - sp.x[ind];
      }
      const double inv_r = 1.0 / (r < x0 ? x0 : r);
      double rad = 0.0;
      int last_f = -1;
      for (int lm = 0; lm < sp.total; lm++) {
        const int l = sp.lm_l[lm], mv = sp.lm_m[lm], fi = sp.lm_f[lm];
        if (fi != last_f) {
          const double *f = sp.f + (long long)fi * sp.size;
          const double *b = sp.spl + (long long)fi * 3 * sp.size;
          if (r > xl)
            rad = 0.0;
          else if (r < x0)
            rad = f[0];
          else
            rad = f[ind] + rem * (b[ind] + rem * (b[sp.size + ind] + rem * b[2 * sp.size + ind]));
          rad *= inv_r;
          last_f = fi;
        }
        const int am = mv < 0 ? -mv : mv;
        const double y = sp.lm_coef[lm] * P[l][am] * rad;
        const double cs = er[am], ss = mv < 0 ? -ei[am] : ei[am];
        val[sg.site_val + (long long)lm * sg.site_npts + (sg.pt_off - sg.site_pt) + pos] =
            make_float2((float)(y * cs), (float)(y * ss));
      }
      for (int kq = 0; kq < nkp; kq++) {
        const double *kf = kfrac + 3 * kq;
        double a = 0;
        for (int d = 0; d < 3; d++) a += kf[d] * (s.coord[d] + shift[d]);
        a = 2.0 * (a - rint(a));  // in units of pi, reduced to [-1, 1]
        double sv, cv;
        sincospi(a, &sv, &cv);
        phase[(long long)kq * npts + pt] = make_float2((float)cv, (float)sv);
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) base_s += chunk;
    __syncthreads();
  }
}

void launch_ae_count(const SiteDesc *sites, const int2 *slabs, int nslabs, const double *lattice, const int *fftg,
                     int *counts) {
  if (nslabs <= 0) return;
  PAWPY_LAUNCH("ae_tables", k_ae_count<<<nslabs, 256, 0, stream()>>>(sites, slabs, lattice, fftg, counts));
}

void launch_ae_fill(const SiteDesc *sites, const SegFill *segs, int nseg, const AeSpeciesDev *species,
                    const double *lattice, const int *fftg, const double *kfrac, int nkp, long long npts, int *cell,
                    float2 *val, float2 *phase) {
  if (nseg <= 0) return;
  PAWPY_LAUNCH("ae_tables", k_ae_fill<<<nseg, 128, 0, stream()>>>(sites, segs, species, lattice, fftg, kfrac, nkp,
                                                                   npts, cell, val, phase));
}

// grid[b][(g1 N2 + g2) N3 + g3] = C[b][t] at the wrapped plane-wave indices (grids zeroed
// before); grid (W / 256, nb)
__global__ void k_scatter_bands(const float2 *__restrict__ C, int Wpad, const int *__restrict__ g, int W, int N1,
                                int N2, int N3, float2 *__restrict__ grid) {
  const int b = blockIdx.y;
  const long long n3d = (long long)N1 * N2 * N3;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < W; t += gridDim.x * blockDim.x) {
    const int g1 = ((g[3 * t] % N1) + N1) % N1, g2 = ((g[3 * t + 1] % N2) + N2) % N2,
              g3 = ((g[3 * t + 2] % N3) + N3) % N3;
    grid[b * n3d + ((long long)g1 * N2 + g2) * N3 + g3] = C[(long long)b * Wpad + t];
  }
}

void launch_scatter_bands(const float2 *C, int Wpad, const int *gsorted, int W, int N1, int N2, int N3,
                          float2 *grid, int nb) {
  if (nb <= 0) return;
  PAWPY_CUDA(cudaMemsetAsync(grid, 0, sizeof(float2) * (size_t)nb * N1 * N2 * N3, stream()));
  if (W <= 0) return;
  dim3 g(ceil_div(W, 256), nb);
  PAWPY_LAUNCH("ae_grids", k_scatter_bands<<<g, 256, 0, stream()>>>(C, Wpad, gsorted, W, N1, N2, N3, grid));
}

// grid *= V^-1/2 exp(2 pi i k.(i/N1, j/N2, k/N3)) (fft3d's scale and realspace_state's Bloch
// factor, density.c:251-263); grid (N1 N2, nb)
__global__ void k_bloch(float2 *__restrict__ grid, int N1, int N2, int N3, double kx, double ky, double kz,
                        double scale) {
  const int ij = blockIdx.x, b = blockIdx.y;
  const int i = ij / N2, j = ij % N2;
  float2 *row = grid + ((long long)b * N1 * N2 + ij) * N3;
  const double base = kx * i / N1 + ky * j / N2;
  for (int k = threadIdx.x; k < N3; k += blockDim.x) {
    double a = base + kz * k / N3;
    a = 2.0 * (a - rint(a));
    double sv, cv;
    sincospi(a, &sv, &cv);
    const float2 x = row[k];
    const double re = x.x * scale, im = x.y * scale;
    row[k] = make_float2((float)(re * cv - im * sv), (float)(re * sv + im * cv));
  }
}

void launch_bloch(float2 *grid, int N1, int N2, int N3, const double *kfrac, double scale, int nb) {
  if (nb <= 0) return;
  dim3 g(N1 * N2, nb);
  PAWPY_LAUNCH("ae_grids", k_bloch<<<g, 128, 0, stream()>>>(grid, N1, N2, N3, kfrac[0], kfrac[1], kfrac[2], scale));
}

// grid[b][ucell[u]] += sum over the cell's entries e (site order) of
//   phase[k][pt_e] sum_n val[site_e][n][pt_e] P[b][pcol[site_e] + n]
// grid (ncell / 128, nb)
__global__ void k_ae_add(AeSpread c, const float2 *__restrict__ P, int Pstride, int kq, float2 *__restrict__ grid,
                         long long n3d) {
  const int b = blockIdx.y;
  const float2 *pb = P + (long long)b * Pstride;
  const float2 *ph = c.phase + (long long)kq * c.npts;
  for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < c.ncell; u += gridDim.x * blockDim.x) {
    float2 acc = make_float2(0.f, 0.f);
    for (int e = c.ent_first[u]; e < c.ent_first[u + 1]; e++) {
      const int s = c.ent_site[e];
      const long long pt = c.ent_pt[e];
      const int np = c.site_npts[s], T = c.site_total[s];
      const float2 *v = c.val + c.site_val[s] + (pt - c.site_pt[s]);
      const float2 *pp = pb + c.site_pcol[s];
      float2 y = make_float2(0.f, 0.f);
      for (int q = 0; q < T; q++) {
        const float2 a = __ldg(pp + q), w = __ldg(v + (long long)q * np);
        y.x += a.x * w.x - a.y * w.y;
        y.y += a.x * w.y + a.y * w.x;
      }
      const float2 f = __ldg(ph + pt);
      acc.x += y.x * f.x - y.y * f.y;
      acc.y += y.x * f.y + y.y * f.x;
    }
    float2 *x = grid + b * n3d + c.ucell[u];
    x->x += acc.x;
    x->y += acc.y;
  }
}

void launch_ae_add(const AeSpread &c, const float2 *P, int Pstride, int kq, float2 *grid, long long n3d, int nb) {
  if (nb <= 0 || c.ncell <= 0) return;
  dim3 g(ceil_div(c.ncell, 128), nb);
  PAWPY_LAUNCH("ae_grids", k_ae_add<<<g, 128, 0, stream()>>>(c, P, Pstride, kq, grid, n3d));
}

// rho[i] += sum_b w[b] |grid[b][i]|^2 in double precision, bands in order
__global__ void k_density(const float2 *__restrict__ grid, const double *__restrict__ w, int nb, long long n3d,
                          double *__restrict__ rho) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n3d; i += (long long)gridDim.x * blockDim.x) {
    double acc = rho[i];
    for (int b = 0; b < nb; b++) {
      const float2 x = grid[b * n3d + i];
      acc += w[b] * ((double)x.x * x.x + (double)x.y * x.y);
    }
    rho[i] = acc;
  }
}

void launch_density(const float2 *grid, const double *w, int nb, long long n3d, double *rho) {
  if (nb <= 0 || n3d <= 0) return;
  PAWPY_LAUNCH("ae_density", k_density<<<ceil_div(n3d, 256), 256, 0, stream()>>>(grid, w, nb, n3d, rho));
}

// x[i] *= exp(-2 pi i k.(i/N1, j/N2, k/N3)) in double precision (remove_phase)
__global__ void k_remove_phase(double2 *__restrict__ x, int N1, int N2, int N3, double kx, double ky, double kz) {
  const int ij = blockIdx.x;
  const int i = ij / N2, j = ij % N2;
  double2 *row = x + (long long)ij * N3;
  const double base = kx * i / N1 + ky * j / N2;
  for (int k = threadIdx.x; k < N3; k += blockDim.x) {
    double a = base + kz * k / N3;
    a = 2.0 * (a - rint(a));
    double sv, cv;
    sincospi(a, &sv, &cv);
    const double2 v = row[k];
    row[k] = make_double2(v.x * cv + v.y * sv, v.y * cv - v.x * sv);
  }
}

void launch_remove_phase(double2 *x, int N1, int N2, int N3, const double *kfrac) {
  dim3 g(N1 * N2);
  PAWPY_LAUNCH("ae_grids", k_remove_phase<<<g, 128, 0, stream()>>>(x, N1, N2, N3, kfrac[0], kfrac[1], kfrac[2]));
}

}  // namespace pawpy

// Launch wrappers of the device kernels of libpawpy_gpu (kernels.cu, gemm.cu).
#pragma once

#include <cuda_runtime.h>

#include "common.h"
#include "fft_block.cuh"

namespace pawpy {

// ---- coefficients ----
// C[b][t] = Cu[b][perm[t]] for t < W, 0 for W <= t < Wpad (b < nb)
void launch_permute(const float2 *Cu, int W, const int *perm, float2 *C, int Wpad, int nb);

// ---- FFT (backward, exp(+i)) ----
struct PlaneGeom {
  int N1, N2, N3;
  int g1min, n1;  // planes g1 in [g1min, g1min + n1)
};
// H[b][p][j*N3+k] = sum over the plane's coefficients (2D transform of plane p)
void launch_fft_planes(const float2 *C, int Wpad, const int *plane_start, const int *plane_off,
                       const PlaneGeom &g, const Radices &r2, const Radices &r3, const float2 *tw2,
                       const float2 *tw3, float2 *H, int nb);
// u[b][i][j][k] = scale * sum_p H[b][p][j][k] exp(2 pi i (g1min+p) i / N1)
void launch_fft_x(const float2 *H, const PlaneGeom &g, const Radices &r1, const float2 *tw1,
                  float scale, float2 *u, int nb);
// Generic in-place transform of full grids along one axis (single-band paths).
void launch_fft_axis(float2 *grid, int nb, int N1, int N2, int N3, int axis, const Radices &r,
                     const float2 *tw);
// Zero grid and scatter coefficients at (G mod N) (single-band paths).
void launch_scatter_grid(const int *Gs, const float2 *Cs, int nw, int N1, int N2, int N3, float2 *grid);
void launch_scale_to_c128(const float2 *grid, long n, double scale, double2 *out);

// ---- sphere tables (double precision tabulation) ----
struct SpeciesDev {      // radial data of one element, device pointers
  const double *f;       // [nfunc][size] values on the linear grid x_j = rmax_grid*j/size
  const double *spl;     // [nfunc][3][size] spline b,c,d
  int size;              // grid points (ndata)
  int nfunc;
  int total;             // lm channels
  double rmax;           // radius of the table: rmax (projectors) or wave_rmax (smooth)
  double grid_rmax;      // the linear grid's rmax
  int r0_size;           // proj_gridsize used for the cutoff denominator
  int lm_l[32], lm_m[32], lm_f[32];
};
struct SiteDesc {
  double coord[3];
  int species;
  int g[3], c[3];        // half box and centre (grid units)
  double R0;
  long long pt_off;      // first point of this site in the concatenated tables
  long long val_off;     // first table value of this site (tables are [total][npts] per site)
  int npts;
  int lm_off;            // first lm channel of this site in the output vector
  int total;
};
// pass 1: count points inside each sphere -> counts[s]
void launch_sphere_count(const SiteDesc *sites, int nsites, const double *lattice, const int *fftg,
                         int *counts);
// pass 2: indices, conj(radial*Ylm)*dV in lm-major tables, and exp(i k.path) for nkp k-points
void launch_sphere_fill(const SiteDesc *sites, int nsites, const SpeciesDev *species,
                        const double *lattice, const int *fftg, double dv, const double *kcart,
                        int nkp, long long total_pts, int *idx, float2 *tab, float2 *phase);
// P[b][lm_off+lm] = sum_pt tab[lm][pt] * u[b][idx[pt]] * phase[pt]  (one k-point)
void launch_sphere_gather(const SiteDesc *sites, int nsites, const int *idx, const float2 *tab,
                          const float2 *phase, const float2 *u, long long grid, float2 *P, int Ptot,
                          int nb, int max_total);

// ---- overlap GEMM (FP32 complex, SIMT) ----
// For each batch z < nz: out_z[n][m] = sum_k conj(A_z[m][k]) * B_z[n][k], with the K range split
// in two segments (A1/B1 of length K1, then A2/B2 of length K2; each a multiple of 16).
struct GemmBatch {
  const float2 *A1, *B1, *A2, *B2;
  long long lda1, ldb1, lda2, ldb2;  // row strides (elements)
  int K1, K2;                        // segment lengths, multiples of 16 (may differ per batch)
  float2 *out;                       // [N][M] row-major, leading dimension M
};
// One grouped launch over nz batches (uneven K allowed). splits > 1 needs a
// workspace of splits*nz*N*M float2 and reduces in split order.
void launch_zgemm_f32(const GemmBatch *batches_dev, int nz, int M, int N, int splits, float2 *workspace);

// ---- augmentation columns of the PAW terms ----
// A[kslice][b][c] = src[c] < Pt ? P[kslice][b][src[c]] : WP[kslice][b][src[c]-Pt]; zero for c >= Kc
void launch_aug_a(const float2 *P, int Pt, const float2 *WP, int Pw, int nb, int nk, const int *src, int Kc,
                  int Kcpad, double2 *A64, float2 *A32);
// B[k][b][c] = phase(k, pair[c]) * sum_e val[e] * (P|WP)[k][b0+b][col[e]] for bands b < nb
void launch_aug_b(const float2 *P, int Pt, const float2 *WP, int Pw, int nbtot, int b0, int nb, int nk,
                  const int *ptr, const int *col, const double2 *val, const int *pair, const double2 *phase,
                  int npairs, int Kc, int Kcpad, double2 *B64, float2 *B32);
// out[bS][bR][k] = (complex double) S[k][bS][bR]
void launch_to_host_layout(const float2 *S, int nk, int nbS, int nbR, double2 *out);
// out[bR][k] = S[k][band][bR]
void launch_extract_band(const float2 *S, int nk, int nbS, int nbR, int band, double2 *out);

// ---- compensation (FP64) ----
// out[m] (+)= sum_k conj(A[m][k]) * b[k] for rows m < M; K terms (complex double)
void launch_zgemv_f64(const double2 *A, long long lda, int M, int K, const double2 *b, double2 *out);

}  // namespace pawpy

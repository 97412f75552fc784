// Launch wrappers of the device kernels of libpawpy_gpu (kernels.cu, gemm.cu).
#pragma once

#include <cuda_runtime.h>

#include <mutex>
#include <vector>

#include "common.h"
#include "fft_block.cuh"

namespace pawpy {

// ---- coefficients ----
// C[b][t] = Cu[b][perm[t]] for t < W, 0 for W <= t < Wpad (b < nb)
void launch_permute(const float2 *Cu, int W, const int *perm, float2 *C, int Wpad, int nb);
// C[b][invperm[w]] = host_bands[b][w] read straight from pageable host memory (devices that
// access it through the host page tables), zero for the padding W <= t < Wpad
void launch_load_host_bands(const float2 *const *host_bands, int W, const int *invperm, float2 *C, int Wpad,
                            int nb);

// ---- FFT (backward, exp(+i)) ----
struct PlaneGeom {
  int N1, N2, N3;
  int g1min, n1;  // planes g1 in [g1min, g1min + n1)
  // rows g2 in [g2min, g2min + n2) and columns g3 in [g3min, g3min + n3)
  // (mod N2, N3) hold every coefficient of every plane
  int g2min = 0, n2 = 0, g3min = 0, n3 = 0;
  int maxcnt = 0;  // most coefficients in one plane
};
// H[b][p][j*N3+k] = sum over the plane's coefficients (2D transform of plane p)
void launch_fft_planes(const float2 *C, int Wpad, const int *plane_start, const int *plane_off,
                       const PlaneGeom &g, const Radices &r2, const Radices &r3, const float2 *tw2,
                       const float2 *tw3, float2 *H, int nb);
// The same two passes with register line transforms (fft_fast.cu) for the
// grid lengths compiled there; fft_fast_supported tells whether g is one.
bool fft_fast_supported(const PlaneGeom &g);
void launch_fft_planes_fast(const float2 *C, int Wpad, const int *plane_start, const int *plane_off,
                            const PlaneGeom &g, float2 *H, int nb);
struct GatherSeg;
// The sphere points in plane order: points [plane_first[j], plane_first[j + 1])
// lie in plane j of the second axis; cell is the point's offset i*LD + k in the
// transformed plane's shared tile (LD the padded row length), xo the position in
// the picked-point vector, phase[kq*npts + q] the Bloch phase.
// ent[q] = (offset of the point in the transformed plane's shared tile, offset of its value in
// a band's picked row: K-block word offset (pos / 16) * kb_words + pos % 16 of the split form,
// or the position pos in a complex64 row)
struct PickList {
  const int *plane_first = nullptr;
  uint2 *ent = nullptr;
  float2 *phase = nullptr;
  long long npts = 0;
  int max_plane_pts = 0;
};
// lo_words > 0: the rows are written in the split BF16 form (bf16split.cuh), lo plane lo_words
// 32-bit words after the hi plane
// gamma: the k-point is Gamma (every Bloch phase is 1, the phase list is not read)
void launch_fft_x_pick_fast(const float2 *H, const PlaneGeom &g, const PickList &pl, int kq, float2 *X,
                            long long xstride, int nb, long long lo_words = 0, bool gamma = false);
// the device's SM count (tc_gemm.cu)
int sm_count();
// pass B on the tensor cores (xpick_tc.cu): Gamma point, split rows (lo_words > 0), n1 <= 64,
// 2 N1 <= 256, N3 <= 128
bool xpick_tc_supported(const PlaneGeom &g);
void launch_xpick_tc(const float2 *H, const PlaneGeom &g, const PickList &pl, float2 *X, int nb, long long lo_words);
// Resident real-space wavefunctions of one k-point, bands in tiles of 16: the value of band b at
// cell c (= (x N2 + y) N3 + z) is at grid_value_index(b, c, n3d).
__host__ __device__ inline long long grid_value_index(int b, long long cell, long long n3d) {
  return ((long long)(b >> 4) * n3d + cell) * 16 + (b & 15);
}
// pass B writing whole grids of bands [b0, b0 + nb) of one k-point (register sizes only)
void launch_fft_x_grid(const float2 *H, const PlaneGeom &g, float2 *grid, int b0, int nb);
// fills pl.ent/phase from segments sorted by plane; base[si] = first flat position of segment si;
// kb_words > 0: row offsets of the split form (K blocks kb_words words apart), 0: complex64 rows
void launch_flatten_pick(const GatherSeg *segs, const int *base, int nsegs, int nkp, int N3, long long kb_words,
                         PickList &pl);
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
  // sqrt((2l+1)/(4 pi) (l-|m|)!/(l+|m|)!) of each channel, times (-1)^|m| (l-|m|)!/(l+|m|)!
  // for m < 0 (P_l^-|m| from P_l^|m|): Y_lm = lm_coef P_l^|m|(cos theta) e^{i m phi}
  double lm_coef[32];
  double h, inv_h;       // grid_rmax / size and its inverse (spline interval)
};
struct SiteDesc {
  double coord[3];
  int species;
  int g[3], c[3];        // half box and centre (grid units)
  double R0;             // sphere cutoff
  int lm_off;            // first lm channel of this site in the output vector
  int total;             // lm channels
};
// one slab of a site's box (fixed box row jb along the second axis) with points
struct SegFill {
  int site, jb;
  long long pt_off;      // first point of the segment in the set's point arrays
  int npts;
  long long site_pt;     // first point of the segment's site
  int site_npts;         // points of the site
  long long site_val;    // first table value of the site (tables are [total][site_npts] per site)
};
// a segment as the point pick sees it
struct GatherSeg {
  const int *idx;        // i*N3 + k inside the plane
  const float2 *phase;   // exp(i k.path): phase[kq*phase_stride + p]
  long long phase_stride;
  long long x_off;       // position of the segment's first point in the picked-point vector
  int npts;
};
// a chunk (<= CHUNK_PTS consecutive points) of one site as the contraction sees it
constexpr int CHUNK_PTS = 256;
struct ChunkContract {
  const float2 *tab;     // the site's table [total][site_npts], offset to the chunk's first point
  long long x_off;       // first point of the chunk in the picked-point vector
  int site_npts;         // row stride of the site's table
  int npts, total;
  int part_off;          // offset of the chunk's partial sums in the per-band partial vector
};
// Source of the staged contraction (launch_contract_staged): the picked-point
// rows X[row][xstride], or (grid != nullptr) the real-space grids of rows
// R = r0 + row ([R][n3d], R = k nband + band) read at gcell[xo] times
// gphase[k][xo] (npts points per k).
struct ContractSource {
  const float2 *X = nullptr;
  long long xstride = 0;
  long long xrows = 0;  // split form (tensor-core contraction): rows per plane of X
  const float2 *grid = nullptr;  // k-point kq at grid + kq gstride, grid_value_index layout
  long long n3d = 0, r0 = 0, npts = 0, gstride = 0;
  int nband = 1;
  bool gamma = false;  // every k-point of the rows is Gamma (all Bloch phases 1)
  const int *gcell = nullptr;
  const float2 *gphase = nullptr;
};
// partial[row][part_off + l] = sum over the chunk's points of source(row, point) * tab[l][point];
// npts (the merged point space) sizes the declared work
void launch_contract_staged(const ChunkContract *chunks, int nchunks, int max_total, const ContractSource &src,
                            float2 *partial, int ptot, int nb, long long npts);
// Tensor-core form of the contraction (sphere_tc.cu). One site of one set: its K range
// starts at the even point a_x of the merged point space and spans nkb blocks of 16 points;
// its table occupies rows [b_row, b_row + width) of the table planes; P of row R (global
// (k-point, band) row) is written to out[R * ld + c] for channels c < total.
struct TcSite {
  long long a_x = 0;
  int nkb = 0, b_row = 0, total = 0, ld = 0;
  float2 *out = nullptr;
};
// Source of one site's table planes: tab[c][npts] (site_npts stride), shifted by lead points.
struct TcTable {
  const float2 *tab = nullptr;
  int npts = 0, lead = 0, total = 0, nkb = 0, b_row = 0;
};
// Zeroes K blocks blocks[0..nblocks) of the split picked rows (rows [0, nb), both planes;
// kb_words 32-bit words from one block to the next).
void launch_zero_picked_blocks(float2 *X, const long long *blocks, int nblocks, long long kb_words, int nb,
                               long long lo_words);
// table width (2 x channels, padded) for the widest site: 32, 48 or 64
int tc_sphere_width(int max_total);
// BF16 hi/lo table planes [2][brows][lb] of every site
void launch_tc_tables(const TcTable *tabs_dev, int nsites, int max_nkb, int bn, int brows, long long lb,
                      void *planes);
// P of every site for the rows [r0, r0 + nb) of src (picked rows: xtot points per row)
void launch_tc_sphere(const TcSite *sites_dev, int nsites, int bn, const void *planes, int brows, long long lb,
                      const ContractSource &src, int nb, long long npts, long long xtot);
// the global cell and Bloch phase of every point of the merged point space
void launch_point_index(const GatherSeg *segs, const int *seg_j, int nsegs, int N2, int N3, int nkp, long long Q,
                        int *gcell, float2 *gphase);
// pass 1: count the inside points of every slab
void launch_slab_count(const SiteDesc *sites, const int2 *slabs, int nslabs, const double *lattice,
                       const int *fftg, int *counts);
// pass 2: compact and tabulate every non-empty slab (FP64, stored complex64)
// hmin: half the smallest lattice-plane spacing (points nearer their site skip the image search)
void launch_seg_fill(const SiteDesc *sites, const SegFill *segs, int nseg, const SpeciesDev *species,
                     const double *lattice, const int *fftg, double wscale, double hmin, const double *kcart, int nkp,
                     long long total_pts, int *idx, float2 *tab, float2 *phase, int what = 3);
// x-axis transform of each plane j of nb bands, then X[b][x_off + p] = u(point p) exp(i k.path_p) for
// the segments of plane j (segs sorted by plane; plane_start[N2+1])
// (npicked: the points the segments pick, for the launch's algorithmic bytes)
void launch_fft_x_pick(const float2 *H, const PlaneGeom &g, const Radices &r1, const float2 *tw1,
                       const GatherSeg *segs, const int *plane_start, int kq, float2 *X, long long xstride, int nb,
                       long long lo_words, long long npicked);
// P[(band_base + b)*Ptot + o] = sum over c < col[o].y of partial[b][col[o].x + c*col[o].z]: the
// chunks of column o's site, in chunk order
void launch_chunk_reduce(const float2 *partial, int ptot, const int4 *col, float2 *P, int Ptot, int nb,
                         long long band_base);

// ---- overlap GEMM (FP32 complex, SIMT) ----
// For each batch z < nz: out_z[n][m] = sum_k conj(A_z[m][k]) * B_z[n][k], with the K range split
// in two segments (A1/B1 of length K1, then A2/B2 of length K2; each a multiple of 16).
struct GemmBatch {
  const float2 *A1, *B1, *A2, *B2;
  long long lda1, ldb1, lda2, ldb2;  // row strides (elements)
  int K1, K2;                        // segment lengths, multiples of 16 (may differ per batch)
  float2 *out;                       // [N][M] row-major, leading dimension M
  // an optional third K segment (K3 = 0: none), after the first two
  const float2 *A3 = nullptr, *B3 = nullptr;
  long long lda3 = 0, ldb3 = 0;
  int K3 = 0;
};
// One grouped launch over nz batches (uneven K allowed). splits > 1 needs a
// workspace of splits*nz*N*M float2 and reduces in split order.
void launch_zgemm_f32(const GemmBatch *batches_dev, int nz, int M, int N, int splits, float2 *workspace);
// The same grouped contraction on the tensor cores (tc_gemm.cu): split-BF16
// 3-term (tf32 false) or TF32 operands, FP32 accumulation. hb is the host copy
// of batches_dev. splits_hint <= 0 picks the K split from the SM count.
// A pipeline wait of the kernel that ran out makes the next sync() throw.
// Tile width of the tensor-core contraction: 64 or 128 defect bands, 0 = timed per shape.
void set_tc_tile(int bn);
struct TcGemmInfo {
  int splits = 0, Kc = 0, ctas = 0, bn = 0;  // bn: defect bands per tile
};
// The split planes of the first segment of operand A (a resident basis's coefficients, the
// same device arrays call after call), built on the first call that gives it and read by the
// later ones (after ready): only the augmentation columns are split per call. Owned by the
// basis; one precision and shape (a call of another shape splits everything itself).
struct TcSplitCache {
  std::mutex mu;
  bool built = false, tf32 = false;
  int nz = 0, Mpad = 0, K1 = 0;
  std::vector<const float2 *> src;
  DevBuf<unsigned char> planes;
  cudaEvent_t ready = nullptr;
  ~TcSplitCache() {
    if (ready) cudaEventDestroy(ready);
  }
};
void launch_zgemm_tc(const GemmBatch *batches_dev, const std::vector<GemmBatch> &hb, int M, int N, bool tf32,
                     int splits_hint, TcGemmInfo *info, TcSplitCache *cacheA = nullptr);
// The two kernels behind launch_zgemm_f32 (64x64 tiles, 256 threads; grid (M/64, N/64, nz*splits)
// and (M*N/1024, nz)), for callers that launch them on their own stream.
__global__ void __launch_bounds__(256) k_zgemm_f32(const GemmBatch *batches, int M, int N, int splits,
                                                   float2 *ws, int nz);
__global__ void k_split_reduce(const GemmBatch *batches, const float2 *ws, int M, int N, int splits, int nz);
// The same two kernels for one batch whose descriptor is a launch argument (nothing
// read from device memory before the tile starts): grid (M/64, N/64, splits), and
// out[e] = sum over splits of ws[sp*M*N + e] in split order.
__global__ void __launch_bounds__(256) k_zgemm_f32_one(const GemmBatch bt, int M, int N, int splits, float2 *ws);
__global__ void k_split_reduce_one(float2 *out, const float2 *ws, int M, int N, int splits);

// ---- aug_recip augmentation coefficients (recip.cu) ----
// The sphere points of a set grouped per grid cell, per real-space plane j of
// the second axis: cells [cell_first[j], cell_first[j+1]) of plane j at
// ucell[u] = i*N3 + k, each summing the entries [ent_first[u], ent_first[u+1])
// (point ent_pt[e] of set site ent_site[e], in site order).
struct RecipSpread {
  const int *cell_first = nullptr, *ucell = nullptr, *ent_first = nullptr, *ent_site = nullptr;
  const long long *ent_pt = nullptr;
  const long long *site_pt = nullptr, *site_val = nullptr;  // per set site: first point, first table value
  const int *site_npts = nullptr, *site_total = nullptr;    // points, lm channels
  const int *site_pcol = nullptr;                           // first column of the site in the P rows
  const float2 *tab = nullptr;                              // the set's tables [total][site points] per site
  const float2 *phase = nullptr;                            // exp(i k.path) [nkp][npts]
  long long npts = 0;
};
// pass 1: H[b][p][j][k] = sum_i y_b(i, j, k) exp(+2 pi i g1(p) i / N1) with y_b the spread of band b
// (P rows [b][Pstride] of k-point kq); grid (N2 planes, nb bands)
void launch_recip_xspread(const RecipSpread &c, const float2 *P, int Pstride, int nkp, int kq, const PlaneGeom &g,
                          const Radices &r1, const float2 *tw1, float2 *H, int nb);
// pass 2: CA[b][t] = conj(2D backward transform of H[b][p] at coefficient t of plane p); D = C + CA when
// D is given; grid (n1 planes, nb bands)
void launch_recip_planes_pick(const float2 *H, const PlaneGeom &g, const int *pstart, const int *poff,
                              const Radices &r2, const Radices &r3, const float2 *tw2, const float2 *tw3,
                              const float2 *C, int Wpad, float2 *CA, float2 *D, int nb);

// ---- all-electron real-space wavefunctions (realspace.cu) ----
struct AeSpeciesDev {    // (phi - phit)(r) of one element on its logarithmic grid, device pointers
  const double *x;       // [size] the grid
  const double *f;       // [nfunc][size]
  const double *spl;     // [nfunc][3][size] spline b, c, d
  int size, nfunc, total;
  double logstep;        // log(x[1] / x[0])
  int lm_l[32], lm_m[32], lm_f[32];
  double lm_coef[32];    // as SpeciesDev
};
// The sphere points of a wavefunction's sites grouped per grid cell: cells ucell[u] (global
// (i N2 + j) N3 + k), each summing entries [ent_first[u], ent_first[u+1]) in site order.
struct AeSpread {
  int ncell = 0;
  const int *ucell = nullptr, *ent_first = nullptr, *ent_site = nullptr;
  const long long *ent_pt = nullptr;
  const long long *site_pt = nullptr, *site_val = nullptr;
  const int *site_npts = nullptr, *site_total = nullptr, *site_pcol = nullptr;
  const float2 *val = nullptr;    // [total][site points] per site: (phi - phit)/r Y_lm
  const float2 *phase = nullptr;  // [nkp][npts] exp(2 pi i k.(R + T))
  long long npts = 0;
};
void launch_ae_count(const SiteDesc *sites, const int2 *slabs, int nslabs, const double *lattice, const int *fftg,
                     int *counts);
void launch_ae_fill(const SiteDesc *sites, const SegFill *segs, int nseg, const AeSpeciesDev *species,
                    const double *lattice, const int *fftg, const double *kfrac, int nkp, long long npts, int *cell,
                    float2 *val, float2 *phase);
// nb zeroed grids [b][N1][N2][N3] with C[b][t] at the wrapped plane-wave indices gsorted[3t..3t+2]
void launch_scatter_bands(const float2 *C, int Wpad, const int *gsorted, int W, int N1, int N2, int N3,
                          float2 *grid, int nb);
// every grid point times scale exp(2 pi i k.(i/N1, j/N2, k/N3))
void launch_bloch(float2 *grid, int N1, int N2, int N3, const double *kfrac, double scale, int nb);
// the sphere terms of every band's projector coefficients (rows P[b][Pstride], k-point kq) added per cell
void launch_ae_add(const AeSpread &c, const float2 *P, int Pstride, int kq, float2 *grid, long long n3d, int nb);
// rho[i] += sum_b w[b] |grid[b][i]|^2 (double precision)
void launch_density(const float2 *grid, const double *w, int nb, long long n3d, double *rho);
// x[i] *= exp(-2 pi i k.r_frac) on a host-layout double grid
void launch_remove_phase(double2 *x, int N1, int N2, int N3, const double *kfrac);

// ---- augmentation columns of the PAW terms ----
// A[kslice][b][c] = src[c] < Pt ? P[kslice][b][src[c]] : WP[kslice][b][src[c]-Pt]; zero for c >= Kc
void launch_aug_a(const float2 *P, int Pt, const float2 *WP, int Pw, int nb, int nk, const int *src, int Kc,
                  int Kcpad, double2 *A64, float2 *A32);
// B[k][b][c] = phase(k, pair[c]) * sum_e val[e] * (P|WP)[k][b0+b][col[e]] for bands b < nb
void launch_aug_b(const float2 *P, int Pt, const float2 *WP, int Pw, int nbtot, int b0, int nb, int nk,
                  const int *ptr, const int *col, const double2 *val, const int *pair, const double2 *phase,
                  int npairs, int Kc, int Kcpad, double2 *B64, float2 *B32);
// val32[k][e] = val[e] (times phase[k][e_pair[e]] where e_pair[e] >= 0) in FP32, e < ne (zero from n on)
void launch_aug_val32(const double2 *val, const int *e_pair, int n, int ne, const double2 *phase, int npairs, int nk,
                      float2 *val32);
// FP32 form for the batched contraction: val32 [nk][nent] = entries times their column's pair phase
void launch_aug_b32(const float2 *P, int Pt, const float2 *WP, int Pw, int nbtot, int nb, int nk, const int *ptr,
                    const int *col, const float2 *val32, int nent, int Kc, int Kcpad, float2 *B32);
// out[bS][bR][k] = (complex double) S[k][bS][bR]
void launch_to_host_layout(const float2 *S, int nk, int nbS, int nbR, double2 *out);
// out[bR][k] = S[k][band][bR]
// v[bS*nch + ch] = sum over (bR, k) of channel ch of |S[k][bS][bR]|^2 wv[bR*nk + k], c likewise
// with wc; one channel (nch = 1) or two spin channels (nch = 2, k >= nwk is spin 1)
void launch_band_character(const float2 *S, int nk, int nbS, int nbR, const double *wv, const double *wc, int nwk,
                           int nch, double *v, double *c);
void launch_extract_band(const float2 *S, int nk, int nbS, int nbR, int band, double2 *out);

// ---- compensation (FP64) ----
// out[m] (+)= sum_k conj(A[m][k]) * b[k] for rows m < M; K terms (complex double)
void launch_zgemv_f64(const double2 *A, long long lda, int M, int K, const double2 *b, double2 *out);

}  // namespace pawpy

// Augmentation-sphere tables, the sphere-point pick fused into the last FFT
// pass, and the per-site contraction that gives <p_lm|psi>.
//
// A site's sphere (setup_site, utils.c:590-696) is cut into slabs: the grid
// points of its box with one fixed index j along the second lattice axis.
// Non-empty slabs are "segments". Tables are built per segment, in double
// precision, with the points of a segment in (i, k) order:
//   idx  = i*N3 + k (position inside the N1 x N3 plane j)
//   tab  = conj(p(r) Y_lm(theta, phi)) * dV * V^-1/2   [total][site points]
//   phase= exp(i k.path) for every k-point              [nkp][all points]
// (onto_projector_helper, projector.c:223-274, applies dV and exp(i k.path);
// fft3d, linalg.c:33-38, the V^-1/2 that is folded in here.)
//
// The x-axis FFT kernel owns one plane j of one band in shared memory after
// its transform and writes u(point) exp(i k.path) for every sphere point in
// that plane into a compact vector X (the real-space grid never goes to HBM).
// The contraction sum_p X[b][p] tab[lm][p] of each site then runs as a small
// register-blocked complex product over (bands x lm channels).
#include <cuda_runtime.h>

#include "bf16split.cuh"
#include "fft_tmpl.cuh"
#include "kernels.h"

namespace pawpy {

__device__ __forceinline__ void s_to_cart(const double *f, const double *L, double *o) {
  double t0 = f[0] * L[0] + f[1] * L[3] + f[2] * L[6];
  double t1 = f[0] * L[1] + f[1] * L[4] + f[2] * L[7];
  double t2 = f[0] * L[2] + f[1] * L[5] + f[2] * L[8];
  o[0] = t0;
  o[1] = t1;
  o[2] = t2;
}

// |v| rounded once, as the reference's pow(x, 0.5) (a correctly rounded square root) gives it
__device__ __forceinline__ double s_norm(const double *v) { return sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }

__device__ __forceinline__ int box_i(const SiteDesc &s, int a, int off) { return off - s.g[a] + s.c[a]; }

// grid point (i, j, k) of slab (site s, box row jb), linear (i,k) index q; returns inside and the path
__device__ __forceinline__ bool slab_point(const SiteDesc &s, int jb, int q, const double *L, const int *N,
                                           int *ijk, double *path) {
  int w2 = 2 * s.g[2] + 1;
  ijk[0] = box_i(s, 0, q / w2);
  ijk[1] = box_i(s, 1, jb);
  ijk[2] = box_i(s, 2, q % w2);
  double fr[3] = {(double)ijk[0] / N[0] - s.coord[0], (double)ijk[1] / N[1] - s.coord[1],
                  (double)ijk[2] / N[2] - s.coord[2]};
  s_to_cart(fr, L, path);
  return s_norm(path) < s.R0;
}

// Single-precision pre-test of slab_point: the displacement in grid units times the
// lattice rows over N, squared length against R0^2 widened by a relative margin of 1e-4
// (far above the single-precision error, about 1e-6 here). 1: inside, 0: outside, -1:
// within the margin (slab_point decides).
struct FastTest {
  float lf[9];   // L[a][c] / N[a]
  float cn[3];   // site position in grid units
  float r2lo, r2hi;
  __device__ void init(const SiteDesc &s, const double *L, const int *N) {
    // single precision throughout (every thread runs this; FP64 division is slow on this part)
    for (int a = 0; a < 3; a++) {
      cn[a] = (float)(s.coord[a] * N[a]);
      const float inv = 1.0f / (float)N[a];
      for (int c = 0; c < 3; c++) lf[3 * a + c] = (float)L[3 * a + c] * inv;
    }
    const double r2 = s.R0 * s.R0;
    r2lo = (float)(r2 * (1.0 - 1e-4));
    r2hi = (float)(r2 * (1.0 + 1e-4));
  }
  __device__ int test(const int *ijk) const {
    const float u0 = (float)ijk[0] - cn[0], u1 = (float)ijk[1] - cn[1], u2 = (float)ijk[2] - cn[2];
    const float x = u0 * lf[0] + u1 * lf[3] + u2 * lf[6];
    const float y = u0 * lf[1] + u1 * lf[4] + u2 * lf[7];
    const float z = u0 * lf[2] + u1 * lf[5] + u2 * lf[8];
    const float r2 = x * x + y * y + z * z;
    return r2 < r2lo ? 1 : (r2 > r2hi ? 0 : -1);
  }
};

// slab_point's verdict through the pre-test; the FP64 path only within the margin
__device__ __forceinline__ bool slab_inside(const SiteDesc &s, const FastTest &ft, int jb, int q, const double *L,
                                            const int *N) {
  const int w2 = 2 * s.g[2] + 1;
  const int ijk[3] = {box_i(s, 0, q / w2), box_i(s, 1, jb), box_i(s, 2, q % w2)};
  const int v = ft.test(ijk);
  if (v >= 0) return v == 1;
  int ijk2[3];
  double path[3];
  return slab_point(s, jb, q, L, N, ijk2, path);
}

__global__ void k_slab_count(const SiteDesc *__restrict__ sites, const int2 *__restrict__ slabs,
                             const double *__restrict__ Lg, const int *__restrict__ Ng, int *__restrict__ counts) {
  __shared__ int total;
  const int2 sl = slabs[blockIdx.x];
  const SiteDesc s = sites[sl.x];
  double L[9];
  int N[3] = {Ng[0], Ng[1], Ng[2]};
  for (int i = 0; i < 9; i++) L[i] = Lg[i];
  FastTest ft;
  ft.init(s, L, N);
  if (threadIdx.x == 0) total = 0;
  __syncthreads();
  int n = (2 * s.g[0] + 1) * (2 * s.g[2] + 1), c = 0;
  for (int q = threadIdx.x; q < n; q += blockDim.x)
    if (slab_inside(s, ft, sl.y, q, L, N)) c++;
  atomicAdd(&total, c);
  __syncthreads();
  if (threadIdx.x == 0) counts[blockIdx.x] = total;
}

void launch_slab_count(const SiteDesc *sites, const int2 *slabs, int nslabs, const double *lattice,
                       const int *fftg, int *counts) {
  if (nslabs <= 0) return;
  PAWPY_LAUNCH("sphere_count", k_slab_count<<<nslabs, 256, 0, stream()>>>(sites, slabs, lattice, fftg, counts));
}

// The table values of one inside point of a site (ijk: its unwrapped box position, path: the
// displacement from the site): conj(radial * Y_lm) * dV * V^-1/2 of every channel lm at
// tab[sg.site_val + lm site_npts + point], point = pos within the segment.
__device__ __forceinline__ void fill_point_tables(const SiteDesc &s, const SpeciesDev &sp, const SegFill &sg,
                                                  const double *L, const int *N, const int *ijk,
                                                  const double *path, double hmin, double wscale, int pos,
                                                  float2 *__restrict__ tab) {
  int ii = ((ijk[0] % N[0]) + N[0]) % N[0];
  int jj = ((ijk[1] % N[1]) + N[1]) % N[1];
  int kk = ((ijk[2] % N[2]) + N[2]) % N[2];
  // minimum-image displacement from the site to the wrapped grid point (utils.c:51-73):
  // nearer than hmin, the unwrapped box displacement is the unique minimum image;
  // otherwise search the 27 images
  double t[3] = {path[0], path[1], path[2]}, r = s_norm(path);
  if (!(r < hmin)) {
    // the image of least squared distance is the image of least distance (the square root
    // is monotone and correctly rounded), so one square root at the end gives the same r
    double gp[3] = {(double)ii / N[0], (double)jj / N[1], (double)kk / N[2]};
    double r2 = INFINITY;
    for (int a = -1; a <= 1; a++)
      for (int b = -1; b <= 1; b++)
        for (int c = -1; c <= 1; c++) {
          double f[3] = {gp[0] + a - s.coord[0], gp[1] + b - s.coord[1], gp[2] + c - s.coord[2]};
          double v[3];
          s_to_cart(f, L, v);
          double dd = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
          if (dd < r2) {
            r2 = dd;
            t[0] = v[0];
            t[1] = v[1];
            t[2] = v[2];
          }
        }
    r = sqrt(r2);
  }
  // Y_lm(theta, phi) of the displacement t without transcendental calls:
  // cos(theta) = t_z / r and exp(i phi) = (t_x + i t_y) / rho give the same angles the
  // reference takes from acos (utils.c:553-561; phi = 0 on the polar axis and at r = 0).
  // (FP64 division is slow on this part: one reciprocal each for r and rho)
  double ct = 1.0, cp = 1.0, sp_ = 0.0;
  if (r != 0) {
    ct = t[2] * (1.0 / r);
    double rho = sqrt(t[0] * t[0] + t[1] * t[1]);
    if (rho != 0 && r - fabs(t[2]) != 0) {
      const double irho = 1.0 / rho;
      cp = t[0] * irho;
      sp_ = t[1] * irho;
    }
  }
  // The channel values in single precision (the table is stored in single precision; the
  // geometry above and the spline index below stay in double precision)
  const float ctf = (float)ct, cpf = (float)cp, spf = (float)sp_;
  const float stf = sqrtf(fmaxf(0.f, (float)(1.0 - ct * ct)));
  // associated Legendre P_l^m (Condon-Shortley phase), 0 <= m <= l <= 3, by recurrence:
  // P_l^m = ((2l-1) ct P_{l-1}^m - (l+m-1) P_{l-2}^m) / (l-m)
  float P[4][4];
  P[0][0] = 1.f;
  for (int m = 1; m <= 3; m++) P[m][m] = -(2 * m - 1) * stf * P[m - 1][m - 1];
  for (int m = 0; m < 3; m++) P[m + 1][m] = (2 * m + 1) * ctf * P[m][m];
  P[2][0] = (3.f * ctf * P[1][0] - 1.f * P[0][0]) * 0.5f;
  P[3][0] = (5.f * ctf * P[2][0] - 2.f * P[1][0]) * (1.f / 3.f);
  P[3][1] = (5.f * ctf * P[2][1] - 3.f * P[1][1]) * 0.5f;
  float er[4] = {1.f, cpf, 0.f, 0.f}, ei[4] = {0.f, spf, 0.f, 0.f};
  for (int m = 2; m <= 3; m++) {
    er[m] = er[m - 1] * cpf - ei[m - 1] * spf;
    ei[m] = er[m - 1] * spf + ei[m - 1] * cpf;
  }
  // linear-grid spline interpolation (proj_interpolate, utils.c:461-475); x_j = rmax/size*j
  double xlast = sp.h * (sp.size - 1);
  int ind = (int)(r * sp.inv_h);
  if (ind > sp.size - 2) ind = sp.size - 2;
  const float dd = (float)(r - sp.h * ind);
  const float ws = (float)wscale;
  float rad = 0.f;
  int last_f = -1;
  for (int lm = 0; lm < sp.total; lm++) {
    int l = sp.lm_l[lm], mm = sp.lm_m[lm], fi = sp.lm_f[lm];
    if (fi != last_f) {
      const double *f = sp.f + (long long)fi * sp.size;
      const double *sb = sp.spl + (long long)fi * 3 * sp.size;
      rad = r > xlast ? 0.f
                      : (float)f[ind] + dd * ((float)sb[ind] + dd * ((float)sb[sp.size + ind] +
                                                                      dd * (float)sb[2 * sp.size + ind]));
      last_f = fi;
    }
    int am = mm < 0 ? -mm : mm;
    float plm = l <= 3 ? P[l][am] : 0.f;
    // lm_coef carries the m < 0 factor of P_l^{-|m|} (utils.c:379-380)
    float y = (float)sp.lm_coef[lm] * plm * rad * ws;
    float cs = er[am], sn = mm < 0 ? -ei[am] : ei[am];
    // conj(radial * Y_lm) * dV * V^-1/2
    tab[sg.site_val + (long long)lm * sg.site_npts + (sg.pt_off - sg.site_pt) + pos] = make_float2(y * cs, -y * sn);
  }
}

// One CTA per segment: compact the slab's inside points in (i, k) order and
// tabulate them (double precision, rounded to complex64 at the end).
__global__ void k_seg_fill(const SiteDesc *__restrict__ sites, const SegFill *__restrict__ segs,
                           const SpeciesDev *__restrict__ species, const double *__restrict__ Lg,
                           const int *__restrict__ Ng, double wscale, double hmin,
                           const double *__restrict__ kcart, int nkp,
                           long long total_pts, int *__restrict__ idx, float2 *__restrict__ tab,
                           float2 *__restrict__ phase, int what) {
  __shared__ int warp_cnt[32];
  __shared__ int base_s;
  __shared__ double invN[3];
  const SegFill sg = segs[blockIdx.x];
  const SiteDesc s = sites[sg.site];
  const SpeciesDev &sp = species[s.species];
  double L[9];
  int N[3] = {Ng[0], Ng[1], Ng[2]};
  for (int i = 0; i < 9; i++) L[i] = Lg[i];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  FastTest ft;
  ft.init(s, L, N);
  if (threadIdx.x == 0) {
    base_s = 0;
    for (int a = 0; a < 3; a++) invN[a] = 1.0 / N[a];
  }
  __syncthreads();
  if (what == 2 && 2 * s.g[0] + 1 <= N[0] && 2 * s.g[2] + 1 <= N[2]) {
    // tables alone, after the index fill: the segment's inside points are idx[pt_off + pos]
    // (wrapped cells i N3 + k, each the image of exactly one box point, the box being no wider
    // than the cell): one thread per point, the same displacement and values as below
    const int lo0 = box_i(s, 0, 0), lo2 = box_i(s, 2, 0);
    for (int pos = threadIdx.x; pos < sg.npts; pos += blockDim.x) {
      const int c = idx[sg.pt_off + pos], ii = c / N[2], kk = c - ii * N[2];
      const int ijk[3] = {lo0 + ((ii - lo0) % N[0] + N[0]) % N[0], box_i(s, 1, sg.jb),
                          lo2 + ((kk - lo2) % N[2] + N[2]) % N[2]};
      const double fr[3] = {ijk[0] * invN[0] - s.coord[0], ijk[1] * invN[1] - s.coord[1],
                            ijk[2] * invN[2] - s.coord[2]};
      double path[3];
      s_to_cart(fr, L, path);
      fill_point_tables(s, sp, sg, L, N, ijk, path, hmin, wscale, pos, tab);
    }
    return;
  }
  const int n = (2 * s.g[0] + 1) * (2 * s.g[2] + 1);
  const int w2 = 2 * s.g[2] + 1;
  for (int start = 0; start < n; start += blockDim.x) {
    int q = start + threadIdx.x;
    int ijk[3];
    double path[3];
    bool in = q < n && slab_inside(s, ft, sg.jb, q, L, N);
    if (in) {
      // the displacement of an inside point (its membership was decided exactly above)
      ijk[0] = box_i(s, 0, q / w2);
      ijk[1] = box_i(s, 1, sg.jb);
      ijk[2] = box_i(s, 2, q % w2);
      const double fr[3] = {ijk[0] * invN[0] - s.coord[0], ijk[1] * invN[1] - s.coord[1],
                            ijk[2] * invN[2] - s.coord[2]};
      s_to_cart(fr, L, path);
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
    // what & 1: the point's plane index and Bloch phases (the pick needs only these); what & 2:
    // its table values
    if (in && pos < sg.npts && (what & 1)) {
      const int ii = ((ijk[0] % N[0]) + N[0]) % N[0];
      const int kk = ((ijk[2] % N[2]) + N[2]) % N[2];
      idx[sg.pt_off + pos] = ii * N[2] + kk;
    }
    if (in && pos < sg.npts && (what & 2)) fill_point_tables(s, sp, sg, L, N, ijk, path, hmin, wscale, pos, tab);
    if (in && pos < sg.npts && (what & 1)) {
      // exp(i k.path): the argument in units of pi reduced to [-1, 1] in double precision,
      // then the single-precision sincospi (the phase is stored in single precision)
      for (int kq = 0; kq < nkp; kq++) {
        double kr = kcart[3 * kq] * path[0] + kcart[3 * kq + 1] * path[1] + kcart[3 * kq + 2] * path[2];
        double u = kr * 0.31830988618379067154;  // 1 / pi
        u -= 2.0 * rint(0.5 * u);
        float sn, cs;
        sincospif((float)u, &sn, &cs);
        phase[(long long)kq * total_pts + sg.pt_off + pos] = make_float2(cs, sn);
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) base_s += chunk;
    __syncthreads();
  }
}

void launch_seg_fill(const SiteDesc *sites, const SegFill *segs, int nseg, const SpeciesDev *species,
                     const double *lattice, const int *fftg, double wscale, double hmin, const double *kcart, int nkp,
                     long long total_pts, int *idx, float2 *tab, float2 *phase, int what) {
  if (nseg <= 0) return;
  PAWPY_LAUNCH("sphere_fill", k_seg_fill<<<nseg, 128, 0, stream()>>>(sites, segs, species, lattice, fftg, wscale,
                                                                    hmin, kcart, nkp, total_pts, idx, tab, phase,
                                                                    what));
}

// ---------------------------------------------------------------------------
// x-axis transform of plane j, then pick the sphere points lying in it.

__global__ void __launch_bounds__(256) k_fft_x_pick(const float2 *__restrict__ H, PlaneGeom g, Radices r1,
                                                    const float2 *__restrict__ tw1g,
                                                    const GatherSeg *__restrict__ segs,
                                                    const int *__restrict__ plane_start, int kq,
                                                    float2 *__restrict__ X, long long xstride, long long lo_words) {
  extern __shared__ float2 sm[];
  const int tile = g.N1 * g.N3;
  float2 *a = sm, *b = sm + tile, *tw1 = sm + 2 * tile;
  const int j = blockIdx.x, band = blockIdx.y;
  for (int i = threadIdx.x; i < g.N1; i += blockDim.x) tw1[i] = tw1g[i];
  for (int i = threadIdx.x; i < tile; i += blockDim.x) {
    int row = i / g.N3, k = i - row * g.N3;
    int p = row - g.g1min;
    p = ((p % g.N1) + g.N1) % g.N1;
    float2 v = make_float2(0.f, 0.f);
    if (p < g.n1) v = H[(((long long)band * g.n1 + p) * g.N2 + j) * g.N3 + k];
    a[i] = v;
  }
  __syncthreads();
  const float2 *u = block_fft_any<1, false>(a, b, r1, g.N3, 1, g.N3, tw1);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  for (int si = plane_start[j] + warp; si < plane_start[j + 1]; si += nwarp) {
    const GatherSeg sg = segs[si];
    const float2 *ph = sg.phase + (long long)kq * sg.phase_stride;
    for (int p = lane; p < sg.npts; p += 32)
      put_picked(X, band, xstride, lo_words, (int)(sg.x_off + p), cmul(u[sg.idx[p]], ph[p]));
  }
}

void launch_fft_x_pick(const float2 *H, const PlaneGeom &g, const Radices &r1, const float2 *tw1,
                       const GatherSeg *segs, const int *plane_start, int kq, float2 *X, long long xstride, int nb,
                       long long lo_words, long long npicked) {
  if (nb <= 0) return;
  size_t smem = sizeof(float2) * (2 * (size_t)g.N1 * g.N3 + g.N1);
  PAWPY_REQUIRE(smem <= 227 * 1024, "FFT tile does not fit in shared memory");
  allow_dynamic_smem((const void *)k_fft_x_pick, smem);
  dim3 grid(g.N2, nb);
  PAWPY_LAUNCH("fft_x_pick", k_fft_x_pick<<<grid, 256, smem, stream()>>>(H, g, r1, tw1, segs, plane_start, kq, X,
                                                                        xstride, lo_words));
  note_work("fft_x_pick", 8.0 * ((double)g.n1 * g.N2 * g.N3 + (double)npicked) * nb);
}

// ---------------------------------------------------------------------------
// <p_lm|psi_b> = sum_p X[b][p] tab[lm][p], chunk by chunk (the sum over the
// grid points of one site in onto_projector, projector.c:266-311, for every
// band at once). A chunk is <= CHUNK_PTS points of one site with a compile-time
// bound of 8, 18 or 32 lm channels.
//
// One CTA per (chunk, block of TC rows), one row per thread. The chunk's points
// are taken in tiles of TP: the tile's picked values are copied with cp.async,
// each warp reading along points (consecutive addresses) into shared memory
// transposed to [point][row], so that the row threads read them conflict-free;
// the tile's table slice [lm][point] is read as broadcasts. Tiles are
// double-buffered: the copies of tile t + 1 are in flight while tile t is
// summed. Two sources: the rows of the picked-point vector X (the projection
// pass's output) or, for a wavefunction held in real space, its grid values at
// the points' cells (the pick itself, fused: no X is written); there the CTA's
// rows belong to one k-point and its Bloch phase is folded into the staged
// table slice.
namespace {
constexpr int TC = 128;          // rows per CTA
constexpr int TP = 16;           // points per staged tile (divides 32)
constexpr int XS = TC + 1;       // row stride of a staged tile (float2)

__device__ __forceinline__ void cpa8(void *dst, const void *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(static_cast<uint32_t>(__cvta_generic_to_shared(dst))),
               "l"(src)
               : "memory");
}
__device__ __forceinline__ void cpa_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cpa_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
}  // namespace

template <int NL, bool GATHER>
__global__ void __launch_bounds__(TC) k_contract_staged(const ChunkContract *__restrict__ chunks,
                                                        ContractSource src, float2 *__restrict__ partial, int ptot,
                                                        int nb) {
  extern __shared__ float4 smem4[];
  float2 *xs = reinterpret_cast<float2 *>(smem4);  // [2][TP][XS]
  float2 *tt = xs + 2 * TP * XS;                   // [2][NL][TP]
  const ChunkContract cc = chunks[blockIdx.x];
  const int n = cc.npts;
  // rows [row0, row1) of the batch; with GATHER a block never crosses a k-point
  int row0, row1;
  long long kq = 0;
  if (GATHER) {
    const int bpk = (src.nband + TC - 1) / TC;
    kq = src.r0 / src.nband + blockIdx.y / bpk;
    const long long lo = kq * src.nband + (long long)(blockIdx.y % bpk) * TC;  // global row
    const long long hi = min(min(lo + TC, (kq + 1) * src.nband), src.r0 + nb);
    row0 = (int)(max(lo, src.r0) - src.r0);
    row1 = (int)(hi - src.r0);
  } else {
    row0 = blockIdx.y * TC;
    row1 = min(row0 + TC, nb);
  }
  const int nrows = row1 - row0;
  if (nrows <= 0) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ntiles = (n + TP - 1) / TP;

  auto load_tile = [&](int t, int buf) {
    const int p0 = t * TP;
    float2 *tb = tt + buf * NL * TP;
    for (int e = threadIdx.x; e < NL * TP; e += TC) {
      const int l = e / TP, q = e - l * TP, pp = p0 + q;
      float2 v = make_float2(0.f, 0.f);
      if (l < cc.total && pp < n) {
        v = cc.tab[(long long)l * cc.site_npts + pp];
        if (GATHER) {
          const float2 f = src.gphase[kq * src.npts + cc.x_off + pp];
          v = make_float2(v.x * f.x - v.y * f.y, v.x * f.y + v.y * f.x);
        }
      }
      tb[e] = v;
    }
    // a warp instruction copies 32 / TP rows of TP points: lane -> (point pl, row rfirst + k RSTEP)
    const int pl = lane % TP, rsub = lane / TP;
    constexpr int RSTEP = (TC / 32) * (32 / TP);  // rows per pass of the whole CTA
    const int p = p0 + pl;
    if (p < n) {
      const long long xo = cc.x_off + p;
      float2 *dst = xs + ((long long)buf * TP + pl) * XS;
      const int rfirst = warp * (32 / TP) + rsub;
      if (GATHER) {
        const float2 *gk = src.grid + kq * src.gstride;
        const int b0 = (int)(src.r0 + row0 - kq * src.nband);
        const int cell = src.gcell[xo];
        for (int r = rfirst; r < nrows; r += RSTEP) cpa8(dst + r, gk + grid_value_index(b0 + r, cell, src.n3d));
      } else {
        const float2 *x = src.X + (long long)row0 * src.xstride + xo;
        for (int r = rfirst; r < nrows; r += RSTEP) cpa8(dst + r, x + (long long)r * src.xstride);
      }
    }
    cpa_commit();
  };

  float ar[NL], ai[NL];
#pragma unroll
  for (int l = 0; l < NL; l++) ar[l] = ai[l] = 0.f;
  load_tile(0, 0);
  for (int t = 0; t < ntiles; t++) {
    const int buf = t & 1;
    if (t + 1 < ntiles) {
      load_tile(t + 1, buf ^ 1);
      cpa_wait<1>();
    } else {
      cpa_wait<0>();
    }
    __syncthreads();  // tile t (copies and table slice) is visible to every thread
    const int m = min(TP, n - t * TP);
    const float2 *xt = xs + (long long)buf * TP * XS + threadIdx.x;
    const float2 *tb = tt + buf * NL * TP;
    int q = 0;
    for (; q + 1 < m; q += 2) {
      const float2 v0 = xt[q * XS], v1 = xt[(q + 1) * XS];
#pragma unroll
      for (int l = 0; l < NL; l++) {
        const float4 w = *reinterpret_cast<const float4 *>(tb + l * TP + q);
        ar[l] = fmaf(w.x, v0.x, fmaf(-w.y, v0.y, ar[l]));
        ai[l] = fmaf(w.x, v0.y, fmaf(w.y, v0.x, ai[l]));
        ar[l] = fmaf(w.z, v1.x, fmaf(-w.w, v1.y, ar[l]));
        ai[l] = fmaf(w.z, v1.y, fmaf(w.w, v1.x, ai[l]));
      }
    }
    if (q < m) {
      const float2 v0 = xt[q * XS];
#pragma unroll
      for (int l = 0; l < NL; l++) {
        const float2 w = tb[l * TP + q];
        ar[l] = fmaf(w.x, v0.x, fmaf(-w.y, v0.y, ar[l]));
        ai[l] = fmaf(w.x, v0.y, fmaf(w.y, v0.x, ai[l]));
      }
    }
    __syncthreads();  // tile t is consumed before tile t + 2 overwrites its buffer
  }
  if ((int)threadIdx.x >= nrows) return;
  float2 *o = partial + (long long)(row0 + threadIdx.x) * ptot + cc.part_off;
#pragma unroll
  for (int l = 0; l < NL; l++)
    if (l < cc.total) o[l] = make_float2(ar[l], ai[l]);
}

template <int NL, bool GATHER>
static void contract_staged(const ChunkContract *chunks, int nchunks, const ContractSource &src, float2 *partial,
                            int ptot, int nb) {
  const size_t smem = sizeof(float2) * (2 * (size_t)TP * XS + 2 * (size_t)NL * TP);
  allow_dynamic_smem((const void *)k_contract_staged<NL, GATHER>, smem);
  int blocks_y = ceil_div(nb, TC);
  if (GATHER) {
    // row blocks per k-point, over the k-points the batch [r0, r0 + nb) touches
    const long long k0 = src.r0 / src.nband, k1 = (src.r0 + nb - 1) / src.nband;
    blocks_y = (int)(k1 - k0 + 1) * ceil_div(src.nband, TC);
  }
  dim3 grid(nchunks, blocks_y);
  PAWPY_LAUNCH("sphere_contract",
               (k_contract_staged<NL, GATHER><<<grid, TC, smem, stream()>>>(chunks, src, partial, ptot, nb)));
}

void launch_contract_staged(const ChunkContract *chunks, int nchunks, int max_total, const ContractSource &src,
                            float2 *partial, int ptot, int nb, long long npts) {
  if (nchunks <= 0 || nb <= 0) return;
  note_work("sphere_contract", 8.0 * (double)npts * nb);
  if (max_total > 32) throw Error(ERR_UNSUPPORTED, "more than 32 projector channels on one site");
  const bool gather = src.grid != nullptr;
  PAWPY_REQUIRE(gather || src.X, "contraction without a source");
  PAWPY_REQUIRE(!gather || src.nband > 0, "contraction source without a band count");
  if (max_total <= 8)
    gather ? contract_staged<8, true>(chunks, nchunks, src, partial, ptot, nb)
           : contract_staged<8, false>(chunks, nchunks, src, partial, ptot, nb);
  else if (max_total <= 18)
    gather ? contract_staged<18, true>(chunks, nchunks, src, partial, ptot, nb)
           : contract_staged<18, false>(chunks, nchunks, src, partial, ptot, nb);
  else
    gather ? contract_staged<32, true>(chunks, nchunks, src, partial, ptot, nb)
           : contract_staged<32, false>(chunks, nchunks, src, partial, ptot, nb);
}

// gcell[xo] = (i N2 + j) N3 + k and gphase[kq][xo] = the segment's Bloch phase, for every point xo
// of the merged point space (segment si lies in plane seg_j[si] of the second axis)
__global__ void k_point_index(const GatherSeg *__restrict__ segs, const int *__restrict__ seg_j, int N2, int N3,
                              int nkp, long long Q, int *__restrict__ gcell, float2 *__restrict__ gphase) {
  const GatherSeg sg = segs[blockIdx.x];
  const int j = seg_j[blockIdx.x];
  for (int p = threadIdx.x; p < sg.npts; p += blockDim.x) {
    const int c = sg.idx[p], i = c / N3, k = c - i * N3;
    const long long xo = sg.x_off + p;
    gcell[xo] = (i * N2 + j) * N3 + k;
    for (int q = 0; q < nkp; q++) gphase[q * Q + xo] = sg.phase[q * sg.phase_stride + p];
  }
}

void launch_point_index(const GatherSeg *segs, const int *seg_j, int nsegs, int N2, int N3, int nkp, long long Q,
                        int *gcell, float2 *gphase) {
  if (nsegs <= 0) return;
  PAWPY_LAUNCH("pick_list", k_point_index<<<nsegs, 128, 0, stream()>>>(segs, seg_j, N2, N3, nkp, Q, gcell, gphase));
}

// P[(band_base + b) * Ptot + o] = sum over the chunks c < n of the column's
// site of partial[b][first + c * stride] (col = {first, n, stride}), in chunk
// order. Grid (Ptot / 128, bands).
__global__ void k_chunk_reduce(const float2 *__restrict__ partial, int ptot, const int4 *__restrict__ col,
                               float2 *__restrict__ P, int Ptot, int nb, long long band_base) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (o >= Ptot || b >= nb) return;
  const int4 c = col[o];
  const float2 *pb = partial + (long long)b * ptot + c.x;
  float re = 0.f, im = 0.f;
  for (int e = 0; e < c.y; e++) {
    const float2 v = pb[e * c.z];
    re += v.x;
    im += v.y;
  }
  P[(band_base + b) * Ptot + o] = make_float2(re, im);
}

void launch_chunk_reduce(const float2 *partial, int ptot, const int4 *col, float2 *P, int Ptot, int nb,
                         long long band_base) {
  if (Ptot <= 0 || nb <= 0) return;
  dim3 grid(ceil_div(Ptot, 128), nb);
  PAWPY_LAUNCH("sphere_reduce",
               k_chunk_reduce<<<grid, 128, 0, stream()>>>(partial, ptot, col, P, Ptot, nb, band_base));
}

}  // namespace pawpy

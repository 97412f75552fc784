// Radial (per-element) setup of the PAW datasets on the device, in double
// precision: get_projector_list (projector.c:20-171) with the spherical Bessel
// transforms of sbt.c:24-215 (Talman, Comput. Phys. Commun. 180 (2009) 332)
// and make_pwave_overlap_matrices (projector.c:507-558).
//
// The parallel, transcendental-heavy part runs on the device: the transform's
// multiplier table (one thread per t) and the forward and inverse Bessel
// transforms (one CTA per function, 2N-point FP64 FFT in shared memory with
// tabulated twiddles). The O(n) serial recurrences (cubic-spline solves, the
// running-product grid, spline integrals) stay on the calling host core: a
// single GPU thread runs such FP64 dependency chains far slower than a CPU
// core. The result is returned once, in ppot_t structs with the reference's
// layout and ownership (the ABI returns host structs).
#include <cuda_runtime.h>

#include <atomic>
#include <cstring>
#include <mutex>

#include <cmath>
#include <cstdlib>
#include <map>
#include <vector>

#include "host.h"
#include "kernels.h"

namespace pawpy {

namespace {

struct ElemDev {
  int ngrid, lmax;
  const double *wave_grid;  // [ngrid]
  double *ks, *rs;          // [2 ngrid]
  double2 *M;               // [(lmax+1)][2 ngrid]
  double2 *tw;              // [2 ngrid] exp(+2 pi i m / 2 ngrid)
};

struct FuncDev {
  int elem, l;
  const double *diff;  // [ngrid] r*(phi - phit)
  double *kwave;       // [ngrid]
  double *smooth;      // [ngrid] inverse transform of the filtered kwave, on the dense grid
};

// transform grids and twiddles of each element (one CTA per element)
__global__ void k_rad_grids(ElemDev *__restrict__ els, double encut_sbt) {
  ElemDev e = els[blockIdx.x];
  int N = 2 * e.ngrid;
  double drho = log(e.wave_grid[1] / e.wave_grid[0]);
  double kmin = pow(encut_sbt * 0.262465831, 0.5) * exp(-(N / 2 - 1) * drho);
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    e.ks[i] = kmin * exp(i * drho);
    e.rs[i] = e.wave_grid[0] * exp((i - N / 2) * drho);
    double s, c;
    sincospi(2.0 * i / N, &s, &c);
    e.tw[i] = make_double2(c, s);
  }
}

// multiplier table M_l(t) of the transform (sbt.c:47-86): arg Gamma(1/2 + i t) by a
// 10-step shift and Stirling's series; one thread per t, all l
__global__ void k_rad_mtable(ElemDev *__restrict__ els, double encut_sbt) {
  ElemDev e = els[blockIdx.y];
  int N = 2 * e.ngrid;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  int lmax = e.lmax == 0 ? 1 : e.lmax;
  double drho = log(e.wave_grid[1] / e.wave_grid[0]);
  double dt = 2 * M_PI / N / drho;
  double kmin = pow(encut_sbt * 0.262465831, 0.5) * exp(-(N / 2 - 1) * drho);
  double kappamin = log(kmin);
  double rhomin = log(e.wave_grid[0] * exp((0 - N / 2) * drho));
  double t = i * dt;
  double rad = sqrt(10.5 * 10.5 + t * t);
  double ph = atan((2 * t) / 21);
  double g = -10 * ph - t * log(rad) + t + sin(ph) / (12 * rad) - sin(3 * ph) / (360 * pow(rad, 3.0)) +
             sin(5 * ph) / (1260 * pow(rad, 5.0)) - sin(7 * ph) / (1680 * pow(rad, 7.0));
  for (int j = 1; j <= 10; j++) g += atan((2 * t) / (2 * j - 1));
  double h = -atan(tanh(M_PI * t / 2));
  double phase = g + h + (kappamin + rhomin) * t;
  double mag = sqrt(M_PI / 2) / N * (i == 0 ? 0.5 : 1.0);
  double s, c;
  sincos(phase, &s, &c);
  double2 m0 = make_double2(mag * c, mag * s);
  e.M[i] = m0;
  double a = 2 * (-h - atan(2 * t));
  sincos(a, &s, &c);
  e.M[N + i] = make_double2(c * m0.x - s * m0.y, c * m0.y + s * m0.x);
  for (int l = 1; l < lmax; l++) {
    double b = 2 * -atan(2 * t / (2 * l + 1));
    sincos(b, &s, &c);
    double2 p = e.M[(l - 1) * N + i];
    e.M[(l + 1) * N + i] = make_double2(c * p.x - s * p.y, c * p.y + s * p.x);
  }
}

__device__ __forceinline__ double2 zmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// exp(+i) unnormalised transform of x[n] in shared memory (Stockham; radix 4
// first, then primes; a prime factor above 16 becomes one direct stage that
// reads its inputs from shared memory). tw[m] = exp(+2 pi i m/n).
__device__ double2 *d_block_fft(double2 *x, double2 *y, int n, const double2 *tw) {
  int span = 1;
  double2 *src = x, *dst = y;
  int m = n;
  while (m > 1) {
    int R = (m % 4 == 0) ? 4 : 2;
    if (m % R) {
      R = 3;
      while (m % R) R += 2;
    }
    const int M = n / R, tstep = n / (span * R), rstep = n / R;
    for (int j = threadIdx.x; j < M; j += blockDim.x) {
      int k = j % span;
      int base = (j / span) * span * R + k;
      if (R <= 16) {
        double2 v[16];
        for (int r = 0; r < R; r++) {
          double2 a = src[j + r * M];
          if (r > 0 && k > 0) a = zmul(a, tw[k * r * tstep]);
          v[r] = a;
        }
        for (int q = 0; q < R; q++) {
          double2 acc = v[0];
          for (int r = 1; r < R; r++) {
            double2 w = tw[((r * q) % R) * rstep];
            acc.x += v[r].x * w.x - v[r].y * w.y;
            acc.y += v[r].x * w.y + v[r].y * w.x;
          }
          dst[base + q * span] = acc;
        }
      } else {
        for (int q = 0; q < R; q++) {
          double2 acc = make_double2(0, 0);
          for (int r = 0; r < R; r++) {
            double2 a = zmul(src[j + r * M], tw[(k * r * tstep) % n]);
            double2 w = tw[((r * q) % R) * rstep];
            acc.x += a.x * w.x - a.y * w.y;
            acc.y += a.x * w.y + a.y * w.x;
          }
          dst[base + q * span] = acc;
        }
      }
    }
    __syncthreads();
    double2 *t = src;
    src = dst;
    dst = t;
    span *= R;
    m /= R;
  }
  return src;
}

// forward transform of r*(phi - phit) (sbt.c:102-154): one CTA per function
__global__ void k_sbt_forward(const ElemDev *__restrict__ els, const FuncDev *__restrict__ fns) {
  extern __shared__ double2 zs[];
  const FuncDev fn = fns[blockIdx.x];
  const ElemDev e = els[fn.elem];
  const int N = 2 * e.ngrid, n = e.ngrid, l = fn.l;
  double2 *a = zs, *b = zs + N;
  double C = fn.diff[0] / pow(e.rs[n], l + 1.0);
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    double f = i < n ? C * pow(e.rs[i], l + 1.0) : fn.diff[i - n];
    a[i] = make_double2(pow(e.rs[i], 0.5) * f, 0.0);
  }
  __syncthreads();
  double2 *r = d_block_fft(a, b, N, e.tw);
  for (int i = threadIdx.x; i < N; i += blockDim.x) r[i] = i < n ? zmul(r[i], e.M[l * N + i]) : make_double2(0, 0);
  __syncthreads();
  double2 *o = r == a ? b : a;
  r = d_block_fft(r, o, N, e.tw);
  for (int p = threadIdx.x; p < n; p += blockDim.x) fn.kwave[p] = r[p].x * 2 / pow(e.ks[p], 1.5);
}

// keep k below sqrt(c grid_encut), inverse transform (projector.c:127-137, sbt.c:156-215)
__global__ void k_sbt_inverse(const ElemDev *__restrict__ els, const FuncDev *__restrict__ fns, double kcut) {
  extern __shared__ double2 zs[];
  const FuncDev fn = fns[blockIdx.x];
  const ElemDev e = els[fn.elem];
  const int N = 2 * e.ngrid, n = e.ngrid, l = fn.l;
  double2 *a = zs, *b = zs + N;
  __shared__ int qcut;
  if (threadIdx.x == 0) {
    int q = 0;
    while (q < n && e.ks[q] < kcut) q++;
    qcut = q;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    double f = i < qcut ? fn.kwave[i] : 0.0;
    a[i] = make_double2(i < n ? pow(e.ks[i], 1.5) * f : 0.0, 0.0);
  }
  __syncthreads();
  double2 *r = d_block_fft(a, b, N, e.tw);
  for (int i = threadIdx.x; i < N; i += blockDim.x) r[i] = i < n ? zmul(r[i], e.M[l * N + i]) : make_double2(0, 0);
  __syncthreads();
  double2 *o = r == a ? b : a;
  r = d_block_fft(r, o, N, e.tw);
  for (int p = threadIdx.x; p < n; p += blockDim.x)
    fn.smooth[p] = r[p + n].x / M_PI * 2 * 2 / pow(e.rs[p + n], 1.5);
}

}  // namespace

// ------------------------------------------------------------------ off-site pairs
//
// reciprocal_offsite_wave_overlap (radial.c:116-196) integrates, for each L,
//   f1(k) f2(k) k^2 j_L(k R)
// with a cubic spline on a 500-point log k grid between the two elements' grid
// limits. The spline integral is linear in the sampled values, so it equals
// sum_q w_q g(k_q) with weights w that depend only on the grid: they are
// computed once per element pair (one thread per unit vector), the sampled
// f(k_q) once per function, and each pair then needs dot products only.

namespace {

constexpr int KQ = 500;  // KGRID_SIZE of radial.c:12

struct PairGrid {
  double kmin, kmax;
  double *kg, *w;  // [KQ]
};

struct KFunc {
  const double *kgrid, *f, *b, *c, *d;  // element k grid and the function's spline there
  int n;
  double *out;  // [KQ] f(kg_q)
};

// f(kg_q) by log-grid spline interpolation (wave_interpolate, utils.c:477-489)
__global__ void k_pair_sample(const KFunc *__restrict__ fs, const double *__restrict__ kg) {
  KFunc f = fs[blockIdx.y];
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= KQ) return;
  double r = kg[q], v;
  const double *x = f.kgrid;
  if (r > x[f.n - 1]) {
    v = 0;
  } else if (r < x[0]) {
    v = f.f[0];
  } else {
    int i = (int)(log(r / x[0]) / log(x[1] / x[0]));
    if (i > f.n - 2) i = f.n - 2;
    double t = r - x[i];
    v = f.f[i] + t * (f.b[i] + t * (f.c[i] + t * f.d[i]));
  }
  f.out[q] = v;
}

struct PairJob {
  const double *kg, *w;   // the element pair's grid and weights
  const double *F1, *F2;  // [nf1][KQ], [nf2][KQ]
  int nf1, nf2, Lmax;
  double R;
  double *I;              // [nf1][nf2][Lmax+1]
};

// spherical Bessel j_L by upward recurrence, zero-guarded (sbf, utils.c:804-824)
__device__ double d_sbf(double x, int l) {
  if (x < 10e-6) return l == 0 ? 1 : 0;
  double a = sin(x) / x, b = sin(x) / (x * x) - cos(x) / x;
  if (l == 0) return a;
  if (l == 1) return b;
  double c = 0;
  for (int q = 1; q < l; q++) {
    c = (2 * q + 1) / x * b - a;
    a = b;
    b = c;
  }
  return c;
}

// one CTA per pair: I[f1][f2][L] = sum_q w_q F1 F2 k_q^2 j_L(k_q R)
__global__ void k_pair_integrals(const PairJob *__restrict__ jobs) {
  __shared__ double J[7][KQ];
  __shared__ double wk[KQ];
  const PairJob pj = jobs[blockIdx.x];
  for (int q = threadIdx.x; q < KQ; q += blockDim.x) {
    double k = pj.kg[q];
    wk[q] = pj.w[q] * k * k;
    for (int L = 0; L <= pj.Lmax; L++) J[L][q] = d_sbf(k * pj.R, L);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int combos = pj.nf1 * pj.nf2 * (pj.Lmax + 1);
  for (int cix = warp; cix < combos; cix += nw) {
    int L = cix % (pj.Lmax + 1), r = cix / (pj.Lmax + 1);
    int f2 = r % pj.nf2, f1 = r / pj.nf2;
    const double *a = pj.F1 + (long long)f1 * KQ, *b = pj.F2 + (long long)f2 * KQ;
    double acc = 0;
    for (int q = lane; q < KQ; q += 32) acc += wk[q] * a[q] * b[q] * J[L][q];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) pj.I[cix] = acc;
  }
}

}  // namespace

// Radial integrals I[p][f1][f2][L] of every N_RS pair on the device (FP64).
void offsite_radial_integrals(const ppot_t *ppR, const ppot_t *ppS, const std::vector<int> &eR,
                              const std::vector<int> &eS, const std::vector<double> &R,
                              std::vector<std::vector<double>> &I, std::vector<int> &Lmax_out) {
  int np = (int)eR.size();
  I.assign(np, {});
  Lmax_out.assign(np, 0);
  if (np == 0) return;
  // element pairs in use
  std::map<std::pair<int, int>, int> pidx;
  for (int p = 0; p < np; p++) pidx.emplace(std::make_pair(eR[p], eS[p]), (int)pidx.size());
  int ne = (int)pidx.size();
  DevBuf<double> kg((size_t)ne * KQ), w((size_t)ne * KQ);
  // per element pair: grid, weights, sampled functions (device copies of kwave and its spline)
  std::vector<DevBuf<double>> fbuf;
  std::vector<KFunc> kf;
  std::vector<long> F1off(ne), F2off(ne);
  std::vector<int> nf1(ne), nf2(ne);
  long nsamp = 0;
  for (auto &it : pidx) {
    int e = it.second;
    nf1[e] = ppR[it.first.first].num_projs;
    nf2[e] = ppS[it.first.second].num_projs;
    F1off[e] = nsamp;
    nsamp += (long)nf1[e] * KQ;
    F2off[e] = nsamp;
    nsamp += (long)nf2[e] * KQ;
  }
  DevBuf<double> F(std::max(1L, nsamp));
  for (auto &it : pidx) {
    int e = it.second;
    const ppot_t &a = ppR[it.first.first], &b = ppS[it.first.second];
    PairGrid g;
    g.kmin = std::max(a.kwave_grid[0], b.kwave_grid[0]);
    g.kmax = std::min(a.kwave_grid[a.wave_gridsize - 1], b.kwave_grid[b.wave_gridsize - 1]);
    g.kg = kg.p + (size_t)e * KQ;
    g.w = w.p + (size_t)e * KQ;
    std::vector<double> hk(KQ), hw(KQ);
    for (int q = 0; q < KQ; q++) hk[q] = g.kmin * std::pow(g.kmax / g.kmin, (double)q / KQ);
    spline_integral_weights(hk.data(), KQ, hw.data());
    kg.upload(hk.data(), KQ, (size_t)e * KQ);
    w.upload(hw.data(), KQ, (size_t)e * KQ);
    for (int side = 0; side < 2; side++) {
      const ppot_t &pp = side == 0 ? a : b;
      int n = pp.wave_gridsize;
      for (int f = 0; f < pp.num_projs; f++) {
        fbuf.emplace_back((size_t)4 * n);
        DevBuf<double> &fb = fbuf.back();
        fb.upload(pp.kwave_grid, n, 0);
        fb.upload(pp.funcs[f].kwave, n, n);
        std::vector<double> spl(3 * (size_t)n);
        for (int c = 0; c < 3; c++)
          for (int q = 0; q < n; q++) spl[(size_t)c * n + q] = pp.funcs[f].kwave_spline[c][q];
        DevBuf<double> sb(3 * (size_t)n);
        sb.upload(spl.data(), spl.size());
        fbuf.emplace_back(std::move(sb));
        const double *base = fbuf[fbuf.size() - 2].p, *sp = fbuf.back().p;
        KFunc k;
        k.kgrid = base;
        k.f = base + n;
        k.b = sp;
        k.c = sp + n;
        k.d = sp + 2 * n;
        k.n = n;
        k.out = F.p + (side == 0 ? F1off[e] : F2off[e]) + (long)f * KQ;
        kf.push_back(k);
      }
    }
    DevBuf<KFunc> kfd(kf.size());
    kfd.upload(kf.data(), kf.size());
    PAWPY_LAUNCH("pair_sample", k_pair_sample<<<dim3(ceil_div(KQ, 128), (unsigned)kf.size()), 128, 0, stream()>>>(kfd.p, g.kg));
    sync();
    kf.clear();
  }
  std::vector<PairJob> jobs(np);
  std::vector<long> ioff(np);
  long itot = 0;
  for (int p = 0; p < np; p++) {
    int e = pidx[std::make_pair(eR[p], eS[p])];
    int l1max = 0, l2max = 0;
    for (int f = 0; f < ppR[eR[p]].num_projs; f++) l1max = std::max(l1max, ppR[eR[p]].funcs[f].l);
    for (int f = 0; f < ppS[eS[p]].num_projs; f++) l2max = std::max(l2max, ppS[eS[p]].funcs[f].l);
    PairJob &j = jobs[p];
    j.kg = kg.p + (size_t)e * KQ;
    j.w = w.p + (size_t)e * KQ;
    j.F1 = F.p + F1off[e];
    j.F2 = F.p + F2off[e];
    j.nf1 = nf1[e];
    j.nf2 = nf2[e];
    j.Lmax = l1max + l2max;
    PAWPY_REQUIRE(j.Lmax <= 6, "pair matrices need l <= 3");
    j.R = R[p];
    ioff[p] = itot;
    itot += (long)j.nf1 * j.nf2 * (j.Lmax + 1);
    Lmax_out[p] = j.Lmax;
  }
  DevBuf<double> Id(std::max(1L, itot));
  for (int p = 0; p < np; p++) jobs[p].I = Id.p + ioff[p];
  DevBuf<PairJob> jd(np);
  jd.upload(jobs.data(), np);
  PAWPY_LAUNCH("pair_integrals", k_pair_integrals<<<np, 256, 0, stream()>>>(jd.p));
  std::vector<double> h(itot);
  Id.download(h.data(), itot);
  sync();
  for (int p = 0; p < np; p++)
    I[p].assign(h.begin() + ioff[p], h.begin() + ioff[p] + (long)jobs[p].nf1 * jobs[p].nf2 * (jobs[p].Lmax + 1));
}

static double *dupd(const std::vector<double> &v) {
  double *p = static_cast<double *>(std::malloc(sizeof(double) * std::max<size_t>(1, v.size())));
  if (!p) throw std::bad_alloc();
  std::copy(v.begin(), v.end(), p);
  return p;
}

// malloc'd spline coefficients in the reference's double*[3] layout
static double **new_spline3(const double *x, const double *y, int n) {
  double **s = static_cast<double **>(std::malloc(3 * sizeof(double *)));
  if (!s) throw std::bad_alloc();
  for (int q = 0; q < 3; q++) {
    s[q] = static_cast<double *>(std::malloc(sizeof(double) * n));
    if (!s[q]) throw std::bad_alloc();
  }
  spline_coeffs(x, y, n, s[0], s[1], s[2]);
  return s;
}

// ---- results of get_projector_list by exact input, returned as deep copies

namespace {

template <typename T>
T *dup_array(const T *src, size_t n) {
  if (!src) return nullptr;
  T *d = static_cast<T *>(std::malloc(sizeof(T) * std::max<size_t>(1, n)));
  if (!d) throw std::bad_alloc();
  std::memcpy(d, src, sizeof(T) * n);
  return d;
}

double **dup_spline(double *const *s, int n) {
  if (!s) return nullptr;
  double **d = static_cast<double **>(std::calloc(3, sizeof(double *)));
  if (!d) throw std::bad_alloc();
  for (int q = 0; q < 3; q++) d[q] = dup_array(s[q], (size_t)n);
  return d;
}

// deep copy of an element array made by device_projector_list (every pointer it sets)
ppot_t *copy_ppot_array(const ppot_t *src, int n) {
  ppot_t *pps = static_cast<ppot_t *>(std::calloc(n, sizeof(ppot_t)));
  if (!pps) throw std::bad_alloc();
  try {
    for (int e = 0; e < n; e++) {
      const ppot_t &a = src[e];
      ppot_t &b = pps[e];
      b = a;
      b.funcs = nullptr;
      b.pspw_overlap_matrix = b.aepw_overlap_matrix = b.diff_overlap_matrix = nullptr;
      b.wave_grid = b.kwave_grid = b.proj_grid = b.smooth_grid = b.dense_kgrid = nullptr;
      const int ng = a.wave_gridsize, nd = a.proj_gridsize, np = a.num_projs;
      b.wave_grid = dup_array(a.wave_grid, ng);
      b.kwave_grid = dup_array(a.kwave_grid, ng);
      b.proj_grid = dup_array(a.proj_grid, nd);
      b.smooth_grid = dup_array(a.smooth_grid, nd);
      b.pspw_overlap_matrix = dup_array(a.pspw_overlap_matrix, (size_t)np * np);
      b.aepw_overlap_matrix = dup_array(a.aepw_overlap_matrix, (size_t)np * np);
      b.diff_overlap_matrix = dup_array(a.diff_overlap_matrix, (size_t)np * np);
      b.funcs = static_cast<funcset_t *>(std::calloc(np, sizeof(funcset_t)));
      if (!b.funcs) throw std::bad_alloc();
      for (int k = 0; k < np; k++) {
        const funcset_t &f = a.funcs[k];
        funcset_t &g = b.funcs[k];
        g.l = f.l;
        g.proj = dup_array(f.proj, nd);
        g.proj_spline = dup_spline(f.proj_spline, nd);
        g.aewave = dup_array(f.aewave, ng);
        g.aewave_spline = dup_spline(f.aewave_spline, ng);
        g.pswave = dup_array(f.pswave, ng);
        g.pswave_spline = dup_spline(f.pswave_spline, ng);
        g.diffwave = dup_array(f.diffwave, ng);
        g.diffwave_spline = dup_spline(f.diffwave_spline, ng);
        g.kwave = dup_array(f.kwave, ng);
        g.kwave_spline = dup_spline(f.kwave_spline, ng);
        g.smooth_diffwave = dup_array(f.smooth_diffwave, nd);
        g.smooth_diffwave_spline = dup_spline(f.smooth_diffwave_spline, nd);
      }
    }
  } catch (...) {
    free_ppot_array(pps, n);
    throw;
  }
  return pps;
}

struct ListCache {
  std::mutex mu;
  std::vector<std::pair<std::vector<unsigned char>, ppot_t *>> entries;  // (inputs, master copy)
  std::vector<int> counts;                                               // elements of each entry
};
std::atomic<bool> g_list_cache_on{true};

ListCache &list_cache() {
  static ListCache c;
  return c;
}

void append_bytes(std::vector<unsigned char> &k, const void *p, size_t n) {
  const unsigned char *c = static_cast<const unsigned char *>(p);
  k.insert(k.end(), c, c + n);
}

}  // namespace

ppot_t *cached_projector_list(int num_els, const int *labels, const int *ls, const double *wave_grids,
                              const double *projectors, const double *aewaves, const double *pswaves,
                              const double *rmaxs, double grid_encut) {
  PAWPY_REQUIRE(num_els > 0 && labels && ls && wave_grids && projectors && aewaves && pswaves && rmaxs,
                "get_projector_list: missing input array");
  if (!g_list_cache_on.load())
    return device_projector_list(num_els, labels, ls, wave_grids, projectors, aewaves, pswaves, rmaxs, grid_encut);
  long npt = 0, ngt = 0, ndp = 0, ngp = 0;
  for (int e = 0; e < num_els; e++) {
    const long np = labels[4 * e + 1], nd = labels[4 * e + 2], ng = labels[4 * e + 3];
    PAWPY_REQUIRE(np >= 1 && nd >= 3 && ng >= 3, "get_projector_list: bad element dimensions");
    npt += np;
    ngt += ng;
    ndp += np * nd;
    ngp += np * ng;
  }
  std::vector<unsigned char> key;
  key.reserve(sizeof(int) * (4 * num_els + npt) + sizeof(double) * (ngt + ndp + 2 * ngp + num_els + 1) + 8);
  append_bytes(key, &num_els, sizeof(int));
  append_bytes(key, labels, sizeof(int) * 4 * (size_t)num_els);
  append_bytes(key, ls, sizeof(int) * (size_t)npt);
  append_bytes(key, wave_grids, sizeof(double) * (size_t)ngt);
  append_bytes(key, projectors, sizeof(double) * (size_t)ndp);
  append_bytes(key, aewaves, sizeof(double) * (size_t)ngp);
  append_bytes(key, pswaves, sizeof(double) * (size_t)ngp);
  append_bytes(key, rmaxs, sizeof(double) * (size_t)num_els);
  append_bytes(key, &grid_encut, sizeof(double));
  ListCache &c = list_cache();
  {
    std::lock_guard<std::mutex> lk(c.mu);
    for (auto &en : c.entries)
      if (en.first == key) return copy_ppot_array(en.second, num_els);
  }
  ppot_t *master = device_projector_list(num_els, labels, ls, wave_grids, projectors, aewaves, pswaves, rmaxs,
                                         grid_encut);
  ppot_t *out = nullptr;
  try {
    out = copy_ppot_array(master, num_els);
  } catch (...) {
    free_ppot_array(master, num_els);
    throw;
  }
  std::lock_guard<std::mutex> lk(c.mu);
  if (c.entries.size() >= 16) {  // oldest first out
    free_ppot_array(c.entries.front().second, c.counts.front());
    c.entries.erase(c.entries.begin());
    c.counts.erase(c.counts.begin());
  }
  c.entries.emplace_back(std::move(key), master);
  c.counts.push_back(num_els);
  return out;
}

void set_projector_list_cache(bool on) { g_list_cache_on = on; }

ppot_t *device_projector_list(int num_els, const int *labels, const int *ls, const double *wave_grids,
                              const double *projectors, const double *aewaves, const double *pswaves,
                              const double *rmaxs, double grid_encut) {
  PAWPY_REQUIRE(num_els > 0 && labels && ls && wave_grids && projectors && aewaves && pswaves && rmaxs,
                "get_projector_list: missing input array");
  const double encut_sbt = 1e7;  // top of the transform's k grid (projector.c:115)
  ppot_t *pps = static_cast<ppot_t *>(std::calloc(num_els, sizeof(ppot_t)));
  if (!pps) throw std::bad_alloc();
  try {
    // ---- host: grids, difference waves and their splines (serial recurrences)
    long wg = 0, pr = 0, wv = 0, l_off = 0;
    int nf = 0;
    std::vector<std::vector<double>> dense(num_els);
    for (int e = 0; e < num_els; e++) {
      ppot_t &pp = pps[e];
      pp.num_projs = labels[4 * e + 1];
      pp.proj_gridsize = labels[4 * e + 2];
      pp.wave_gridsize = labels[4 * e + 3];
      pp.rmax = rmaxs[e];
      int nd = pp.proj_gridsize, ng = pp.wave_gridsize, np = pp.num_projs;
      PAWPY_REQUIRE(nd >= 3 && ng >= 3 && np >= 1, "get_projector_list: bad element dimensions");
      pp.wave_grid = dupd(std::vector<double>(wave_grids + wg, wave_grids + wg + ng));
      wg += ng;
      pp.wave_rmax = pp.wave_grid[ng - 1];
      std::vector<double> pg(nd), sg(nd);
      for (int j = 0; j < nd; j++) {
        pg[j] = pp.rmax / nd * j;
        sg[j] = pp.wave_rmax / nd * j;
      }
      pp.proj_grid = dupd(pg);
      pp.smooth_grid = dupd(sg);
      // the reference rebuilds the log grid as a running product of its first ratio (projector.c:62-67)
      dense[e].resize(ng);
      dense[e][0] = pp.wave_grid[0];
      double ratio = std::pow(pp.wave_grid[1] / pp.wave_grid[0], 1.0);
      for (int i = 1; i < ng; i++) dense[e][i] = dense[e][i - 1] * ratio;
      pp.funcs = static_cast<funcset_t *>(std::calloc(np, sizeof(funcset_t)));
      if (!pp.funcs) throw std::bad_alloc();
      pp.lmax = 0;
      pp.total_projs = 0;
      for (int k = 0; k < np; k++) {
        funcset_t &f = pp.funcs[k];
        f.l = ls[l_off++];
        PAWPY_REQUIRE(f.l >= 0 && f.l <= 3, "get_projector_list: projector channels need 0 <= l <= 3");
        pp.lmax = std::max(pp.lmax, f.l);
        pp.total_projs += 2 * f.l + 1;
        f.aewave = dupd(std::vector<double>(aewaves + wv, aewaves + wv + ng));
        f.pswave = dupd(std::vector<double>(pswaves + wv, pswaves + wv + ng));
        wv += ng;
        std::vector<double> df(ng);
        for (int i = 0; i < ng; i++) df[i] = f.aewave[i] - f.pswave[i];
        f.diffwave = dupd(df);
        f.proj = dupd(std::vector<double>(projectors + pr, projectors + pr + nd));
        pr += nd;
        // (their splines are fitted while the device transforms run, below)
      }
      nf += np;
    }
    // ---- device: transform grids, multiplier tables, forward + filtered inverse transforms
    long g_ng = 0, g_m = 0, g_f = 0;
    for (int e = 0; e < num_els; e++) {
      g_ng += pps[e].wave_gridsize;
      g_m += (long)(std::max(1, pps[e].lmax) + 1) * 2 * pps[e].wave_gridsize;
      g_f += (long)pps[e].num_projs * pps[e].wave_gridsize;
    }
    DevBuf<double> d_wg(g_ng), ks(2 * g_ng), rs(2 * g_ng), d_diff(g_f), kwave(g_f), smooth(g_f);
    DevBuf<double2> Mt(g_m), tw(2 * g_ng);
    std::vector<ElemDev> els(num_els);
    std::vector<FuncDev> fns;
    std::vector<long> f_off;
    int maxN = 0;
    {
      long o_ng = 0, o_m = 0, o_f = 0;
      for (int e = 0; e < num_els; e++) {
        ppot_t &pp = pps[e];
        int ng = pp.wave_gridsize;
        d_wg.upload(pp.wave_grid, ng, o_ng);
        ElemDev &d = els[e];
        d.ngrid = ng;
        d.lmax = pp.lmax;
        d.wave_grid = d_wg.p + o_ng;
        d.ks = ks.p + 2 * o_ng;
        d.rs = rs.p + 2 * o_ng;
        d.tw = tw.p + 2 * o_ng;
        d.M = Mt.p + o_m;
        maxN = std::max(maxN, 2 * ng);
        for (int k = 0; k < pp.num_projs; k++) {
          d_diff.upload(pp.funcs[k].diffwave, ng, o_f);
          FuncDev fn;
          fn.elem = e;
          fn.l = pp.funcs[k].l;
          fn.diff = d_diff.p + o_f;
          fn.kwave = kwave.p + o_f;
          fn.smooth = smooth.p + o_f;
          fns.push_back(fn);
          f_off.push_back(o_f);
          o_f += ng;
        }
        o_ng += ng;
        o_m += (long)(std::max(1, pp.lmax) + 1) * 2 * ng;
      }
    }
    DevBuf<ElemDev> d_els(num_els);
    d_els.upload(els.data(), num_els);
    DevBuf<FuncDev> d_fns(nf);
    d_fns.upload(fns.data(), nf);
    PAWPY_LAUNCH("radial_grids", k_rad_grids<<<num_els, 256, 0, stream()>>>(d_els.p, encut_sbt));
    PAWPY_LAUNCH("radial_mtable", k_rad_mtable<<<dim3(ceil_div(maxN, 128), num_els), 128, 0, stream()>>>(d_els.p, encut_sbt));
    size_t zsm = 2 * sizeof(double2) * maxN;
    PAWPY_REQUIRE(zsm <= 48 * 1024, "radial grid too long for the transform's shared memory");
    PAWPY_LAUNCH("radial_sbt", k_sbt_forward<<<nf, 256, zsm, stream()>>>(d_els.p, d_fns.p));
    double kcut = std::pow(0.262465831 * grid_encut, 0.5);
    PAWPY_LAUNCH("radial_sbt", k_sbt_inverse<<<nf, 256, zsm, stream()>>>(d_els.p, d_fns.p, kcut));
    // the host splines of the input functions, one function per host thread, beside the transforms
    {
      std::vector<std::pair<int, int>> fk;
      for (int e = 0; e < num_els; e++)
        for (int k = 0; k < pps[e].num_projs; k++) fk.push_back({e, k});
      host_parallel_for((int)fk.size(), [&](int i) {
        ppot_t &pp = pps[fk[i].first];
        funcset_t &f = pp.funcs[fk[i].second];
        const int nd = pp.proj_gridsize, ng = pp.wave_gridsize;
        f.proj_spline = new_spline3(pp.proj_grid, f.proj, nd);
        f.aewave_spline = new_spline3(pp.wave_grid, f.aewave, ng);
        f.pswave_spline = new_spline3(pp.wave_grid, f.pswave, ng);
        f.diffwave_spline = new_spline3(pp.wave_grid, f.diffwave, ng);
      });
    }
    std::vector<double> h_ks(ks.n), h_kw(kwave.n), h_sm(smooth.n);
    ks.download(h_ks.data(), ks.n);
    kwave.download(h_kw.data(), kwave.n);
    smooth.download(h_sm.data(), smooth.n);
    sync();
    HostPhase hp_post("projector_list_splines");
    // ---- host: splines of the transforms, the smooth difference on the linear grid, overlaps;
    // the functions and the overlap integrals are independent: one host thread each
    std::vector<int> f_el, f_k;
    {
      long o_ng = 0;
      for (int e = 0; e < num_els; e++) {
        ppot_t &pp = pps[e];
        pp.kwave_grid = dupd(std::vector<double>(h_ks.begin() + 2 * o_ng, h_ks.begin() + 2 * o_ng + pp.wave_gridsize));
        for (int k = 0; k < pp.num_projs; k++) {
          f_el.push_back(e);
          f_k.push_back(k);
        }
        o_ng += pp.wave_gridsize;
        const int np = pp.num_projs;
        pp.pspw_overlap_matrix = static_cast<double *>(std::calloc(np * np, sizeof(double)));
        pp.aepw_overlap_matrix = static_cast<double *>(std::calloc(np * np, sizeof(double)));
        pp.diff_overlap_matrix = static_cast<double *>(std::calloc(np * np, sizeof(double)));
        if (!pp.pspw_overlap_matrix || !pp.aepw_overlap_matrix || !pp.diff_overlap_matrix) throw std::bad_alloc();
      }
    }
    host_parallel_for((int)f_el.size(), [&](int f) {
      const int e = f_el[f], k = f_k[f];
      ppot_t &pp = pps[e];
      const int ng = pp.wave_gridsize, nd = pp.proj_gridsize;
      funcset_t &fs = pp.funcs[k];
      fs.kwave = dupd(std::vector<double>(h_kw.begin() + f_off[f], h_kw.begin() + f_off[f] + ng));
      fs.kwave_spline = new_spline3(pp.kwave_grid, fs.kwave, ng);
      const double *sm = h_sm.data() + f_off[f];
      double **ss = new_spline3(dense[e].data(), sm, ng);
      std::vector<double> sdw(nd);
      for (int p = 1; p < nd; p++) sdw[p] = interp_log(pp.smooth_grid[p], ng, dense[e].data(), sm, ss);
      sdw[0] = fs.l > 0 ? 0.0 : sdw[1];
      for (int q = 0; q < 3; q++) std::free(ss[q]);
      std::free(ss);
      fs.smooth_diffwave = dupd(sdw);
      fs.smooth_diffwave_spline = new_spline3(pp.smooth_grid, fs.smooth_diffwave, nd);
    });
    // overlap integrals <ps|ps>, <ae|ae>, <ae-ps|ae-ps> of the function pairs of equal l
    struct OvTask {
      int e, i, j, w;
    };
    std::vector<OvTask> ov;
    for (int e = 0; e < num_els; e++)
      for (int i = 0; i < pps[e].num_projs; i++)
        for (int j = i; j < pps[e].num_projs; j++)
          if (pps[e].funcs[i].l == pps[e].funcs[j].l)
            for (int w = 0; w < 3; w++) ov.push_back({e, i, j, w});
    host_parallel_for((int)ov.size(), [&](int t) {
      const OvTask &o = ov[t];
      ppot_t &pp = pps[o.e];
      const int ng = pp.wave_gridsize, np = pp.num_projs;
      const funcset_t &a1 = pp.funcs[o.i], &a2 = pp.funcs[o.j];
      std::vector<double> prod(ng), b(ng), c(ng), d(ng);
      for (int q = 0; q < ng; q++) {
        if (o.w == 0) prod[q] = a1.pswave[q] * a2.pswave[q];
        else if (o.w == 1) prod[q] = a1.aewave[q] * a2.aewave[q];
        else prod[q] = (a1.aewave[q] - a1.pswave[q]) * (a2.aewave[q] - a2.pswave[q]);
      }
      spline_coeffs(pp.wave_grid, prod.data(), ng, b.data(), c.data(), d.data());
      const double v = spline_integral(pp.wave_grid, prod.data(), b.data(), c.data(), d.data(), ng);
      double *mat = o.w == 0 ? pp.pspw_overlap_matrix : o.w == 1 ? pp.aepw_overlap_matrix : pp.diff_overlap_matrix;
      mat[o.i * np + o.j] = v;
      mat[o.j * np + o.i] = v;
    });
  } catch (...) {
    free_ppot_array(pps, num_els);
    throw;
  }
  return pps;
}

}  // namespace pawpy

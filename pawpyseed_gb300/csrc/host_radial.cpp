// Radial (per-element) setup of the PAW datasets, in double precision:
// get_projector_list (projector.c:20-171), make_pwave_overlap_matrices
// (projector.c:507-558), the spherical Bessel transforms they use
// (sbt.c:24-215; Talman's NumSBT, Comput. Phys. Commun. 180 (2009) 332) and
// the off-site partial-wave overlap of a site pair (radial.c:116-196).
//
// The results must equal the reference's to rounding, so the algorithms are
// the reference's: the same spline (a clamped-start / natural-end cubic whose
// first slope is the first secant, utils.c:699-749), the same 2N-point
// logarithmic extension and multiplier table of the transform, the same
// k-space filter at sqrt(c*grid_encut), the same 500-point k quadrature.
// Each is written here in its own form.
#include <cmath>
#include <complex>
#include <cstdlib>
#include <vector>

#include "host.h"

namespace pawpy {

using cd = std::complex<double>;
static const double kC = 0.262465831;

// ------------------------------------------------------------------ splines

void spline_coeffs(const double *x, const double *y, int n, double *b, double *c, double *d) {
  // Tridiagonal sweep for the second derivatives M_i (kept in c), then the
  // polynomial coefficients of each interval.
  double s0 = (y[1] - y[0]) / (x[1] - x[0]);
  if (s0 > 0.99e30) {
    c[0] = 0;
    b[0] = 0;
  } else {
    c[0] = -0.5;
    b[0] = (3 / (x[1] - x[0])) * ((y[1] - y[0]) / (x[1] - x[0]) - s0);
  }
  for (int i = 1; i < n - 1; i++) {
    double sig = (x[i] - x[i - 1]) / (x[i + 1] - x[i - 1]);
    double p = sig * c[i - 1] + 2;
    c[i] = (sig - 1) / p;
    double dd = (y[i + 1] - y[i]) / (x[i + 1] - x[i]) - (y[i] - y[i - 1]) / (x[i] - x[i - 1]);
    b[i] = (6 * dd / (x[i + 1] - x[i - 1]) - sig * b[i - 1]) / p;
  }
  b[n - 1] = 0;
  c[n - 1] = 0;
  d[n - 1] = 0;
  for (int i = n - 2; i >= 0; i--) c[i] = c[i] * c[i + 1] + b[i];
  for (int i = 0; i < n - 1; i++) {
    double h = x[i + 1] - x[i];
    double q = (c[i + 1] - c[i]) / 6;
    d[i] = q / h;
    c[i] = c[i] / 2;
    b[i] = (y[i + 1] - y[i]) / h - (c[i] + q) * h;
  }
}

double spline_integral(const double *x, const double *y, const double *b, const double *c,
                       const double *d, int n) {
  double s = 0;
  for (int i = 0; i < n - 1; i++) {
    double h = x[i + 1] - x[i];
    s += h * (y[i] + h * (b[i] / 2 + h * (c[i] / 3 + d[i] * h / 4)));
  }
  return s;
}

double interp_log(double r, int n, const double *x, const double *f, double *const *s) {
  if (r > x[n - 1]) return 0;
  if (r < x[0]) return f[0];
  int i = (int)(std::log(r / x[0]) / std::log(x[1] / x[0]));
  if (i > n - 2) i = n - 2;
  double t = r - x[i];
  return f[i] + t * (s[0][i] + t * (s[1][i] + t * s[2][i]));
}

static double **new_spline(const double *x, const double *y, int n) {
  double **s = static_cast<double **>(std::malloc(3 * sizeof(double *)));
  if (!s) throw std::bad_alloc();
  for (int j = 0; j < 3; j++) {
    s[j] = static_cast<double *>(std::malloc(sizeof(double) * n));
    if (!s[j]) throw std::bad_alloc();
  }
  spline_coeffs(x, y, n, s[0], s[1], s[2]);
  return s;
}

static double *dup(const double *src, int n) {
  double *p = static_cast<double *>(std::malloc(sizeof(double) * (n > 0 ? n : 1)));
  if (!p) throw std::bad_alloc();
  for (int i = 0; i < n; i++) p[i] = src[i];
  return p;
}

// ------------------------------------------------- 1D FFT for the transform

// Mixed-radix Stockham transform with the exp(+i) sign of a DFTI backward
// transform (unnormalised), for the 2N-point lengths of the Bessel transform.
struct Fft1 {
  int n;
  std::vector<int> radix;
  std::vector<cd> w;  // exp(+2 pi i m/n)
  explicit Fft1(int len) : n(len), w(len) {
    int m = len;
    for (int q = 2; m > 1; q++)
      while (m % q == 0) {
        radix.push_back(q);
        m /= q;
      }
    for (int i = 0; i < len; i++) {
      double a = 2.0 * M_PI * i / len;
      w[i] = cd(std::cos(a), std::sin(a));
    }
  }
  void operator()(std::vector<cd> &x) const {
    std::vector<cd> y(n), v(64), o(64);
    cd *src = x.data(), *dst = y.data();
    long span = 1;
    for (int R : radix) {
      long m = n / R;
      for (long j = 0; j < m; j++) {
        long k = j % span;
        long tstep = n / (span * R);
        for (int r = 0; r < R; r++) v[r] = src[j + r * m] * w[(k * r * tstep) % n];
        for (int q = 0; q < R; q++) {
          cd acc = 0;
          for (int r = 0; r < R; r++) acc += v[r] * w[(long)((r * q) % R) * (n / R)];
          o[q] = acc;
        }
        long base = (j / span) * span * R + k;
        for (int q = 0; q < R; q++) dst[base + q * span] = o[q];
      }
      std::swap(src, dst);
      span *= R;
    }
    if (src != x.data()) std::copy(src, src + n, x.begin());
  }
};

// ---------------------------------------------- spherical Bessel transform

struct Sbt {
  int N, lmax;
  std::vector<double> ks, rs;
  std::vector<std::vector<cd>> M;
  Fft1 fft;
  // r: logarithmic grid of n points; encut sets the top of the k grid.
  Sbt(double encut, int lmax_in, int n, const double *r)
      : N(2 * n), lmax(lmax_in == 0 ? 1 : lmax_in), ks(2 * n), rs(2 * n), fft(2 * n) {
    double drho = std::log(r[1] / r[0]);
    double dt = 2 * M_PI / N / drho;
    double kmin = std::pow(encut * kC, 0.5) * std::exp(-(N / 2 - 1) * drho);
    double kappamin = std::log(kmin);
    for (int i = 0; i < N; i++) {
      ks[i] = kmin * std::exp(i * drho);
      rs[i] = r[0] * std::exp((i - N / 2) * drho);
    }
    double rhomin = std::log(rs[0]);
    M.assign(lmax + 1, std::vector<cd>(N));
    for (int i = 0; i < N; i++) {
      double t = i * dt;
      // arg Gamma(1/2 + i t): shift by 10 then Stirling's series
      double rad = std::sqrt(10.5 * 10.5 + t * t);
      double ph = std::atan((2 * t) / 21);
      double g = -10 * ph - t * std::log(rad) + t + std::sin(ph) / (12 * rad) -
                 std::sin(3 * ph) / (360 * std::pow(rad, 3)) +
                 std::sin(5 * ph) / (1260 * std::pow(rad, 5)) -
                 std::sin(7 * ph) / (1680 * std::pow(rad, 7));
      for (int j = 1; j <= 10; j++) g += std::atan((2 * t) / (2 * j - 1));
      double h = -std::atan(std::tanh(M_PI * t / 2));
      double phase = g + h + (kappamin + rhomin) * t;
      cd m0 = std::sqrt(M_PI / 2) * std::exp(cd(0, phase)) / (double)N;
      if (i == 0) m0 *= 0.5;
      M[0][i] = m0;
      M[1][i] = std::exp(cd(0, 2 * (-h - std::atan(2 * t)))) * m0;
      for (int l = 1; l < lmax; l++)
        M[l + 1][i] = std::exp(cd(0, 2 * -std::atan(2 * t / (2 * l + 1)))) * M[l - 1][i];
    }
  }
  // transform of r*f given on the original grid (n points) -> n values on ks[0..n)
  std::vector<double> forward(const double *f, int l) const {
    int n = N / 2;
    std::vector<cd> x(N);
    double C = f[0] / std::pow(rs[n], l + 1);
    for (int i = 0; i < N; i++) {
      double fs = i < n ? C * std::pow(rs[i], l + 1) : f[i - n];
      x[i] = std::pow(rs[i], 0.5) * fs;
    }
    fft(x);
    for (int i = 0; i < N; i++) x[i] = i < n ? x[i] * M[l][i] : cd(0);
    fft(x);
    std::vector<double> out(n);
    for (int p = 0; p < n; p++) out[p] = x[p].real() * 2 / std::pow(ks[p], 1.5);
    return out;
  }
  // inverse of forward (roles of the two grids exchanged)
  std::vector<double> inverse(const double *fk, int l) const {
    int n = N / 2;
    std::vector<cd> x(N);
    for (int i = 0; i < N; i++) x[i] = i < n ? std::pow(ks[i], 1.5) * fk[i] : 0.0;
    fft(x);
    for (int i = 0; i < N; i++) x[i] = i < n ? x[i] * M[l][i] : cd(0);
    fft(x);
    std::vector<double> out(n);
    for (int p = 0; p < n; p++) out[p] = x[p + n].real() / M_PI * 2 * 2 / std::pow(rs[p + n], 1.5);
    return out;
  }
};

// ------------------------------------------------------- element datasets

ppot_t *build_projector_list(int num_els, const int *labels, const int *ls, const double *wave_grids,
                             const double *projectors, const double *aewaves, const double *pswaves,
                             const double *rmaxs, double grid_encut) {
  PAWPY_REQUIRE(num_els > 0 && labels && ls && wave_grids && projectors && aewaves && pswaves && rmaxs,
                "get_projector_list: missing input array");
  ppot_t *pps = static_cast<ppot_t *>(std::calloc(num_els, sizeof(ppot_t)));
  if (!pps) throw std::bad_alloc();
  long wg_off = 0, p_off = 0, w_off = 0, l_off = 0;
  try {
    for (int e = 0; e < num_els; e++) {
      ppot_t &pp = pps[e];
      pp.num_projs = labels[4 * e + 1];
      pp.proj_gridsize = labels[4 * e + 2];
      pp.wave_gridsize = labels[4 * e + 3];
      pp.rmax = rmaxs[e];
      int nd = pp.proj_gridsize, ng = pp.wave_gridsize, np = pp.num_projs;
      PAWPY_REQUIRE(nd >= 3 && ng >= 3 && np >= 1, "get_projector_list: bad element dimensions");
      pp.wave_grid = dup(wave_grids + wg_off, ng);
      wg_off += ng;
      pp.kwave_grid = static_cast<double *>(std::calloc(ng, sizeof(double)));
      pp.proj_grid = static_cast<double *>(std::malloc(sizeof(double) * nd));
      pp.smooth_grid = static_cast<double *>(std::malloc(sizeof(double) * nd));
      pp.funcs = static_cast<funcset_t *>(std::calloc(np, sizeof(funcset_t)));
      if (!pp.kwave_grid || !pp.proj_grid || !pp.smooth_grid || !pp.funcs) throw std::bad_alloc();
      for (int j = 0; j < nd; j++) pp.proj_grid[j] = pp.rmax / nd * j;
      pp.wave_rmax = pp.wave_grid[ng - 1];
      for (int j = 0; j < nd; j++) pp.smooth_grid[j] = pp.wave_rmax / nd * j;
      // the reference rebuilds the log grid as a running product of its first ratio
      std::vector<double> dense(ng);
      dense[0] = pp.wave_grid[0];
      double ratio = std::pow(pp.wave_grid[1] / pp.wave_grid[0], 1.0);
      for (int i = 1; i < ng; i++) dense[i] = dense[i - 1] * ratio;
      pp.lmax = 0;
      pp.total_projs = 0;
      for (int k = 0; k < np; k++) {
        funcset_t &f = pp.funcs[k];
        f.l = ls[l_off++];
        if (f.l > pp.lmax) pp.lmax = f.l;
        pp.total_projs += 2 * f.l + 1;
        f.aewave = dup(aewaves + w_off, ng);
        f.pswave = dup(pswaves + w_off, ng);
        f.diffwave = static_cast<double *>(std::malloc(sizeof(double) * ng));
        if (!f.diffwave) throw std::bad_alloc();
        for (int i = 0; i < ng; i++) f.diffwave[i] = f.aewave[i] - f.pswave[i];
        w_off += ng;
        f.proj = dup(projectors + p_off, nd);
        p_off += nd;
        f.proj_spline = new_spline(pp.proj_grid, f.proj, nd);
        f.aewave_spline = new_spline(pp.wave_grid, f.aewave, ng);
        f.pswave_spline = new_spline(pp.wave_grid, f.pswave, ng);
        f.diffwave_spline = new_spline(pp.wave_grid, f.diffwave, ng);
      }
      Sbt sbt(1e7, pp.lmax, ng, pp.wave_grid);
      for (int i = 0; i < ng; i++) pp.kwave_grid[i] = sbt.ks[i];
      double kcut = std::pow(kC * grid_encut, 0.5);
      for (int k = 0; k < np; k++) {
        funcset_t &f = pp.funcs[k];
        std::vector<double> kw = sbt.forward(f.diffwave, f.l);
        f.kwave = dup(kw.data(), ng);
        f.kwave_spline = new_spline(pp.kwave_grid, f.kwave, ng);
        // drop every k at or above sqrt(c * grid_encut), transform back
        std::vector<double> lowk(ng, 0.0);
        for (int q = 0; q < ng && pp.kwave_grid[q] < kcut; q++) lowk[q] = f.kwave[q];
        std::vector<double> sm = sbt.inverse(lowk.data(), f.l);
        double **ss = new_spline(dense.data(), sm.data(), ng);
        double *sdw = static_cast<double *>(std::malloc(sizeof(double) * nd));
        if (!sdw) throw std::bad_alloc();
        for (int p = 1; p < nd; p++) sdw[p] = interp_log(pp.smooth_grid[p], ng, dense.data(), sm.data(), ss);
        sdw[0] = f.l > 0 ? 0.0 : sdw[1];
        for (int j = 0; j < 3; j++) std::free(ss[j]);
        std::free(ss);
        f.smooth_diffwave = sdw;
        f.smooth_diffwave_spline = new_spline(pp.smooth_grid, sdw, nd);
      }
      // partial-wave overlap integrals between channels of equal l
      pp.pspw_overlap_matrix = static_cast<double *>(std::calloc(np * np, sizeof(double)));
      pp.aepw_overlap_matrix = static_cast<double *>(std::calloc(np * np, sizeof(double)));
      pp.diff_overlap_matrix = static_cast<double *>(std::calloc(np * np, sizeof(double)));
      if (!pp.pspw_overlap_matrix || !pp.aepw_overlap_matrix || !pp.diff_overlap_matrix)
        throw std::bad_alloc();
      std::vector<double> prod(ng), sb(ng), sc(ng), sd(ng);
      for (int i = 0; i < np; i++)
        for (int j = i; j < np; j++) {
          if (pp.funcs[i].l != pp.funcs[j].l) continue;
          const funcset_t &a = pp.funcs[i], &b = pp.funcs[j];
          double *mats[3] = {pp.pspw_overlap_matrix, pp.aepw_overlap_matrix, pp.diff_overlap_matrix};
          for (int which = 0; which < 3; which++) {
            for (int q = 0; q < ng; q++) {
              if (which == 0) prod[q] = a.pswave[q] * b.pswave[q];
              else if (which == 1) prod[q] = a.aewave[q] * b.aewave[q];
              else prod[q] = (a.aewave[q] - a.pswave[q]) * (b.aewave[q] - b.pswave[q]);
            }
            spline_coeffs(pp.wave_grid, prod.data(), ng, sb.data(), sc.data(), sd.data());
            double v = spline_integral(pp.wave_grid, prod.data(), sb.data(), sc.data(), sd.data(), ng);
            mats[which][i * np + j] = v;
            mats[which][j * np + i] = v;
          }
        }
    }
  } catch (...) {
    free_ppot_array(pps, num_els);
    throw;
  }
  return pps;
}

// ---------------------------------------------------- off-site pair matrix

static double fact(int n) {
  double t = 1;
  for (int m = 1; m <= n; m++) t *= m;
  return t;
}

// associated Legendre P_l^m(x), Condon-Shortley phase, as utils.c:377-386
static double plm(int l, int m, double x) {
  if (m < 0) return std::pow(-1.0, m) * fact(l + m) / fact(l - m) * plm(l, -m, x);
  double acc = 0;
  for (int n = l; n >= 0 && 2 * n - l - m >= 0; n--)
    acc += std::pow(x, 2 * n - l - m) * fact(2 * n) / fact(2 * n - l - m) / fact(n) / fact(l - n) *
           std::pow(-1, l - n);
  return acc * std::pow(-1, m) * std::pow(1 - x * x, m / 2.0) / std::pow(2, l);
}

static cd ylm(int l, int m, double theta, double phi) {
  double nrm = std::pow((2 * l + 1) / (4 * M_PI) * fact(l - m) / fact(l + m), 0.5);
  return nrm * plm(l, m, std::cos(theta)) * std::exp(cd(0, m * phi));
}

// spherical Bessel j_l by upward recurrence, zero-guarded as utils.c:804-824
static double bessel_up(double x, int l) {
  if (x < 10e-6) return l == 0 ? 1 : 0;
  double a = std::sin(x) / x, b = std::sin(x) / (x * x) - std::cos(x) / x;
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

// w3j(l1 l2 l3; 0 0 0) * w3j(l1 l2 l3; -m1 m2 m1-m2) * sqrt((2l1+1)(2l2+1)(2l3+1)/4pi),
// the table the reference generates in gaunt.py:11-31 (Racah's formula here).
static double w3j(int j1, int j2, int j3, int m1, int m2, int m3) {
  if (m1 + m2 + m3 != 0 || std::abs(m1) > j1 || std::abs(m2) > j2 || std::abs(m3) > j3) return 0;
  if (j3 < std::abs(j1 - j2) || j3 > j1 + j2) return 0;
  double tri = fact(j1 + j2 - j3) * fact(j1 - j2 + j3) * fact(-j1 + j2 + j3) / fact(j1 + j2 + j3 + 1);
  double pre = std::sqrt(tri * fact(j1 + m1) * fact(j1 - m1) * fact(j2 + m2) * fact(j2 - m2) *
                         fact(j3 + m3) * fact(j3 - m3));
  int kmin = std::max(0, std::max(j2 - j3 - m1, j1 - j3 + m2));
  int kmax = std::min(j1 + j2 - j3, std::min(j1 - m1, j2 + m2));
  double s = 0;
  for (int k = kmin; k <= kmax; k++)
    s += ((k & 1) ? -1.0 : 1.0) / (fact(k) * fact(j3 - j2 + k + m1) * fact(j3 - j1 + k - m2) *
                                   fact(j1 + j2 - j3 - k) * fact(j1 - k - m1) * fact(j2 - k + m2));
  return (((j1 - j2 - m3) & 1) ? -1.0 : 1.0) * pre * s;
}

static double bessel_fac(int lx, int ly, int L, int mx, int my) {
  return w3j(lx, ly, L, 0, 0, 0) * w3j(lx, ly, L, -mx, my, mx - my) *
         std::sqrt((2 * lx + 1) * (2 * ly + 1) * (2 * L + 1) / 4.0 / M_PI);
}

static cd offsite_one(const double *dc, const ppot_t *p1, int f1, const ppot_t *p2, int f2, int l1,
                      int m1, int l2, int m2) {
  int lx = l1, ly = l2, mx = m1, my = m2;
  if (l1 < l2) {
    lx = l2;
    ly = l1;
    mx = m2;
    my = m1;
  }
  if (my < 0) {
    mx = -mx;
    my = -my;
  }
  const double *k1 = p1->kwave_grid, *k2 = p2->kwave_grid;
  int n1 = p1->wave_gridsize, n2 = p2->wave_gridsize;
  double kmax = std::min(k1[n1 - 1], k2[n2 - 1]);
  double kmin = std::max(k1[0], k2[0]);
  double R = std::pow(dc[0] * dc[0] + dc[1] * dc[1] + dc[2] * dc[2], 0.5), th = 0, ph = 0;
  if (R < 10e-12) {
    R = 0;
  } else {
    th = std::acos(dc[2] / R);
    ph = R - std::fabs(dc[2]) < 10e-12 ? 0 : std::acos(dc[0] / std::pow(dc[0] * dc[0] + dc[1] * dc[1], 0.5));
    if (dc[1] < 0) ph = 2 * M_PI - ph;
  }
  const int K = 500;
  std::vector<double> kg(K), fn(K), b(K), c(K), d(K);
  cd total = 0;
  double sign = std::pow(-1, m1) * 8;
  int lo = std::abs(l1 - l2);
  for (int L = lo; L <= l1 + l2; L += 2) {
    for (int q = 0; q < K; q++) {
      kg[q] = kmin * std::pow(kmax / kmin, (double)q / K);
      double kk = kg[q];
      fn[q] = interp_log(kk, n1, k1, p1->funcs[f1].kwave, p1->funcs[f1].kwave_spline) *
              interp_log(kk, n2, k2, p2->funcs[f2].kwave, p2->funcs[f2].kwave_spline) * kk * kk *
              bessel_up(kk * R, L);
    }
    spline_coeffs(kg.data(), fn.data(), K, b.data(), c.data(), d.data());
    double integ = spline_integral(kg.data(), fn.data(), b.data(), c.data(), d.data(), K);
    if (R > 10e-10) {
      static const cd ipow[4] = {cd(1, 0), cd(0, 1), cd(-1, 0), cd(0, -1)};
      total += integ * bessel_fac(lx, ly, L, mx, my) * ylm(L, m1 - m2, th, ph) *
               ipow[((l2 + L - l1) % 4 + 4) % 4] * sign;
    } else if (L == 0 && l1 == l2 && m1 == m2) {
      total += integ * 2 / M_PI;
    }
  }
  return total;
}

void offsite_pair_matrix(const ppot_t *p1, const ppot_t *p2, const double *dcoord, pawpy_c128 *out) {
  int t1 = 0;
  for (int j = 0; j < p1->num_projs; j++) {
    int l1 = p1->funcs[j].l;
    for (int m1 = -l1; m1 <= l1; m1++, t1++) {
      int t2 = 0;
      for (int k = 0; k < p2->num_projs; k++) {
        int l2 = p2->funcs[k].l;
        for (int m2 = -l2; m2 <= l2; m2++, t2++)
          out[(long)t1 * p2->total_projs + t2] = std::conj(offsite_one(dcoord, p1, j, p2, k, l1, m1, l2, m2));
      }
    }
  }
}

void min_image_path(const double *coord, const double *center, const double *L, double *path, double *r) {
  *r = INFINITY;
  for (int i = -1; i <= 1; i++)
    for (int j = -1; j <= 1; j++)
      for (int k = -1; k <= 1; k++) {
        double f0 = coord[0] + i - center[0], f1 = coord[1] + j - center[1], f2 = coord[2] + k - center[2];
        double v0 = f0 * L[0] + f1 * L[3] + f2 * L[6];
        double v1 = f0 * L[1] + f1 * L[4] + f2 * L[7];
        double v2 = f0 * L[2] + f1 * L[5] + f2 * L[8];
        double dd = std::pow(v0 * v0 + v1 * v1 + v2 * v2, 0.5);
        if (dd < *r) {
          path[0] = v0;
          path[1] = v1;
          path[2] = v2;
          *r = dd;
        }
      }
}

}  // namespace pawpy

// Host double-precision pieces of the radial work: the reference's spline
// (a clamped-start / natural-end cubic whose first slope is the first secant,
// utils.c:699-749) and its integral, log-grid interpolation (utils.c:477-489),
// and the off-site partial-wave overlap of a site pair (radial.c:116-196)
// with its 500-point k quadrature. The per-element setup runs on the device
// (radial.cu).
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
  // polynomial coefficients of each interval. The start slope is the first
  // secant (clamped end; b[0] is then exactly 0); a secant above 0.99e30 selects
  // the natural end instead. That test is kept only so that the sweep follows the
  // reference's (utils.c:699-749) operation for operation; the radial functions
  // of a POTCAR never take it.
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

// Weights w with spline_integral(x, y, spline_coeffs(x, y)) = sum_i w_i y_i for
// every y: the spline (utils.c:699-749) and its integral are linear in y, so w
// is the gradient of the integral, obtained in O(n) by running the recurrences
// in reverse. Per interval the integral is h (y_i + y_{i+1})/2 - h^3 (M_i + M_{i+1})/24
// with M the second derivatives of the tridiagonal sweep.
void spline_integral_weights(const double *x, int n, double *w) {
  std::vector<double> h(n), cc(n), alpha(n), beta(n), gam(n, 0.0), Mbar(n, 0.0), bbar(n, 0.0), ddbar(n, 0.0);
  for (int i = 0; i < n - 1; i++) h[i] = x[i + 1] - x[i];
  // forward sweep coefficients (depend on x only): b_i = alpha_i dd_i + beta_i b_{i-1}, M_i = c_i M_{i+1} + b_i
  cc[0] = -0.5;
  for (int i = 1; i < n - 1; i++) {
    double sig = (x[i] - x[i - 1]) / (x[i + 1] - x[i - 1]);
    double p = sig * cc[i - 1] + 2;
    cc[i] = (sig - 1) / p;
    alpha[i] = 6 / (x[i + 1] - x[i - 1]) / p;
    beta[i] = -sig / p;
  }
  cc[n - 1] = 0;
  for (int i = 0; i < n; i++) w[i] = 0;
  for (int i = 0; i < n - 1; i++) {
    w[i] += h[i] / 2;
    w[i + 1] += h[i] / 2;
    double g = -h[i] * h[i] * h[i] / 24;
    gam[i] += g;
    gam[i + 1] += g;
  }
  // adjoint of M_i = c_i M_{i+1} + b_i (computed for i = n-2 .. 0; M_{n-1} = 0)
  for (int i = 0; i <= n - 2; i++) {
    Mbar[i] += gam[i];
    Mbar[i + 1] += cc[i] * Mbar[i];
    bbar[i] += Mbar[i];
  }
  // adjoint of b_i = alpha_i dd_i + beta_i b_{i-1} (i = 1 .. n-2; b_0 = 0 because the first
  // slope equals the first secant)
  for (int i = n - 2; i >= 1; i--) {
    ddbar[i] += alpha[i] * bbar[i];
    bbar[i - 1] += beta[i] * bbar[i];
  }
  // adjoint of dd_i = (y_{i+1} - y_i)/h_i - (y_i - y_{i-1})/h_{i-1}
  for (int i = 1; i <= n - 2; i++) {
    w[i + 1] += ddbar[i] / h[i];
    w[i] -= ddbar[i] / h[i] + ddbar[i] / h[i - 1];
    w[i - 1] += ddbar[i] / h[i - 1];
  }
}

double interp_log(double r, int n, const double *x, const double *f, double *const *s) {
  if (r > x[n - 1]) return 0;
  if (r < x[0]) return f[0];
  int i = (int)(std::log(r / x[0]) / std::log(x[1] / x[0]));
  if (i > n - 2) i = n - 2;
  double t = r - x[i];
  return f[i] + t * (s[0][i] + t * (s[1][i] + t * s[2][i]));
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

// |d| and the angles of the pair displacement, as radial.c:146-160
static void pair_geometry(const double *dc, double *R, double *th, double *ph) {
  *R = std::pow(dc[0] * dc[0] + dc[1] * dc[1] + dc[2] * dc[2], 0.5);
  *th = 0;
  *ph = 0;
  if (*R < 10e-12) {
    *R = 0;
    return;
  }
  *th = std::acos(dc[2] / *R);
  *ph = *R - std::fabs(dc[2]) < 10e-12 ? 0 : std::acos(dc[0] / std::pow(dc[0] * dc[0] + dc[1] * dc[1], 0.5));
  if (dc[1] < 0) *ph = 2 * M_PI - *ph;
}

double pair_distance(const double *dcoord) {
  double R, th, ph;
  pair_geometry(dcoord, &R, &th, &ph);
  return R;
}

namespace {
// bessel_fac(lx, ly, L, mx, my) for lx >= ly, 0 <= my <= ly <= lx <= 3, |mx| <= lx, L <= 6: the
// same values, computed once (the pair matrices ask for them ~10^5 times per 216-atom pair set)
struct BesselFacTable {
  double v[4][4][7][7][4];
  BesselFacTable() {
    for (int lx = 0; lx < 4; lx++)
      for (int ly = 0; ly <= lx; ly++)
        for (int L = 0; L < 7; L++)
          for (int mx = -lx; mx <= lx; mx++)
            for (int my = 0; my <= ly; my++) v[lx][ly][L][mx + 3][my] = bessel_fac(lx, ly, L, mx, my);
  }
};
const BesselFacTable &bessel_fac_table() {
  static const BesselFacTable t;
  return t;
}
}  // namespace

void offsite_pair_matrix(const ppot_t *p1, const ppot_t *p2, const double *dcoord, const double *I, int Lmax,
                         pawpy_c128 *out) {
  double R, th, ph;
  pair_geometry(dcoord, &R, &th, &ph);
  static const cd ipow[4] = {cd(1, 0), cd(0, 1), cd(-1, 0), cd(0, -1)};
  const BesselFacTable &bf = bessel_fac_table();
  // Y_L^m of the pair direction for every (L, m) the sums below reach (m = m1 - m2)
  cd Y[7][13];
  if (R > 10e-10)
    for (int L = 0; L <= Lmax && L < 7; L++)
      for (int m = -L; m <= L; m++) Y[L][m + 6] = ylm(L, m, th, ph);
  int nf2 = p2->num_projs;
  int t1 = 0;
  for (int f1 = 0; f1 < p1->num_projs; f1++) {
    int l1 = p1->funcs[f1].l;
    for (int m1 = -l1; m1 <= l1; m1++, t1++) {
      int t2 = 0;
      for (int f2 = 0; f2 < nf2; f2++) {
        int l2 = p2->funcs[f2].l;
        for (int m2 = -l2; m2 <= l2; m2++, t2++) {
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
          cd total = 0;
          double sign = std::pow(-1, m1) * 8;
          int lo = std::abs(l1 - l2);
          for (int L = lo; L <= l1 + l2; L += 2) {
            double integ = I[((long)f1 * nf2 + f2) * (Lmax + 1) + L];
            if (R > 10e-10) {
              // ylm(L, m, .) is zero for |m| > L (plm's factorials of negative arguments)
              cd y = std::abs(m1 - m2) <= L ? Y[L][m1 - m2 + 6] : ylm(L, m1 - m2, th, ph);
              total += integ * bf.v[lx][ly][L][mx + 3][my] * y * ipow[((l2 + L - l1) % 4 + 4) % 4] * sign;
            } else if (L == 0 && l1 == l2 && m1 == m2) {
              total += integ * 2 / M_PI;
            }
          }
          out[(long)t1 * p2->total_projs + t2] = std::conj(total);
        }
      }
    }
  }
}

// Upper bound on the grid points inside an element's largest sphere, as
// add_num_cart_gridpts (projector.c:455-505) computes it for ppot_t.num_cart_gridpts.
int cart_gridpts_bound(const ppot_t &pp, const double *lat, const int *fftg) {
  auto dot = [](const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; };
  auto mag = [&](const double *a) { return std::pow(dot(a, a), 0.5); };
  auto cross = [](const double *a, const double *b, double *o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
  };
  double m1 = mag(lat), m2 = mag(lat + 3), m3 = mag(lat + 6), v[3];
  double rmax = pp.rmax;
  if (pp.wave_grid[pp.wave_gridsize - 1] > rmax) rmax = pp.wave_grid[pp.wave_gridsize - 1];
  double p12 = std::acos(dot(lat, lat + 3) / (m1 * m2));
  cross(lat, lat + 3, v);
  double s = dot(lat + 6, v) / (mag(v) * m3);
  double a1 = rmax * fftg[0] / (m1 * std::fabs(std::sin(p12))) + 1;
  double a2 = rmax * fftg[1] / (m2 * std::fabs(std::sin(p12))) + 1;
  double a3 = rmax * fftg[2] / (m3 * std::fabs(s)) + 1;
  int nA = (int)(4.0 / 3.0 * M_PI * a1 * a2 * a3) + 1;
  double p13 = std::acos(dot(lat, lat + 6) / (m1 * m3));
  cross(lat, lat + 6, v);
  s = dot(lat + 3, v) / (mag(v) * m2);
  double b1 = rmax * fftg[0] / (m1 * std::fabs(std::sin(p13))) + 1;
  double b2 = rmax * fftg[1] / (m2 * std::fabs(s)) + 1;
  double b3 = rmax * fftg[2] / (m3 * std::fabs(std::sin(p13))) + 1;
  int nB = (int)(4.0 / 3.0 * M_PI * b1 * b2 * b3) + 1;
  double p23 = std::acos(dot(lat + 3, lat + 6) / (m2 * m3));
  cross(lat + 3, lat + 6, v);
  s = dot(lat, v) / (mag(v) * m1);
  double c1 = rmax * fftg[0] / (m1 * std::fabs(s)) + 1;
  double c2 = rmax * fftg[1] / (m2 * std::fabs(std::sin(p23))) + 1;
  double c3 = rmax * fftg[2] / (m3 * std::fabs(std::sin(p23))) + 1;
  int nC = (int)(4.0 / 3.0 * M_PI * c1 * c2 * c3) + 1;
  return std::max(nA, std::max(nB, nC));
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

/* TEST INFRASTRUCTURE -- the oracle (checker) for the band-projection path.
 * See oracle.h. A restatement of the reference algorithm in plain C; the
 * product library never links this file. Double precision throughout. */
#include "oracle.h"

#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define O_PI 3.14159265358979323846
#define O_C 0.262465831 /* hbar^2/2m, projector.c:17 */

/* ------------------------------------------------------------------------ */
/* spline (utils.c:699-749) and its integral (utils.c:751-764)               */
/* ------------------------------------------------------------------------ */

void oracle_spline_coeff(const double *x, const double *y, int n, double *b,
                         double *c, double *d) {
  /* b/c/d play the roles of coeff[0]/coeff[1]/coeff[2] of the reference. */
  double slope0 = (y[1] - y[0]) / (x[1] - x[0]);
  if (slope0 > 0.99e30) {
    c[0] = 0;
    b[0] = 0;
  } else {
    c[0] = -0.5;
    b[0] = (3 / (x[1] - x[0])) * ((y[1] - y[0]) / (x[1] - x[0]) - slope0);
  }
  for (int i = 1; i < n - 1; i++) {
    double s = (x[i] - x[i - 1]) / (x[i + 1] - x[i - 1]);
    double r = s * c[i - 1] + 2;
    c[i] = (s - 1) / r;
    b[i] = (6 * ((y[i + 1] - y[i]) / (x[i + 1] - x[i]) - (y[i] - y[i - 1]) / (x[i] - x[i - 1])) /
                (x[i + 1] - x[i - 1]) -
            s * b[i - 1]) /
           r;
  }
  b[n - 1] = c[n - 1] = d[n - 1] = 0;
  for (int i = n - 2; i >= 0; i--) c[i] = c[i] * c[i + 1] + b[i];
  for (int i = 0; i < n - 1; i++) {
    double h = x[i + 1] - x[i];
    double r = (c[i + 1] - c[i]) / 6;
    d[i] = r / h;
    c[i] = c[i] / 2;
    b[i] = (y[i + 1] - y[i]) / h - (c[i] + r) * h;
  }
}

double oracle_spline_integral(const double *x, const double *a, const double *b,
                              const double *c, const double *d, int n) {
  double acc = 0;
  for (int i = 0; i < n - 1; i++) {
    double h = x[i + 1] - x[i];
    acc += h * (a[i] + h * (b[i] / 2 + h * (c[i] / 3 + d[i] * h / 4)));
  }
  return acc;
}

/* proj_interpolate, utils.c:461-475 (linear grid x[j] = rmax*j/size) */
static double lin_interp(double r, double rmax, int size, const double *x,
                         const double *f, const double *b, const double *c,
                         const double *d) {
  if (r > x[size - 1]) return 0;
  if (r < x[0]) return f[0];
  int ind = (int)(r / rmax * size);
  if (ind > size - 2) ind = size - 2;
  double t = r - x[ind];
  return f[ind] + t * (b[ind] + t * (c[ind] + t * d[ind]));
}

/* wave_interpolate, utils.c:477-489 (log grid) */
static double log_interp(double r, int size, const double *x, const double *f,
                         const double *b, const double *c, const double *d) {
  if (r > x[size - 1]) return 0;
  if (r < x[0]) return f[0];
  int ind = (int)(log(r / x[0]) / log(x[1] / x[0]));
  if (ind > size - 2) ind = size - 2;
  double t = r - x[ind];
  return f[ind] + t * (b[ind] + t * (c[ind] + t * d[ind]));
}

/* ------------------------------------------------------------------------ */
/* Legendre / Y_lm, complex Condon-Shortley (utils.c:377-386, 431-448)       */
/* ------------------------------------------------------------------------ */

static double ofac(int n) {
  double t = 1;
  for (int m = 1; m <= n; m++) t *= m;
  return t;
}

double oracle_legendre(int l, int m, double x) {
  if (m < 0) return pow(-1.0, m) * ofac(l + m) / ofac(l - m) * oracle_legendre(l, -m, x);
  double acc = 0;
  for (int n = l; n >= 0 && 2 * n - l - m >= 0; n--)
    acc += pow(x, 2 * n - l - m) * ofac(2 * n) / ofac(2 * n - l - m) / ofac(n) / ofac(l - n) *
           pow(-1, l - n);
  return acc * pow(-1, m) * pow(1 - x * x, m / 2.0) / pow(2, l);
}

void oracle_ylm(int l, int m, double theta, double phi, double *re, double *im) {
  double nrm = sqrt((2 * l + 1) / (4 * O_PI) * ofac(l - m) / ofac(l + m));
  double v = nrm * oracle_legendre(l, m, cos(theta));
  *re = v * cos(m * phi);
  *im = v * sin(m * phi);
}

/* angles of a displacement as utils.c:553-561 */
static void angles(const double *t, double r, double *theta, double *phi) {
  *theta = acos(t[2] / r);
  if (r - fabs(t[2]) == 0)
    *phi = 0;
  else
    *phi = acos(t[0] / sqrt(t[0] * t[0] + t[1] * t[1]));
  if (t[1] < 0) *phi = 2 * O_PI - *phi;
}

/* ------------------------------------------------------------------------ */
/* double precision mixed-radix Stockham FFT                                  */
/* ------------------------------------------------------------------------ */

typedef struct {
  int n, nf, f[40];
  double complex *w; /* exp(+2 pi i m / n) */
} oplan;

static void oplan_init(oplan *p, int n) {
  p->n = n;
  p->nf = 0;
  int m = n;
  for (int q = 2; m > 1; q++)
    while (m % q == 0) {
      p->f[p->nf++] = q;
      m /= q;
    }
  p->w = (double complex *)malloc(sizeof(double complex) * (n > 0 ? n : 1));
  for (int i = 0; i < n; i++) {
    double a = 2.0 * O_PI * (double)i / (double)n;
    p->w[i] = cos(a) + I * sin(a);
  }
}

static void oplan_free(oplan *p) { free(p->w); }

static inline double complex wpow(const oplan *p, long e, int sign) {
  double complex v = p->w[e % p->n];
  return sign > 0 ? v : conj(v);
}

/* In-place transform of x[n] using work[n]; sign +1 = exp(+i..) (backward). */
static void offt(const oplan *p, double complex *x, double complex *work, int sign) {
  int n = p->n;
  double complex *src = x, *dst = work;
  long ns = 1;
  double complex v[64], o[64];
  for (int s = 0; s < p->nf; s++) {
    int R = p->f[s];
    long stride = n / R;
    for (long j = 0; j < stride; j++) {
      long k = j % ns;
      for (int r = 0; r < R; r++)
        v[r] = src[j + r * stride] * wpow(p, k * r * (n / (ns * R)), sign);
      for (int q = 0; q < R; q++) {
        double complex acc = 0;
        for (int r = 0; r < R; r++) acc += v[r] * wpow(p, (long)((r * q) % R) * (n / R), sign);
        o[q] = acc;
      }
      long base = (j / ns) * ns * R + k;
      for (int q = 0; q < R; q++) dst[base + q * ns] = o[q];
    }
    double complex *t = src;
    src = dst;
    dst = t;
    ns *= R;
  }
  if (src != x) memcpy(x, src, sizeof(double complex) * n);
}

/* backward (exp(+i)) unnormalised 3D transform of a C-ordered grid */
static void offt3d(double complex *g, const int *N, oplan *pl, double complex *line,
                   double complex *work) {
  long n0 = N[0], n1 = N[1], n2 = N[2];
  for (long a = 0; a < n0 * n1; a++) offt(&pl[2], g + a * n2, work, +1);
  for (long a = 0; a < n0; a++)
    for (long c = 0; c < n2; c++) {
      for (long b = 0; b < n1; b++) line[b] = g[(a * n1 + b) * n2 + c];
      offt(&pl[1], line, work, +1);
      for (long b = 0; b < n1; b++) g[(a * n1 + b) * n2 + c] = line[b];
    }
  for (long b = 0; b < n1; b++)
    for (long c = 0; c < n2; c++) {
      for (long a = 0; a < n0; a++) line[a] = g[(a * n1 + b) * n2 + c];
      offt(&pl[0], line, work, +1);
      for (long a = 0; a < n0; a++) g[(a * n1 + b) * n2 + c] = line[a];
    }
}

/* fft3d restatement (linalg.c:14-45): zero, scatter at (G mod N), backward
 * transform scaled by vol^-1/2, with caller-owned plans and scratch lines. */
static void fft3d_with(double complex *x, const int *Gs, const float *Cs, int nw,
                       const int *fftg, double vol, oplan *pl, double complex *line,
                       double complex *work) {
  long tot = (long)fftg[0] * fftg[1] * fftg[2];
  memset(x, 0, sizeof(double complex) * tot);
  for (int w = 0; w < nw; w++) {
    int g1 = (Gs[3 * w] + fftg[0]) % fftg[0];
    int g2 = (Gs[3 * w + 1] + fftg[1]) % fftg[1];
    int g3 = (Gs[3 * w + 2] + fftg[2]) % fftg[2];
    x[((long)g1 * fftg[1] + g2) * fftg[2] + g3] = Cs[2 * w] + I * Cs[2 * w + 1];
  }
  offt3d(x, fftg, pl, line, work);
  double s = pow(vol, -0.5);
  for (long i = 0; i < tot; i++) x[i] *= s;
}

void oracle_fft3d(double *xv, const int *Gs, const float *Cs, int nw, const int *fftg,
                  double vol) {
  oplan pl[3];
  int mx = 0;
  for (int a = 0; a < 3; a++) {
    oplan_init(&pl[a], fftg[a]);
    if (fftg[a] > mx) mx = fftg[a];
  }
  double complex *line = malloc(sizeof(double complex) * mx);
  double complex *work = malloc(sizeof(double complex) * mx);
  fft3d_with((double complex *)xv, Gs, Cs, nw, fftg, vol, pl, line, work);
  free(line);
  free(work);
  for (int a = 0; a < 3; a++) oplan_free(&pl[a]);
}

/* ------------------------------------------------------------------------ */
/* spherical Bessel transform (sbt.c:24-215)                                  */
/* ------------------------------------------------------------------------ */

typedef struct {
  int N, lmax;
  double kmin, kappamin, rmin, rhomin, drho, dt;
  double *ks, *rs;
  double complex *M; /* (lmax+1) x N */
} osbt;

static void osbt_setup(osbt *d, double encut, double enbuf, int lmax, int n,
                       const double *r, double *inpks) {
  int N = 2 * n;
  if (lmax == 0) lmax = 1;
  d->N = N;
  d->lmax = lmax;
  d->ks = malloc(sizeof(double) * N);
  d->rs = calloc((size_t)N, sizeof(double));
  d->M = calloc((size_t)(lmax + 1) * N, sizeof(double complex));
  double drho = log(r[1] / r[0]);
  double dt = 2 * O_PI / N / drho;
  double rmin = r[0];
  double kmin = pow((encut + enbuf) * O_C, 0.5) * exp(-(N / 2 - 1) * drho);
  double kappamin = log(kmin);
  for (int i = 0; i < N; i++) {
    d->ks[i] = kmin * exp(i * drho);
    d->rs[i] = rmin * exp((i - N / 2) * drho);
  }
  if (inpks)
    for (int i = 0; i < N / 2; i++) inpks[i] = d->ks[i];
  double rhomin = log(d->rs[0]);
  /* M_l(t): phase of Gamma(1/2+it) by a 10-step shift and the Stirling series,
   * Talman, Comput. Phys. Commun. 180 (2009) 332. */
  for (int i = 0; i < N; i++) {
    double t = i * dt;
    double rad = sqrt(10.5 * 10.5 + t * t);
    double p3 = (kappamin + rhomin) * t;
    double ph = atan((2 * t) / 21);
    double p1 = -10 * ph - t * log(rad) + t + sin(ph) / (12 * rad) -
                sin(3 * ph) / (360 * pow(rad, 3)) + sin(5 * ph) / (1260 * pow(rad, 5)) -
                sin(7 * ph) / (1680 * pow(rad, 7));
    for (int j = 1; j <= 10; j++) p1 += atan((2 * t) / (2 * j - 1));
    double p2 = -atan(tanh(O_PI * t / 2));
    double tot = p1 + p2 + p3;
    double complex m0 = sqrt(O_PI / 2) * cexp(I * tot) / N;
    if (i == 0) m0 *= 0.5;
    d->M[0 * N + i] = m0;
    double a = -p2 - atan(2 * t);
    d->M[1 * N + i] = cexp(2 * I * a) * m0;
    for (int l = 1; l < lmax; l++) {
      double b = -atan(2 * t / (2 * l + 1));
      d->M[(l + 1) * N + i] = cexp(2 * I * b) * d->M[(l - 1) * N + i];
    }
  }
  d->kmin = kmin;
  d->kappamin = kappamin;
  d->rmin = rmin;
  d->rhomin = rhomin;
  d->drho = drho;
  d->dt = dt;
}

static void osbt_free(osbt *d) {
  free(d->ks);
  free(d->rs);
  free(d->M);
}

/* wave_spherical_bessel_transform (sbt.c:102-154); out[n/2] */
static void osbt_fwd(const osbt *d, const double *f, int l, double *out) {
  int N = d->N;
  oplan pl;
  oplan_init(&pl, N);
  double complex *x = calloc(N, sizeof(double complex));
  double complex *w = malloc(sizeof(double complex) * N);
  double C = f[0] / pow(d->rs[N / 2], l + 1);
  for (int i = 0; i < N; i++) {
    double fs = i < N / 2 ? C * pow(d->rs[i], l + 1) : f[i - N / 2];
    x[i] = pow(d->rs[i], 0.5) * fs;
  }
  offt(&pl, x, w, +1);
  for (int i = 0; i < N; i++) x[i] = i < N / 2 ? x[i] * d->M[l * N + i] : 0;
  offt(&pl, x, w, +1);
  for (int p = 0; p < N / 2; p++) out[p] = creal(x[p]) * 2 / pow(d->ks[p], 1.5);
  free(x);
  free(w);
  oplan_free(&pl);
}

/* inverse_wave_spherical_bessel_transform (sbt.c:156-215); out[n/2] */
static void osbt_inv(const osbt *d, const double *fk, int l, double *out) {
  int N = d->N;
  oplan pl;
  oplan_init(&pl, N);
  double complex *x = calloc(N, sizeof(double complex));
  double complex *w = malloc(sizeof(double complex) * N);
  for (int i = 0; i < N; i++) x[i] = i < N / 2 ? pow(d->ks[i], 1.5) * fk[i] : 0;
  offt(&pl, x, w, +1);
  for (int i = 0; i < N; i++) x[i] = i < N / 2 ? x[i] * d->M[l * N + i] : 0;
  offt(&pl, x, w, +1);
  for (int p = 0; p < N / 2; p++)
    out[p] = creal(x[p + N / 2]) / O_PI * 2 * 2 / pow(d->rs[p + N / 2], 1.5);
  free(x);
  free(w);
  oplan_free(&pl);
}

void oracle_sbt_forward(double encut, int lmax, int n, const double *r, const double *f,
                        int l, double *ks, double *out) {
  osbt d;
  osbt_setup(&d, encut, 0, lmax, n, r, ks);
  osbt_fwd(&d, f, l, out);
  osbt_free(&d);
}

void oracle_sbt_inverse(double encut, int lmax, int n, const double *r, const double *fk,
                        int l, double *out) {
  osbt d;
  osbt_setup(&d, encut, 0, lmax, n, r, NULL);
  osbt_inv(&d, fk, l, out);
  osbt_free(&d);
}

/* ------------------------------------------------------------------------ */
/* species setup (projector.c:20-171 per element; 507-558)                    */
/* ------------------------------------------------------------------------ */

void oracle_species_setup(int nproj, const int *ls, int ndata, int ngrid, double rmax,
                          const double *wg, const double *proj, const double *ae,
                          const double *ps, double grid_encut, double *proj_grid,
                          double *proj_spl, double *smooth_grid, double *sdw,
                          double *sdw_spl, double *kgrid, double *kwave,
                          double *kwave_spl, double *aeov, double *psov, double *diov) {
  int lmax = 0;
  for (int k = 0; k < nproj; k++)
    if (ls[k] > lmax) lmax = ls[k];
  for (int j = 0; j < ndata; j++) proj_grid[j] = rmax / ndata * j;
  /* dense grid: a cumulative product of the first ratio (projector.c:62-67) */
  double *dense = malloc(sizeof(double) * ngrid);
  dense[0] = wg[0];
  double factor = pow(wg[1] / wg[0], 1.0);
  for (int p = 1; p < ngrid; p++) dense[p] = dense[p - 1] * factor;
  double wave_rmax = wg[ngrid - 1];
  for (int j = 0; j < ndata; j++) smooth_grid[j] = wave_rmax / ndata * j;
  double *diff = malloc(sizeof(double) * ngrid);
  osbt d;
  osbt_setup(&d, 1e7, 0, lmax, ngrid, wg, kgrid);
  double *fk = malloc(sizeof(double) * ngrid);
  double *sm = malloc(sizeof(double) * ngrid);
  double *sb = malloc(sizeof(double) * ngrid * 3);
  double kcut = pow(O_C * grid_encut, 0.5);
  for (int k = 0; k < nproj; k++) {
    const double *pk = proj + (long)k * ndata;
    double *ps3 = proj_spl + (long)k * 3 * ndata;
    oracle_spline_coeff(proj_grid, pk, ndata, ps3, ps3 + ndata, ps3 + 2 * ndata);
    for (int j = 0; j < ngrid; j++) diff[j] = ae[(long)k * ngrid + j] - ps[(long)k * ngrid + j];
    double *kw = kwave + (long)k * ngrid;
    osbt_fwd(&d, diff, ls[k], kw);
    double *ks3 = kwave_spl + (long)k * 3 * ngrid;
    oracle_spline_coeff(kgrid, kw, ngrid, ks3, ks3 + ngrid, ks3 + 2 * ngrid);
    /* keep k below sqrt(c*grid_encut), inverse transform (projector.c:127-137) */
    memset(fk, 0, sizeof(double) * ngrid);
    for (int q = 0; q < ngrid && kgrid[q] < kcut; q++) fk[q] = kw[q];
    osbt_inv(&d, fk, ls[k], sm);
    oracle_spline_coeff(dense, sm, ngrid, sb, sb + ngrid, sb + 2 * ngrid);
    double *s = sdw + (long)k * ndata;
    if (ls[k] > 0) s[0] = 0;
    for (int p = 1; p < ndata; p++)
      s[p] = log_interp(smooth_grid[p], ngrid, dense, sm, sb, sb + ngrid, sb + 2 * ngrid);
    if (ls[k] == 0) s[0] = s[1];
    double *ss3 = sdw_spl + (long)k * 3 * ndata;
    oracle_spline_coeff(smooth_grid, s, ndata, ss3, ss3 + ndata, ss3 + 2 * ndata);
  }
  /* partial-wave overlap matrices (projector.c:507-558) */
  double *prod = malloc(sizeof(double) * ngrid);
  double *pb = malloc(sizeof(double) * ngrid * 3);
  memset(aeov, 0, sizeof(double) * nproj * nproj);
  memset(psov, 0, sizeof(double) * nproj * nproj);
  memset(diov, 0, sizeof(double) * nproj * nproj);
  for (int i = 0; i < nproj; i++)
    for (int j = i; j < nproj; j++) {
      if (ls[i] != ls[j]) continue;
      const double *p1 = ps + (long)i * ngrid, *p2 = ps + (long)j * ngrid;
      const double *a1 = ae + (long)i * ngrid, *a2 = ae + (long)j * ngrid;
      for (int which = 0; which < 3; which++) {
        for (int q = 0; q < ngrid; q++) {
          if (which == 0) prod[q] = p1[q] * p2[q];
          else if (which == 1) prod[q] = a1[q] * a2[q];
          else prod[q] = (a1[q] - p1[q]) * (a2[q] - p2[q]);
        }
        oracle_spline_coeff(wg, prod, ngrid, pb, pb + ngrid, pb + 2 * ngrid);
        double v = oracle_spline_integral(wg, prod, pb, pb + ngrid, pb + 2 * ngrid, ngrid);
        double *m = which == 0 ? psov : which == 1 ? aeov : diov;
        m[i * nproj + j] = v;
        m[j * nproj + i] = v;
      }
    }
  free(prod);
  free(pb);
  free(fk);
  free(sm);
  free(sb);
  free(diff);
  free(dense);
  osbt_free(&d);
}

/* ------------------------------------------------------------------------ */
/* sphere tables (utils.c:51-73 min_cart_path, 547-576, 590-696 setup_site)   */
/* ------------------------------------------------------------------------ */

static void to_cart(const double *f, const double *L, double *out) {
  double t0 = f[0] * L[0] + f[1] * L[3] + f[2] * L[6];
  double t1 = f[0] * L[1] + f[1] * L[4] + f[2] * L[7];
  double t2 = f[0] * L[2] + f[1] * L[5] + f[2] * L[8];
  out[0] = t0;
  out[1] = t1;
  out[2] = t2;
}

static double norm3(const double *v) { return pow(v[0] * v[0] + v[1] * v[1] + v[2] * v[2], 0.5); }

static void min_image(const double *coord, const double *center, const double *L,
                      double *path, double *r) {
  *r = INFINITY;
  for (int i = -1; i <= 1; i++)
    for (int j = -1; j <= 1; j++)
      for (int k = -1; k <= 1; k++) {
        double f[3] = {coord[0] + i - center[0], coord[1] + j - center[1], coord[2] + k - center[2]};
        double v[3];
        to_cart(f, L, v);
        double dd = norm3(v);
        if (dd < *r) {
          path[0] = v[0];
          path[1] = v[1];
          path[2] = v[2];
          *r = dd;
        }
      }
}

static void cross3(const double *a, const double *b, double *o) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}

int oracle_site_table(const double *L, const int *fftg, const double *coord, double rmax,
                      int size, int r0_size, const double *x, int nproj, const int *ls,
                      const double *f, const double *spl, int cap, int *indices,
                      double *paths, double *values) {
  double vol = L[0] * L[4] * L[8] + L[1] * L[5] * L[6] + L[2] * L[3] * L[7] -
               L[2] * L[4] * L[6] - L[1] * L[3] * L[8] - L[0] * L[5] * L[7];
  int total = 0;
  for (int j = 0; j < nproj; j++) total += 2 * ls[j] + 1;
  double res[3];
  cross3(L + 3, L + 6, res);
  int g1 = (int)(norm3(res) * rmax / vol * fftg[0]) + 1;
  cross3(L + 0, L + 6, res);
  int g2 = (int)(norm3(res) * rmax / vol * fftg[1]) + 1;
  cross3(L + 0, L + 3, res);
  int g3 = (int)(norm3(res) * rmax / vol * fftg[2]) + 1;
  int c1 = (int)round(coord[0] * fftg[0]);
  int c2 = (int)round(coord[1] * fftg[1]);
  int c3 = (int)round(coord[2] * fftg[2]);
  double R0 = (size - 1) * rmax / r0_size;
  int n = 0;
  for (int i = -g1 + c1; i <= g1 + c1; i++)
    for (int j = -g2 + c2; j <= g2 + c2; j++)
      for (int k = -g3 + c3; k <= g3 + c3; k++) {
        double fr[3] = {(double)i / fftg[0] - coord[0], (double)j / fftg[1] - coord[1],
                        (double)k / fftg[2] - coord[2]};
        double tc[3];
        to_cart(fr, L, tc);
        if (!(norm3(tc) < R0)) continue;
        if (n >= cap) return -1;
        int ii = (i % fftg[0] + fftg[0]) % fftg[0];
        int jj = (j % fftg[1] + fftg[1]) % fftg[1];
        int kk = (k % fftg[2] + fftg[2]) % fftg[2];
        indices[n] = (ii * fftg[1] + jj) * fftg[2] + kk;
        paths[3 * n] = tc[0];
        paths[3 * n + 1] = tc[1];
        paths[3 * n + 2] = tc[2];
        double gp[3] = {(double)ii / fftg[0], (double)jj / fftg[1], (double)kk / fftg[2]};
        double t[3] = {0, 0, 0}, r = 0;
        min_image(gp, coord, L, t, &r);
        int p = 0;
        for (int q = 0; q < nproj; q++) {
          const double *fq = f + (long)q * size;
          const double *sq = spl + (long)q * 3 * size;
          double rad = lin_interp(r, rmax, size, x, fq, sq, sq + size, sq + 2 * size);
          for (int m = -ls[q]; m <= ls[q]; m++, p++) {
            double yr, yi;
            if (r == 0) {
              oracle_ylm(ls[q], m, 0, 0, &yr, &yi);
            } else {
              double th, ph;
              angles(t, r, &th, &ph);
              oracle_ylm(ls[q], m, th, ph, &yr, &yi);
            }
            values[2 * ((long)n * total + p)] = rad * yr;
            values[2 * ((long)n * total + p) + 1] = rad * yi;
          }
        }
        n++;
      }
  return n;
}

/* ------------------------------------------------------------------------ */
/* FFT + sphere gather for many bands (onto_projector, projector.c:223-357)   */
/* ------------------------------------------------------------------------ */

void oracle_project_bands(int nb, const float *Cs, long stride, const int *Gs, int nw,
                          const int *fftg, const double *L, const double *kcart,
                          int nsites, const int *npts, const long *toff, const long *voff,
                          const int *total, const int *ooff, int ntot, const int *indices,
                          const double *paths, const double *values, double *out) {
  double vol = L[0] * L[4] * L[8] + L[1] * L[5] * L[6] + L[2] * L[3] * L[7] -
               L[2] * L[4] * L[6] - L[1] * L[3] * L[8] - L[0] * L[5] * L[7];
  long tot = (long)fftg[0] * fftg[1] * fftg[2];
  double dv = vol / fftg[0] / fftg[1] / fftg[2];
#pragma omp parallel
  {
    double complex *x = malloc(sizeof(double complex) * tot);
    int maxp = 0;
    for (int s = 0; s < nsites; s++)
      if (npts[s] > maxp) maxp = npts[s];
    double complex *xv = malloc(sizeof(double complex) * (maxp > 0 ? maxp : 1));
    oplan pl[3];
    int mx = 0;
    for (int a = 0; a < 3; a++) {
      oplan_init(&pl[a], fftg[a]);
      if (fftg[a] > mx) mx = fftg[a];
    }
    double complex *line = malloc(sizeof(double complex) * mx);
    double complex *work = malloc(sizeof(double complex) * mx);
#pragma omp for schedule(dynamic)
    for (int b = 0; b < nb; b++) {
      fft3d_with(x, Gs, Cs + 2 * (long)b * stride, nw, fftg, vol, pl, line, work);
      for (int s = 0; s < nsites; s++) {
        const int *ind = indices + toff[s];
        const double *pth = paths + 3 * toff[s];
        for (int i = 0; i < npts[s]; i++) {
          double kr = kcart[0] * pth[3 * i] + kcart[1] * pth[3 * i + 1] + kcart[2] * pth[3 * i + 2];
          xv[i] = x[ind[i]] * dv * cexp(I * kr);
        }
        const double complex *val = (const double complex *)(values) + voff[s];
        for (int p = 0; p < total[s]; p++) {
          double complex acc = 0;
          for (int i = 0; i < npts[s]; i++) acc += conj(val[(long)i * total[s] + p]) * xv[i];
          long o = (long)b * ntot + ooff[s] + p;
          out[2 * o] = creal(acc);
          out[2 * o + 1] = cimag(acc);
        }
      }
    }
    free(x);
    free(xv);
    free(line);
    free(work);
    for (int a = 0; a < 3; a++) oplan_free(&pl[a]);
  }
}

/* ------------------------------------------------------------------------ */
/* aug_recip augmentation coefficients (get_aug_freqs, projector.c:276-331,    */
/* 420-453; fwd_fft3d, linalg.c:47-79)                                          */
/* ------------------------------------------------------------------------ */

/* For nb bands: x(r) = sum over the table's sites s and channels p of
 * P[b][pcol[s] + p] * values_s,p(r) * exp(-i k.path) (get_aug_freqs_helper,
 * projector.c:305-329), the forward transform of x scaled by sqrt(V)/N^3 and
 * read at the nw plane waves Gs (fwd_fft3d). The forward transform is the
 * conjugate of the backward one of conj(x). P: complex128 [nb][pstride];
 * out: complex128 [nb][nw]. */
void oracle_aug_coefficients(int nb, const double *P, long pstride, const int *pcol, const int *Gs, int nw,
                             const int *fftg, const double *L, const double *kcart, int nsites,
                             const int *npts, const long *toff, const long *voff, const int *total,
                             const int *indices, const double *paths, const double *values, double *out) {
  double vol = L[0] * L[4] * L[8] + L[1] * L[5] * L[6] + L[2] * L[3] * L[7] -
               L[2] * L[4] * L[6] - L[1] * L[3] * L[8] - L[0] * L[5] * L[7];
  long tot = (long)fftg[0] * fftg[1] * fftg[2];
  double scale = sqrt(vol) / tot;
#pragma omp parallel
  {
    double complex *x = malloc(sizeof(double complex) * tot);
    oplan pl[3];
    int mx = 0;
    for (int a = 0; a < 3; a++) {
      oplan_init(&pl[a], fftg[a]);
      if (fftg[a] > mx) mx = fftg[a];
    }
    double complex *line = malloc(sizeof(double complex) * mx);
    double complex *work = malloc(sizeof(double complex) * mx);
#pragma omp for schedule(dynamic)
    for (int b = 0; b < nb; b++) {
      memset(x, 0, sizeof(double complex) * tot);
      const double complex *pb = (const double complex *)P + (long)b * pstride;
      for (int s = 0; s < nsites; s++) {
        const int *ind = indices + toff[s];
        const double *pth = paths + 3 * toff[s];
        const double complex *val = (const double complex *)(values) + voff[s];
        for (int i = 0; i < npts[s]; i++) {
          double kr = kcart[0] * pth[3 * i] + kcart[1] * pth[3 * i + 1] + kcart[2] * pth[3 * i + 2];
          double complex ph = cexp(-I * kr);
          for (int p = 0; p < total[s]; p++) x[ind[i]] += pb[pcol[s] + p] * val[(long)i * total[s] + p] * ph;
        }
      }
      for (long i = 0; i < tot; i++) x[i] = conj(x[i]);
      offt3d(x, fftg, pl, line, work);
      for (int w = 0; w < nw; w++) {
        int g1 = (Gs[3 * w] + fftg[0]) % fftg[0];
        int g2 = (Gs[3 * w + 1] + fftg[1]) % fftg[1];
        int g3 = (Gs[3 * w + 2] + fftg[2]) % fftg[2];
        double complex v = conj(x[((long)g1 * fftg[1] + g2) * fftg[2] + g3]) * scale;
        out[2 * ((long)b * nw + w)] = creal(v);
        out[2 * ((long)b * nw + w) + 1] = cimag(v);
      }
    }
    free(x);
    free(line);
    free(work);
    for (int a = 0; a < 3; a++) oplan_free(&pl[a]);
  }
}

/* ------------------------------------------------------------------------ */
/* off-site overlap (radial.c:116-196; sbf utils.c:804-824)                   */
/* ------------------------------------------------------------------------ */

static double osbf(double x, int l) {
  if (x < 10e-6) return l == 0 ? 1 : 0;
  double jm1 = sin(x) / x;
  double j = sin(x) / (x * x) - cos(x) / x;
  double jp1 = 0;
  if (l == 0) return jm1;
  if (l == 1) return j;
  for (int ll = 1; ll < l; ll++) {
    jp1 = (2 * ll + 1) / x * j - jm1;
    jm1 = j;
    j = jp1;
  }
  return jp1;
}

#define KGRID 500

void oracle_offsite(const double *dc, const double *k1, const double *f1, const double *s1,
                    int size1, const double *k2, const double *f2, const double *s2,
                    int size2, int l1, int m1, int l2, int m2, const double *sbtfacs,
                    double *re, double *im) {
  int lx, ly, mx, my;
  if (l1 < l2) {
    lx = l2; ly = l1; mx = m2; my = m1;
  } else {
    lx = l1; ly = l2; mx = m1; my = m2;
  }
  if (my < 0) {
    mx = -mx;
    my = -my;
  }
  double kmax = k1[size1 - 1] < k2[size2 - 1] ? k1[size1 - 1] : k2[size2 - 1];
  double kmin = k1[0] > k2[0] ? k1[0] : k2[0];
  double theta = 0, phi = 0, R = norm3(dc);
  if (R < 10e-12) {
    R = 0;
  } else {
    theta = acos(dc[2] / R);
    if (R - fabs(dc[2]) < 10e-12)
      phi = 0;
    else
      phi = acos(dc[0] / pow(dc[0] * dc[0] + dc[1] * dc[1], 0.5));
    if (dc[1] < 0) phi = 2 * O_PI - phi;
  }
  double kg[KGRID], fn[KGRID], b[KGRID], c[KGRID], d[KGRID];
  double complex total = 0;
  double mult = pow(-1, m1) * 8;
  int lo = abs(l1 - l2);
  for (int L = lo; L <= l1 + l2; L += 2) {
    for (int q = 0; q < KGRID; q++) {
      kg[q] = kmin * pow(kmax / kmin, (double)q / KGRID);
      double kk = kg[q];
      fn[q] = log_interp(kk, size1, k1, f1, s1, s1 + size1, s1 + 2 * size1) *
              log_interp(kk, size2, k2, f2, s2, s2 + size2, s2 + 2 * size2) * kk * kk *
              osbf(kk * R, L);
    }
    oracle_spline_coeff(kg, fn, KGRID, b, c, d);
    double integ = oracle_spline_integral(kg, fn, b, c, d, KGRID);
    if (R > 10e-10) {
      double fac = sbtfacs[(((lx * 4 + ly) * 4 + (L - lo) / 2) * 7 + (lx + mx)) * 4 + my];
      double yr, yi;
      oracle_ylm(L, m1 - m2, theta, phi, &yr, &yi);
      int e = ((l2 + L - l1) % 4 + 4) % 4;
      double complex ip = e == 0 ? 1 : e == 1 ? I : e == 2 ? -1 : -I;
      total += integ * fac * (yr + I * yi) * ip * mult;
    } else if (L == 0 && l1 == l2 && m1 == m2) {
      total += integ * 2 / O_PI;
    }
  }
  *re = creal(total);
  *im = cimag(total);
}

/* The whole pair matrix Q[tj][tk] = conj(offsite(lm_j of site 1, lm_k of site 2)) of one
 * N_RS pair (projector.c:699-712), each element as oracle_offsite. f and s hold every
 * channel of an element back to back (size and 3 size values per channel); n, l, m list the
 * element's lm channels in projector order. out: 2 T1 T2 doubles (re, im). */
void oracle_offsite_matrix(const double *dc, const double *k1, const double *f1, const double *s1,
                           int size1, int T1, const int *n1, const int *l1, const int *m1,
                           const double *k2, const double *f2, const double *s2, int size2, int T2,
                           const int *n2, const int *l2, const int *m2, const double *sbtfacs,
                           double *out) {
#pragma omp parallel for schedule(dynamic)
  for (int t = 0; t < T1 * T2; t++) {
    int tj = t / T2, tk = t % T2;
    double re, im;
    oracle_offsite(dc, k1, f1 + (long)n1[tj] * size1, s1 + (long)n1[tj] * 3 * size1, size1, k2,
                   f2 + (long)n2[tk] * size2, s2 + (long)n2[tk] * 3 * size2, size2, l1[tj], m1[tj],
                   l2[tk], m2[tk], sbtfacs, &re, &im);
    out[2 * t] = re;
    out[2 * t + 1] = -im;
  }
}

/* ------------------------------------------------------------------------ */
/* pseudoprojection for all S bands at one k (pseudoprojector.c:63-90)        */
/* ------------------------------------------------------------------------ */

void oracle_pseudo_k(int nbR, int nbS, int nw, const float *CR, long strideR,
                     const float *CS, long strideS, int fp32, double *out) {
#pragma omp parallel for schedule(dynamic)
  for (int bR = 0; bR < nbR; bR++) {
    const float *a = CR + 2 * (long)bR * strideR;
    for (int bS = 0; bS < nbS; bS++) {
      const float *b = CS + 2 * (long)bS * strideS;
      long o = (long)bS * nbR + bR;
      if (fp32) {
        float complex acc = 0;
        for (int w = 0; w < nw; w++)
          acc += conjf(a[2 * w] + I * a[2 * w + 1]) * (b[2 * w] + I * b[2 * w + 1]);
        out[2 * o] = crealf(acc);
        out[2 * o + 1] = cimagf(acc);
      } else {
        double complex acc = 0;
        for (int w = 0; w < nw; w++)
          acc += conj((double)a[2 * w] + I * (double)a[2 * w + 1]) *
                 ((double)b[2 * w] + I * (double)b[2 * w + 1]);
        out[2 * o] = creal(acc);
        out[2 * o + 1] = cimag(acc);
      }
    }
  }
}

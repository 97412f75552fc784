/* Implementation of the MKL stand-in declared in mkl.h (test infrastructure).
 *
 * The transform is a textbook recursive mixed-radix decimation-in-time
 * Cooley-Tukey FFT in double precision: split N = p*m by its smallest prime
 * factor p, transform the p interleaved subsequences, combine with twiddles
 * exp(s 2 pi i r k / N) evaluated from (r*k mod N) so that every twiddle is a
 * directly computed cos/sin. Multi-dimensional transforms apply the 1D
 * transform along each axis of the C-ordered array. */
#include "mkl.h"

#include <complex.h>
#include <math.h>
#include <stdarg.h>
#include <stdlib.h>
#include <string.h>

struct pawpy_shim_dfti {
  int dim;
  MKL_LONG len[3];
  double fscale, bscale;
};

static const double TWO_PI = 6.283185307179586476925286766559;

static void fft1d(double complex *x, long n, long stride, int sign,
                  double complex *work) {
  if (n == 1) return;
  long p = 2;
  while (p * p <= n && n % p) p++;
  if (n % p) p = n;
  long m = n / p;
  /* gather subsequences: sub r holds x[(r + p*j)*stride], j < m */
  for (long r = 0; r < p; r++)
    for (long j = 0; j < m; j++) work[r * m + j] = x[(r + p * j) * stride];
  if (m > 1) {
    double complex *w2 = (double complex *)malloc(sizeof(double complex) * m);
    for (long r = 0; r < p; r++) fft1d(work + r * m, m, 1, sign, w2);
    free(w2);
  }
  for (long k = 0; k < n; k++) {
    double complex acc = 0;
    long km = k % m;
    for (long r = 0; r < p; r++) {
      long e = (r * k) % n;
      double a = sign * TWO_PI * (double)e / (double)n;
      acc += work[r * m + km] * (cos(a) + I * sin(a));
    }
    x[k * stride] = acc;
  }
}

static void fft_axis(double complex *x, const MKL_LONG *len, int dim, int axis,
                     int sign) {
  long n = len[axis], inner = 1, outer = 1;
  for (int d = axis + 1; d < dim; d++) inner *= len[d];
  for (int d = 0; d < axis; d++) outer *= len[d];
  double complex *work = (double complex *)malloc(sizeof(double complex) * n);
  for (long o = 0; o < outer; o++)
    for (long i = 0; i < inner; i++)
      fft1d(x + o * n * inner + i, n, inner, sign, work);
  free(work);
}

MKL_LONG DftiCreateDescriptor(DFTI_DESCRIPTOR_HANDLE *h, enum DFTI_CONFIG_VALUE prec,
                              enum DFTI_CONFIG_VALUE domain, MKL_LONG dim, ...) {
  if (prec != DFTI_DOUBLE || domain != DFTI_COMPLEX || dim < 1 || dim > 3) return 1;
  struct pawpy_shim_dfti *d = (struct pawpy_shim_dfti *)calloc(1, sizeof(*d));
  va_list ap;
  va_start(ap, dim);
  if (dim == 1) {
    d->len[0] = va_arg(ap, MKL_LONG);
  } else {
    MKL_LONG *l = va_arg(ap, MKL_LONG *);
    for (int i = 0; i < dim; i++) d->len[i] = l[i];
  }
  va_end(ap);
  d->dim = (int)dim;
  d->fscale = d->bscale = 1.0;
  *h = d;
  return 0;
}

MKL_LONG DftiSetValue(DFTI_DESCRIPTOR_HANDLE h, enum DFTI_CONFIG_PARAM p, ...) {
  va_list ap;
  va_start(ap, p);
  double v = va_arg(ap, double);
  va_end(ap);
  if (p == DFTI_FORWARD_SCALE) h->fscale = v;
  else if (p == DFTI_BACKWARD_SCALE) h->bscale = v;
  else return 1;
  return 0;
}

MKL_LONG DftiCommitDescriptor(DFTI_DESCRIPTOR_HANDLE h) { return h ? 0 : 1; }

static MKL_LONG compute(DFTI_DESCRIPTOR_HANDLE h, void *xv, int sign, double scale) {
  double complex *x = (double complex *)xv;
  long total = 1;
  for (int d = 0; d < h->dim; d++) total *= h->len[d];
  for (int a = 0; a < h->dim; a++) fft_axis(x, h->len, h->dim, a, sign);
  if (scale != 1.0)
    for (long i = 0; i < total; i++) x[i] *= scale;
  return 0;
}

MKL_LONG DftiComputeBackward(DFTI_DESCRIPTOR_HANDLE h, void *x, ...) {
  return compute(h, x, +1, h->bscale);
}
MKL_LONG DftiComputeForward(DFTI_DESCRIPTOR_HANDLE h, void *x, ...) {
  return compute(h, x, -1, h->fscale);
}
MKL_LONG DftiFreeDescriptor(DFTI_DESCRIPTOR_HANDLE *h) {
  free(*h);
  *h = NULL;
  return 0;
}
char *DftiErrorMessage(MKL_LONG status) {
  (void)status;
  return (char *)"mkl shim error";
}

void cblas_cdotc_sub(const int n, const void *x, const int incx, const void *y,
                     const int incy, void *dotc) {
  const float complex *a = (const float complex *)x, *b = (const float complex *)y;
  float complex acc = 0;
  for (int i = 0; i < n; i++) acc += conjf(a[i * incx]) * b[i * incy];
  *(float complex *)dotc = acc;
}
void cblas_zdotc_sub(const int n, const void *x, const int incx, const void *y,
                     const int incy, void *dotc) {
  const double complex *a = (const double complex *)x, *b = (const double complex *)y;
  double complex acc = 0;
  for (int i = 0; i < n; i++) acc += conj(a[i * incx]) * b[i * incy];
  *(double complex *)dotc = acc;
}

void *mkl_malloc(size_t size, int align) {
  void *p = NULL;
  if (align < (int)sizeof(void *)) align = sizeof(void *);
  if (posix_memalign(&p, (size_t)align, size ? size : 1)) return NULL;
  return p;
}
void *mkl_calloc(size_t num, size_t size, int align) {
  void *p = mkl_malloc(num * size, align);
  if (p) memset(p, 0, num * size);
  return p;
}
void mkl_free(void *ptr) { free(ptr); }
void mkl_free_buffers(void) {}

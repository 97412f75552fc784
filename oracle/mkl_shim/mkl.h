/* Project-written stand-in for the subset of Intel MKL that the pawpyseed C
 * core calls (DFTI 1D/3D complex double transforms, cblas_cdotc_sub,
 * cblas_zdotc_sub, mkl_malloc/calloc/free). Test infrastructure only: it lets
 * the reference sources compile unmodified in this container, where MKL is
 * absent, so that their outputs can pin the oracle restatement.
 *
 * Conventions kept from MKL's documented behaviour: a backward transform uses
 * exp(+2 pi i jk/N) and is multiplied by DFTI_BACKWARD_SCALE, a forward one
 * uses exp(-2 pi i jk/N) times DFTI_FORWARD_SCALE (both default 1); a
 * multi-dimensional descriptor works on a C-ordered (last index fastest)
 * array in place. */
#ifndef PAWPY_MKL_SHIM_H
#define PAWPY_MKL_SHIM_H
#include <stddef.h>
#include "mkl_types.h"

enum DFTI_CONFIG_PARAM { DFTI_FORWARD_SCALE = 4, DFTI_BACKWARD_SCALE = 5 };
enum DFTI_CONFIG_VALUE { DFTI_COMPLEX = 32, DFTI_DOUBLE = 36, DFTI_SINGLE = 35 };

typedef struct pawpy_shim_dfti *DFTI_DESCRIPTOR_HANDLE;

MKL_LONG DftiCreateDescriptor(DFTI_DESCRIPTOR_HANDLE *h, enum DFTI_CONFIG_VALUE prec,
                              enum DFTI_CONFIG_VALUE domain, MKL_LONG dim, ...);
MKL_LONG DftiSetValue(DFTI_DESCRIPTOR_HANDLE h, enum DFTI_CONFIG_PARAM p, ...);
MKL_LONG DftiCommitDescriptor(DFTI_DESCRIPTOR_HANDLE h);
MKL_LONG DftiComputeBackward(DFTI_DESCRIPTOR_HANDLE h, void *x, ...);
MKL_LONG DftiComputeForward(DFTI_DESCRIPTOR_HANDLE h, void *x, ...);
MKL_LONG DftiFreeDescriptor(DFTI_DESCRIPTOR_HANDLE *h);
char *DftiErrorMessage(MKL_LONG status);

void cblas_cdotc_sub(const int n, const void *x, const int incx, const void *y,
                     const int incy, void *dotc);
void cblas_zdotc_sub(const int n, const void *x, const int incx, const void *y,
                     const int incy, void *dotc);

void *mkl_malloc(size_t size, int align);
void *mkl_calloc(size_t num, size_t size, int align);
void mkl_free(void *ptr);
void mkl_free_buffers(void);
#endif

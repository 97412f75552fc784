/* Project-written stand-in for the few MKL type names the pawpyseed C core
 * uses. Test infrastructure only: it exists so that the reference sources can
 * be compiled unmodified (without Intel MKL) to pin the oracle. */
#ifndef PAWPY_MKL_SHIM_TYPES_H
#define PAWPY_MKL_SHIM_TYPES_H
typedef long MKL_LONG;
#endif

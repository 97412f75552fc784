"""ctypes binding of libpawpy_gpu.so (the C ABI declared in include/pawpy_gpu.h).

The library is built in-tree (``pawpyseed_gb300/lib/libpawpy_gpu.so``) by
``pawpyseed_gb300.build``. Loading fails loudly if it is missing: there is no
other implementation of the path behind this package.
"""

import ctypes as C
import os

import numpy as np

from . import structs as S

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libpawpy_gpu.so")

_lib = None

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_zp = np.ctypeslib.ndpointer(dtype=np.complex128, flags="C_CONTIGUOUS")
_cp = np.ctypeslib.ndpointer(dtype=np.complex64, flags="C_CONTIGUOUS")
_wfp = C.POINTER(S.pswf_t)
_ppp = C.POINTER(S.ppot_t)
_vp = C.c_void_p

PRECISIONS = {"fp32": 0, "bf16x3": 1, "tf32": 2}


class PAWpyGPUError(RuntimeError):
    """A failure reported by libpawpy_gpu (status code and message)."""

    def __init__(self, code, msg):
        super().__init__("libpawpy_gpu error %d: %s" % (code, msg))
        self.code = code


def _declare(L):
    L.pawpy_gpu_last_error.restype = C.c_int
    L.pawpy_gpu_error_string.restype = C.c_char_p
    L.pawpy_gpu_read_wavefunctions.restype = _wfp
    L.pawpy_gpu_read_wavefunctions.argtypes = [C.c_char_p, _dp]
    L.pawpy_gpu_read_wavefunctions_from_str.restype = _wfp
    L.pawpy_gpu_read_wavefunctions_from_str.argtypes = [C.c_char_p, _dp]
    L.pawpy_gpu_read_wavefunctions_from_bytes.restype = _wfp
    L.pawpy_gpu_read_wavefunctions_from_bytes.argtypes = [C.c_char_p, C.c_size_t, _dp]
    L.pawpy_gpu_gvectors.restype = C.c_int
    L.pawpy_gpu_gvectors.argtypes = [_dp, _dp, C.c_double, C.c_void_p, C.c_int]
    L.pawpy_gpu_wavefunction_from_arrays.restype = _wfp
    L.pawpy_gpu_wavefunction_from_arrays.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, _dp, _dp, _dp,
                                                    _ip, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                                                    _dp, _dp, C.c_int]
    L.pawpy_gpu_free_pswf.argtypes = [_wfp]
    L.pawpy_gpu_free_ppot_list.argtypes = [_ppp, C.c_int]
    L.pawpy_gpu_release.argtypes = [_wfp]
    L.pawpy_gpu_upload.argtypes = [_wfp]
    L.pawpy_gpu_upload.restype = C.c_int
    L.get_projector_list.restype = _ppp
    L.get_projector_list.argtypes = [C.c_int, _ip, _ip, _dp, _dp, _dp, _dp, _dp, C.c_double]
    L.setup_projections.argtypes = [_wfp, _ppp, C.c_int, C.c_int, _ip, _ip, _dp]
    L.overlap_setup_real.argtypes = [_wfp, _wfp, _ip, _ip, _dp, _dp, _vp, _vp, _vp, _vp,
                                     C.c_int, C.c_int, C.c_int]
    L.overlap_setup_recip.argtypes = L.overlap_setup_real.argtypes
    L.pseudoprojection.argtypes = [_zp, _wfp, _wfp, C.c_int, C.c_int]
    L.compensation_terms.argtypes = [_zp, C.c_int, _wfp, _wfp, C.c_int, C.c_int, C.c_int, C.c_int,
                                     _vp, _vp, _vp, _vp, _vp, _vp, _ip, _dp, _ip, _dp, _ip, C.c_int]
    L.compensation_terms_recip.argtypes = L.compensation_terms.argtypes
    L.pawpy_gpu_project_all.restype = C.c_int
    L.pawpy_gpu_project_all.argtypes = [_zp, _wfp, _wfp, C.c_int, C.c_int, C.c_int, C.c_int,
                                        _vp, _vp, _vp, _vp, _vp, _vp, C.c_int]
    L.pawpy_gpu_band_character.restype = C.c_int
    L.pawpy_gpu_band_character.argtypes = [_dp, _dp, _wfp, _wfp, C.c_int, C.c_int, C.c_int, C.c_int,
                                           _vp, _vp, _vp, _vp, _vp, _vp, _dp, _dp, C.c_int, C.c_int]
    L.fft3d.argtypes = [_zp, _vp, _dp, _dp, _ip, _vp, C.c_int, _ip]
    L.realspace_state.argtypes = [_zp, C.c_int, C.c_int, _wfp, _ip, _ip, _dp]
    L.remove_phase.argtypes = [_zp, C.c_int, _wfp, _ip]
    L.ae_state_density.argtypes = [_dp, C.c_int, C.c_int, _wfp, _ip, _ip, _dp]
    L.ae_chg_density.argtypes = [_dp, _wfp, _ip, _ip, _dp]
    L.ncl_realspace_state.argtypes = [_zp, C.c_int, C.c_int, _wfp, _ip, _ip, _dp]
    L.ncl_ae_chg_density.argtypes = [_dp, _wfp, _ip, _ip, _dp]
    L.project_realspace_state.argtypes = [_zp, C.c_int, _wfp, _wfp, _ip, _ip, _dp, _ip, _dp]
    L.pawpy_gpu_project_realspace_all.restype = C.c_int
    L.pawpy_gpu_project_realspace_all.argtypes = [_zp, _wfp, _wfp, _ip, _ip, _dp, _ip, _dp]
    L.onto_projector.argtypes = [C.POINTER(S.kpoint_t), C.c_int, C.POINTER(S.real_proj_site_t), C.c_int,
                                 _vp, _dp, _dp, C.c_int, _ip]
    L.pawpy_gpu_set_precision.argtypes = [C.c_int]
    L.pawpy_gpu_get_precision.restype = C.c_int
    L.pawpy_gpu_set_tc_splits.argtypes = [C.c_int]
    L.pawpy_gpu_set_tc_tile.argtypes = [C.c_int]
    L.pawpy_gpu_set_sphere_contraction.argtypes = [C.c_int]
    L.pawpy_gpu_set_element_cache.argtypes = [C.c_int]
    L.pawpy_gpu_prepare_basis.restype = C.c_int
    L.pawpy_gpu_prepare_basis.argtypes = [_wfp, C.c_int]
    L.pawpy_gpu_thread_stream.restype = C.c_int
    L.pawpy_gpu_thread_stream.argtypes = [C.c_int]
    L.pawpy_gpu_server_create.restype = C.c_void_p
    L.pawpy_gpu_server_create.argtypes = [C.c_longlong, C.c_int]
    L.pawpy_gpu_server_add_basis.restype = C.c_int
    L.pawpy_gpu_server_add_basis.argtypes = [C.c_void_p, _wfp, _ip, _dp, C.c_int, C.c_int]
    L.pawpy_gpu_server_submit.restype = C.c_longlong
    L.pawpy_gpu_server_submit.argtypes = [C.c_void_p, C.POINTER(S.pawpy_gpu_request_t)]
    L.pawpy_gpu_server_wait.restype = C.c_int
    L.pawpy_gpu_server_wait.argtypes = [C.c_void_p, C.c_longlong, C.POINTER(C.c_double),
                                        C.POINTER(C.c_longlong), C.c_char_p, C.c_int]
    L.pawpy_gpu_server_counts.argtypes = [C.c_void_p, C.POINTER(C.c_longlong), C.POINTER(C.c_int),
                                          C.POINTER(C.c_int), C.POINTER(C.c_longlong)]
    L.pawpy_gpu_server_destroy.argtypes = [C.c_void_p]
    L.pawpy_gpu_overlap_matrix.restype = C.c_int
    L.pawpy_gpu_overlap_matrix.argtypes = [_cp, _cp, C.c_int, C.c_int, C.c_int, _ip, _cp, C.c_int]
    L.pawpy_gpu_set_host_projections.argtypes = [C.c_int]
    L.pawpy_gpu_timer_stop_ms.restype = C.c_float
    L.pawpy_gpu_launch_count.restype = C.c_longlong
    L.pawpy_gpu_launch_count.argtypes = [C.c_int]
    L.pawpy_gpu_profile.argtypes = [C.c_int]
    L.pawpy_gpu_kernel_stats.restype = C.c_int
    L.pawpy_gpu_kernel_stats.argtypes = [C.c_char_p, C.c_int, C.c_int]
    L.pawpy_gpu_device_bytes.restype = C.c_longlong
    L.pawpy_gpu_pageable_memory_access.restype = C.c_int
    L.pawpy_gpu_host_pool_check.restype = C.c_int
    L.pawpy_gpu_host_pool_check.argtypes = [C.c_int, C.c_int]
    L.pawpy_gpu_struct_layout.restype = C.c_int
    L.pawpy_gpu_struct_layout.argtypes = [C.c_char_p, C.c_int]


def lib():
    """The loaded library (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libpawpy_gpu.so is not built (run python -m pawpyseed_gb300.build): %s"
                              % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        _declare(L)
        _lib = L
    return _lib


def check():
    """Raise PAWpyGPUError if the last library call on this thread failed."""
    L = lib()
    code = L.pawpy_gpu_last_error()
    if code:
        msg = L.pawpy_gpu_error_string().decode(errors="replace")
        L.pawpy_gpu_clear_error()
        raise PAWpyGPUError(code, msg)


def ptr(a):
    """ctypes void* of a numpy array, or NULL when it is empty (as pawpyc.pyx:660-665)."""
    return None if a is None or len(a) == 0 else a.ctypes.data_as(C.c_void_p)


def set_precision(name):
    lib().pawpy_gpu_set_precision(PRECISIONS[name])


def get_precision():
    v = lib().pawpy_gpu_get_precision()
    return {b: a for a, b in PRECISIONS.items()}[v]


def overlap_matrix(As, Bs, precision="fp32"):
    """out[z] = conj(As[z]) @ Bs[z].T for lists of complex64 matrices that
    share their row counts (M and N) and may differ in K; returns nz x N x M
    complex64 (out[z][n][m] = <A_z[m] | B_z[n]>)."""
    M, N, nz = As[0].shape[0], Bs[0].shape[0], len(As)
    K = np.array([a.shape[1] for a in As], np.int32)
    for a, b in zip(As, Bs):
        if a.shape[0] != M or b.shape[0] != N or a.shape[1] != b.shape[1]:
            raise ValueError("overlap_matrix: inconsistent shapes")
    A = np.ascontiguousarray(np.concatenate([np.ascontiguousarray(a, np.complex64).ravel() for a in As]))
    B = np.ascontiguousarray(np.concatenate([np.ascontiguousarray(b, np.complex64).ravel() for b in Bs]))
    out = np.zeros((nz, N, M), np.complex64)
    lib().pawpy_gpu_overlap_matrix(A, B, M, N, nz, K, out, PRECISIONS[precision])
    check()
    return out


def kernel_stats(reset=True, spans=False, work=False):
    """{family: (ms, launches)} of the launches profiled since the last reset; with spans,
    {family: (ms, launches, first start, last end)}, the times in ms after profiling was
    switched on (host phases "host.<name>" on the host clock from the same moment); with work,
    {family: (ms, launches, work)}: the algorithmic bytes (or, for the overlap contractions,
    useful flops) the family's launches declared."""
    L = lib()
    n = L.pawpy_gpu_kernel_stats(None, 0, 0)
    buf = C.create_string_buffer(max(n, 1))
    L.pawpy_gpu_kernel_stats(buf, len(buf), int(reset))
    check()
    out = {}
    for line in buf.value.decode().splitlines():
        name, ms, cnt, t0, t1, wk = line.split()
        if work:
            out[name] = (float(ms), int(cnt), float(wk))
        else:
            out[name] = (float(ms), int(cnt), float(t0), float(t1)) if spans else (float(ms), int(cnt))
    return out


def struct_layout():
    L = lib()
    n = L.pawpy_gpu_struct_layout(None, 0)
    buf = C.create_string_buffer(n)
    L.pawpy_gpu_struct_layout(buf, n)
    rows = []
    for line in buf.value.decode().splitlines():
        s, m, off = line.split()
        rows.append((s, m, int(off)))
    return rows

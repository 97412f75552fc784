"""ctypes mirrors of the pawpyseed C structs that cross the C ABI.

The member order and types are the binary layout of
``pawpyseed/core/utils.h:30-166`` (``funcset_t``, ``ppot_t``, ``projection_t``,
``band_t``, ``rayleigh_set_t``, ``kpoint_t``, ``pswf_t``, ``real_proj_t``,
``real_proj_site_t``).  They must stay identical: the Cython layer of
pawpyseed reads ``pswf_t`` members directly (``pawpyc.pyx:537`` reads
``wf_ptr.kpts[k].bands[b].occ``), and the drop-in library receives these
structs by pointer.  ``include/pawpy_gpu.h`` declares the same layout in C,
and a CPU test compares the offsets the library reports with these.
"""

import ctypes as C

c_int_p = C.POINTER(C.c_int)
c_double_p = C.POINTER(C.c_double)
c_double_pp = C.POINTER(c_double_p)


class funcset_t(C.Structure):
    _fields_ = [
        ("l", C.c_int),
        ("proj", c_double_p), ("proj_spline", c_double_pp),
        ("aewave", c_double_p), ("aewave_spline", c_double_pp),
        ("pswave", c_double_p), ("pswave_spline", c_double_pp),
        ("diffwave", c_double_p), ("diffwave_spline", c_double_pp),
        ("kwave", c_double_p), ("kwave_spline", c_double_pp),
        ("smooth_diffwave", c_double_p), ("smooth_diffwave_spline", c_double_pp),
        ("dense_kwave", c_double_p), ("dense_kwave_spline", c_double_pp),
    ]


class ppot_t(C.Structure):
    _fields_ = [
        ("num_projs", C.c_int), ("total_projs", C.c_int), ("lmax", C.c_int),
        ("funcs", C.POINTER(funcset_t)),
        ("rmax", C.c_double), ("wave_rmax", C.c_double),
        ("pspw_overlap_matrix", c_double_p), ("aepw_overlap_matrix", c_double_p),
        ("diff_overlap_matrix", c_double_p),
        ("proj_gridsize", C.c_int), ("wave_gridsize", C.c_int), ("num_cart_gridpts", C.c_int),
        ("wave_grid", c_double_p), ("kwave_grid", c_double_p), ("proj_grid", c_double_p),
        ("smooth_grid", c_double_p), ("dense_kgrid", c_double_p),
    ]


class projection_t(C.Structure):
    _fields_ = [
        ("num_projs", C.c_int), ("total_projs", C.c_int),
        ("ns", c_int_p), ("ls", c_int_p), ("ms", c_int_p),
        ("overlaps", c_double_p),  # double complex*, read as pairs of doubles
    ]


class band_t(C.Structure):
    _fields_ = [
        ("n", C.c_int), ("num_waves", C.c_int),
        ("occ", C.c_double), ("N", C.c_double), ("energy", C.c_double),
        ("Cs", C.c_void_p),    # float complex*
        ("CRs", C.c_void_p),   # double complex*
        ("CAs", C.c_void_p),   # float complex*
        ("projections", C.POINTER(projection_t)),
        ("up_projections", C.POINTER(projection_t)),
        ("down_projections", C.POINTER(projection_t)),
        ("wave_projections", C.POINTER(projection_t)),
    ]


class rayleigh_set_t(C.Structure):
    _fields_ = [("l", C.c_int), ("terms", C.c_void_p)]


class kpoint_t(C.Structure):
    _fields_ = [
        ("up", C.c_short), ("num_waves", C.c_int), ("Gs", c_int_p), ("k", c_double_p),
        ("weight", C.c_double), ("num_bands", C.c_int),
        ("bands", C.POINTER(C.POINTER(band_t))),
        ("expansion", C.c_void_p),
    ]


class pswf_t(C.Structure):
    _fields_ = [
        ("encut", C.c_double), ("num_elems", C.c_int), ("num_projs", c_int_p),
        ("num_sites", C.c_int), ("pps", C.POINTER(ppot_t)), ("G_bounds", c_int_p),
        ("kpts", C.POINTER(C.POINTER(kpoint_t))),
        ("nspin", C.c_int), ("nband", C.c_int), ("nwk", C.c_int),
        ("lattice", c_double_p), ("reclattice", c_double_p), ("fftg", c_int_p),
        ("is_ncl", C.c_int), ("wp_num", C.c_int), ("num_aug_overlap_sites", C.c_int),
        ("dcoords", c_double_p), ("overlaps", C.c_void_p),  # double complex**
    ]


class real_proj_t(C.Structure):
    _fields_ = [("l", C.c_int), ("m", C.c_int), ("func_num", C.c_int), ("values", C.c_void_p)]


class real_proj_site_t(C.Structure):
    _fields_ = [
        ("index", C.c_int), ("elem", C.c_int), ("num_projs", C.c_int), ("total_projs", C.c_int),
        ("num_indices", C.c_int), ("gridsize", C.c_int), ("rmax", C.c_double),
        ("coord", c_double_p), ("indices", c_int_p), ("paths", c_double_p),
        ("projs", C.POINTER(real_proj_t)),
    ]


class pawpy_gpu_request_t(C.Structure):
    """A projection request of the library's server (include/pawpy_gpu.h)."""

    _fields_ = [
        ("basis", C.c_int),
        ("wf", C.POINTER(pswf_t)),
        ("pps", C.POINTER(ppot_t)),
        ("num_elems", C.c_int),
        ("num_sites", C.c_int),
        ("fftg", C.c_void_p),
        ("labels", C.c_void_p),
        ("coords", C.c_void_p),
        ("num_M", C.c_int),
        ("num_N_R", C.c_int),
        ("num_N_S", C.c_int),
        ("num_N_RS", C.c_int),
        ("M_R", C.c_void_p),
        ("M_S", C.c_void_p),
        ("N_R", C.c_void_p),
        ("N_S", C.c_void_p),
        ("N_RS_R", C.c_void_p),
        ("N_RS_S", C.c_void_p),
        ("out", C.c_void_p),
    ]


STRUCTS = [funcset_t, ppot_t, projection_t, band_t, rayleigh_set_t, kpoint_t, pswf_t,
           real_proj_t, real_proj_site_t, pawpy_gpu_request_t]


def layout_table():
    """(struct name, member, offset) for every member, plus each struct's size."""
    rows = []
    for s in STRUCTS:
        for name, _ in s._fields_:
            rows.append((s.__name__, name, getattr(s, name).offset))
        rows.append((s.__name__, "__sizeof__", C.sizeof(s)))
    return rows

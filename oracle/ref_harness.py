"""Drive the reference pawpyseed C core (``oracle/_ref/libpawpy_ref.so``) through ctypes.

TEST INFRASTRUCTURE ONLY. Used in the development container, where the
reference sources exist, to generate golden vectors and to pin the oracle
restatement.  It replays the call sequence of the reference's Python/Cython
layer for ``Projector(wf, basis).single_band_projection(b)`` with the default
``aug_real`` method:

* ``Wavefunction._make_c_projectors`` (wavefunction.py:386-415) and
  ``CWavefunction._c_projector_setup`` (pawpyc.pyx:352-412): species packing,
  ``grid_encut = max((pi*dim/abc)^2/0.262)``, ``get_projector_list``,
  ``setup_projections`` -- basis first, then wf (projector.py:106-108);
* ``Projector.make_site_lists`` (projector.py:115-160), including its use of
  ``sites[i]`` for the S-side rmax (projector.py:157);
* ``CProjector._setup_overlap`` -> ``overlap_setup_real`` (pawpyc.pyx:651-683);
* per band ``pseudoprojection`` + ``compensation_terms`` (projector.py:210-223,
  pawpyc.pyx:311-325, 685-702);
* for the ``aug_recip`` method, ``overlap_setup_recip`` (pawpyc.pyx:674-678) and per band
  ``pseudoprojection`` + ``compensation_terms_recip`` (projector.py:225-236,
  pawpyc.pyx:704-721).
"""

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from pawpyseed_gb300 import structs as S  # noqa: E402
from pawpyseed_gb300 import vaspio  # noqa: E402

REF_LIB = os.path.join(HERE, "_ref", "libpawpy_ref.so")

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_zp = np.ctypeslib.ndpointer(dtype=np.complex128, flags="C_CONTIGUOUS")


def load_ref():
    lib = C.CDLL(REF_LIB)
    lib.read_wavefunctions.restype = C.POINTER(S.pswf_t)
    lib.read_wavefunctions.argtypes = [C.c_char_p, _dp]
    lib.get_projector_list.restype = C.POINTER(S.ppot_t)
    lib.get_projector_list.argtypes = [C.c_int, _ip, _ip, _dp, _dp, _dp, _dp, _dp, C.c_double]
    lib.setup_projections.argtypes = [C.POINTER(S.pswf_t), C.POINTER(S.ppot_t), C.c_int, C.c_int,
                                      _ip, _ip, _dp]
    lib.overlap_setup_real.argtypes = [C.POINTER(S.pswf_t), C.POINTER(S.pswf_t), _ip, _ip, _dp, _dp,
                                       C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_int, C.c_int, C.c_int]
    lib.pseudoprojection.argtypes = [_zp, C.POINTER(S.pswf_t), C.POINTER(S.pswf_t), C.c_int, C.c_int]
    lib.compensation_terms.argtypes = [_zp, C.c_int, C.POINTER(S.pswf_t), C.POINTER(S.pswf_t),
                                       C.c_int, C.c_int, C.c_int, C.c_int,
                                       C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_void_p, _ip, _dp, _ip, _dp, _ip, C.c_int]
    lib.overlap_setup_recip.argtypes = lib.overlap_setup_real.argtypes
    lib.compensation_terms_recip.argtypes = lib.compensation_terms.argtypes
    lib.fft3d.argtypes = [_zp, C.c_void_p, _dp, _dp, _ip, C.c_void_p, C.c_int, _ip]
    lib.free_pswf.argtypes = [C.POINTER(S.pswf_t)]
    return lib


def _ptr(a):
    return None if a is None or len(a) == 0 else a.ctypes.data_as(C.c_void_p)


def pack_species(cr):
    """Flat arrays of CWavefunction._c_projector_setup (pawpyc.pyx:359-381)."""
    labels, ls, wg, pr, ae, ps, rm = [], [], [], [], [], [], []
    for num, sym in enumerate(cr.pps):
        pp = cr.pps[sym]
        labels += [num, len(pp.ls), pp.ndata, len(pp.grid)]
        rm.append(pp.rmax)
        ls += list(pp.ls)
        wg += list(pp.grid)
        for i in range(len(pp.ls)):
            pr += list(pp.realprojs[i])
            ae += list(pp.aewaves[i])
            ps += list(pp.pswaves[i])
    f = lambda x: np.ascontiguousarray(x, dtype=np.float64)  # noqa: E731
    return (np.array(labels, np.int32), np.array(ls, np.int32), f(wg), f(pr), f(ae), f(ps), f(rm))


def site_lists(basis_struct, wf_struct, basis_cr, wf_cr):
    """Restatement of Projector.make_site_lists (projector.py:115-160), quirk included."""
    ref, cur = basis_struct, wf_struct
    M_R, M_S = [], []
    for i in range(len(ref)):
        for j in range(len(cur)):
            if ref.distance(i, cur, j) <= 0.02 and ref.species[i] == cur.species[j]:
                M_R.append(i)
                M_S.append(j)
    N_R = [i for i in range(len(ref)) if i not in M_R]
    N_S = [j for j in range(len(cur)) if j not in M_S]
    N_RS = []
    for i in N_R:
        for j in N_S:
            rmax1 = basis_cr.pps[ref.species[i]].rmax
            rmax2 = wf_cr.pps[cur.species[i]].rmax  # sites[i], as projector.py:157
            if ref.distance(i, cur, j) < rmax1 + rmax2:
                N_RS.append((i, j))
    return M_R, M_S, N_R, N_S, N_RS


class RefWavefunction:
    def __init__(self, lib, path):
        self.lib = lib
        self.struct = vaspio.read_poscar(os.path.join(path, "CONTCAR"))
        self.cr = vaspio.CoreRegion(os.path.join(path, "POTCAR"))
        vr = vaspio.Vasprun(os.path.join(path, "vasprun.xml"))
        self.dim = np.array([vr.parameters[n] for n in ("NGX", "NGY", "NGZ")], np.int32)
        self.kws = np.ascontiguousarray(vr.actual_kpoints_weights, dtype=np.float64)
        self.kpts = vr.actual_kpoints
        self.ptr = lib.read_wavefunctions(os.path.join(path, "WAVECAR").encode(), self.kws)
        w = self.ptr.contents
        self.nband, self.nwk, self.nspin = w.nband, w.nwk, w.nspin
        labels = {e: n for n, e in enumerate(self.cr.pps)}
        self.nums = np.array([labels[s] for s in self.struct.species], np.int32)
        self.coords = np.ascontiguousarray(self.struct.frac_coords.reshape(-1), dtype=np.float64)

    def setup_projectors(self):
        grid_encut = float(np.max((np.pi * self.dim / self.struct.abc) ** 2 / 0.262))
        labels, ls, wg, pr, ae, ps, rm = pack_species(self.cr)
        self._keep = (labels, ls, wg, pr, ae, ps, rm)
        pps = self.lib.get_projector_list(len(self.cr.pps), labels, ls, wg, pr, ae, ps, rm, grid_encut)
        self.lib.setup_projections(self.ptr, pps, len(self.cr.pps), len(self.struct), self.dim,
                                   self.nums, self.coords)
        self.grid_encut = grid_encut

    def projections(self, band, kidx, which="projections"):
        """Per-site <p|psi> (projections, or up_projections / down_projections of a spinor band),
        or the wave_projections, of one band as a list of complex arrays."""
        kp = self.ptr.contents.kpts[kidx].contents
        bd = kp.bands[band].contents
        arr = getattr(bd, which)
        n = self.ptr.contents.wp_num if which == "wave_projections" else len(self.struct)
        out = []
        for s in range(n):
            p = arr[s]
            v = np.ctypeslib.as_array(p.overlaps, shape=(2 * p.total_projs,)).copy()
            out.append(v[0::2] + 1j * v[1::2])
        return out

    def aug_coefficients(self, band, kidx):
        """band->CAs of one band (complex64 in the file's plane-wave order), or None."""
        kp = self.ptr.contents.kpts[kidx].contents
        bd = kp.bands[band].contents
        if not bd.CAs:
            return None
        v = np.ctypeslib.as_array(C.cast(bd.CAs, C.POINTER(C.c_float)), shape=(2 * kp.num_waves,)).copy()
        return (v[0::2] + 1j * v[1::2]).astype(np.complex64)

    def free(self):
        if self.ptr:
            self.lib.free_pswf(self.ptr)
            self.ptr = None


class RefProjector:
    """The reference aug_real (or, with recip, aug_recip) projection of wf (S) onto basis (R)."""

    def __init__(self, lib, basis, wf, recip=False):
        self.lib, self.basis, self.wf = lib, basis, wf
        self.recip = recip
        basis.setup_projectors()
        wf.setup_projectors()
        M_R, M_S, N_R, N_S, N_RS = site_lists(basis.struct, wf.struct, basis.cr, wf.cr)
        N_RS_R = [a for a, _ in N_RS]
        N_RS_S = [b for _, b in N_RS]
        a = lambda x: np.array(x, dtype=np.int32)  # noqa: E731
        self.lists = dict(M_R=a(M_R), M_S=a(M_S), N_R=a(N_R), N_S=a(N_S),
                          N_RS_R=a(N_RS_R), N_RS_S=a(N_RS_S))
        L = self.lists
        setup = lib.overlap_setup_recip if recip else lib.overlap_setup_real
        setup(basis.ptr, wf.ptr, basis.nums, wf.nums, basis.coords, wf.coords,
              _ptr(L["N_R"]), _ptr(L["N_S"]), _ptr(L["N_RS_R"]), _ptr(L["N_RS_S"]),
              len(N_R), len(N_S), len(N_RS))

    def pseudo(self, band, flip_spin=False):
        nk = self.basis.nwk * self.basis.nspin
        res = np.zeros(self.basis.nband * nk, dtype=np.complex128)
        self.lib.pseudoprojection(res, self.basis.ptr, self.wf.ptr, band, int(flip_spin))
        return res

    def single_band_projection(self, band, flip_spin=False):
        res = self.pseudo(band, flip_spin)
        L = self.lists
        comp = self.lib.compensation_terms_recip if self.recip else self.lib.compensation_terms
        comp(res, band, self.wf.ptr, self.basis.ptr,
             len(L["M_R"]), len(L["N_R"]), len(L["N_S"]), len(L["N_RS_R"]),
             _ptr(L["M_R"]), _ptr(L["M_S"]), _ptr(L["N_R"]), _ptr(L["N_S"]),
             _ptr(L["N_RS_R"]), _ptr(L["N_RS_S"]),
             self.wf.nums, self.wf.coords, self.basis.nums, self.basis.coords,
             self.wf.dim, int(flip_spin))
        return res

    def overlaps_NRS(self):
        """The N_RS pair matrices Q (overlap_setup_real, projector.c:682-719) and dcoords."""
        w = self.wf.ptr.contents
        n = w.num_aug_overlap_sites
        out = []
        if n == 0:
            return out, np.zeros((0, 3))
        ptrs = C.cast(w.overlaps, C.POINTER(C.POINTER(C.c_double)))
        pps_b, pps_w = self.basis.cr, self.wf.cr
        for i in range(n):
            s1, s2 = self.lists["N_RS_R"][i], self.lists["N_RS_S"][i]
            t1 = sum(2 * l + 1 for l in pps_b.pps[self.basis.struct.species[s1]].ls)
            t2 = sum(2 * l + 1 for l in pps_w.pps[self.wf.struct.species[s2]].ls)
            v = np.ctypeslib.as_array(ptrs[i], shape=(2 * t1 * t2,)).copy()
            out.append((v[0::2] + 1j * v[1::2]).reshape(t1, t2))
        dc = np.ctypeslib.as_array(w.dcoords, shape=(3 * n,)).copy().reshape(n, 3)
        return out, dc

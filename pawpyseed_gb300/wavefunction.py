"""``Wavefunction``: the pawpyseed wavefunction object over the GB300 library.

Mirrors ``pawpyseed.core.wavefunction.Wavefunction`` (wavefunction.py:169-606)
and its Cython base classes (``PseudoWavefunction``/``CWavefunction``,
pawpyc.pyx:227-540) for the projection path: construction from VASP files,
``check_c_projectors`` (species packing and ``setup_projections``),
``pseudoprojection`` and the occupation/energy accessors. The C structs are
the reference's (``pswf_t``), created by the library's WAVECAR reader.
"""

import ctypes as C
import bz2
import gzip
import os
import time

import numpy as np

from . import _lib
from .vaspio import CoreRegion, PAWpyError, Structure, Vasprun, read_poscar


class Timer:
    """Accumulated wall-clock times of the setup stages (pawpyc.pyx:37-49)."""

    ALL_SETUP_TIME = 0.0
    ALL_OVERLAP_TIME = 0.0
    ALL_AUGMENTATION_TIME = 0.0

    @staticmethod
    def setup_time(t):
        Timer.ALL_SETUP_TIME += t

    @staticmethod
    def overlap_time(t):
        Timer.ALL_OVERLAP_TIME += t

    @staticmethod
    def augmentation_time(t):
        Timer.ALL_AUGMENTATION_TIME += t


def pack_species(cr):
    """Flat species arrays in the layout get_projector_list expects (pawpyc.pyx:359-381).

    Elements are numbered in POTCAR order, as Wavefunction._make_c_projectors
    labels them (wavefunction.py:396-402).
    """
    labels, ls, wg, pr, ae, ps, rm = [], [], [], [], [], [], []
    for num, sym in enumerate(cr.pps):
        pp = cr.pps[sym]
        labels += [num, len(pp.ls), pp.ndata, len(pp.grid)]
        rm.append(pp.rmax)
        ls += list(pp.ls)
        wg.append(np.asarray(pp.grid, dtype=np.float64))
        for i in range(len(pp.ls)):
            pr.append(np.asarray(pp.realprojs[i][: pp.ndata], dtype=np.float64))
            ae.append(np.asarray(pp.aewaves[i], dtype=np.float64))
            ps.append(np.asarray(pp.pswaves[i], dtype=np.float64))
    cat = lambda x: np.ascontiguousarray(np.concatenate(x), dtype=np.float64)  # noqa: E731
    return (np.array(labels, np.int32), np.array(ls, np.int32), cat(wg), cat(pr), cat(ae), cat(ps),
            np.array(rm, np.float64))


class Wavefunction:
    """PAW wavefunction of one structure (plane-wave part in device memory on demand).

    Attributes (as the reference): structure, cr, dim, nband, nwk, nspin, encut,
    kpts, kws, ncl, symprec.
    """

    _NCL = False  # the collinear class refuses spinor wavefunctions, as the reference does

    def __init__(self, struct, pwf, cr, dim, kpts=None, kws=None, symprec=1e-4, setup_projectors=False):
        self._ptr = None
        if not pwf:
            raise PAWpyError("NULL wavefunction pointer")
        self._ptr = pwf
        w = pwf.contents
        self.nband, self.nwk, self.nspin, self.encut = w.nband, w.nwk, w.nspin, w.encut
        self.ncl = bool(w.is_ncl)
        if self.ncl and not self._NCL:
            raise PAWpyError("Pseudowavefunction is noncollinear! Call NCLWavefunction(...) instead")
        if self._NCL and not self.ncl:
            raise PAWpyError("Pseudowavefunction is collinear! Call Wavefunction(...) instead")
        self.structure = struct
        self.cr = cr
        self.symprec = symprec
        self.dim = np.array(dim, dtype=np.int32)
        if len(dim) != 3:
            raise PAWpyError("Grid dimensions must be length 3")
        if kpts is None:
            kpts = np.array([[w.kpts[k].contents.k[a] for a in range(3)] for k in range(self.nwk)])
        self.kpts = np.array(kpts, dtype=np.float64)
        if kws is None:
            kws = np.array([w.kpts[k].contents.weight for k in range(self.nwk)])
        self.kws = np.array(kws, dtype=np.float64)
        self.projector_owner = 0
        labels = {e: n for n, e in enumerate(cr.pps)}
        self.nums = np.array([labels[s] for s in struct.species], dtype=np.int32)
        self.coords = np.ascontiguousarray(struct.frac_coords.reshape(-1), dtype=np.float64)
        if setup_projectors:
            self.check_c_projectors()

    # -- construction ------------------------------------------------------

    @classmethod
    def from_files(cls, struct="CONTCAR", wavecar="WAVECAR", cr="POTCAR", vr="vasprun.xml",
                   setup_projectors=False):
        """Wavefunction.from_files (wavefunction.py:281-322)."""
        for fname in [struct, wavecar, cr, vr]:
            if not os.path.isfile(fname):
                raise FileNotFoundError(f"File {fname} does not exist.")
        vr = Vasprun(vr)
        dim = np.array([vr.parameters["NGX"], vr.parameters["NGY"], vr.parameters["NGZ"]])
        kws = np.ascontiguousarray(vr.actual_kpoints_weights, dtype=np.float64)
        path = str(wavecar)
        # compressed WAVECARs are inflated in memory and read from the bytes (pawpyc.pyx:217-222
        # reads them through zopen for names containing .gz or .bz2)
        opener = gzip.open if ".gz" in path else bz2.open if ".bz2" in path else None
        if opener is not None:
            with opener(path, "rb") as src:
                data = src.read()
            ptr = _lib.lib().pawpy_gpu_read_wavefunctions_from_bytes(data, len(data), kws)
        else:
            ptr = _lib.lib().pawpy_gpu_read_wavefunctions(path.encode(), kws)
        _lib.check()
        return cls(read_poscar(struct), ptr, CoreRegion(cr), dim, vr.actual_kpoints, kws,
                            vr.parameters["SYMPREC"], setup_projectors)

    @classmethod
    def from_directory(cls, path, setup_projectors=False):
        files = [os.path.join(path, d) for d in ["CONTCAR", "WAVECAR", "POTCAR", "vasprun.xml"]]
        return cls.from_files(*files, setup_projectors)

    @classmethod
    def from_arrays(cls, struct, cr, dim, data, setup_projectors=False):
        """Build from in-memory WAVECAR content (dict of synth.wavefunction_data; a
        noncollinear dict has ``ncl`` set, spinor coefficients of twice the G count)."""
        nk = data["nspin"] * data["nwk"]
        ncl = bool(data.get("ncl", False))
        nplane = np.array([(2 if ncl else 1) * g.shape[0] for g in data["gs"]], dtype=np.int32)
        gs = [np.ascontiguousarray(g, dtype=np.int32) for g in data["gs"]]
        cs = [np.ascontiguousarray(c, dtype=np.complex64) for c in data["coeffs"]]
        gp = (C.c_void_p * nk)(*[g.ctypes.data for g in gs])
        cp = (C.c_void_p * nk)(*[c.ctypes.data for c in cs])
        lat = np.ascontiguousarray(np.asarray(data["lattice"]).reshape(-1), dtype=np.float64)
        kp = np.ascontiguousarray(np.asarray(data["kpts"]).reshape(-1), dtype=np.float64)
        kws = np.ascontiguousarray(data["weights"], dtype=np.float64)
        en = np.ascontiguousarray(np.asarray(data["energies"]).reshape(-1), dtype=np.float64)
        oc = np.ascontiguousarray(np.asarray(data["occs"]).reshape(-1), dtype=np.float64)
        ptr = _lib.lib().pawpy_gpu_wavefunction_from_arrays(data["nspin"], data["nwk"], data["nband"],
                                                           float(data["encut"]), lat, kp, kws, nplane,
                                                           gp, cp, en, oc, 1 if ncl else 0)
        _lib.check()
        return cls(struct, ptr, cr, dim, data["kpts"], kws, 1e-4, setup_projectors)

    def detach(self):
        """Give up the pswf_t without freeing it (its new owner frees it)."""
        self._ptr = None

    def __del__(self):
        if getattr(self, "_ptr", None):
            try:
                _lib.lib().pawpy_gpu_free_pswf(self._ptr)
            except Exception:
                pass
            self._ptr = None

    # -- accessors ---------------------------------------------------------

    @property
    def wf_ptr(self):
        return self._ptr

    def check_band_index(self, b):
        if b < 0 or b >= self.nband:
            raise ValueError("Invalid band {}. Should be in range [{}, {}]".format(b, 0, self.nband - 1))

    def _get_occs(self):
        """Occupations in [band][spin*nwk + k] order (pawpyc.pyx:532-538)."""
        nk = self.nwk * self.nspin
        w = self._ptr.contents
        res = np.zeros(self.nband * nk)
        for k in range(nk):
            kp = w.kpts[k].contents
            for b in range(self.nband):
                res[b * nk + k] = kp.bands[b].contents.occ
        return res

    def _get_energy_list(self, bands):
        w = self._ptr.contents
        out = {}
        for b in bands:
            self.check_band_index(b)
            out[b] = []
            for s in range(self.nspin):
                for k in range(self.nwk):
                    bd = w.kpts[k + s * self.nwk].contents.bands[b].contents
                    out[b].append([bd.energy, bd.occ])
        return out

    def upload(self):
        """Make the plane-wave coefficients resident in device memory now."""
        _lib.lib().pawpy_gpu_upload(self._ptr)
        _lib.check()

    # -- projector setup ---------------------------------------------------

    def grid_encut(self):
        """(pi*dim/abc)^2/0.262 maximised over the axes (wavefunction.py:411)."""
        return float(np.max((np.pi * self.dim / self.structure.abc) ** 2 / 0.262))

    def _make_c_projectors(self):
        L = _lib.lib()
        labels, ls, wg, pr, ae, ps, rm = pack_species(self.cr)
        pps = L.get_projector_list(len(self.cr.pps), labels, ls, wg, pr, ae, ps, rm, self.grid_encut())
        _lib.check()
        self.dimv = np.ascontiguousarray(self.dim, dtype=np.int32)
        L.setup_projections(self._ptr, pps, len(self.cr.pps), len(self.structure), self.dimv, self.nums,
                            self.coords)
        _lib.check()
        self.projector_owner = 1

    def check_c_projectors(self):
        """Set up the projector functions and <p|psi> if that has not happened yet."""
        if not self.projector_owner:
            start = time.monotonic()
            self._make_c_projectors()
            Timer.setup_time(time.monotonic() - start)

    # -- all-electron real-space wavefunctions (wavefunction.py:431-590, pawpyc.pyx:425-523) --------
    #
    # The grid is given explicitly (dim); the reference sets it through update_dim, which also
    # changes the wavefunction's own grid. States default to the wavefunction's grid, densities
    # to the doubled grid, as there.

    def _grid(self, dim, fine):
        g = self.dim * (2 if fine else 1) if dim is None else np.asarray(dim)
        return np.ascontiguousarray(g, dtype=np.int32)

    def _check_bks(self, b, k, s):
        if b < 0 or b >= self.nband:
            raise ValueError("Invalid band choice")
        if k < 0 or k >= self.nwk:
            raise ValueError("Invalid k-point choice")
        if s < 0 or s >= self.nspin:
            raise ValueError("Invalid spin choice")

    def get_state_realspace(self, b, k, s, dim=None, remove_phase=False):
        """All-electron wavefunction of band b, k-point k, spin s on the grid dim (default the
        wavefunction's own): complex128 [N1, N2, N3] (realspace_state, density.c:245-310). With
        remove_phase the exp(2 pi i k.r) factor is divided out."""
        self.check_c_projectors()
        self._check_bks(b, k, s)
        g = self._grid(dim, False)
        res = np.zeros(int(np.prod(g)), dtype=np.complex128)
        L = _lib.lib()
        L.realspace_state(res, int(b), int(k + s * self.nwk), self._ptr, g, self.nums, self.coords)
        _lib.check()
        if remove_phase:
            L.remove_phase(res, int(k + s * self.nwk), self._ptr, g)
            _lib.check()
        return res.reshape(tuple(g))

    def get_state_realspace_density(self, b, k, s, dim=None):
        """|psi|^2 of one band on the grid dim (default twice the wavefunction's grid)
        (ae_state_density, density.c:27-37)."""
        self.check_c_projectors()
        self._check_bks(b, k, s)
        g = self._grid(dim, True)
        res = np.zeros(int(np.prod(g)), dtype=np.float64)
        _lib.lib().ae_state_density(res, int(b), int(k + s * self.nwk), self._ptr, g, self.nums, self.coords)
        _lib.check()
        return res.reshape(tuple(g))

    def get_realspace_density(self, dim=None, bands=None):
        """All-electron charge density on the grid dim (default twice the wavefunction's grid):
        every occupied band (ae_chg_density, density.c:158-178), or with bands (an int or a list)
        those bands weighted by k-point weight / nspin (pawpyc.pyx:455-494)."""
        self.check_c_projectors()
        g = self._grid(dim, True)
        n = int(np.prod(g))
        L = _lib.lib()
        res = np.zeros(n, dtype=np.float64)
        if bands is None:
            L.ae_chg_density(res, self._ptr, g, self.nums, self.coords)
            _lib.check()
        else:
            for b in ([bands] if isinstance(bands, (int, np.integer)) else list(bands)):
                if b < 0 or b >= self.nband:
                    raise ValueError("Invalid band choice")
                for k in range(self.nwk * self.nspin):
                    work = np.zeros(n, dtype=np.float64)
                    L.ae_state_density(work, int(b), int(k), self._ptr, g, self.nums, self.coords)
                    _lib.check()
                    res += work * self.kws[k % self.nwk] / self.nspin
        return res.reshape(tuple(g))

    def _write_volumetric(self, filename, values, dim, scale):
        """A VASP volumetric file: the structure header of _convert_to_vasp_volumetric
        (wavefunction.py:481-510), the grid dimensions, then the values times scale with the
        first index fastest, five per line, as write_volumetric (density.c:461-477) prints them."""
        st = self.structure
        syms, counts = [], []
        for sp in st.species:
            if syms and syms[-1] == sp:
                counts[-1] += 1
            else:
                syms.append(sp)
                counts.append(1)
        lines = [filename, "   1.00000000000000"]
        for row in np.asarray(st.lattice).reshape(3, 3):
            lines.append(" %12.6f%12.6f%12.6f" % tuple(row))
        lines.append("".join("%5s" % x for x in syms))
        lines.append("".join("%6d" % x for x in counts))
        lines.append("Direct")
        for fc in st.frac_coords:
            lines.append("%10.6f%10.6f%10.6f" % tuple(fc))
        lines.append(" ")
        lines.append("%d %d %d" % tuple(int(x) for x in dim))
        vals = (np.asarray(values).reshape(tuple(dim)).transpose(2, 1, 0).ravel() * scale)
        body = []
        for i in range(0, vals.size, 5):
            body.append("".join("%E   " % v for v in vals[i:i + 5]))
        with open(filename, "w") as fh:
            fh.write("\n".join(lines) + "\n" + "\n".join(body) + ("\n" if body else ""))

    def write_state_realspace(self, b, k, s, fileprefix="", dim=None, scale=1, remove_phase=False):
        """Writes the real and imaginary parts of one band to <prefix>B<b>K<k>S<s>_REAL.vasp and
        _IMAG.vasp (wavefunction.py:512-555); returns the complex grid."""
        res = self.get_state_realspace(b, k, s, dim, remove_phase)
        base = "%sB%dK%dS%d" % (fileprefix, b, k, s)
        self._write_volumetric("%s_REAL.vasp" % base, np.real(res), res.shape, scale)
        self._write_volumetric("%s_IMAG.vasp" % base, np.imag(res), res.shape, scale)
        return res

    def write_density_realspace(self, filename="PYAECCAR.vasp", dim=None, scale=1, bands=None):
        """Writes the all-electron charge density (wavefunction.py:557-590); returns it."""
        res = self.get_realspace_density(dim, bands)
        self._write_volumetric(filename, res, res.shape, scale)
        return res

    def pseudoprojection(self, band_num, basis, flip_spin=False):
        """<psi~_basis,b,k|psi~_self,band_num,k> for all basis bands b and k (pawpyc.pyx:311-325)."""
        res = np.zeros(basis.nband * basis.nwk * basis.nspin, dtype=np.complex128)
        _lib.lib().pseudoprojection(res, basis._ptr, self._ptr, int(band_num), int(flip_spin))
        _lib.check()
        return res


class NCLWavefunction(Wavefunction):
    """Noncollinear (spinor) wavefunction (noncollinear.py:4-32).

    setup_projections fills every band's ``up_projections`` and
    ``down_projections`` (onto_projector_ncl, projector.c:359-392): the two
    spinor halves share the G list and are transformed and projected as two
    bands on the device. Overlaps of noncollinear wavefunctions are not part of
    the reference's projection path (``Projector`` refuses them)."""

    _NCL = True

    def get_state_realspace(self, b, k, s, dim=None, remove_phase=False):
        """All-electron spinor components of band b, k-point k, spin s on the grid dim (default the
        wavefunction's own): (up, down), complex128 [N1, N2, N3] each (ncl_realspace_state,
        density.c:328-408; pawpyc.pyx:563-580)."""
        self.check_c_projectors()
        self._check_bks(b, k, s)
        g = self._grid(dim, False)
        n = int(np.prod(g))
        res = np.zeros(2 * n, dtype=np.complex128)
        L = _lib.lib()
        L.ncl_realspace_state(res, int(b), int(k + s * self.nwk), self._ptr, g, self.nums, self.coords)
        _lib.check()
        up, down = res[:n].copy(), res[n:].copy()
        if remove_phase:
            for half in (up, down):
                L.remove_phase(half, int(k + s * self.nwk), self._ptr, g)
                _lib.check()
        return up.reshape(tuple(g)), down.reshape(tuple(g))

    def get_state_realspace_density(self, b, k, s, dim=None):
        """|psi_up|^2 + |psi_down|^2 of one band on the grid dim (default twice the wavefunction's)."""
        up, down = self.get_state_realspace(b, k, s, self._grid(dim, True))
        return np.abs(up) ** 2 + np.abs(down) ** 2

    def get_realspace_density(self, dim=None, bands=None):
        """All-electron charge density of the occupied bands on the grid dim (default twice the
        wavefunction's grid): ncl_ae_chg_density (density.c:181-204; pawpyc.pyx:582-588)."""
        if bands is not None:
            raise ValueError("band-resolved densities are not defined for noncollinear wavefunctions")
        self.check_c_projectors()
        g = self._grid(dim, True)
        res = np.zeros(int(np.prod(g)), dtype=np.float64)
        _lib.lib().ncl_ae_chg_density(res, self._ptr, g, self.nums, self.coords)
        _lib.check()
        return res.reshape(tuple(g))

    def write_state_realspace(self, b, k, s, fileprefix="", dim=None, scale=1, remove_phase=False):
        """Writes the real and imaginary parts of both spinor components to
        <prefix>B<b>K<k>S<s>_UP_REAL.vasp, _UP_IMAG, _DOWN_REAL, _DOWN_IMAG (noncollinear.py:98-147);
        returns (up, down)."""
        up, down = self.get_state_realspace(b, k, s, dim, remove_phase)
        base = "%sB%dK%dS%d" % (fileprefix, b, k, s)
        for tag, v in (("UP", up), ("DOWN", down)):
            self._write_volumetric("%s_%s_REAL.vasp" % (base, tag), np.real(v), v.shape, scale)
            self._write_volumetric("%s_%s_IMAG.vasp" % (base, tag), np.imag(v), v.shape, scale)
        return up, down

    def spinor_projections(self, band, k):
        """(<p|psi_up>, <p|psi_down>) of one band at k-point index k (spin-major), complex128
        over every site's lm channels in site order."""
        self.check_c_projectors()
        kp = self.wf_ptr.contents.kpts[k].contents
        bd = kp.bands[band].contents
        out = []
        for lst in (bd.up_projections, bd.down_projections):
            vals = []
            for s in range(len(self.structure)):
                p = lst[s]
                v = np.ctypeslib.as_array(p.overlaps, shape=(2 * p.total_projs,))
                vals.append(v[0::2] + 1j * v[1::2])
            out.append(np.concatenate(vals))
        return out[0], out[1]

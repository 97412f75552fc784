"""TEST INFRASTRUCTURE -- the oracle (checker) for the band-projection path.

Python driver over ``oracle/liboracle.so`` (the C restatement in oracle.c)
that reproduces the reference's Python-level flow:

* species setup per element, in POTCAR order (wavefunction.py:386-415,
  pawpyc.pyx:352-412, projector.c:20-171);
* sphere tables for all sites and FFT + gather for every band
  (projector.c:193-209, 560-602; utils.c:590-696);
* ``make_site_lists`` (projector.py:115-160, with its ``sites[i]`` quirk);
* ``overlap_setup_real`` (projector.c:604-725): smooth-(phi-phit) tables of the
  other structure's sites, their projections, the N_RS pair matrices
  ``conj(reciprocal_offsite_wave_overlap)`` (radial.c:116-196);
* ``pseudoprojection`` (pseudoprojector.c:63-90) and ``compensation_terms``
  (projector.c:850-963) for every defect band, as full matrices;
* ``realspace_state`` and ``ae_chg_density`` (density.c:158-310): all-electron
  states and charge densities on a real-space grid.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
bench.py use this module; the product path never imports it.  The
compensation sums are evaluated with numpy in double precision.
"""

import ctypes as C
import math
import os
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from pawpyseed_gb300 import vaspio  # noqa: E402

LIB_PATH = os.path.join(HERE, "liboracle.so")
_lib = None

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_lp = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_fp = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")


def build():
    subprocess.check_call(["make", "-s", "-C", HERE, "liboracle.so"])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.oracle_species_setup.argtypes = [C.c_int, _ip, C.c_int, C.c_int, C.c_double, _dp, _dp, _dp,
                                           _dp, C.c_double] + [_dp] * 11
        L.oracle_site_table.restype = C.c_int
        L.oracle_site_table.argtypes = [_dp, _ip, _dp, C.c_double, C.c_int, C.c_int, _dp, C.c_int,
                                        _ip, _dp, _dp, C.c_int, _ip, _dp, _dp]
        L.oracle_project_bands.argtypes = [C.c_int, _fp, C.c_long, _ip, C.c_int, _ip, _dp, _dp,
                                           C.c_int, _ip, _lp, _lp, _ip, _ip, C.c_int, _ip, _dp, _dp, _dp]
        L.oracle_offsite.argtypes = [_dp, _dp, _dp, _dp, C.c_int, _dp, _dp, _dp, C.c_int,
                                     C.c_int, C.c_int, C.c_int, C.c_int, _dp,
                                     C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.oracle_offsite_matrix.argtypes = [_dp, _dp, _dp, _dp, C.c_int, C.c_int, _ip, _ip, _ip,
                                            _dp, _dp, _dp, C.c_int, C.c_int, _ip, _ip, _ip, _dp, _dp]
        L.oracle_pseudo_k.argtypes = [C.c_int, C.c_int, C.c_int, _fp, C.c_long, _fp, C.c_long,
                                      C.c_int, _dp]
        L.oracle_fft3d.argtypes = [_dp, _ip, _fp, C.c_int, _ip, C.c_double]
        L.oracle_aug_coefficients.argtypes = [C.c_int, _dp, C.c_long, _ip, _ip, C.c_int, _ip, _dp, _dp, C.c_int,
                                              _ip, _lp, _lp, _ip, _ip, _dp, _dp, _dp]
        L.oracle_spline_coeff.argtypes = [_dp, _dp, C.c_int, _dp, _dp, _dp]
        L.oracle_legendre.restype = C.c_double
        L.oracle_legendre.argtypes = [C.c_int, C.c_int, C.c_double]
        L.oracle_ylm.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double,
                                 C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.oracle_sbt_forward.argtypes = [C.c_double, C.c_int, C.c_int, _dp, _dp, C.c_int, _dp, _dp]
        _lib = L
    return _lib


# --------------------------------------------------------------------------
# Gaunt-type factors (regenerated from the Wigner 3j symbols, gaunt.py:11-31)
# --------------------------------------------------------------------------


def wigner3j(j1, j2, j3, m1, m2, m3):
    """Racah's closed form of the Wigner 3j symbol for integer arguments."""
    if m1 + m2 + m3 != 0 or abs(m1) > j1 or abs(m2) > j2 or abs(m3) > j3:
        return 0.0
    if j3 < abs(j1 - j2) or j3 > j1 + j2:
        return 0.0
    f = math.factorial
    tri = f(j1 + j2 - j3) * f(j1 - j2 + j3) * f(-j1 + j2 + j3) / f(j1 + j2 + j3 + 1)
    pre = math.sqrt(tri * f(j1 + m1) * f(j1 - m1) * f(j2 + m2) * f(j2 - m2) * f(j3 + m3) * f(j3 - m3))
    s = 0.0
    kmin = max(0, j2 - j3 - m1, j1 - j3 + m2)
    kmax = min(j1 + j2 - j3, j1 - m1, j2 + m2)
    for k in range(kmin, kmax + 1):
        s += (-1) ** k / (f(k) * f(j3 - j2 + k + m1) * f(j3 - j1 + k - m2) * f(j1 + j2 - j3 - k)
                          * f(j1 - k - m1) * f(j2 - k + m2))
    return (-1) ** (j1 - j2 - m3) * pre * s


def sbtfacs():
    """SBTFACS[l1][l2][(L-|l1-l2|)/2][l1+m1][m2], flat float64 [4*4*4*7*4]."""
    t = np.zeros((4, 4, 4, 7, 4))
    for l1 in range(4):
        for l2 in range(l1 + 1):
            for l3 in range(abs(l1 - l2), l1 + l2 + 1, 2):
                for m1 in range(-l1, l1 + 1):
                    for m2 in range(0, l2 + 1):
                        v = wigner3j(l1, l2, l3, 0, 0, 0) * wigner3j(l1, l2, l3, -m1, m2, m1 - m2)
                        v *= math.sqrt((2 * l1 + 1) * (2 * l2 + 1) * (2 * l3 + 1) / 4 / math.pi)
                        t[l1, l2, (l3 - abs(l1 - l2)) // 2, l1 + m1, m2] = v
    return np.ascontiguousarray(t.reshape(-1))


# --------------------------------------------------------------------------
# species and sites
# --------------------------------------------------------------------------


class OSpecies:
    def __init__(self, pp, grid_encut):
        L = lib()
        self.ls = np.array(pp.ls, dtype=np.int32)
        self.nproj = len(pp.ls)
        self.ndata = int(pp.ndata)
        self.ngrid = len(pp.grid)
        self.rmax = float(pp.rmax)
        self.total = int(sum(2 * l + 1 for l in pp.ls))
        wg = np.ascontiguousarray(pp.grid, dtype=np.float64)
        proj = np.ascontiguousarray(np.concatenate([p[: self.ndata] for p in pp.realprojs]))
        ae = np.ascontiguousarray(np.concatenate(pp.aewaves))
        ps = np.ascontiguousarray(np.concatenate(pp.pswaves))
        nd, ng, npj = self.ndata, self.ngrid, self.nproj
        self.wave_grid = wg
        self.proj = proj
        self.proj_grid = np.zeros(nd)
        self.proj_spl = np.zeros(npj * 3 * nd)
        self.smooth_grid = np.zeros(nd)
        self.sdw = np.zeros(npj * nd)
        self.sdw_spl = np.zeros(npj * 3 * nd)
        self.kgrid = np.zeros(ng)
        self.kwave = np.zeros(npj * ng)
        self.kwave_spl = np.zeros(npj * 3 * ng)
        self.aeov = np.zeros(npj * npj)
        self.psov = np.zeros(npj * npj)
        self.diov = np.zeros(npj * npj)
        L.oracle_species_setup(npj, self.ls, nd, ng, self.rmax, wg, proj, ae, ps, grid_encut,
                               self.proj_grid, self.proj_spl, self.smooth_grid, self.sdw,
                               self.sdw_spl, self.kgrid, self.kwave, self.kwave_spl,
                               self.aeov, self.psov, self.diov)
        self.wave_rmax = float(wg[-1])
        # all-electron minus pseudo partial wave per channel (projector.c:95-99)
        self.diffwave = [np.asarray(a, dtype=np.float64) - np.asarray(b, dtype=np.float64)
                         for a, b in zip(pp.aewaves, pp.pswaves)]
        self._ae_spl = {}
        # (n, l, m) of each lm channel, in the order of setup_site (utils.c:622-635)
        self.nlm = [(n, int(l), m) for n, l in enumerate(pp.ls) for m in range(-int(l), int(l) + 1)]
        D = (self.aeov - self.psov).reshape(npj, npj)
        T = self.total
        self.Dfull = np.zeros((T, T))
        for i, (ni, li, mi) in enumerate(self.nlm):
            for j, (nj, lj, mj) in enumerate(self.nlm):
                if li == lj and mi == mj:
                    self.Dfull[i, j] = D[ni, nj]


class SiteTables:
    """Concatenated sphere tables of a list of sites (setup_site, utils.c:590-696)."""

    def __init__(self, lattice, fftg, site_nums, labels, coords, species, smooth):
        L = lib()
        lat = np.ascontiguousarray(lattice, dtype=np.float64).reshape(-1)
        fg = np.ascontiguousarray(fftg, dtype=np.int32)
        idx, pth, val, npts, total = [], [], [], [], []
        for s, p in enumerate(site_nums):
            sp = species[labels[p]]
            r0_size = species[labels[s]].ndata  # pps[labels[s]] as utils.c:651-652
            rmax = sp.wave_rmax if smooth else sp.rmax
            grid = sp.smooth_grid if smooth else sp.proj_grid
            f = sp.sdw if smooth else sp.proj
            spl = sp.sdw_spl if smooth else sp.proj_spl
            box = [int(np.linalg.norm(np.cross(lat.reshape(3, 3)[(a + 1) % 3], lat.reshape(3, 3)[(a + 2) % 3]))
                       * rmax / abs(np.linalg.det(lat.reshape(3, 3))) * fftg[a]) + 1 for a in range(3)]
            cap = int(np.prod([2 * b + 1 for b in box]))
            ind = np.zeros(cap, np.int32)
            pa = np.zeros(3 * cap)
            va = np.zeros(2 * cap * sp.total)
            n = L.oracle_site_table(lat, fg, np.ascontiguousarray(coords[p], dtype=np.float64), rmax,
                                    sp.ndata, r0_size, grid, sp.nproj, sp.ls, f, spl, cap, ind, pa, va)
            if n < 0:
                raise RuntimeError("sphere table overflow")
            idx.append(ind[:n])
            pth.append(pa[: 3 * n])
            val.append(va[: 2 * n * sp.total])
            npts.append(n)
            total.append(sp.total)
        self.npts = np.array(npts, np.int32)
        self.total = np.array(total, np.int32)
        self.toff = np.concatenate([[0], np.cumsum(self.npts)[:-1]]).astype(np.int64)
        self.voff = np.concatenate([[0], np.cumsum(self.npts * self.total)[:-1]]).astype(np.int64)
        self.ooff = np.concatenate([[0], np.cumsum(self.total)[:-1]]).astype(np.int32)
        self.ntot = int(self.total.sum())
        self.indices = np.ascontiguousarray(np.concatenate(idx) if idx else np.zeros(0, np.int32))
        self.paths = np.ascontiguousarray(np.concatenate(pth) if pth else np.zeros(0))
        self.values = np.ascontiguousarray(np.concatenate(val) if val else np.zeros(0))
        self.nsites = len(site_nums)

    def project(self, cs, gs, fftg, lattice, kcart):
        """<T|psi> for all bands cs[nb, W] -> complex128 [nb, ntot]."""
        L = lib()
        nb, nw = cs.shape
        out = np.zeros(2 * nb * self.ntot)
        if self.nsites == 0 or nb == 0:
            return np.zeros((nb, self.ntot), np.complex128)
        cf = np.ascontiguousarray(cs.view(np.float32).reshape(-1))
        L.oracle_project_bands(nb, cf, nw, np.ascontiguousarray(gs.reshape(-1), dtype=np.int32), nw,
                               np.ascontiguousarray(fftg, dtype=np.int32),
                               np.ascontiguousarray(lattice, dtype=np.float64).reshape(-1),
                               np.ascontiguousarray(kcart, dtype=np.float64), self.nsites, self.npts,
                               self.toff, self.voff, self.total, self.ooff, self.ntot, self.indices,
                               self.paths, self.values, out)
        return (out[0::2] + 1j * out[1::2]).reshape(nb, self.ntot)

    def aug_coefficients(self, P, pcol, gs, fftg, lattice, kcart):
        """get_aug_freqs (projector.c:276-331, 420-453) of every band: P complex128 [nb, *] projector
        coefficients (site s of these tables at column pcol[s]) -> CAs complex128 [nb, W]."""
        L = lib()
        nb = P.shape[0]
        nw = gs.shape[0]
        if self.nsites == 0 or nb == 0:
            return np.zeros((nb, nw), np.complex128)
        out = np.zeros(2 * nb * nw)
        Pc = np.ascontiguousarray(P, dtype=np.complex128)
        L.oracle_aug_coefficients(nb, Pc.view(np.float64).reshape(-1), Pc.shape[1],
                                  np.ascontiguousarray(pcol, dtype=np.int32),
                                  np.ascontiguousarray(gs.reshape(-1), dtype=np.int32), nw,
                                  np.ascontiguousarray(fftg, dtype=np.int32),
                                  np.ascontiguousarray(lattice, dtype=np.float64).reshape(-1),
                                  np.ascontiguousarray(kcart, dtype=np.float64), self.nsites, self.npts,
                                  self.toff, self.voff, self.total, self.indices, self.paths, self.values, out)
        return (out[0::2] + 1j * out[1::2]).reshape(nb, nw)


class OracleWavefunction:
    """One structure: WAVECAR data, species tables and <p|psi> for every band."""

    def __init__(self, path=None, data=None, struct=None, cr=None, dim=None):
        if path is not None:
            struct = vaspio.read_poscar(os.path.join(path, "CONTCAR"))
            cr = vaspio.CoreRegion(os.path.join(path, "POTCAR"))
            vr = vaspio.Vasprun(os.path.join(path, "vasprun.xml"))
            dim = [vr.parameters[n] for n in ("NGX", "NGY", "NGZ")]
            data = vaspio.read_wavecar_numpy(os.path.join(path, "WAVECAR"))
            data = dict(data, weights=vr.actual_kpoints_weights)
        self.struct, self.cr = struct, cr
        self.dim = np.array(dim, np.int32)
        self.data = data
        self.nband, self.nwk, self.nspin = data["nband"], data["nwk"], data["nspin"]
        self.nk = self.nwk * self.nspin
        self.lattice = np.asarray(data["lattice"], dtype=np.float64)
        self.kpts = np.asarray(data["kpts"], dtype=np.float64)
        labels = {e: n for n, e in enumerate(cr.pps)}
        self.nums = np.array([labels[s] for s in struct.species], np.int32)
        self.coords = np.ascontiguousarray(struct.frac_coords, dtype=np.float64)
        self.occs = np.asarray(data["occs"])

    def kcart(self, kidx):
        return self.kpts[kidx % self.nwk] @ vaspio.reciprocal_lattice(self.lattice)

    def setup_projectors(self, timer=None, reuse=None):
        """Element setup, sphere tables and <p|psi> of every band. timer (a dict) receives the
        seconds of the phases 'element', 'tables' (band-independent) and 'project' (per band).
        reuse: a wavefunction of the same structure whose element setup and tables are taken
        instead of being built again."""
        t0 = time.perf_counter()
        grid_encut = float(np.max((np.pi * self.dim / self.struct.abc) ** 2 / 0.262))
        self.grid_encut = grid_encut
        self.species = reuse.species if reuse is not None else [OSpecies(self.cr.pps[e], grid_encut)
                                                                for e in self.cr.pps]
        t1 = time.perf_counter()
        self.tables = reuse.tables if reuse is not None else SiteTables(
            self.lattice, self.dim, list(range(len(self.struct))), self.nums, self.coords, self.species,
            smooth=False)
        self.site_off = self.tables.ooff
        t2 = time.perf_counter()
        self.P = [self.tables.project(self.data["coeffs"][k], self.data["gs"][k], self.dim,
                                      self.lattice, self.kcart(k)) for k in range(self.nk)]
        t3 = time.perf_counter()
        if timer is not None:
            for name, dt in (("element", t1 - t0), ("tables", t2 - t1), ("project", t3 - t2)):
                timer[name] = timer.get(name, 0.0) + dt

    def site_block(self, P, s):
        o = self.site_off[s]
        return P[:, o: o + self.tables.total[s]]

    # -- all-electron real-space states (density.c) ------------------------------------------

    def _ae_spline(self, e, n):
        """Cubic-spline coefficients of diffwave channel n of species e on the log wave grid
        (diffwave_spline, projector.c:111-112)."""
        sp = self.species[e]
        if n not in sp._ae_spl:
            x = sp.wave_grid
            f = np.ascontiguousarray(sp.diffwave[n][: len(x)])
            b, c, d = np.zeros(len(x)), np.zeros(len(x)), np.zeros(len(x))
            lib().oracle_spline_coeff(x, f, len(x), b, c, d)
            sp._ae_spl[n] = (f, b, c, d)
        return sp._ae_spl[n]

    def _site_geometry(self, p, N):
        """Grid points of site p within its last wave-grid radius on the grid N (the box and test of
        realspace_state, density.c:267-296): flattened cell, periodic-image shift, radial values
        per channel (wave_interpolate / max(r, x0), utils.c:477-489, 522-531) and Y_lm per (l, m)
        with the angles of wave_value2 (utils.c:533-543). Cached per grid."""
        key = (p, tuple(int(v) for v in N))
        cache = self.__dict__.setdefault("_geom", {})
        if key in cache:
            return cache[key]
        lat = self.lattice
        vol = abs(np.linalg.det(lat))
        e = int(self.nums[p])
        sp = self.species[e]
        wg = sp.wave_grid
        rmax = float(wg[-1])
        c = self.coords[p]
        box = [int(np.linalg.norm(np.cross(lat[(a + 1) % 3], lat[(a + 2) % 3])) * rmax / vol * N[a]) + 1
               for a in range(3)]
        # C round(): halves away from zero
        ctr = [int(math.copysign(math.floor(abs(c[a] * N[a]) + 0.5), c[a] * N[a])) for a in range(3)]
        ax = [np.arange(ctr[a] - box[a], ctr[a] + box[a] + 1) for a in range(3)]
        I, J, K = np.meshgrid(ax[0], ax[1], ax[2], indexing="ij")
        ijk = np.stack([I.ravel(), J.ravel(), K.ravel()], axis=1)
        cart = (ijk / N - c) @ lat
        r = np.sqrt((cart ** 2).sum(axis=1))
        keep = r < rmax
        ijk, cart, r = ijk[keep], cart[keep], r[keep]
        wrapped = np.mod(ijk, N)
        shift = (wrapped - ijk) // N
        with np.errstate(invalid="ignore", divide="ignore"):
            theta = np.arccos(np.clip(cart[:, 2] / np.where(r > 0, r, 1), -1, 1))
            rxy = np.sqrt(cart[:, 0] ** 2 + cart[:, 1] ** 2)
            phi = np.where(r - np.abs(cart[:, 2]) == 0, 0.0,
                           np.arccos(np.clip(cart[:, 0] / np.where(rxy > 0, rxy, 1), -1, 1)))
        phi = np.where(cart[:, 1] < 0, 2 * np.pi - phi, phi)
        theta = np.where(r == 0, 0.0, theta)
        phi = np.where(r == 0, 0.0, phi)
        lg = math.log(wg[1] / wg[0])
        ind = np.minimum((np.log(np.maximum(r, wg[0]) / wg[0]) / lg).astype(np.int64), len(wg) - 2)
        rem = r - wg[ind]
        rads, ys = {}, {}
        for n, l, m in sp.nlm:
            if n not in rads:
                f, sb, sc, sd = self._ae_spline(e, n)
                rad = np.where(r < wg[0], f[0], f[ind] + rem * (sb[ind] + rem * (sc[ind] + rem * sd[ind])))
                rads[n] = rad / np.maximum(r, wg[0])
            if (l, m) not in ys:
                ys[(l, m)] = ylm_c(l, m, theta, phi)
        flat = (wrapped[:, 0] * N[1] + wrapped[:, 1]) * N[2] + wrapped[:, 2]
        cache[key] = (flat, shift, rads, ys)
        return cache[key]

    def realspace_state(self, b, kidx, fftg):
        """realspace_state (density.c:245-310): the pseudo wavefunction of band b at k-point
        index kidx on the grid fftg (fft3d, linalg.c:14-45) times exp(2 pi i k.r), plus for every
        site the partial-wave differences (phi - phit)(r)/r Y_lm weighted by <p|psi> on the grid
        points within the last wave-grid radius, with the Bloch phase of the periodic image.
        Needs setup_projectors. complex128 [N1, N2, N3]."""
        L = lib()
        N = np.asarray(fftg, dtype=np.int32)
        lat = self.lattice
        vol = abs(np.linalg.det(lat))
        gs = np.ascontiguousarray(self.data["gs"][kidx], dtype=np.int32)
        cs = np.ascontiguousarray(self.data["coeffs"][kidx][b], dtype=np.complex64)
        xv = np.zeros(2 * int(np.prod(N)))
        L.oracle_fft3d(xv, gs.reshape(-1), cs.view(np.float32), gs.shape[0], N, vol)
        x = (xv[0::2] + 1j * xv[1::2]).reshape(tuple(N))
        kf = self.kpts[kidx % self.nwk]
        fr = [np.arange(N[a]) / N[a] for a in range(3)]
        kdotr = kf[0] * fr[0][:, None, None] + kf[1] * fr[1][None, :, None] + kf[2] * fr[2][None, None, :]
        x = x * np.exp(2j * np.pi * kdotr)
        P = self.P[kidx]
        xf = x.reshape(-1)
        for p in range(len(self.struct)):
            e = int(self.nums[p])
            sp = self.species[e]
            flat, shift, rads, ys = self._site_geometry(p, N)
            phase = np.exp(2j * np.pi * ((self.coords[p] + shift) @ kf))
            acc = np.zeros(flat.shape[0], np.complex128)
            o = self.site_off[p]
            for q, (n, l, m) in enumerate(sp.nlm):
                acc += rads[n] * ys[(l, m)] * P[b, o + q]
            np.add.at(xf, flat, acc * phase)
        return x

    def ae_chg_density(self, fftg):
        """ae_chg_density (density.c:158-178): sum over k-points and occupied bands of
        |realspace_state|^2 x k-point weight x occupation x 2/nspin."""
        N = tuple(int(v) for v in fftg)
        rho = np.zeros(N)
        occ = np.asarray(self.occs, dtype=np.float64).reshape(self.nk, self.nband)
        w = np.asarray(self.data["weights"], dtype=np.float64)
        for k in range(self.nk):
            for b in range(self.nband):
                if occ[k, b] > 0:
                    x = self.realspace_state(b, k, fftg)
                    rho += (x.real ** 2 + x.imag ** 2) * w[k % self.nwk] * occ[k, b] * (2 / self.nspin)
        return rho


def ylm_c(l, m, theta, phi):
    """Complex Y_lm (Condon-Shortley) of arrays of angles through the C restatement of Ylm
    (utils.c)."""
    L = lib()
    th = np.atleast_1d(np.asarray(theta, dtype=np.float64))
    ph = np.atleast_1d(np.asarray(phi, dtype=np.float64))
    out = np.zeros(th.shape, np.complex128)
    re, im = C.c_double(), C.c_double()
    for i in range(th.size):
        L.oracle_ylm(int(l), int(m), float(th.flat[i]), float(ph.flat[i]), C.byref(re), C.byref(im))
        out.flat[i] = complex(re.value, im.value)
    return out


def band_subset(data, idx):
    """In-memory WAVECAR content restricted to the bands idx (every k-point and spin)."""
    idx = np.asarray(idx, dtype=np.int64)
    return dict(data, nband=len(idx), coeffs=[np.ascontiguousarray(c[idx]) for c in data["coeffs"]],
                energies=np.asarray(data["energies"])[:, idx], occs=np.asarray(data["occs"])[:, idx])


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
            rmax2 = wf_cr.pps[cur.species[i]].rmax
            if ref.distance(i, cur, j) < rmax1 + rmax2:
                N_RS.append((i, j))
    return M_R, M_S, N_R, N_S, N_RS


def min_cart_path(coord, center, lattice):
    """utils.c:51-73 (first strict minimum over the 27 images, i outer)."""
    best, path = np.inf, None
    for i in (-1, 0, 1):
        for j in (-1, 0, 1):
            for k in (-1, 0, 1):
                v = (np.asarray(coord) + [i, j, k] - np.asarray(center)) @ lattice
                d = math.sqrt(float(v @ v))
                if d < best:
                    best, path = d, v
    return path, best


class OracleProjector:
    """aug_real projection of wf (S) onto basis (R), full matrices in FP64."""

    def __init__(self, wf, basis, lists=None, timer=None, reuse=None, recip=False):
        """timer (a dict) receives the seconds of the overlap setup's phases: 'smooth_tables'
        (band-independent), 'wp_defect' (per defect band), 'wp_basis' (per basis band) and
        'pair_matrices' (band-independent). reuse: a projector of the same two structures and
        lists whose band-independent parts (smoothed-wave tables, pair matrices) are taken.
        recip: the aug_recip method (overlap_setup_recip, projector.c:727-848): instead of
        real-space smoothed-wave projections, the augmentation coefficients CA_R (R's bands on
        its N_R sites) and CA_S (S's bands on its N_S sites), complex128 [nk][nband][W]."""
        self.recip = recip
        self.wf, self.basis = wf, basis
        tm = {} if timer is None else timer

        def tick(name, t0):
            tm[name] = tm.get(name, 0.0) + time.perf_counter() - t0
        L = lib()
        for w in (basis, wf):
            if not hasattr(w, "P"):
                w.setup_projectors()
        if lists is None:
            lists = site_lists(basis.struct, wf.struct, basis.cr, wf.cr)
        self.M_R, self.M_S, self.N_R, self.N_S, N_RS = lists
        self.N_RS_R = [a for a, _ in N_RS]
        self.N_RS_S = [b for _, b in N_RS]
        nk = basis.nk
        # <(phi-phit)_R|psi_S> on N_R sites of R in S's grid (projector.c:625-646)
        self.WP_S = [np.zeros((wf.nband, 0), np.complex128)] * nk
        self.WP_R = [np.zeros((basis.nband, 0), np.complex128)] * nk
        if recip:
            self._setup_recip(reuse, tick)
        elif self.N_R:
            t0 = time.perf_counter()
            tab = reuse.tab_NR if reuse is not None else SiteTables(wf.lattice, wf.dim, self.N_R, basis.nums,
                                                                    basis.coords, basis.species, True)
            self.tab_NR = tab
            tick("smooth_tables", t0)
            t0 = time.perf_counter()
            self.WP_S = [tab.project(wf.data["coeffs"][k], wf.data["gs"][k], wf.dim, wf.lattice,
                                     wf.kcart(k)) for k in range(nk)]
            tick("wp_defect", t0)
        if self.N_S and not recip:
            t0 = time.perf_counter()
            tab = reuse.tab_NS if reuse is not None else SiteTables(basis.lattice, basis.dim, self.N_S, wf.nums,
                                                                    wf.coords, wf.species, True)
            self.tab_NS = tab
            tick("smooth_tables", t0)
            t0 = time.perf_counter()
            self.WP_R = [tab.project(basis.data["coeffs"][k], basis.data["gs"][k], basis.dim,
                                     basis.lattice, basis.kcart(k)) for k in range(nk)]
            tick("wp_basis", t0)
        # N_RS pair matrices (projector.c:682-719)
        t0 = time.perf_counter()
        facs = sbtfacs()
        self.Q, self.dcoords = [], []
        if reuse is not None:
            self.Q, self.dcoords = reuse.Q, reuse.dcoords
        for s1, s2 in zip(self.N_RS_R, self.N_RS_S) if reuse is None else ():
            sp1 = basis.species[basis.nums[s1]]
            sp2 = wf.species[wf.nums[s2]]
            dc, _ = min_cart_path(wf.coords[s2], basis.coords[s1], basis.lattice)
            dc = np.ascontiguousarray(dc, dtype=np.float64)
            T1, T2 = sp1.total, sp2.total
            n1, l1, m1 = [np.ascontiguousarray([x[i] for x in sp1.nlm], dtype=np.int32) for i in range(3)]
            n2, l2, m2 = [np.ascontiguousarray([x[i] for x in sp2.nlm], dtype=np.int32) for i in range(3)]
            q = np.zeros(2 * T1 * T2)
            # conj of the off-site overlap per (lm, lm') (projector.c:706), looped in C
            L.oracle_offsite_matrix(dc, sp1.kgrid, sp1.kwave, sp1.kwave_spl, sp1.ngrid, T1, n1, l1, m1,
                                    sp2.kgrid, sp2.kwave, sp2.kwave_spl, sp2.ngrid, T2, n2, l2, m2, facs, q)
            Q = (q[0::2] + 1j * q[1::2]).reshape(T1, T2)
            self.Q.append(Q)
            self.dcoords.append(dc)
        tick("pair_matrices", t0)

    def _setup_recip(self, reuse, tick):
        b, w = self.basis, self.wf
        nk = b.nk
        self.CA_R = [np.zeros((b.nband, b.data["coeffs"][k].shape[1]), np.complex128) for k in range(nk)]
        self.CA_S = [np.zeros((w.nband, w.data["coeffs"][k].shape[1]), np.complex128) for k in range(nk)]
        for side, (W, lst, name) in enumerate(((b, self.N_R, "tab_NR"), (w, self.N_S, "tab_NS"))):
            if not lst:
                continue
            t0 = time.perf_counter()
            tab = getattr(reuse, name) if reuse is not None else SiteTables(W.lattice, W.dim, lst, W.nums,
                                                                            W.coords, W.species, True)
            setattr(self, name, tab)
            tick("smooth_tables", t0)
            t0 = time.perf_counter()
            pcol = [int(W.site_off[s]) for s in lst]
            out = self.CA_R if side == 0 else self.CA_S
            for k in range(nk):
                out[k] = tab.aug_coefficients(W.P[k], pcol, W.data["gs"][k], W.dim, W.lattice, W.kcart(k))
            tick("wp_basis" if side == 0 else "wp_defect", t0)

    def cross_full(self, flip_spin=False, fp32=False):
        """aug_recip cross terms <CA_R|C_S> + <C_R|CA_S> (compensation_terms_recip,
        projector.c:1000-1016), [nk, nbS, nbR]. fp32: as the reference evaluates them (CAs stored
        as complex64, cblas_cdotc_sub accumulating in single precision)."""
        L = lib()
        b, w = self.basis, self.wf
        out = np.zeros((b.nk, w.nband, b.nband), np.complex128)

        def dots(A, B):
            A = np.ascontiguousarray(A, dtype=np.complex64)
            B = np.ascontiguousarray(B, dtype=np.complex64)
            tmp = np.zeros(2 * B.shape[0] * A.shape[0])
            L.oracle_pseudo_k(A.shape[0], B.shape[0], A.shape[1], A.view(np.float32).reshape(-1), A.shape[1],
                              B.view(np.float32).reshape(-1), B.shape[1], 1, tmp)
            return (tmp[0::2] + 1j * tmp[1::2]).reshape(B.shape[0], A.shape[0])

        for k in range(b.nk):
            kR = self._kR(k, flip_spin)
            CR, CS = b.data["coeffs"][kR], w.data["coeffs"][k]
            if fp32:
                if self.N_R:
                    out[k] += dots(self.CA_R[kR], CS)
                if self.N_S:
                    out[k] += dots(CR, self.CA_S[k])
            else:
                out[k] = (CS.astype(np.complex128) @ self.CA_R[kR].conj().T +
                          self.CA_S[k] @ CR.astype(np.complex128).conj().T)
        return out

    def _kR(self, k, flip):
        b = self.basis
        if b.nspin == 2 and flip:
            return k + b.nwk if k < b.nwk else k - b.nwk
        return k

    def pseudo_full(self, flip_spin=False, fp32=False):
        """S[k][bS, bR] = <C_R,bR,kR|C_S,bS,k> (complex128 [nk, nbS, nbR])."""
        L = lib()
        b, w = self.basis, self.wf
        out = np.zeros((b.nk, w.nband, b.nband), np.complex128)
        for k in range(b.nk):
            kR = self._kR(k, flip_spin)
            CR = np.ascontiguousarray(b.data["coeffs"][kR].view(np.float32).reshape(-1))
            CS = np.ascontiguousarray(w.data["coeffs"][k].view(np.float32).reshape(-1))
            nw = b.data["coeffs"][k].shape[1]
            tmp = np.zeros(2 * w.nband * b.nband)
            L.oracle_pseudo_k(b.nband, w.nband, nw, CR, b.data["coeffs"][kR].shape[1], CS,
                              w.data["coeffs"][k].shape[1], int(fp32), tmp)
            out[k] = (tmp[0::2] + 1j * tmp[1::2]).reshape(w.nband, b.nband)
        return out

    def comp_full(self, flip_spin=False):
        """The PAW terms O_M + O_R + O_S + O_N (projector.c:850-963), [nk, nbS, nbR]; for aug_recip
        O_M + O_N only (compensation_terms_recip, projector.c:1018-1075; see cross_full)."""
        b, w = self.basis, self.wf
        out = np.zeros((b.nk, w.nband, b.nband), np.complex128)
        for k in range(b.nk):
            kR = self._kR(k, flip_spin)
            PR, PS = b.P[kR], w.P[k]
            acc = np.zeros((b.nband, w.nband), np.complex128)
            for s1, s2 in zip(self.M_R, self.M_S):
                sp = b.species[b.nums[s1]]
                acc += b.site_block(PR, s1).conj() @ sp.Dfull @ w.site_block(PS, s2).T
            for si, s in enumerate([] if self.recip else self.N_R):
                pr = b.site_block(PR, s)
                o = self.tab_NR.ooff[si]
                ws = self.WP_S[k][:, o:o + self.tab_NR.total[si]]
                acc += pr.conj() @ ws.T
            for si, s in enumerate([] if self.recip else self.N_S):
                ps = w.site_block(PS, s)
                o = self.tab_NS.ooff[si]
                wr = self.WP_R[kR][:, o:o + self.tab_NS.total[si]]
                acc += wr.conj() @ ps.T
            kv = b.kpts[kR % b.nwk]
            for Q, dc, s1, s2 in zip(self.Q, self.dcoords, self.N_RS_R, self.N_RS_S):
                ph = np.exp(2j * np.pi * float(kv @ dc))
                acc += (b.site_block(PR, s1).conj() @ Q @ w.site_block(PS, s2).T) * ph
            out[k] = acc.T
        return out

    def full(self, flip_spin=False, fp32=False):
        tot = self.pseudo_full(flip_spin, fp32) + self.comp_full(flip_spin)
        if self.recip:
            tot += self.cross_full(flip_spin, fp32)
        return tot

    @staticmethod
    def band_vector(full, band):
        """single_band_projection layout: res[bR*nk + k] from a [nk, nbS, nbR] matrix."""
        return np.ascontiguousarray(full[:, band, :].T.reshape(-1))

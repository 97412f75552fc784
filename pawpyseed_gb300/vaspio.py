"""VASP-format file I/O for the band-projection path.

Host-side readers and writers for the four files a pawpyseed ``Wavefunction``
is built from: POSCAR/CONTCAR (structure), POTCAR (PAW datasets), vasprun.xml
(FFT grid and k-point weights) and WAVECAR (plane-wave coefficients).

The WAVECAR binary layout and the plane-wave enumeration order are format
facts that any reader must share with VASP; they follow the reference reader
``pawpyseed/core/reader.c:55-127`` (``setup``: reciprocal lattice with 2*pi and
the nb{1,2,3}max bounds) and ``reader.c:129-315`` (``read_wavecar``: record
layout, G loop ig3 outer / ig2 / ig1 inner, wrap ``ig > nbmax -> ig-2*nbmax-1``
computed in double and truncated to int, keep ``|k+G|^2/c <= ENCUT``).
The C reader that the library ships (``csrc/host_wavecar.cpp``) implements the same
order; this module is the writer used for synthetic inputs.

The POTCAR text follows the keyword layout that the reference parser splits on
(``pawpyseed/core/wavefunction.py:58-137``).
"""

import os
import re
import xml.etree.ElementTree as ET

import numpy as np

# hbar^2/2m in eV*Angstrom^2, the constant of pawpyseed/core/reader.c:11
C_EV = 0.262465831


class PAWpyError(Exception):
    """Raised on API misuse, as pawpyseed/core/utils.py:5-13 does."""

    def __init__(self, msg):
        super().__init__(msg)
        self.msg = msg


# --------------------------------------------------------------------------
# structure
# --------------------------------------------------------------------------


class Structure:
    """Minimal periodic structure: lattice rows (Angstrom), species, fractional coords.

    Stands in for the pymatgen ``Structure`` the reference API carries; it keeps
    only what the projection path reads (lattice, species symbols, positions,
    periodic minimum-image distances).
    """

    def __init__(self, lattice, species, frac_coords):
        self.lattice = np.array(lattice, dtype=np.float64).reshape(3, 3)
        self.species = list(species)
        self.frac_coords = np.array(frac_coords, dtype=np.float64).reshape(-1, 3)
        if len(self.species) != self.frac_coords.shape[0]:
            raise PAWpyError("species and coordinates differ in length")

    def __len__(self):
        return len(self.species)

    @property
    def volume(self):
        return float(abs(np.linalg.det(self.lattice)))

    @property
    def abc(self):
        return np.linalg.norm(self.lattice, axis=1)

    def same_lattice(self, other, tol=1e-8):
        return np.allclose(self.lattice, other.lattice, atol=tol, rtol=0)

    def distance(self, i, other, j):
        """Periodic minimum-image distance between site i of self and site j of other.

        pymatgen's ``PeriodicSite.distance`` (used by the reference
        ``make_site_lists``, projector.py:135-159) is the minimum over lattice images.
        """
        return float(self.distance_matrix(other, [i], [j])[0, 0])

    def distance_matrix(self, other, rows=None, cols=None):
        """Periodic minimum-image distances between the sites rows of self (default all) and the
        sites cols of other: [len(rows), len(cols)], the 27 nearest images of the wrapped
        fractional difference, as ``distance``."""
        fa = self.frac_coords if rows is None else self.frac_coords[np.asarray(rows, dtype=int)]
        fb = other.frac_coords if cols is None else other.frac_coords[np.asarray(cols, dtype=int)]
        d = fb[None, :, :] - fa[:, None, :]
        d = d - np.round(d)
        L = self.lattice
        dc = d @ L
        best = np.full(d.shape[:2], np.inf)
        for a in (-1, 0, 1):
            for b in (-1, 0, 1):
                for c in (-1, 0, 1):
                    v = dc + np.array([a, b, c], dtype=np.float64) @ L
                    np.minimum(best, np.einsum("ijk,ijk->ij", v, v), out=best)
        # the square root is monotone and correctly rounded: the root of the least square
        return np.sqrt(best)


def write_poscar(path, struct, comment="synthetic"):
    symbols = []
    counts = []
    for s in struct.species:
        if symbols and symbols[-1] == s:
            counts[-1] += 1
        else:
            symbols.append(s)
            counts.append(1)
    if len(set(symbols)) != len(symbols):
        # POSCAR groups species; reorder would change site indices, so refuse.
        raise PAWpyError("POSCAR writer needs sites grouped by species")
    lines = [comment, "   1.00000000000000"]
    for row in struct.lattice:
        lines.append("  %22.16f%22.16f%22.16f" % tuple(row))
    lines.append("   " + "   ".join(symbols))
    lines.append("   " + "   ".join(str(c) for c in counts))
    lines.append("Direct")
    for f in struct.frac_coords:
        lines.append("  %20.16f%20.16f%20.16f" % tuple(f))
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


def read_poscar(path):
    with open(path) as fh:
        lines = [ln.rstrip("\n") for ln in fh]
    scale = float(lines[1].split()[0])
    lattice = np.array([[float(x) for x in lines[i].split()[:3]] for i in (2, 3, 4)])
    lattice = lattice * scale
    symbols = lines[5].split()
    counts = [int(x) for x in lines[6].split()]
    pos = 7
    if lines[pos].strip()[:1].lower() == "s":
        pos += 1
    cart = lines[pos].strip()[:1].lower() in ("c", "k")
    pos += 1
    n = sum(counts)
    coords = np.array([[float(x) for x in lines[pos + i].split()[:3]] for i in range(n)])
    if cart:
        coords = np.linalg.solve(lattice.T, (coords * scale).T).T
    species = []
    for s, c in zip(symbols, counts):
        species += [s] * c
    return Structure(lattice, species, coords)


# --------------------------------------------------------------------------
# vasprun.xml (the two things the path reads from it)
# --------------------------------------------------------------------------


def write_vasprun(path, kpts, weights, dim, symprec=1e-4):
    out = ['<?xml version="1.0" encoding="ISO-8859-1"?>', "<modeling>", " <kpoints>"]
    out.append('  <varray name="kpointlist" >')
    for k in np.asarray(kpts).reshape(-1, 3):
        out.append("   <v> %18.12f %18.12f %18.12f </v>" % tuple(k))
    out.append("  </varray>")
    out.append('  <varray name="weights" >')
    for w in np.asarray(weights).reshape(-1):
        out.append("   <v> %18.14f </v>" % w)
    out.append("  </varray>")
    out.append(" </kpoints>")
    out.append(" <parameters>")
    out.append('  <separator name="grids" >')
    for name, v in zip(("NGX", "NGY", "NGZ"), dim):
        out.append('   <i type="int" name="%s">%6d</i>' % (name, int(v)))
    out.append("  </separator>")
    out.append('  <separator name="symmetry" >')
    out.append('   <i name="SYMPREC">%16.8f</i>' % symprec)
    out.append("  </separator>")
    out.append(" </parameters>")
    out.append("</modeling>")
    with open(path, "w") as fh:
        fh.write("\n".join(out) + "\n")


class Vasprun:
    """Reads the FFT grid, SYMPREC and the k-point list/weights from vasprun.xml.

    The reference reads the same fields through pymatgen
    (wavefunction.py:310-313 for NGX/NGY/NGZ/SYMPREC, pawpyc.pyx:213-214 for
    ``actual_kpoints`` and ``actual_kpoints_weights``).
    """

    def __init__(self, path):
        root = ET.parse(path).getroot()
        self.parameters = {}
        for node in root.iter("i"):
            name = node.get("name")
            if name in ("NGX", "NGY", "NGZ"):
                self.parameters[name] = int(node.text.split()[0])
            elif name == "SYMPREC":
                self.parameters[name] = float(node.text.split()[0])
        self.parameters.setdefault("SYMPREC", 1e-5)
        kp = root.find("kpoints")
        if kp is None:
            raise PAWpyError("vasprun.xml has no <kpoints> block")
        kl, wl = None, None
        for va in kp.findall("varray"):
            rows = [[float(x) for x in v.text.split()] for v in va.findall("v")]
            if va.get("name") == "kpointlist":
                kl = rows
            elif va.get("name") == "weights":
                wl = [r[0] for r in rows]
        self.actual_kpoints = np.array(kl, dtype=np.float64)
        self.actual_kpoints_weights = np.array(wl, dtype=np.float64)
        for name in ("NGX", "NGY", "NGZ"):
            if name not in self.parameters:
                raise PAWpyError("vasprun.xml lacks %s" % name)


# --------------------------------------------------------------------------
# POTCAR
# --------------------------------------------------------------------------


def _fmt_block(vals, per_line=5):
    vals = np.asarray(vals, dtype=np.float64).reshape(-1)
    lines = []
    for i in range(0, len(vals), per_line):
        lines.append("  " + " ".join("%16.9E" % v for v in vals[i : i + per_line]))
    return "\n".join(lines) + "\n"


def potcar_dataset_text(symbol, ls, rmax, ndata, realprojs, grid, aewaves, pswaves, T=1.0):
    """One element's POTCAR dataset, in the keyword layout the pawpyseed parser splits on.

    ``realprojs[i]`` holds the real-space projector p_i on the linear grid
    rmax*j/ndata (j < ndata); ``aewaves``/``pswaves`` hold r*phi on ``grid``.
    The text ends with ``End of Dataset\\n`` (15 characters), which the
    reference strips with ``data[:-15]`` (wavefunction.py:166).
    """
    ls = list(ls)
    parts = []
    parts.append("  PAW_PBE %s 01Jan2000\n 4.00000000000000000\n" % symbol)
    parts.append(" parameters from PSCTR are:\n   VRHFIN =%s: synthetic\n" % symbol)
    parts.append("   POMASS =   10.000; ZVAL   =    4.000    mass and valenz\n")
    parts.append(" Description\n     l       E        TYP  RCUT    TYP  RCUT\n")
    parts.append("   Error from kinetic energy argument (eV)\n")
    parts.append("   NDATA  =  %6d\n   STEP   =  20.000   1.050\n" % ndata)
    parts.append("   END of PSCTR-controll parameters\n")
    parts.append(" local part\n")
    parts.append(_fmt_block(np.linspace(1.0, 0.0, 11)))
    parts.append(" core charge-density (partial)\n")
    parts.append(_fmt_block(np.zeros(10)))
    parts.append(" atomic pseudo charge-density\n")
    parts.append(_fmt_block(np.zeros(10)))
    # float at text[-22:-4] just before the first "Non local Part" (wavefunction.py:96)
    parts.append("%18.10f\n   " % T)
    # group consecutive equal l into one Non local Part block
    groups = []
    for i, l in enumerate(ls):
        if groups and groups[-1][0] == l:
            groups[-1][1].append(i)
        else:
            groups.append((l, [i]))
    for l, idxs in groups:
        parts.append("Non local Part\n")
        parts.append("  %d  %d  %18.12f\n" % (l, len(idxs), rmax))
        parts.append(_fmt_block(np.ones(len(idxs) * len(idxs))))
        for i in idxs:
            parts.append(" Reciprocal Space Part\n")
            parts.append(_fmt_block(np.zeros(10)))
            parts.append(" Real Space Part\n")
            parts.append(_fmt_block(realprojs[i]))
        parts.append(" ")
    parts.append("PAW radial sets\n")
    parts.append("  %d  %18.12f\n" % (len(grid), rmax))
    parts.append(" augmentation charges (non sperical)\n")
    parts.append(_fmt_block(np.zeros(len(ls) * len(ls))))
    parts.append(" uccopancies in atom\n")
    parts.append(_fmt_block(np.zeros(len(ls))))
    parts.append(" grid\n")
    parts.append(_fmt_block(grid))
    parts.append(" aepotential\n")
    parts.append(_fmt_block(np.zeros(len(grid))))
    parts.append(" core charge-density\n")
    parts.append(_fmt_block(np.zeros(len(grid))))
    parts.append(" pspotential\n")
    parts.append(_fmt_block(np.zeros(len(grid))))
    parts.append(" core charge-density (pseudized)\n")
    parts.append(_fmt_block(np.zeros(len(grid))))
    for i in range(len(ls)):
        parts.append(" pseudo wavefunction\n")
        parts.append(_fmt_block(pswaves[i]))
        parts.append(" ae wavefunction\n")
        parts.append(_fmt_block(aewaves[i]))
    parts.append("End of Dataset\n")
    return "".join(parts)


def _nums(text):
    toks = text.split()
    out = []
    for t in toks:
        try:
            out.append(float(t))
        except ValueError:
            break
    return np.array(out, dtype=np.float64)


class Pseudopotential:
    """The fields of one POTCAR dataset that the projection path uses.

    Splits the dataset text on the same keywords as the reference parser
    (pawpyseed/core/wavefunction.py:58-137): ``PAW radial sets``,
    ``pseudo wavefunction``/``ae wavefunction``, ``grid``, ``aepotential``,
    ``Non local Part``, ``Reciprocal Space Part``/``Real Space Part``,
    ``NDATA`` (the token before ``STEP   =``). Attributes keep the reference
    names: ``ls``, ``rmax``, ``ndata``, ``grid``, ``realprojs``, ``aewaves``,
    ``pswaves``, ``projgrid``.
    """

    def __init__(self, data):
        nonradial, radial = data.split("PAW radial sets", 1)
        pw = radial.split("pseudo wavefunction")
        head, pw = pw[0], pw[1:]
        self.pswaves, self.aewaves = [], []
        for chunk in pw:
            ps, ae = chunk.split("ae wavefunction", 1)
            self.pswaves.append(_nums(ps))
            self.aewaves.append(_nums(ae))
        gridstr = head.split("grid", 1)[1].split("aepotential", 1)[0]
        self.grid = _nums(gridstr)
        blocks = nonradial.split("Non local Part")
        top, blocks = blocks[0], blocks[1:]
        self.ls, self.realprojs = [], []
        self.rmax = None
        for blk in blocks:
            pieces = blk.split("Reciprocal Space Part")
            header = pieces[0].split()
            l = int(round(float(header[0])))
            self.rmax = float(header[2])
            for p in pieces[1:]:
                real = p.split("Real Space Part", 1)[1]
                self.realprojs.append(_nums(real))
                self.ls.append(l)
        m = re.search(r"(\S+)\s+STEP\s+=", top)
        if m is None:
            raise PAWpyError("POTCAR dataset lacks NDATA")
        self.ndata = int(m.group(1))
        n = len(self.realprojs[0])
        self.projgrid = np.arange(n) * self.rmax / n


class CoreRegion:
    """Element symbol -> Pseudopotential, in POTCAR order (wavefunction.py:143-166)."""

    def __init__(self, path_or_text):
        if os.path.exists(str(path_or_text)):
            with open(path_or_text) as fh:
                text = fh.read()
        else:
            text = str(path_or_text)
        self.pps = {}
        for chunk in text.split("End of Dataset"):
            if "PAW radial sets" not in chunk:
                continue
            m = re.search(r"PAW_\S+\s+(\S+)", chunk)
            sym = m.group(1) if m else "X%d" % len(self.pps)
            self.pps[sym] = Pseudopotential(chunk)


# --------------------------------------------------------------------------
# WAVECAR
# --------------------------------------------------------------------------


def reciprocal_lattice(lattice):
    """Rows b_i with a_i.b_j = 2*pi*delta_ij (reader.c:58-65)."""
    a = np.asarray(lattice, dtype=np.float64).reshape(3, 3)
    vol = np.dot(a[0], np.cross(a[1], a[2]))
    b = np.array([np.cross(a[1], a[2]), np.cross(a[2], a[0]), np.cross(a[0], a[1])])
    return b * (2.0 * np.pi / vol)


def nbmax(lattice, encut):
    """The double-valued bounds nb{1,2,3}max of reader.c:55-127."""
    b = reciprocal_lattice(lattice)
    mag = np.sqrt((b * b).sum(1))
    kc = np.sqrt(encut * C_EV)

    def ang(i, j):
        return np.arccos(np.dot(b[i], b[j]) / (mag[i] * mag[j]))

    def sinphi(top, i, j):
        v = np.cross(b[i], b[j])
        return np.dot(b[top], v) / (np.sqrt(v @ v) * mag[top])

    s12, s13, s23 = abs(np.sin(ang(0, 1))), abs(np.sin(ang(0, 2))), abs(np.sin(ang(1, 2)))
    A = [kc / (mag[0] * s12) + 1, kc / (mag[1] * s12) + 1, kc / (mag[2] * abs(sinphi(2, 0, 1))) + 1]
    B = [kc / (mag[0] * s13) + 1, kc / (mag[1] * abs(sinphi(1, 0, 2))) + 1, kc / (mag[2] * s13) + 1]
    C = [kc / (mag[0] * abs(sinphi(0, 1, 2))) + 1, kc / (mag[1] * s23) + 1, kc / (mag[2] * s23) + 1]
    return [max(A[i], B[i], C[i]) for i in range(3)]


def _wrap_axis(nb):
    """Indices in loop order 0..2*nb (double bound), wrapped as reader.c:232-243."""
    out = []
    i = 0
    while i <= 2.0 * nb:
        out.append(int(i - 2.0 * nb - 1.0) if i > nb else i)
        i += 1
    return np.array(out, dtype=np.int64)


def gvectors(lattice, kpt, encut, return_energy=False):
    """The plane-wave list of one k-point in WAVECAR order (reader.c:230-271).

    Returns int32 [W, 3] with ig1 fastest, ig3 slowest; keeps |k+G|^2/c <= encut.
    """
    b = reciprocal_lattice(lattice)
    n1, n2, n3 = nbmax(lattice, encut)
    i1, i2, i3 = _wrap_axis(n1), _wrap_axis(n2), _wrap_axis(n3)
    g3, g2, g1 = np.meshgrid(i3, i2, i1, indexing="ij")
    g = np.stack([g1.ravel(), g2.ravel(), g3.ravel()], axis=1)
    kg = (kpt[0] + g[:, 0:1]) * b[0] + (kpt[1] + g[:, 1:2]) * b[1] + (kpt[2] + g[:, 2:3]) * b[2]
    e = (kg * kg).sum(1) / C_EV
    keep = e <= encut
    if return_energy:
        return g[keep].astype(np.int32), e
    return g[keep].astype(np.int32)


def cutoff_margin(lattice, kpt, encut):
    """Smallest relative distance of any |k+G|^2/c from ENCUT (a boundary-ambiguity check)."""
    _, e = gvectors(lattice, kpt, encut, return_energy=True)
    return float(np.min(np.abs(e - encut)) / encut)


def write_wavecar(path, lattice, encut, kpts, coeffs, energies, occs, nspin=1):
    """Write a complex64 (rtag 45200) WAVECAR.

    ``coeffs[iwk]`` is complex64 [nband, W_k] for iwk = spin*nwk + k, in the
    plane-wave order of :func:`gvectors`; ``energies``/``occs`` are [nspin*nwk, nband].
    Record layout as read by reader.c:129-299.
    """
    kpts = np.asarray(kpts, dtype=np.float64).reshape(-1, 3)
    nwk = kpts.shape[0]
    nband = coeffs[0].shape[0]
    maxw = max(c.shape[1] for c in coeffs)
    nrecl = max(8 * maxw, 8 * (4 + 3 * nband), 8 * 12)
    nrecl = (nrecl + 7) // 8 * 8
    with open(path, "wb") as fh:
        rec = np.zeros(nrecl // 8, dtype=np.float64)
        rec[:3] = [nrecl, nspin, 45200]
        fh.write(rec.tobytes())
        rec = np.zeros(nrecl // 8, dtype=np.float64)
        rec[0], rec[1], rec[2] = nwk, nband, encut
        rec[3:12] = np.asarray(lattice, dtype=np.float64).reshape(-1)
        fh.write(rec.tobytes())
        for iwk in range(nspin * nwk):
            c = np.ascontiguousarray(coeffs[iwk], dtype=np.complex64)
            rec = np.zeros(nrecl // 8, dtype=np.float64)
            rec[0] = c.shape[1]
            rec[1:4] = kpts[iwk % nwk]
            e = np.asarray(energies[iwk], dtype=np.float64)
            o = np.asarray(occs[iwk], dtype=np.float64)
            rec[4 : 4 + 3 * nband : 3] = e
            rec[6 : 6 + 3 * nband : 3] = o
            fh.write(rec.tobytes())
            for b in range(nband):
                row = np.zeros(nrecl // 8, dtype=np.complex64)
                row[: c.shape[1]] = c[b]
                fh.write(row.tobytes())


def read_wavecar_numpy(path):
    """Pure-numpy WAVECAR reader (structure of reader.c:129-299), for tests and tools.

    Returns dict(nspin, nwk, nband, encut, lattice, kpts[nwk,3], gs[list], coeffs[list],
    energies, occs).
    """
    raw = np.fromfile(path, dtype=np.float64, count=3)
    nrecl, nspin = int(round(raw[0])), int(round(raw[1]))
    rec = np.fromfile(path, dtype=np.float64, count=nrecl // 8, offset=nrecl)
    nwk, nband, encut = int(round(rec[0])), int(round(rec[1])), float(rec[2])
    lattice = rec[3:12].reshape(3, 3).copy()
    kpts, coeffs, gs, energies, occs = [], [], [], [], []
    for iwk in range(nspin * nwk):
        irec = iwk * (1 + nband)
        hdr = np.fromfile(path, dtype=np.float64, count=nrecl // 8, offset=(irec + 2) * nrecl)
        nplane = int(round(hdr[0]))
        k = hdr[1:4].copy()
        if iwk < nwk:
            kpts.append(k)
        energies.append(hdr[4 : 4 + 3 * nband : 3].copy())
        occs.append(hdr[6 : 6 + 3 * nband : 3].copy())
        g = gvectors(lattice, k, encut)
        if 2 * g.shape[0] == nplane:
            g = np.concatenate([g, g], axis=0)
        gs.append(g)
        c = np.empty((nband, nplane), dtype=np.complex64)
        for b in range(nband):
            c[b] = np.fromfile(path, dtype=np.complex64, count=nplane, offset=(irec + 3 + b) * nrecl)
        coeffs.append(c)
    return dict(nspin=nspin, nwk=nwk, nband=nband, encut=encut, lattice=lattice,
                kpts=np.array(kpts), gs=gs, coeffs=coeffs,
                energies=np.array(energies), occs=np.array(occs))

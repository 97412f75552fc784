"""Seeded synthetic inputs for the band-projection path.

No public dataset exists for this path; these generators stand in for VASP
outputs with the shapes, sizes and value distributions of the four named
workloads (8-atom / 64-atom / 216-atom cubic diamond cells and a 96-atom
orthorhombic cell).  Every choice the workload text leaves open is fixed here
and listed in ``CHOICES`` (k-point sets, species split, displacement reading).

Radial functions (all on a 400-point log grid r = 1e-4 .. 2.0 Angstrom,
projectors on the POTCAR linear grid rmax*j/NDATA, NDATA = 100):

  p_{l,n}(r)   = r^l exp(-r^2/(0.5 s_n)^2) (1-(r/rc)^2)^2   for r < rc, else 0
  phit_{l,n}(r) = r^l exp(-r^2/(0.6 s_n)^2)
  phi_{l,n}(r)  = phit_{l,n}(r) + 0.3 r^l sin((n+1) pi r/rc)   for r < rc

with s_0 = 1 and s_1 = 1.25 for the two channels n of each l, and the second
channel's all-electron correction carrying one more node (the workload text
gives one formula per l; distinct channels make channel-index mistakes in the
PAW sums visible), rc = 1.0 A for
species A (l = 0,0,1,1) and 1.2 A for species B (l = 0,0,1,1,2,2).  The POTCAR
stores the projector p(r) and the partial waves as r*phi(r).

Plane-wave coefficients: complex64 (N(0,1) + i N(0,1)) exp(-|k+G|^2/(2*4^2)),
each band normalised to sum |C|^2 = 1, drawn from numpy default_rng(seed).
"""

import os

import numpy as np

from . import vaspio
from .vaspio import C_EV, Structure

CHOICES = {
    "channels": "second channel of each l: widths 0.5*1.25 / 0.6*1.25 and sin(2 pi r/rc) in phi",
    "cfg0_kpoints": "Gamma, (1/4,1/4,1/4), (1/4,1/4,-1/4), (1/4,-1/4,-1/4); equal weights",
    "cfg1_species": "A on the first fcc sublattice, B on the second (32:32)",
    "cfg1_kpoints": "2x2x2 Monkhorst-Pack (+-1/4,+-1/4,+-1/4); equal weights",
    "cfg2_species": "A:B = 3:1 by a seeded permutation; defect substitutes 2 seeded A sites by B",
    "cfg2_displacement": "every defect atom moved by a uniform random vector in [-0.05,0.05]^3 A",
    "cfg3_structure": "4x4x6 jittered grid (+-0.2 A) in 10x12x14 A, species 50/50 seeded; "
                      "defect = atom 0 moved +0.1 A along x",
    "cfg3_grid": "36 x 45 x 50, the smallest 2,3,5-smooth N_i >= 2*g_max,i + 1",
    "occupations": "lower half of the bands occupied (occ = 1), upper half empty",
    "energies": "linspace(-5, 5, nband) eV",
}

NDATA = 100
NGRID = 400
RMIN, RMAXGRID = 1e-4, 2.0

DIAMOND = np.array([
    [0.00, 0.00, 0.00], [0.00, 0.50, 0.50], [0.50, 0.00, 0.50], [0.50, 0.50, 0.00],
    [0.25, 0.25, 0.25], [0.25, 0.75, 0.75], [0.75, 0.25, 0.75], [0.75, 0.75, 0.25],
])

SPECIES = {
    "A": dict(rc=1.0, ls=[0, 0, 1, 1]),
    "B": dict(rc=1.2, ls=[0, 0, 1, 1, 2, 2]),
}


def log_grid():
    return RMIN * (RMAXGRID / RMIN) ** (np.arange(NGRID) / (NGRID - 1))


def species_arrays(sym):
    """POTCAR arrays of a synthetic species: ls, rmax, ndata, realprojs, grid, aewaves, pswaves."""
    sp = SPECIES[sym]
    rc, ls = sp["rc"], sp["ls"]
    grid = log_grid()
    pgrid = rc * np.arange(NDATA) / NDATA
    realprojs, aewaves, pswaves = [], [], []
    seen = {}
    for l in ls:
        n = seen.get(l, 0)
        seen[l] = n + 1
        s = 1.0 + 0.25 * n
        p = pgrid ** l * np.exp(-pgrid ** 2 / (0.5 * s) ** 2) * (1 - (pgrid / rc) ** 2) ** 2
        p[pgrid >= rc] = 0.0
        pt = grid ** l * np.exp(-grid ** 2 / (0.6 * s) ** 2)
        ae = pt + np.where(grid < rc, 0.3 * grid ** l * np.sin((n + 1) * np.pi * grid / rc), 0.0)
        realprojs.append(p)
        pswaves.append(grid * pt)
        aewaves.append(grid * ae)
    return dict(ls=ls, rmax=rc, ndata=NDATA, realprojs=realprojs, grid=grid,
                aewaves=aewaves, pswaves=pswaves)


def potcar_text(symbols):
    txt = ""
    for sym in symbols:
        a = species_arrays(sym)
        txt += vaspio.potcar_dataset_text(sym, a["ls"], a["rmax"], a["ndata"], a["realprojs"],
                                          a["grid"], a["aewaves"], a["pswaves"])
    return txt


# --------------------------------------------------------------------------
# structures
# --------------------------------------------------------------------------


def _supercell(a0, n):
    fr = []
    for i in range(n):
        for j in range(n):
            for k in range(n):
                fr.append((DIAMOND + [i, j, k]) / n)
    return np.concatenate(fr, axis=0), np.eye(3) * a0 * n


def _group_by_species(species, coords, order=("A", "B")):
    idx = [i for s in order for i in range(len(species)) if species[i] == s]
    return [species[i] for i in idx], coords[idx]


def structures(cfg, seed=0):
    """(basis, defect) Structure pair of a named workload."""
    rng = np.random.default_rng(1000 + seed)
    if cfg == 0:
        coords, lat = _supercell(5.43, 1)
        basis = Structure(lat, ["A"] * 8, coords)
        dc = coords.copy()
        dc[0, 0] += 0.1 / 5.43
        defect = Structure(lat, ["A"] * 8, dc)
    elif cfg == 1:
        coords, lat = _supercell(5.43, 2)
        species = ["A" if (i % 8) < 4 else "B" for i in range(64)]
        species, coords = _group_by_species(species, coords)
        basis = Structure(lat, species, coords)
        defect = Structure(lat, species[1:], coords[1:])
    elif cfg == 2:
        coords, lat = _supercell(5.43, 3)
        perm = rng.permutation(216)
        species = ["A"] * 216
        for i in perm[:54]:
            species[i] = "B"
        dspecies = list(species)
        a_sites = [i for i in range(216) if species[i] == "A"]
        for i in rng.choice(a_sites, size=2, replace=False):
            dspecies[i] = "B"
        disp = rng.uniform(-0.05, 0.05, size=(216, 3)) / 16.29
        order = sorted(range(216), key=lambda i: (species[i], i))
        basis = Structure(lat, [species[i] for i in order], coords[order])
        dorder = sorted(range(216), key=lambda i: (dspecies[i], i))
        defect = Structure(lat, [dspecies[i] for i in dorder], (coords + disp)[dorder])
    elif cfg == 3:
        lat = np.diag([10.0, 12.0, 14.0])
        g = np.stack(np.meshgrid(np.arange(4), np.arange(4), np.arange(6), indexing="ij"), -1)
        fr = (g.reshape(-1, 3) + 0.5) / np.array([4, 4, 6])
        fr = fr + rng.uniform(-0.2, 0.2, size=fr.shape) / np.diag(lat)
        sp = np.array(["A"] * 48 + ["B"] * 48)[rng.permutation(96)].tolist()
        sp, fr = _group_by_species(sp, fr)
        basis = Structure(lat, sp, fr)
        dc = fr.copy()
        dc[0, 0] += 0.1 / 10.0
        defect = Structure(lat, sp, dc)
    else:
        raise ValueError("unknown workload %r" % cfg)
    return basis, defect


def workload(cfg):
    """Sampling parameters of a named workload: encut, dim, kpts, weights, nband, nspin."""
    if cfg == 0:
        k = np.array([[0, 0, 0], [0.25, 0.25, 0.25], [0.25, 0.25, -0.25], [0.25, -0.25, -0.25]])
        return dict(encut=300.0, dim=(24, 24, 24), kpts=k, nband=32, nspin=1)
    if cfg == 1:
        k = np.array([[x, y, z] for x in (0.25, -0.25) for y in (0.25, -0.25) for z in (0.25, -0.25)])
        return dict(encut=400.0, dim=(60, 60, 60), kpts=k, nband=256, nspin=1)
    if cfg == 2:
        return dict(encut=400.0, dim=(90, 90, 90), kpts=np.zeros((1, 3)), nband=1024, nspin=1)
    if cfg == 3:
        rng = np.random.default_rng(3003)
        k = rng.uniform(-0.5, 0.5, size=(24, 3))
        return dict(encut=450.0, dim=(36, 45, 50), kpts=k, nband=128, nspin=2)
    raise ValueError("unknown workload %r" % cfg)


def small_workload(cfg, nband=None, nk=None):
    """A reduced copy of a workload (fewer bands / k-points), same cell and grid."""
    w = dict(workload(cfg))
    if nband is not None:
        w["nband"] = nband
    if nk is not None:
        w["kpts"] = w["kpts"][:nk]
    return w


# --------------------------------------------------------------------------
# coefficients
# --------------------------------------------------------------------------


def band_coefficients(rng, lattice, kpt, gs, nband):
    b = vaspio.reciprocal_lattice(lattice)
    kg = (kpt[0] + gs[:, 0:1]) * b[0] + (kpt[1] + gs[:, 1:2]) * b[1] + (kpt[2] + gs[:, 2:3]) * b[2]
    env = np.exp(-(kg * kg).sum(1) / (2.0 * 4.0 ** 2))
    w = gs.shape[0]
    c = (rng.standard_normal((nband, w), dtype=np.float32)
         + 1j * rng.standard_normal((nband, w), dtype=np.float32)).astype(np.complex64)
    c *= env.astype(np.float32)[None, :]
    nrm = np.sqrt((np.abs(c.astype(np.complex128)) ** 2).sum(1))
    return (c / nrm[:, None].astype(np.float32)).astype(np.complex64)


def wavefunction_data(struct, w, seed, ncl=False):
    """In-memory WAVECAR content for one structure of a workload.

    ncl: noncollinear content; each band is a spinor (up half, then down half,
    each on the k-point's G list) normalised as a whole."""
    rng = np.random.default_rng(seed)
    lattice = struct.lattice
    kpts = np.asarray(w["kpts"], dtype=np.float64).reshape(-1, 3)
    nwk, nspin, nband = kpts.shape[0], w["nspin"], w["nband"]
    for k in kpts:
        m = vaspio.cutoff_margin(lattice, k, w["encut"])
        if m < 1e-9:
            raise RuntimeError("a plane wave sits on the ENCUT sphere; move the k-point")
    gs, coeffs, energies, occs = [], [], [], []
    for iwk in range(nspin * nwk):
        k = kpts[iwk % nwk]
        g = vaspio.gvectors(lattice, k, w["encut"])
        gs.append(g)
        if ncl:
            up = band_coefficients(rng, lattice, k, g, nband)
            dn = band_coefficients(rng, lattice, k, g, nband)
            sp = np.concatenate([up, dn], axis=1).astype(np.complex128)
            sp /= np.sqrt((np.abs(sp) ** 2).sum(1))[:, None]
            coeffs.append(sp.astype(np.complex64))
        else:
            coeffs.append(band_coefficients(rng, lattice, k, g, nband))
        energies.append(np.linspace(-5.0, 5.0, nband))
        occs.append((np.arange(nband) < nband // 2).astype(np.float64))
    return dict(lattice=lattice, encut=w["encut"], kpts=kpts, nspin=nspin, nwk=nwk,
                nband=nband, gs=gs, coeffs=coeffs, energies=np.array(energies),
                occs=np.array(occs), weights=np.full(nwk, 1.0 / nwk), ncl=bool(ncl))


def write_structure_dir(path, struct, data, dim, symbols=None):
    """Write CONTCAR, WAVECAR, POTCAR and vasprun.xml for one structure."""
    os.makedirs(path, exist_ok=True)
    vaspio.write_poscar(os.path.join(path, "CONTCAR"), struct)
    vaspio.write_wavecar(os.path.join(path, "WAVECAR"), data["lattice"], data["encut"],
                         data["kpts"], data["coeffs"], data["energies"], data["occs"],
                         nspin=data["nspin"])
    if symbols is None:
        symbols = []
        for s in struct.species:
            if s not in symbols:
                symbols.append(s)
    with open(os.path.join(path, "POTCAR"), "w") as fh:
        fh.write(potcar_text(symbols))
    vaspio.write_vasprun(os.path.join(path, "vasprun.xml"), data["kpts"], data["weights"], dim)


def write_workload(root, cfg, nband=None, nk=None, seed=0):
    """Write basis/ and defect/ directories for a (possibly reduced) workload.

    Both POTCARs list species A then B (when present in either cell) so that the
    element labels of the two structures agree.
    """
    w = small_workload(cfg, nband=nband, nk=nk)
    basis, defect = structures(cfg, seed)
    syms = [s for s in ("A", "B") if s in basis.species or s in defect.species]
    out = {}
    for name, st, sd in (("basis", basis, 11 + 100 * seed), ("defect", defect, 22 + 100 * seed)):
        d = wavefunction_data(st, w, sd + 7 * cfg)
        write_structure_dir(os.path.join(root, name), st, d, w["dim"], symbols=syms)
        out[name] = os.path.join(root, name)
    return out

"""Generate the golden vectors under tests/golden/ from the reference pawpyseed C core.

Run in a container where the reference sources are present:

    make -C oracle ref            # builds oracle/_ref/libpawpy_ref.so from the reference C
    python tests/golden/make_golden.py

Inputs are the seeded synthetic workloads of ``pawpyseed_gb300.synth`` (reduced
band / k-point counts so the reference finishes in seconds); each fixture
stores a fingerprint of the inputs it was made from, so a test can tell
whether its regenerated inputs are the same bytes.

Fixtures:
* ``fft_ga4.npz``  -- the reference's own fft3d known-answer case
  (pawpyseed/core/tests/tests.c:28-80): band 0, k-point 0 of the Ga4
  test_files/WAVECAR on a 20^3 grid, with the reference fft3d output and a
  direct plane-wave sum.
* ``<name>.npz``   -- reference ``single_band_projection`` (aug_real) for every
  defect band: total PAW overlaps, pseudo overlaps, per-band projector
  coefficients, N_RS pair matrices; and the same projections with the
  ``aug_recip`` method (``recip_total_*``) with the augmentation coefficients
  band->CAs of band 0 of each side that has them, per k-point, first 4096
  plane waves in file order (``recip_CA_<side>_k<k>``).
* ``realspace_cfg0.npz`` -- the real-space functions of density.c on the
  8-atom workload reduced to 4 bands and 2 k-points, on the defect's grid:
  ``realspace_state`` of band 1 at k-point 1 (``state_b1_k1``),
  ``ae_chg_density`` of the defect (``rho``), and
  ``project_realspace_state`` of every defect band onto the basis (``proj``,
  [band][basis band * nk + k]).
* ``realspace_ncl_cfg0.npz`` -- the noncollinear real-space functions of
  density.c (``ncl_realspace_state``, up then down component, of band 3 at
  k-point 1; ``ncl_ae_chg_density``) and the spinor projections of
  ``onto_projector_ncl`` (``P_up``, ``P_down``: [k][band][sites x channels]) on
  a spinor wavefunction of the 8-atom cell (4 bands, 2 k-points).

The reference tree is read from $PAWPY_REFERENCE (default /root/reference).
"""

import ctypes as C
import hashlib
import os
import shutil
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from pawpyseed_gb300 import synth, vaspio  # noqa: E402

REFERENCE = os.environ.get("PAWPY_REFERENCE", "/root/reference")

# realspace_state adds the sites' partial waves from an OpenMP loop over sites whose
# updates of shared grid cells are unsynchronised (density.c:265-306); one thread makes
# the sums deterministic.
os.environ["OMP_NUM_THREADS"] = "1"

CASES = {
    # name: (workload, nband, nk, flips)
    "cfg0": (0, 32, None, (False,)),
    "cfg1s": (1, 8, 2, (False,)),
    "cfg2s": (2, 4, None, (False,)),
    "cfg3s": (3, 4, 2, (False, True)),
}


def fingerprint(path):
    h = hashlib.sha256()
    for name in ("WAVECAR", "POTCAR", "CONTCAR", "vasprun.xml"):
        with open(os.path.join(path, name), "rb") as fh:
            h.update(fh.read())
    return h.hexdigest()


def fft_fixture():
    import ref_harness as rh

    lib = rh.load_ref()
    wc = os.path.join(REFERENCE, "test_files", "WAVECAR")
    d = vaspio.read_wavecar_numpy(wc)
    g = np.ascontiguousarray(d["gs"][0], dtype=np.int32)
    c = np.ascontiguousarray(d["coeffs"][0][0], dtype=np.complex64)
    lat = np.ascontiguousarray(d["lattice"].reshape(-1), dtype=np.float64)
    fftg = np.array([20, 20, 20], np.int32)
    x = np.zeros(8000, np.complex128)
    lib.fft3d(x, None, lat, np.ascontiguousarray(d["kpts"][0]), g.reshape(-1).copy(),
              c.ctypes.data_as(rh.C.c_void_p), g.shape[0], fftg)
    f = np.stack(np.meshgrid(np.arange(20), np.arange(20), np.arange(20), indexing="ij"), -1) / 20.0
    ph = np.exp(2j * np.pi * (f.reshape(-1, 3) @ g.T.astype(np.float64)))
    direct = ph @ c.astype(np.complex128) / np.sqrt(abs(np.linalg.det(d["lattice"])))
    np.savez_compressed(os.path.join(HERE, "fft_ga4.npz"), gs=g, cs=c, lattice=d["lattice"],
                        kpt=d["kpts"][0], fftg=fftg, ref=x, direct=direct)
    print("fft_ga4: max|ref-direct| = %.3e" % np.abs(x - direct).max())


def case_fixture(name, cfg, nband, nk, flips):
    import ref_harness as rh

    lib = rh.load_ref()
    tmp = tempfile.mkdtemp()
    try:
        paths = synth.write_workload(tmp, cfg, nband=nband, nk=nk)
        b = rh.RefWavefunction(lib, paths["basis"])
        d = rh.RefWavefunction(lib, paths["defect"])
        pr = rh.RefProjector(lib, b, d)
        out = dict(fp_basis=fingerprint(paths["basis"]), fp_defect=fingerprint(paths["defect"]),
                   cfg=cfg, nband=nband, nk=-1 if nk is None else nk)
        for flip in flips:
            tag = "flip" if flip else "noflip"
            out["total_" + tag] = np.array([pr.single_band_projection(i, flip) for i in range(d.nband)])
            out["pseudo_" + tag] = np.array([pr.pseudo(i, flip) for i in range(d.nband)])
        nkt = b.nwk * b.nspin
        nbp = min(2, b.nband)
        out["P_basis"] = np.array([[np.concatenate(b.projections(bb, k)) for bb in range(nbp)]
                                   for k in range(nkt)])
        out["P_defect"] = np.array([[np.concatenate(d.projections(bb, k)) for bb in range(nbp)]
                                    for k in range(nkt)])
        Q, dc = pr.overlaps_NRS()
        Q, dc = Q[:6], dc[:6]
        if Q:
            out["Q_shapes"] = np.array([q.shape for q in Q])
            out["Q_flat"] = np.concatenate([q.reshape(-1) for q in Q])
            out["dcoords"] = dc
        for k, v in pr.lists.items():
            out["list_" + k] = v
        # the aug_recip method on fresh wavefunctions (band->CAs are kept per band)
        b2 = rh.RefWavefunction(lib, paths["basis"])
        d2 = rh.RefWavefunction(lib, paths["defect"])
        prr = rh.RefProjector(lib, b2, d2, recip=True)
        for flip in flips:
            tag = "flip" if flip else "noflip"
            out["recip_total_" + tag] = np.array([prr.single_band_projection(i, flip) for i in range(d2.nband)])
        for side, wfr in (("basis", b2), ("defect", d2)):
            for k in range(nkt):
                ca = wfr.aug_coefficients(0, k)
                if ca is not None:
                    out["recip_CA_%s_k%d" % (side, k)] = ca[:4096]
        b2.free()
        d2.free()
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(name, "written", {k: getattr(v, "shape", v) for k, v in out.items() if k.startswith("total")})
        b.free()
        d.free()
    finally:
        shutil.rmtree(tmp)


def realspace_fixture():
    import ref_harness as rh

    lib = rh.load_ref()
    zp = np.ctypeslib.ndpointer(dtype=np.complex128, flags="C_CONTIGUOUS")
    dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
    ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
    wfp = C.POINTER(rh.S.pswf_t)
    lib.realspace_state.argtypes = [zp, C.c_int, C.c_int, wfp, ip, ip, dp]
    lib.ae_chg_density.argtypes = [dp, wfp, ip, ip, dp]
    lib.project_realspace_state.argtypes = [zp, C.c_int, wfp, wfp, ip, ip, dp, ip, dp]
    tmp = tempfile.mkdtemp()
    try:
        paths = synth.write_workload(tmp, 0, nband=4, nk=2)
        b = rh.RefWavefunction(lib, paths["basis"])
        d = rh.RefWavefunction(lib, paths["defect"])
        b.setup_projectors()
        d.setup_projectors()
        fftg = np.ascontiguousarray(d.dim, dtype=np.int32)
        n = int(np.prod(fftg))
        x = np.zeros(n, np.complex128)
        lib.realspace_state(x, 1, 1, d.ptr, fftg, d.nums, d.coords)
        rho = np.zeros(n)
        lib.ae_chg_density(rho, d.ptr, fftg, d.nums, d.coords)
        nk = d.nwk * d.nspin
        proj = np.zeros((d.nband, b.nband * nk), np.complex128)
        for band in range(d.nband):
            row = np.zeros(b.nband * nk, np.complex128)
            lib.project_realspace_state(row, band, d.ptr, b.ptr, fftg, d.nums, d.coords, b.nums, b.coords)
            proj[band] = row
        out = dict(fp_basis=fingerprint(paths["basis"]), fp_defect=fingerprint(paths["defect"]),
                   fftg=fftg, state_b1_k1=x.reshape(tuple(fftg)), rho=rho.reshape(tuple(fftg)), proj=proj)
        np.savez_compressed(os.path.join(HERE, "realspace_cfg0.npz"), **out)
        print("realspace_cfg0 written: grid", tuple(fftg), "sum rho dV =",
              rho.sum() * abs(np.linalg.det(d.struct.lattice)) / n)
        b.free()
        d.free()
    finally:
        shutil.rmtree(tmp)


def ncl_realspace_inputs():
    """The noncollinear case of the real-space fixture: the 8-atom cell, 4 spinor bands, 2
    k-points, species A only, coefficients seed 77 (tests/test_oracle.py rebuilds the same)."""
    w = synth.small_workload(0, nband=4, nk=2)
    bs, _ = synth.structures(0)
    data = synth.wavefunction_data(bs, w, 77, ncl=True)
    return bs, w, data


def ncl_realspace_fixture():
    import ref_harness as rh

    lib = rh.load_ref()
    zp = np.ctypeslib.ndpointer(dtype=np.complex128, flags="C_CONTIGUOUS")
    dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
    ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
    wfp = C.POINTER(rh.S.pswf_t)
    lib.ncl_realspace_state.argtypes = [zp, C.c_int, C.c_int, wfp, ip, ip, dp]
    lib.ncl_ae_chg_density.argtypes = [dp, wfp, ip, ip, dp]
    tmp = tempfile.mkdtemp()
    try:
        bs, w, data = ncl_realspace_inputs()
        path = os.path.join(tmp, "ncl")
        synth.write_structure_dir(path, bs, data, w["dim"], symbols=["A"])
        d = rh.RefWavefunction(lib, path)
        assert d.ptr.contents.is_ncl == 1
        d.setup_projectors()
        fftg = np.ascontiguousarray(d.dim, dtype=np.int32)
        n = int(np.prod(fftg))
        out = dict(fp=fingerprint(path), fftg=fftg)
        nk = d.nwk * d.nspin
        for side in ("up", "down"):
            out["P_" + side] = np.array([[np.concatenate(d.projections(b, k, side + "_projections"))
                                          for b in range(d.nband)] for k in range(nk)])
        x = np.zeros(2 * n, np.complex128)
        lib.ncl_realspace_state(x, 3, 1, d.ptr, fftg, d.nums, d.coords)
        out["state_b3_k1"] = x.reshape((2,) + tuple(fftg))
        rho = np.zeros(n)
        lib.ncl_ae_chg_density(rho, d.ptr, fftg, d.nums, d.coords)
        out["rho"] = rho.reshape(tuple(fftg))
        np.savez_compressed(os.path.join(HERE, "realspace_ncl_cfg0.npz"), **out)
        print("realspace_ncl_cfg0 written: grid", tuple(fftg), "sum rho dV =",
              rho.sum() * abs(np.linalg.det(d.struct.lattice)) / n)
        d.free()
    finally:
        shutil.rmtree(tmp)


if __name__ == "__main__":
    which = sys.argv[1:] or ["fft"] + list(CASES) + ["realspace", "realspace_ncl"]
    for w in which:
        if w == "fft":
            fft_fixture()
        elif w == "realspace":
            realspace_fixture()
        elif w == "realspace_ncl":
            ncl_realspace_fixture()
        else:
            case_fixture(w, *CASES[w])

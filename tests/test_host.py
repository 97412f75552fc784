"""Host-side logic of the library, without a GPU: ABI exports, struct layout,
the WAVECAR reader, the radial (per-element) setup, file formats and site lists."""

import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import CASES, ROOT, fingerprint


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "pawpy_gpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    names = re.findall(r"^[A-Za-z_][\w \*]*?\b(\w+)\s*\(", txt, flags=re.M)
    return sorted(set(n for n in names if n not in ("if", "sizeof")))


def test_library_exports_every_header_symbol():
    from pawpyseed_gb300 import _lib

    L = _lib.lib()
    syms = header_symbols()
    assert "pseudoprojection" in syms and "compensation_terms" in syms and "fft3d" in syms
    for s in syms:
        assert hasattr(L, s), s


def test_struct_layout_matches_reference_layout():
    from pawpyseed_gb300 import _lib, structs

    lib_rows = {(s, m): o for s, m, o in _lib.struct_layout()}
    ct_rows = {(s, m): o for s, m, o in structs.layout_table()}
    assert set(lib_rows) == set(ct_rows)
    for k, v in ct_rows.items():
        assert lib_rows[k] == v, k


def test_wavecar_reader_matches_numpy_reader(workload_dirs):
    from pawpyseed_gb300 import _lib, vaspio

    d = workload_dirs("cfg3s")["basis"]
    ref = vaspio.read_wavecar_numpy(os.path.join(d, "WAVECAR"))
    kws = np.full(ref["nwk"], 1.0 / ref["nwk"])
    L = _lib.lib()
    p = L.pawpy_gpu_read_wavefunctions(os.path.join(d, "WAVECAR").encode(), kws)
    _lib.check()
    try:
        w = p.contents
        assert (w.nspin, w.nwk, w.nband) == (ref["nspin"], ref["nwk"], ref["nband"])
        for k in range(w.nspin * w.nwk):
            kp = w.kpts[k].contents
            g = np.ctypeslib.as_array(kp.Gs, shape=(3 * kp.num_waves,)).reshape(-1, 3)
            assert np.array_equal(g, ref["gs"][k])
            for b in (0, w.nband - 1):
                c = np.ctypeslib.as_array(C.cast(kp.bands[b].contents.Cs, C.POINTER(C.c_float)),
                                          shape=(2 * kp.num_waves,)).view(np.complex64)
                assert np.array_equal(c, ref["coeffs"][k][b])
                assert kp.bands[b].contents.occ == ref["occs"][k][b]
    finally:
        L.pawpy_gpu_free_pswf(p)


@pytest.mark.parametrize("suffix", [".gz", ".bz2"])
def test_compressed_wavecar_reads_as_the_plain_file(suffix, workload_dirs, tmp_path):
    import bz2
    import gzip
    import shutil

    from pawpyseed_gb300.wavefunction import Wavefunction

    d = workload_dirs("cfg0")["defect"]
    for f in ("CONTCAR", "POTCAR", "vasprun.xml"):
        shutil.copy(os.path.join(d, f), tmp_path / f)
    opener = gzip.open if suffix == ".gz" else bz2.open
    with open(os.path.join(d, "WAVECAR"), "rb") as src, opener(tmp_path / ("WAVECAR" + suffix), "wb") as dst:
        shutil.copyfileobj(src, dst)
    plain = Wavefunction.from_directory(d)
    packed = Wavefunction.from_files(str(tmp_path / "CONTCAR"), str(tmp_path / ("WAVECAR" + suffix)),
                                     str(tmp_path / "POTCAR"), str(tmp_path / "vasprun.xml"))
    a, b = plain.wf_ptr.contents, packed.wf_ptr.contents
    assert (a.nspin, a.nwk, a.nband) == (b.nspin, b.nwk, b.nband)
    for k in range(a.nspin * a.nwk):
        ka, kb = a.kpts[k].contents, b.kpts[k].contents
        assert ka.num_waves == kb.num_waves
        for band in (0, a.nband - 1):
            ca = np.ctypeslib.as_array(C.cast(ka.bands[band].contents.Cs, C.POINTER(C.c_float)),
                                       shape=(2 * ka.num_waves,))
            cb = np.ctypeslib.as_array(C.cast(kb.bands[band].contents.Cs, C.POINTER(C.c_float)),
                                       shape=(2 * kb.num_waves,))
            assert np.array_equal(ca, cb)


def test_reference_wavecar_fixture_gsphere(golden):
    """The plane-wave enumeration reproduces the Ga4 WAVECAR's counts (945 at k0)."""
    from pawpyseed_gb300 import vaspio

    g = golden("fft_ga4")
    gs = vaspio.gvectors(g["lattice"], g["kpt"], 320.0)
    assert np.array_equal(gs, g["gs"])


def test_wavecar_from_bytes_reads_as_the_file(workload_dirs):
    """pawpy_gpu_read_wavefunctions_from_bytes / _from_str (read_wavefunctions_from_str,
    reader.c:324-329) give the file reader's wavefunction; a short buffer is an error."""
    from pawpyseed_gb300 import _lib

    d = workload_dirs("cfg3s")["basis"]
    path = os.path.join(d, "WAVECAR")
    data = open(path, "rb").read()
    L = _lib.lib()
    kws = np.ones(64)
    pf = L.pawpy_gpu_read_wavefunctions(path.encode(), kws)
    _lib.check()
    pb = L.pawpy_gpu_read_wavefunctions_from_bytes(data, len(data), kws)
    _lib.check()
    ps = L.pawpy_gpu_read_wavefunctions_from_str(data, kws)
    _lib.check()
    try:
        a = pf.contents
        for p in (pb, ps):
            b = p.contents
            assert (a.nspin, a.nwk, a.nband, a.is_ncl) == (b.nspin, b.nwk, b.nband, b.is_ncl)
            assert [a.G_bounds[i] for i in range(6)] == [b.G_bounds[i] for i in range(6)]
            for k in range(a.nspin * a.nwk):
                ka, kb = a.kpts[k].contents, b.kpts[k].contents
                n = ka.num_waves
                assert kb.num_waves == n
                assert np.array_equal(np.ctypeslib.as_array(ka.Gs, shape=(3 * n,)),
                                      np.ctypeslib.as_array(kb.Gs, shape=(3 * n,)))
                for band in range(a.nband):
                    ca = np.ctypeslib.as_array(C.cast(ka.bands[band].contents.Cs, C.POINTER(C.c_float)),
                                               shape=(2 * n,))
                    cb = np.ctypeslib.as_array(C.cast(kb.bands[band].contents.Cs, C.POINTER(C.c_float)),
                                               shape=(2 * n,))
                    assert np.array_equal(ca, cb)
                    assert ka.bands[band].contents.energy == kb.bands[band].contents.energy
    finally:
        for p in (pf, pb, ps):
            L.pawpy_gpu_free_pswf(p)
    short = data[: len(data) - 8]
    p = L.pawpy_gpu_read_wavefunctions_from_bytes(short, len(short), kws)
    assert not p
    assert L.pawpy_gpu_last_error() == 4
    L.pawpy_gpu_clear_error()


def test_reader_errors_are_reported_not_fatal(tmp_path):
    from pawpyseed_gb300 import _lib

    L = _lib.lib()
    bad = tmp_path / "WAVECAR"
    bad.write_bytes(b"\0" * 16)
    p = L.pawpy_gpu_read_wavefunctions(str(bad).encode(), np.ones(1))
    assert not p
    with pytest.raises(_lib.PAWpyGPUError):
        _lib.check()
    p = L.pawpy_gpu_read_wavefunctions(str(tmp_path / "missing").encode(), np.ones(1))
    assert not p
    assert L.pawpy_gpu_last_error() != 0
    L.pawpy_gpu_clear_error()


def test_potcar_parser_reads_generated_dataset():
    from pawpyseed_gb300 import synth, vaspio

    cr = vaspio.CoreRegion(synth.potcar_text(["A", "B"]))
    assert list(cr.pps) == ["A", "B"]
    a = synth.species_arrays("B")
    pp = cr.pps["B"]
    assert pp.ls == [0, 0, 1, 1, 2, 2] and pp.ndata == 100 and pp.rmax == 1.2
    assert np.allclose(pp.grid, a["grid"], rtol=1e-9)
    for i in range(6):
        assert np.allclose(pp.realprojs[i], a["realprojs"][i], rtol=1e-8, atol=1e-12)
        assert np.allclose(pp.aewaves[i], a["aewaves"][i], rtol=1e-8, atol=1e-12)


def test_potcar_parser_agrees_with_reference_parser():
    """Our POTCAR parser and the reference's Pseudopotential give the same arrays."""
    import importlib.util
    import sys
    import types

    src = os.path.join(os.environ.get("PAWPY_REFERENCE", "/root/reference"), "pawpyseed/core/wavefunction.py")
    if not os.path.exists(src):
        pytest.skip("reference sources not present")
    from pawpyseed_gb300 import synth, vaspio

    stubs = {}
    for name in ["pymatgen", "pymatgen.io", "pymatgen.io.vasp", "pymatgen.io.vasp.inputs",
                 "pymatgen.io.vasp.outputs", "pawpyseed", "pawpyseed.core", "pawpyseed.core.symmetry",
                 "pawpyseed.core.utils"]:
        stubs[name] = types.ModuleType(name)
    stubs["pymatgen.io.vasp.inputs"].Poscar = stubs["pymatgen.io.vasp.inputs"].Potcar = object
    stubs["pymatgen.io.vasp.outputs"].Vasprun = object
    stubs["pawpyseed.core"].pawpyc = types.SimpleNamespace(CWavefunction=object)
    saved = {k: sys.modules.get(k) for k in stubs}
    sys.modules.update(stubs)
    try:
        spec = importlib.util.spec_from_file_location("ref_wavefunction", src)
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        txt = synth.potcar_text(["B"])
        ref = mod.Pseudopotential(txt[:-15])
        mine = vaspio.CoreRegion(txt).pps["B"]
        assert [int(x) for x in ref.ls] == mine.ls and ref.ndata == mine.ndata and ref.rmax == mine.rmax
        assert np.array_equal(ref.grid, mine.grid)
        for i in range(len(mine.ls)):
            assert np.array_equal(ref.realprojs[i], mine.realprojs[i])
            assert np.array_equal(ref.aewaves[i], mine.aewaves[i])
            assert np.array_equal(ref.pswaves[i], mine.pswaves[i])
    finally:
        for k, v in saved.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v


@pytest.mark.parametrize("name", list(CASES))
def test_site_lists_match_reference(name, workload_dirs, golden):
    """Projector.make_site_lists reproduces the reference's classification."""
    from pawpyseed_gb300 import vaspio

    d = workload_dirs(name)
    g = golden(name)
    b = vaspio.read_poscar(os.path.join(d["basis"], "CONTCAR"))
    w = vaspio.read_poscar(os.path.join(d["defect"], "CONTCAR"))
    bcr = vaspio.CoreRegion(os.path.join(d["basis"], "POTCAR"))
    wcr = vaspio.CoreRegion(os.path.join(d["defect"], "POTCAR"))

    class P:  # the Projector method on its own, without a device
        pass

    from pawpyseed_gb300.projector import Projector

    p = P()
    p.basis = type("W", (), {"structure": b, "cr": bcr})()
    p.wf = type("W", (), {"structure": w, "cr": wcr})()
    M_R, M_S, N_R, N_S, N_RS = Projector.make_site_lists(p)
    assert M_R == list(g["list_M_R"]) and M_S == list(g["list_M_S"])
    assert N_R == list(g["list_N_R"]) and N_S == list(g["list_N_S"])
    assert [a for a, _ in N_RS] == list(g["list_N_RS_R"]) and [c for _, c in N_RS] == list(g["list_N_RS_S"])


@pytest.mark.parametrize("name", list(CASES))
def test_synthetic_inputs_are_reproducible(name, workload_dirs, golden):
    """Regenerating a workload gives the bytes the golden fixtures were made from, so the fixture
    comparisons run at rounding level (elsewhere they fall back to tolerances, with a warning)."""
    d = workload_dirs(name)
    g = golden(name)
    assert fingerprint(d["basis"]) == str(g["fp_basis"])
    assert fingerprint(d["defect"]) == str(g["fp_defect"])


def test_collinear_and_noncollinear_classes_refuse_each_other():
    from pawpyseed_gb300 import synth, vaspio
    from pawpyseed_gb300.wavefunction import NCLWavefunction, PAWpyError, Wavefunction

    w = synth.small_workload(0, nband=2, nk=1)
    bs, _ = synth.structures(0)
    cr = vaspio.CoreRegion(synth.potcar_text(["A"]))
    ncl = synth.wavefunction_data(bs, w, 5, ncl=True)
    col = synth.wavefunction_data(bs, w, 5)
    wf = NCLWavefunction.from_arrays(bs, cr, w["dim"], ncl)
    kp = wf.wf_ptr.contents.kpts[0].contents
    assert wf.ncl and kp.num_waves == 2 * ncl["gs"][0].shape[0]
    g = np.ctypeslib.as_array(kp.Gs, shape=(3 * kp.num_waves,)).reshape(-1, 3)
    assert np.array_equal(g[: kp.num_waves // 2], g[kp.num_waves // 2:])
    with pytest.raises(PAWpyError):
        Wavefunction.from_arrays(bs, cr, w["dim"], ncl)
    with pytest.raises(PAWpyError):
        NCLWavefunction.from_arrays(bs, cr, w["dim"], col)


def test_host_worker_pool_runs_concurrent_loops_once_each():
    from pawpyseed_gb300 import _lib

    L = _lib.lib()
    # one caller, then eight callers sharing the workers; a thrown item reaches its caller
    assert L.pawpy_gpu_host_pool_check(1, 37) == 0
    assert L.pawpy_gpu_host_pool_check(8, 1000) == 0
    assert L.pawpy_gpu_host_pool_check(4, 0) == 0
    assert L.pawpy_gpu_host_pool_check(0, 5) == -1
    with pytest.raises(_lib.PAWpyGPUError):
        _lib.check()


@pytest.mark.parametrize("bad", [[-1], [0, 99]])
def test_defect_band_analysis_rejects_out_of_range_bands(bad):
    """aug_real band lists are checked before the batched reduction, with the reference's error
    (single_band_projection raises it for every band it is given, projector.py:270-271)."""
    from pawpyseed_gb300.projector import Projector

    class WF:
        nband, nwk, nspin = 4, 1, 1

        def _get_occs(self):
            return np.array([1.0, 1.0, 0.0, 0.0])

    pr = Projector.__new__(Projector)
    pr.method = "aug_real"
    pr.wf = WF()
    pr.basis = WF()

    def no_device(*a, **k):
        raise AssertionError("reached the device reduction")

    pr.band_character = no_device
    with pytest.raises(ValueError, match="Band index out of range"):
        pr.defect_band_analysis(band_list=bad)


@pytest.mark.parametrize("seed", range(4))
def test_reader_spheres_without_a_device_match_reference_enumeration(seed, tmp_path):
    """Without a CUDA device the reader enumerates the plane-wave spheres on the host threads with
    the reference's expression (gsphere_keep, the test the device path applies to the points it
    leaves undecided): bit-identical lists for triclinic cells, including k-points whose sphere
    has a plane wave exactly on ENCUT."""
    from test_gpu_gsphere import _etot, _rec, reference_gvectors

    from pawpyseed_gb300 import _lib, vaspio

    rng = np.random.default_rng(500 + seed)
    lat = np.diag(rng.uniform(3.0, 5.0, 3)) + rng.uniform(-1.0, 1.0, (3, 3)) * (1 - np.eye(3))
    kpts = np.array([rng.uniform(-0.5, 0.5, 3), np.zeros(3)])
    encut = float(rng.uniform(120.0, 220.0))
    if seed % 2:
        # ENCUT exactly the energy of a plane wave of the second k-point (on the cutoff)
        encut = _etot(_rec(lat), [0.0, 0.0, 0.0], (2, -1, 1))
    gs = [reference_gvectors(lat, k, encut) for k in kpts]
    coeffs = [np.ones((2, g.shape[0]), np.complex64) for g in gs]
    path = str(tmp_path / "WAVECAR")
    vaspio.write_wavecar(path, lat, encut, kpts, coeffs, np.zeros((2, 2)), np.zeros((2, 2)))
    L = _lib.lib()
    p = L.pawpy_gpu_read_wavefunctions(path.encode(), np.full(2, 0.5))
    _lib.check()
    try:
        w = p.contents
        for k in range(2):
            kp = w.kpts[k].contents
            g = np.ctypeslib.as_array(kp.Gs, shape=(3 * kp.num_waves,)).reshape(-1, 3)
            assert np.array_equal(g, gs[k])
    finally:
        L.pawpy_gpu_free_pswf(p)


def test_entry_points_record_argument_errors_instead_of_exiting():
    """The reference's C prints and exits on bad input (utils.c:1100-1118); the library records a
    status and returns. Arguments that are rejected before any device work: the no-allocation
    overlap's output limit and K rule (fake device pointers are never touched), and the
    plane-wave sphere entry point in a process without a device."""
    import ctypes as C

    from pawpyseed_gb300 import _lib

    L = _lib.lib()
    L.pawpy_gpu_overlap_noalloc.restype = C.c_int
    L.pawpy_gpu_overlap_noalloc.argtypes = [C.c_void_p, C.c_longlong, C.c_void_p, C.c_longlong,
                                            C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    fake = C.c_void_p(256)
    assert L.pawpy_gpu_overlap_noalloc(fake, 16, fake, 16, 4096, 4096, 16, fake, None) < 0
    with pytest.raises(_lib.PAWpyGPUError, match="scratch limit"):
        _lib.check()
    assert L.pawpy_gpu_overlap_noalloc(fake, 32, fake, 32, 8, 8, 24, fake, None) < 0
    with pytest.raises(_lib.PAWpyGPUError, match="multiple of 16"):
        _lib.check()
    assert L.pawpy_gpu_overlap_noalloc(None, 16, fake, 16, 8, 8, 16, fake, None) < 0
    with pytest.raises(_lib.PAWpyGPUError, match="NULL"):
        _lib.check()
    assert L.pawpy_gpu_last_error() == 0
    lat = np.eye(3) * 5.0
    n = L.pawpy_gpu_gvectors(np.ascontiguousarray(lat.reshape(-1)), np.zeros(3), 200.0, None, 0)
    if n >= 0:
        pytest.skip("a CUDA device is present: the sphere entry point runs")
    with pytest.raises(_lib.PAWpyGPUError, match="no CUDA device"):
        _lib.check()

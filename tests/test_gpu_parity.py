"""Parity of the CUDA path (through the C ABI) with the reference and the oracle.

Tolerance: the overlaps must agree with the FP64 evaluation (the oracle) to
|error| <= 1e-5 (the accuracy target of the band-pair metric); projector
coefficients to 1e-5 relative to their largest magnitude; the FFT to 1e-5 per
grid point (the reference's own fft_check bound, core/tests/tests.c:61).
"""

import ctypes as C
import os

import numpy as np
import pytest

from conftest import CASES, same_golden_inputs

pytestmark = pytest.mark.gpu

TOL = 1e-5


def load(dirs):
    from pawpyseed_gb300.wavefunction import Wavefunction

    return Wavefunction.from_directory(dirs["basis"]), Wavefunction.from_directory(dirs["defect"])


def host_projections(wf, k, b):
    kp = wf.wf_ptr.contents.kpts[k].contents
    bd = kp.bands[b].contents
    out = []
    for s in range(len(wf.structure)):
        p = bd.projections[s]
        v = np.ctypeslib.as_array(p.overlaps, shape=(2 * p.total_projs,))
        out.append(v[0::2] + 1j * v[1::2])
    return np.concatenate(out)


def test_fft3d_known_answer(golden):
    """fft3d against a direct plane-wave sum on the reference's Ga4 WAVECAR (20^3)."""
    from pawpyseed_gb300 import _lib

    g = golden("fft_ga4")
    L = _lib.lib()
    x = np.zeros(8000, np.complex128)
    cs = np.ascontiguousarray(g["cs"], dtype=np.complex64)
    L.fft3d(x, None, np.ascontiguousarray(g["lattice"].reshape(-1)), np.ascontiguousarray(g["kpt"]),
            np.ascontiguousarray(g["gs"].reshape(-1), dtype=np.int32), cs.ctypes.data_as(C.c_void_p),
            g["gs"].shape[0], np.ascontiguousarray(g["fftg"], dtype=np.int32))
    _lib.check()
    assert np.abs(x - g["direct"]).max() <= 1e-5
    assert np.abs(x - g["ref"]).max() <= 1e-5


def test_projector_list_matches_oracle():
    """get_projector_list (device FP64) against the oracle's element setup."""
    import oracle as orc

    from pawpyseed_gb300 import _lib, synth, vaspio
    from pawpyseed_gb300.wavefunction import pack_species

    cr = vaspio.CoreRegion(synth.potcar_text(["A", "B"]))
    labels, ls, wg, pr, ae, ps, rm = pack_species(cr)
    L = _lib.lib()
    for ge in (640.0, 1150.0):
        pps = L.get_projector_list(2, labels, ls, wg, pr, ae, ps, rm, ge)
        _lib.check()
        for e, sym in enumerate(cr.pps):
            o = orc.OSpecies(cr.pps[sym], ge)
            pp = pps[e]
            nd, ng = pp.proj_gridsize, pp.wave_gridsize
            assert pp.total_projs == o.total and pp.num_projs == o.nproj
            for k in range(pp.num_projs):
                f = pp.funcs[k]
                sdw = np.ctypeslib.as_array(f.smooth_diffwave, shape=(nd,))
                kw = np.ctypeslib.as_array(f.kwave, shape=(ng,))
                # FP64 round-off of two 800-point transforms (device twiddles vs the oracle's)
                assert np.allclose(sdw, o.sdw[k * nd:(k + 1) * nd], rtol=0, atol=1e-10 * np.abs(sdw).max())
                assert np.allclose(kw, o.kwave[k * ng:(k + 1) * ng], rtol=0, atol=1e-10 * np.abs(kw).max())
            n = pp.num_projs
            aeov = np.ctypeslib.as_array(pp.aepw_overlap_matrix, shape=(n * n,))
            psov = np.ctypeslib.as_array(pp.pspw_overlap_matrix, shape=(n * n,))
            assert np.allclose(aeov, o.aeov, atol=1e-13) and np.allclose(psov, o.psov, atol=1e-13)


@pytest.mark.parametrize("name", ["cfg0", "cfg1s"])
def test_projector_coefficients(name, workload_dirs, oracle_projectors, golden):
    basis, wf = load(workload_dirs(name))
    basis.check_c_projectors()
    op = oracle_projectors(name)
    for k in range(basis.nwk * basis.nspin):
        for b in (0, basis.nband - 1):
            mine = host_projections(basis, k, b)
            ref = op.basis.P[k][b]
            assert np.abs(mine - ref).max() <= TOL * np.abs(ref).max()


@pytest.mark.parametrize("name", list(CASES))
def test_single_band_projection(name, workload_dirs, oracle_projectors, golden):
    """Projector.single_band_projection (pseudoprojection + compensation_terms) for every band."""
    from pawpyseed_gb300.projector import Projector

    dirs = workload_dirs(name)
    basis, wf = load(dirs)
    pr = Projector(wf, basis)
    op = oracle_projectors(name)
    g = golden(name)
    same = same_golden_inputs(dirs, g, name)
    flips = [False, True] if "total_flip" in g.files else [False]
    for flip in flips:
        truth = op.full(flip)  # FP64
        mine = np.array([pr.single_band_projection(b, flip_spin=flip) for b in range(wf.nband)])
        tv = np.array([op.band_vector(truth, b) for b in range(wf.nband)])
        assert np.abs(mine - tv).max() <= TOL
        if same:
            assert np.abs(mine - g["total_" + ("flip" if flip else "noflip")]).max() <= TOL
        # the PAW terms alone, against the FP64 sums
        pseudo = np.array([wf.pseudoprojection(b, basis, flip) for b in range(wf.nband)])
        comp_truth = np.array([op.band_vector(op.comp_full(flip), b) for b in range(wf.nband)])
        assert np.abs((mine - pseudo) - comp_truth).max() <= 1e-7


@pytest.mark.parametrize("name", list(CASES))
def test_project_all_matches_band_loop(name, workload_dirs, oracle_projectors):
    """The batched contraction equals the per-band ABI path and the FP64 truth."""
    from pawpyseed_gb300.projector import Projector

    basis, wf = load(workload_dirs(name))
    pr = Projector(wf, basis)
    op = oracle_projectors(name)
    full = pr.project_all()
    loop = np.array([pr.single_band_projection(b) for b in range(wf.nband)])
    truth = op.full()
    tv = np.array([op.band_vector(truth, b) for b in range(wf.nband)])
    assert full.shape == loop.shape
    assert np.abs(full - tv).max() <= TOL
    assert np.abs(full - loop).max() <= 2e-6


@pytest.mark.parametrize("name", ["cfg1s", "cfg2s", "cfg3s"])
def test_deferred_projections_single_fft_pass(name, workload_dirs, oracle_projectors, monkeypatch):
    """With host projection_t output off, <p|psi> and the smoothed-partial-wave projections of a
    wavefunction come from one FFT pass; results equal the FP64 truth. The first pass issued
    early (at setup, on the auxiliary stream, for every k-point) and the interleaved form give
    the same overlaps bit for bit."""
    from pawpyseed_gb300 import _lib
    from pawpyseed_gb300.projector import Projector

    L = _lib.lib()
    L.pawpy_gpu_set_host_projections(0)
    op = oracle_projectors(name)
    truth = op.full()
    try:
        fulls = {}
        for early in ("1", "0"):
            monkeypatch.setenv("PAWPY_GPU_EARLY_FFT", early)
            basis, wf = load(workload_dirs(name))
            pr = Projector(wf, basis)
            full = pr.project_all()
            tv = np.array([op.band_vector(truth, b) for b in range(wf.nband)])
            assert np.abs(full - tv).max() <= TOL
            one = pr.single_band_projection(wf.nband - 1)
            assert np.abs(one - tv[-1]).max() <= TOL
            fulls[early] = full
        assert np.array_equal(fulls["1"], fulls["0"])
    finally:
        L.pawpy_gpu_set_host_projections(1)


def test_copied_and_in_place_coefficients_agree(workload_dirs, monkeypatch):
    """The coefficient upload by copies (hosts whose device cannot read pageable memory) and by
    in-place reads of the host arrays give the same overlaps bit for bit."""
    from pawpyseed_gb300.projector import Projector

    outs = []
    for copy in ("1", ""):
        if copy:
            monkeypatch.setenv("PAWPY_GPU_NO_HOST_READ", copy)
        else:
            monkeypatch.delenv("PAWPY_GPU_NO_HOST_READ", raising=False)
        basis, wf = load(workload_dirs("cfg1s"))
        outs.append(Projector(wf, basis).project_all())
    assert np.array_equal(outs[0], outs[1])


def test_results_deterministic_and_cached(workload_dirs):
    from pawpyseed_gb300.projector import Projector

    basis, wf = load(workload_dirs("cfg0"))
    pr = Projector(wf, basis)
    a = pr.project_all()
    b = pr.project_all()
    assert np.array_equal(a, b)
    x = pr.single_band_projection(3)
    y = pr.single_band_projection(3)
    assert np.array_equal(x, y)


def test_pseudo_method_and_reductions(workload_dirs, oracle_projectors):
    from pawpyseed_gb300.projector import Projector

    basis, wf = load(workload_dirs("cfg0"))
    pr = Projector(wf, basis, method="pseudo")
    op = oracle_projectors("cfg0")
    ps = op.pseudo_full()
    for b in (0, 7, 31):
        assert np.abs(pr.single_band_projection(b) - op.band_vector(ps, b)).max() <= TOL
    v, c = pr.proportion_conduction(4)
    assert abs(v + c - 1) < 1e-12
    res = pr.defect_band_analysis(4, 10, False)
    assert len(res) == 15
    with pytest.raises(ValueError):
        pr.single_band_projection(32)
    with pytest.raises(ValueError):
        pr.single_band_projection(-1)


def test_defect_band_analysis_aug_real(workload_dirs, oracle_projectors):
    """proportion_conduction on aug_real overlaps equals the FP64 reduction."""
    from pawpyseed_gb300.projector import Projector

    basis, wf = load(workload_dirs("cfg3s"))
    pr = Projector(wf, basis)
    op = oracle_projectors("cfg3s")
    truth = op.full()
    occs = basis._get_occs()
    nk = basis.nwk * basis.nspin
    for b in range(wf.nband):
        res = op.band_vector(truth, b)
        v = sum(abs(res[i]) ** 2 * wf.kws[i % basis.nwk] / basis.nspin for i in range(len(res)) if occs[i] > 0.5)
        mv, mc = pr.proportion_conduction(b)
        assert abs(mv - v) < 1e-6
    sp = pr.defect_band_analysis(analyze_all=True, spinpol=True)
    assert len(sp) == basis.nband and len(sp[0][0]) == 2


@pytest.mark.parametrize("name", ["cfg0", "cfg3s"])
def test_band_character_reduction_matches_per_band_reduction(name, workload_dirs):
    """The device reduction of every band's character equals proportion_conduction band by
    band (which reduces the host copy of single_band_projection), with and without spin
    channels."""
    from pawpyseed_gb300.projector import Projector

    basis, wf = load(workload_dirs(name))
    pr = Projector(wf, basis)
    v, c = pr.band_character()
    vs, cs = pr.band_character(spinpol=True)
    assert v.shape == (wf.nband,) and vs.shape == (wf.nband, basis.nspin)
    # the same reductions of the same matrix on the host (only the summation order differs)
    S2 = np.abs(pr.project_all()) ** 2
    nwk, nspin = basis.nwk, basis.nspin
    occ = np.asarray(basis._get_occs(), np.float64)
    kw = np.asarray(wf.kws, np.float64)[np.arange(S2.shape[1]) % nwk]
    full = occ > 0.5
    assert np.allclose(v, S2 @ np.where(full, kw / nspin, 0), rtol=1e-9, atol=1e-12)
    assert np.allclose(c, S2 @ np.where(full, 0, kw / nspin), rtol=1e-9, atol=1e-12)
    spin = (np.arange(S2.shape[1]) // nwk) % nspin
    for s_ in range(nspin):
        m = spin == s_
        assert np.allclose(vs[:, s_], S2[:, m] @ (occ * kw)[m], rtol=1e-9, atol=1e-12)
        assert np.allclose(cs[:, s_], S2[:, m] @ ((1 - occ) * kw)[m], rtol=1e-9, atol=1e-12)
    # and the per-band reduction of single_band_projection (pseudo overlap plus the FP64 PAW
    # terms per band) within the path's bar
    for b in range(wf.nband):
        mv, mc = pr.proportion_conduction(b)
        assert abs(v[b] - mv) <= TOL and abs(c[b] - mc) <= TOL
        sv, sc = pr.proportion_conduction(b, spinpol=True)
        assert np.abs(vs[b] - sv).max() <= TOL and np.abs(cs[b] - sc).max() <= TOL
    res = pr.defect_band_analysis(analyze_all=True)
    assert all(res[b] == (float(v[b]), float(c[b])) for b in range(wf.nband))


def test_self_projection_of_bands_is_identity_on_pseudo_part(workload_dirs):
    """Projecting a structure onto itself: pseudo overlaps of normalised bands have unit diagonal."""
    from pawpyseed_gb300.projector import Projector
    from pawpyseed_gb300.wavefunction import Wavefunction

    d = workload_dirs("cfg0")
    a = Wavefunction.from_directory(d["basis"])
    b = Wavefunction.from_directory(d["basis"])
    pr = Projector(a, b, method="pseudo")
    nk = a.nwk * a.nspin
    for band in (0, 9, 31):
        res = pr.single_band_projection(band)
        diag = res[band * nk:(band + 1) * nk]
        assert np.abs(diag - 1).max() < 2e-6


def test_errors_do_not_abort(workload_dirs):
    """Misuse reaches Python as an exception, never a process exit."""
    from pawpyseed_gb300 import _lib

    basis, wf = load(workload_dirs("cfg0"))
    L = _lib.lib()
    res = np.zeros(basis.nband * basis.nwk, np.complex128)
    L.pseudoprojection(res, basis.wf_ptr, wf.wf_ptr, 1000, 0)
    with pytest.raises(_lib.PAWpyGPUError):
        _lib.check()
    # compensation before overlap_setup_real on this pair
    L.compensation_terms(res, 0, wf.wf_ptr, basis.wf_ptr, 0, 0, 0, 0, None, None, None, None, None, None,
                         wf.nums, wf.coords, basis.nums, basis.coords, wf.dim, 0)
    with pytest.raises(_lib.PAWpyGPUError):
        _lib.check()


@pytest.mark.parametrize("name", list(CASES))
def test_register_fft_matches_shared_memory_fft(name, workload_dirs, monkeypatch):
    """The register line-FFT kernels and the generic shared-memory kernels give the same projections."""
    from pawpyseed_gb300.projector import Projector

    basis, wf = load(workload_dirs(name))
    fast = Projector(wf, basis).project_all()
    monkeypatch.setenv("PAWPY_GPU_FFT", "generic")
    basis2, wf2 = load(workload_dirs(name))
    slow = Projector(wf2, basis2).project_all()
    assert np.abs(fast - slow).max() <= 1e-6


def test_projector_list_cache_returns_independent_copies():
    """A repeated get_projector_list with identical inputs returns an equal deep copy."""
    from pawpyseed_gb300 import _lib, synth, vaspio
    from pawpyseed_gb300.wavefunction import pack_species

    cr = vaspio.CoreRegion(synth.potcar_text(["A", "B"]))
    L = _lib.lib()
    args = pack_species(cr)
    p1 = L.get_projector_list(len(cr.pps), *args, 300.0)
    _lib.check()
    p2 = L.get_projector_list(len(cr.pps), *args, 300.0)
    _lib.check()
    try:
        for e in range(len(cr.pps)):
            a, b = p1[e], p2[e]
            ng, nd, np_ = a.wave_gridsize, a.proj_gridsize, a.num_projs
            assert (ng, nd, np_) == (b.wave_gridsize, b.proj_gridsize, b.num_projs)
            assert C.addressof(a.funcs.contents) != C.addressof(b.funcs.contents)
            for k in range(np_):
                for name, n in (("kwave", ng), ("smooth_diffwave", nd), ("proj", nd)):
                    va = np.ctypeslib.as_array(getattr(a.funcs[k], name), shape=(n,))
                    vb = np.ctypeslib.as_array(getattr(b.funcs[k], name), shape=(n,))
                    assert np.array_equal(va, vb)
                    assert va.ctypes.data != vb.ctypes.data
            ma = np.ctypeslib.as_array(a.diff_overlap_matrix, shape=(np_ * np_,))
            mb = np.ctypeslib.as_array(b.diff_overlap_matrix, shape=(np_ * np_,))
            assert np.array_equal(ma, mb)
    finally:
        L.pawpy_gpu_free_ppot_list(p1, len(cr.pps))
        L.pawpy_gpu_free_ppot_list(p2, len(cr.pps))

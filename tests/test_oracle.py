"""The oracle (CPU FP64 restatement) pinned against the reference's golden vectors.

The golden fixtures were produced by the reference pawpyseed C core itself
(tests/golden/make_golden.py). Inputs are regenerated here from the same seeds;
when the regenerated bytes differ (fingerprint mismatch) a GoldenInputsDiffer
warning is raised and the comparisons run at tolerances that allow for it.
"""

import numpy as np
import pytest

import warnings

from conftest import CASES, GoldenInputsDiffer, fingerprint, same_golden_inputs


@pytest.mark.parametrize("name", list(CASES))
def test_oracle_matches_reference(name, workload_dirs, golden, oracle_projectors):
    g = golden(name)
    d = workload_dirs(name)
    same_inputs = same_golden_inputs(d, g, name)
    op = oracle_projectors(name)
    flips = [False, True] if "total_flip" in g.files else [False]
    for flip in flips:
        tag = "flip" if flip else "noflip"
        ref_total, ref_pseudo = g["total_" + tag], g["pseudo_" + tag]
        # pseudo overlaps accumulated in single precision, like the reference's cblas_cdotc_sub
        p32 = op.pseudo_full(flip, fp32=True)
        p32v = np.array([op.band_vector(p32, b) for b in range(op.wf.nband)])
        comp = op.comp_full(flip)
        compv = np.array([op.band_vector(comp, b) for b in range(op.wf.nband)])
        scale = np.abs(ref_total).max()
        if same_inputs:
            assert np.abs(p32v - ref_pseudo).max() <= 1e-6 * scale
            # PAW terms in FP64: agreement to rounding
            assert np.abs(compv - (ref_total - ref_pseudo)).max() <= 1e-12 * max(1.0, scale)
        else:
            assert np.abs(p32v + compv - ref_total).max() <= 1e-5


@pytest.mark.parametrize("name", list(CASES))
def test_oracle_projections_and_pairs(name, workload_dirs, golden, oracle_projectors):
    g = golden(name)
    d = workload_dirs(name)
    same = same_golden_inputs(d, g, name)
    # rounding level on identical inputs; a few float32 ulps of the coefficients otherwise
    tol = 1e-13 if same else 1e-6
    op = oracle_projectors(name)
    nbp = g["P_basis"].shape[1]
    for k in range(g["P_basis"].shape[0]):
        assert np.abs(op.basis.P[k][:nbp] - g["P_basis"][k]).max() <= tol
        assert np.abs(op.wf.P[k][:nbp] - g["P_defect"][k]).max() <= tol
    if "Q_flat" in g.files:
        off = 0
        for i, shp in enumerate(g["Q_shapes"]):
            n = int(shp[0] * shp[1])
            q = g["Q_flat"][off:off + n].reshape(shp)
            off += n
            assert np.abs(op.Q[i] - q).max() <= 1e-13
            assert np.abs(op.dcoords[i] - g["dcoords"][i]).max() <= 1e-14
    lists = [op.M_R, op.M_S, op.N_R, op.N_S, op.N_RS_R, op.N_RS_S]
    for key, mine in zip(["M_R", "M_S", "N_R", "N_S", "N_RS_R", "N_RS_S"], lists):
        assert list(g["list_" + key]) == list(mine)


def test_oracle_fft_known_answer(golden):
    """The reference's own fft_check case (core/tests/tests.c:28-80): Ga4, 20^3."""
    import oracle as orc

    g = golden("fft_ga4")
    x = np.zeros(2 * 8000)
    orc.lib().oracle_fft3d(x, np.ascontiguousarray(g["gs"].reshape(-1), dtype=np.int32),
                           np.ascontiguousarray(g["cs"].view(np.float32)), g["gs"].shape[0],
                           np.ascontiguousarray(g["fftg"], dtype=np.int32), float(abs(np.linalg.det(g["lattice"]))))
    xc = x[0::2] + 1j * x[1::2]
    assert np.abs(xc - g["direct"]).max() <= 1e-5  # the reference test's tolerance (tests.c:61)
    assert np.abs(xc - g["ref"]).max() <= 1e-12


def test_oracle_ylm_convention():
    """Complex Condon-Shortley Y_lm, as the reference's test_Ylm (test_core.py:68-90) pins."""
    import ctypes as C

    import oracle as orc
    from scipy.special import sph_harm_y

    L = orc.lib()
    rng = np.random.default_rng(0)
    for l in range(4):
        for m in range(-l, l + 1):
            for th, ph in rng.uniform([0, 0], [np.pi, 2 * np.pi], size=(20, 2)):
                re, im = C.c_double(), C.c_double()
                L.oracle_ylm(l, m, th, ph, C.byref(re), C.byref(im))
                ref = sph_harm_y(l, m, th, ph)
                assert abs(complex(re.value, im.value) - ref) < 1e-12


def test_oracle_wigner_table():
    """SBTFACS regenerated from Racah's formula: spot values from sympy-free identities."""
    import oracle as orc

    # w3j(l,l,0;0,0,0)^2 = 1/(2l+1); w3j(1,1,2;0,0,0) = sqrt(2/15)
    for l in range(4):
        assert abs(orc.wigner3j(l, l, 0, 0, 0, 0) ** 2 - 1 / (2 * l + 1)) < 1e-14
    assert abs(orc.wigner3j(1, 1, 2, 0, 0, 0) - np.sqrt(2 / 15)) < 1e-14
    t = orc.sbtfacs().reshape(4, 4, 4, 7, 4)
    assert abs(t[0, 0, 0, 0, 0] - 1 / np.sqrt(4 * np.pi)) < 1e-14


@pytest.fixture(scope="session")
def oracle_recip_projectors(workload_dirs, oracle_projectors):
    """The oracle's aug_recip projector per case (sharing the aug_real projector's wavefunctions)."""
    import oracle as orc

    cache = {}

    def get(name):
        if name not in cache:
            op = oracle_projectors(name)
            cache[name] = orc.OracleProjector(op.wf, op.basis, recip=True)
        return cache[name]

    return get


@pytest.mark.parametrize("name", list(CASES))
def test_oracle_recip_matches_reference(name, workload_dirs, golden, oracle_projectors, oracle_recip_projectors):
    """aug_recip (overlap_setup_recip + compensation_terms_recip) of the oracle against the reference:
    in the reference's arithmetic (complex64 CAs, single-precision dots) to rounding, and in FP64 equal
    to the aug_real overlaps (the reciprocal-space cross terms are the real-space O_R and O_S by
    Parseval on the grid)."""
    g = golden(name)
    d = workload_dirs(name)
    same = same_golden_inputs(d, g, name)
    op = oracle_recip_projectors(name)
    real = oracle_projectors(name)
    flips = [False, True] if "recip_total_flip" in g.files else [False]
    for flip in flips:
        ref = g["recip_total_" + ("flip" if flip else "noflip")]
        f32 = op.full(flip, fp32=True)
        v32 = np.array([op.band_vector(f32, b) for b in range(op.wf.nband)])
        assert np.abs(v32 - ref).max() <= (1e-12 if same else 1e-5)
        f64 = op.full(flip)
        r64 = real.full(flip)
        assert np.abs(f64 - r64).max() <= 1e-12
    # the augmentation coefficients themselves (band 0, the fixture's first 4096 plane waves)
    for key in g.files:
        if not key.startswith("recip_CA_"):
            continue
        side, k = key[len("recip_CA_"):].split("_k")
        CA = op.CA_R if side == "basis" else op.CA_S
        ref = g[key]
        mine = CA[int(k)][0][: ref.shape[0]]
        assert np.abs(mine - ref).max() <= (1e-6 if same else 1e-5) * np.abs(ref).max()


def test_oracle_realspace_matches_reference(realspace_dirs, golden):
    """realspace_state, ae_chg_density and project_realspace_state (density.c:27-310) of the
    oracle against the reference on the same inputs, to rounding."""
    import oracle as orc

    g = golden("realspace_cfg0")
    same = same_golden_inputs(realspace_dirs, g, "realspace_cfg0")
    tol = 1e-12 if same else 1e-5
    w = orc.OracleWavefunction(realspace_dirs["defect"])
    b = orc.OracleWavefunction(realspace_dirs["basis"])
    w.setup_projectors()
    b.setup_projectors()
    N = g["fftg"]
    x = w.realspace_state(1, 1, N)
    assert np.abs(x - g["state_b1_k1"]).max() <= tol
    rho = w.ae_chg_density(N)
    assert np.abs(rho - g["rho"]).max() <= tol
    nk = w.nk
    vol = abs(np.linalg.det(w.lattice))
    n3 = int(np.prod(N))
    proj = np.zeros_like(g["proj"])
    for k in range(nk):
        S = np.array([w.realspace_state(bb, k, N).ravel() for bb in range(w.nband)])
        R = np.array([b.realspace_state(bb, k, N).ravel() for bb in range(b.nband)])
        proj[:, k::nk] = S @ R.conj().T * vol / n3
    assert np.abs(proj - g["proj"]).max() <= tol


def test_oracle_ncl_matches_reference(tmp_path, golden):
    """The spinor projections (onto_projector_ncl, projector.c:359-392), ncl_realspace_state and
    ncl_ae_chg_density (density.c:181-204, 328-408) of the reference on a spinor wavefunction
    against the oracle's collinear functions on each spinor half: up_projections and
    down_projections are the halves' projections, the up and down components of the state are
    the halves' states (each with its own projections), and the density, which carries no spin
    factor, is half the sum of the halves' collinear densities (factor 2 / nspin = 2). This is the
    restatement the noncollinear device functions are checked against."""
    import oracle as orc

    from pawpyseed_gb300 import synth, vaspio

    g = golden("realspace_ncl_cfg0")
    w = synth.small_workload(0, nband=4, nk=2)
    bs, _ = synth.structures(0)
    data = synth.wavefunction_data(bs, w, 77, ncl=True)
    synth.write_structure_dir(str(tmp_path), bs, data, w["dim"], symbols=["A"])
    same = fingerprint(str(tmp_path)) == str(g["fp"])
    if not same:
        warnings.warn(GoldenInputsDiffer("realspace_ncl_cfg0: regenerated inputs differ in bytes from the "
                                         "golden fixture's; comparing at the FP64-truth tolerance instead"))
    tol = 1e-12 if same else 1e-5
    cr = vaspio.CoreRegion(synth.potcar_text(["A"]))
    N = g["fftg"]
    halves = []
    for h in (0, 1):
        half = dict(data, ncl=False)
        half["coeffs"] = [np.ascontiguousarray(c[:, h * gs.shape[0]:(h + 1) * gs.shape[0]])
                          for c, gs in zip(data["coeffs"], data["gs"])]
        ow = orc.OracleWavefunction(data=half, struct=bs, cr=cr, dim=w["dim"])
        ow.setup_projectors()
        halves.append(ow)
    for h, side in ((0, "P_up"), (1, "P_down")):
        for k in range(halves[h].nk):
            assert np.abs(halves[h].P[k] - g[side][k]).max() <= (1e-13 if same else 1e-6)
        x = halves[h].realspace_state(3, 1, N)
        assert np.abs(x - g["state_b3_k1"][h]).max() <= tol
    rho = 0.5 * (halves[0].ae_chg_density(N) + halves[1].ae_chg_density(N))
    assert np.abs(rho - g["rho"]).max() <= tol

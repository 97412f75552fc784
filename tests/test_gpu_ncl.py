"""Noncollinear projections and overlaps. setup_projections on a spinor wavefunction fills
every band's up_projections and down_projections (onto_projector_ncl,
projector.c:359-392) — the two halves share the G list. Checked against the
FP64 oracle run on each half as a collinear wavefunction; tolerance 1e-5
relative to the largest coefficient (as the collinear projector test). The
spinor overlaps (an extension: the reference refuses them) are checked against
the sum of the oracle's overlaps of the two halves."""

import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))


def ncl_case(nband=4, nk=2):
    from pawpyseed_gb300 import synth, vaspio

    w = synth.small_workload(0, nband=nband, nk=nk)
    bs, _ = synth.structures(0)
    cr = vaspio.CoreRegion(synth.potcar_text(["A"]))
    data = synth.wavefunction_data(bs, w, 77, ncl=True)
    return bs, cr, w, data


def half(data, h):
    out = dict(data, ncl=False)
    out["coeffs"] = [np.ascontiguousarray(c[:, h * g.shape[0]:(h + 1) * g.shape[0]]) for c, g in
                     zip(data["coeffs"], data["gs"])]
    return out


def test_ncl_projections_match_oracle_on_each_half():
    import oracle as orc
    from pawpyseed_gb300.wavefunction import NCLWavefunction

    bs, cr, w, data = ncl_case()
    wf = NCLWavefunction.from_arrays(bs, cr, w["dim"], data)
    wf.check_c_projectors()
    for h in (0, 1):
        ow = orc.OracleWavefunction(data=half(data, h), struct=bs, cr=cr, dim=w["dim"])
        ow.setup_projectors()
        for k in range(ow.nk):
            ref = ow.P[k]
            scale = np.abs(ref).max()
            for b in range(ow.nband):
                mine = wf.spinor_projections(b, k)[h]
                assert np.abs(mine - ref[b]).max() <= 1e-5 * scale


def ncl_pair(nband=4, nk=2):
    """A noncollinear basis and defect of the 8-atom cell (atom 0 moved 0.1 A)."""
    from pawpyseed_gb300 import synth, vaspio

    w = synth.small_workload(0, nband=nband, nk=nk)
    bs, ds = synth.structures(0)
    cr = vaspio.CoreRegion(synth.potcar_text(["A"]))
    return bs, ds, cr, w, synth.wavefunction_data(bs, w, 78, ncl=True), synth.wavefunction_data(ds, w, 79, ncl=True)


@pytest.mark.parametrize("precision", ["bf16x3", "fp32"])
def test_ncl_overlaps_match_fp64_sum_over_spinor_halves(precision):
    """Spinor overlaps <psi_R|psi_S> = sum over the up and down components of the PAW overlap of
    each component (pseudo overlap + O_M + O_R + O_S + O_N). The reference defines no overlap of
    noncollinear wavefunctions (projector.py:74-75), so the truth is the FP64 oracle's collinear
    overlaps of each half, summed; tolerance 1e-5. The per-band entry points (pseudoprojection +
    compensation_terms) must give the batched matrix's rows."""
    import oracle as orc

    from pawpyseed_gb300 import _lib
    from pawpyseed_gb300.projector import Projector
    from pawpyseed_gb300.wavefunction import NCLWavefunction

    bs, ds, cr, w, bd, dd = ncl_pair()
    basis = NCLWavefunction.from_arrays(bs, cr, w["dim"], bd)
    wf = NCLWavefunction.from_arrays(ds, cr, w["dim"], dd)
    prec0 = _lib.get_precision()
    _lib.set_precision(precision)
    try:
        pr = Projector(wf, basis, noncollinear=True)
        full = pr.project_all()
        rows = np.array([pr.single_band_projection(b) for b in range(wf.nband)])
    finally:
        _lib.set_precision(prec0)
    truth = 0
    for h in (0, 1):
        ob = orc.OracleWavefunction(data=half(bd, h), struct=bs, cr=cr, dim=w["dim"])
        ow = orc.OracleWavefunction(data=half(dd, h), struct=ds, cr=cr, dim=w["dim"])
        op = orc.OracleProjector(ow, ob)
        truth = truth + np.array([op.band_vector(op.full(), b) for b in range(ow.nband)])
    assert full.shape == truth.shape == (wf.nband, basis.nband * basis.nwk * basis.nspin)
    assert np.abs(full - truth).max() <= 1e-5
    assert np.abs(rows - full).max() <= 1e-6


def test_mixed_collinear_noncollinear_overlaps_are_refused():
    from pawpyseed_gb300 import _lib, synth
    from pawpyseed_gb300.wavefunction import NCLWavefunction, Wavefunction

    bs, cr, w, data = ncl_case(nband=2, nk=1)
    a = NCLWavefunction.from_arrays(bs, cr, w["dim"], data)
    b = Wavefunction.from_arrays(bs, cr, w["dim"], synth.wavefunction_data(bs, w, 5))
    a.check_c_projectors()
    b.check_c_projectors()
    res = np.zeros(b.nband * b.nwk * b.nspin, np.complex128)
    _lib.lib().pseudoprojection(res, b.wf_ptr, a.wf_ptr, 0, 0)
    with pytest.raises(_lib.PAWpyGPUError, match="noncollinear"):
        _lib.check()


def test_ncl_realspace_state_and_density_match_oracle_on_each_half():
    """ncl_realspace_state (density.c:328-408): the up and down components are the collinear
    real-space states of the two halves with their own projections; ncl_ae_chg_density
    (density.c:181-204) sums |up|^2 + |down|^2 x weight x occupation (no spin factor), so it is
    half the sum of the two halves' collinear densities (whose factor is 2 / nspin = 2).
    Tolerance 1e-5 of the largest magnitude, as the collinear real-space test."""
    import oracle as orc

    from pawpyseed_gb300.wavefunction import NCLWavefunction

    bs, cr, w, data = ncl_case()
    wf = NCLWavefunction.from_arrays(bs, cr, w["dim"], data)
    wf.check_c_projectors()
    N = np.asarray(w["dim"], dtype=np.int32)
    halves = []
    for h in (0, 1):
        ow = orc.OracleWavefunction(data=half(data, h), struct=bs, cr=cr, dim=w["dim"])
        ow.setup_projectors()
        halves.append(ow)
    for b, k in ((0, 0), (3, 1)):
        up, down = wf.get_state_realspace(b, k, 0, dim=N)
        for mine, ow in ((up, halves[0]), (down, halves[1])):
            truth = ow.realspace_state(b, k, N)
            assert np.abs(mine - truth).max() <= 1e-5 * np.abs(truth).max()
    rho = wf.get_realspace_density(dim=N)
    rtruth = 0.5 * (halves[0].ae_chg_density(N) + halves[1].ae_chg_density(N))
    assert np.abs(rho - rtruth).max() <= 1e-5 * np.abs(rtruth).max()


def test_collinear_realspace_functions_refuse_noncollinear_wavefunctions():
    from pawpyseed_gb300 import _lib
    from pawpyseed_gb300.wavefunction import NCLWavefunction, Wavefunction

    bs, cr, w, data = ncl_case()
    wf = NCLWavefunction.from_arrays(bs, cr, w["dim"], data)
    wf.check_c_projectors()
    with pytest.raises(_lib.PAWpyGPUError):
        Wavefunction.get_state_realspace(wf, 0, 0, 0)

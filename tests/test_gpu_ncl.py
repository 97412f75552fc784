"""Noncollinear projections: setup_projections on a spinor wavefunction fills
every band's up_projections and down_projections (onto_projector_ncl,
projector.c:359-392) — the two halves share the G list. Checked against the
FP64 oracle run on each half as a collinear wavefunction; tolerance 1e-5
relative to the largest coefficient (as the collinear projector test)."""

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


def test_ncl_overlaps_are_refused():
    from pawpyseed_gb300 import _lib
    from pawpyseed_gb300.wavefunction import NCLWavefunction

    bs, cr, w, data = ncl_case(nband=2, nk=1)
    a = NCLWavefunction.from_arrays(bs, cr, w["dim"], data)
    b = NCLWavefunction.from_arrays(bs, cr, w["dim"], data)
    a.check_c_projectors()
    b.check_c_projectors()
    res = np.zeros(b.nband * b.nwk * b.nspin, np.complex128)
    _lib.lib().pseudoprojection(res, b.wf_ptr, a.wf_ptr, 0, 0)
    with pytest.raises(_lib.PAWpyGPUError):
        _lib.check()

"""The aug_recip method on the device (overlap_setup_recip, compensation_terms_recip and the
batched contraction) against the oracle's FP64 evaluation, the reference's golden vectors, the
reference's augmentation coefficients band->CAs, and the aug_real method on the same inputs.

Tolerances: overlaps within 1e-5 of FP64 (the accuracy target of the band-pair metric); the
augmentation coefficients (single-precision spread and transforms) within 1e-5 of their largest
magnitude; the batched matrix equal to the per-band entry points within 1e-6.
"""

import numpy as np
import pytest

from conftest import CASES, same_golden_inputs

pytestmark = pytest.mark.gpu

TOL = 1e-5


def load(dirs):
    from pawpyseed_gb300.wavefunction import Wavefunction

    return Wavefunction.from_directory(dirs["basis"]), Wavefunction.from_directory(dirs["defect"])


def host_aug_coefficients(wf, k, b):
    """band->CAs of band b at k-point k (complex64, file plane-wave order), or None."""
    kp = wf.wf_ptr.contents.kpts[k].contents
    bd = kp.bands[b].contents
    if not bd.CAs:
        return None
    import ctypes as C

    v = np.ctypeslib.as_array(C.cast(bd.CAs, C.POINTER(C.c_float)), shape=(2 * kp.num_waves,))
    return (v[0::2] + 1j * v[1::2]).astype(np.complex64)


@pytest.mark.parametrize("name", list(CASES))
def test_recip_projections_match_fp64_and_reference(name, workload_dirs, golden, oracle_projectors):
    import oracle as orc

    from pawpyseed_gb300.projector import Projector

    dirs = workload_dirs(name)
    g = golden(name)
    same = same_golden_inputs(dirs, g, name)
    basis, wf = load(dirs)
    pr = Projector(wf, basis, method="aug_recip")
    real = oracle_projectors(name)
    op = orc.OracleProjector(real.wf, real.basis, recip=True)
    flips = [False, True] if "recip_total_flip" in g.files else [False]
    per_band = {}
    for flip in flips:
        truth = op.full(flip)
        tv = np.array([op.band_vector(truth, b) for b in range(wf.nband)])
        mine = np.array([pr.single_band_projection(b, flip_spin=flip) for b in range(wf.nband)])
        assert np.abs(mine - tv).max() <= TOL
        if same:
            assert np.abs(mine - g["recip_total_" + ("flip" if flip else "noflip")]).max() <= TOL
        # the batched contraction over the same terms
        allb = pr.project_all(flip)
        assert np.abs(allb - mine).max() <= 1e-6
        per_band[flip] = mine
    # augmentation coefficients the setup left on the host, against the oracle and the reference
    nk = basis.nwk * basis.nspin
    for side, w, CA in (("basis", basis, op.CA_R), ("defect", wf, op.CA_S)):
        for k in range(nk):
            mine = host_aug_coefficients(w, k, 0)
            ref = g["recip_CA_%s_k%d" % (side, k)] if "recip_CA_%s_k%d" % (side, k) in g.files else None
            if ref is None:
                assert mine is None or not np.any(mine)
                continue
            assert mine is not None
            scale = np.abs(CA[k][0]).max()
            assert np.abs(mine - CA[k][0]).max() <= TOL * scale
            if same:
                assert np.abs(mine[: ref.shape[0]] - ref).max() <= TOL * scale
    # aug_real on the same pair (a new overlap setup) gives the same overlaps
    prr = Projector(wf, basis, method="aug_real")
    for flip in flips:
        mine_real = np.array([prr.single_band_projection(b, flip_spin=flip) for b in range(wf.nband)])
        assert np.abs(mine_real - per_band[flip]).max() <= TOL


def test_recip_and_real_setups_refuse_the_other_terms(workload_dirs):
    """compensation_terms after overlap_setup_recip (and the recip terms after overlap_setup_real)
    report an error instead of mixing the methods."""
    from pawpyseed_gb300 import _lib
    from pawpyseed_gb300.projector import Projector

    basis, wf = load(workload_dirs("cfg0"))
    pr = Projector(wf, basis, method="aug_recip")
    pr.method = "aug_real"
    with pytest.raises(_lib.PAWpyGPUError, match="overlap_setup_real"):
        pr.single_band_projection(0)
    pr2 = Projector(wf, basis, method="aug_real")
    pr2.method = "aug_recip"
    with pytest.raises(_lib.PAWpyGPUError, match="overlap_setup_recip"):
        pr2.single_band_projection(0)

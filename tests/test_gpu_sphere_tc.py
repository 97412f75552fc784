"""The sphere contraction on the tensor cores (split-BF16, csrc/sphere_tc.cu) against the FP32
CUDA-core form and the oracle's FP64 projections.

Every operand source is covered: picked-point rows (the default), the band grids a projection
pass writes for the gathered form (PAWPY_GPU_DEFECT_GRID=1), and the resident real-space grid of a
prepared basis (pawpy_gpu_prepare_basis with real-space storage). Tolerances: projector
coefficients within 1e-5 of the largest coefficient against FP64 (as the collinear projector
test), the two forms within 2e-6 of it of each other, and the overlaps within 1e-5 of FP64 (the
band-pair metric's target).
"""

import os
import sys

import numpy as np
import pytest

from conftest import CASES

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))

TOL = 1e-5


def _projections(wf):
    from test_gpu_parity import host_projections

    nk = wf.nwk * wf.nspin
    return np.array([[host_projections(wf, k, b) for b in range(wf.nband)] for k in range(nk)])


def _with_mode(mode, fn):
    from pawpyseed_gb300 import _lib

    L = _lib.lib()
    L.pawpy_gpu_set_sphere_contraction(mode)
    try:
        return fn()
    finally:
        L.pawpy_gpu_set_sphere_contraction(1)


@pytest.mark.parametrize("defect_grid", ["0", "1"])
@pytest.mark.parametrize("name", list(CASES))
def test_tensor_core_projections_match_fp64_and_cuda_cores(name, defect_grid, workload_dirs, oracle_projectors,
                                                           monkeypatch):
    monkeypatch.setenv("PAWPY_GPU_DEFECT_GRID", defect_grid)
    from pawpyseed_gb300.wavefunction import Wavefunction

    dirs = workload_dirs(name)
    op = oracle_projectors(name)

    def proj():
        w = Wavefunction.from_directory(dirs["defect"])
        w.check_c_projectors()
        return _projections(w)

    tc = _with_mode(2, proj)
    cc = _with_mode(0, proj)
    ref = np.array(op.wf.P)
    scale = np.abs(ref).max()
    assert np.abs(tc - ref).max() <= TOL * scale
    assert np.abs(tc - cc).max() <= 2e-6 * scale


@pytest.mark.parametrize("name", ["cfg0", "cfg2s", "cfg3s"])
@pytest.mark.parametrize("resident", [False, True])
@pytest.mark.parametrize("defect_grid", ["0", "1"])
def test_tensor_core_overlaps_match_fp64(name, resident, defect_grid, workload_dirs, oracle_projectors, monkeypatch):
    """project_all with every sphere contraction on the tensor cores (pseudo overlap in FP32): the
    smoothed-wave projections of both structures, the defect's from picked rows or from the grids of
    its projection pass, the basis's likewise or from its resident real-space grid."""
    monkeypatch.setenv("PAWPY_GPU_DEFECT_GRID", defect_grid)
    from pawpyseed_gb300 import _lib
    from pawpyseed_gb300.projector import Projector
    from pawpyseed_gb300.wavefunction import Wavefunction

    dirs = workload_dirs(name)
    op = oracle_projectors(name)
    t = op.full()
    tv = np.array([op.band_vector(t, b) for b in range(op.wf.nband)])

    def run():
        basis = Wavefunction.from_directory(dirs["basis"])
        wf = Wavefunction.from_directory(dirs["defect"])
        basis.check_c_projectors()
        if resident:
            assert _lib.lib().pawpy_gpu_prepare_basis(basis.wf_ptr, 1) >= 0
            _lib.check()
        return Projector(wf, basis).project_all()

    tc = _with_mode(2, run)
    cc = _with_mode(0, run)
    assert np.abs(tc - tv).max() <= TOL
    assert np.abs(tc - cc).max() <= 2e-6


@pytest.mark.parametrize("defect_grid", ["0", "1"])
def test_tensor_core_spinor_projections(defect_grid, monkeypatch):
    """Spinor halves as rows of the contraction: both halves against the oracle."""
    monkeypatch.setenv("PAWPY_GPU_DEFECT_GRID", defect_grid)
    import oracle as orc
    from test_gpu_ncl import half, ncl_case

    from pawpyseed_gb300.wavefunction import NCLWavefunction

    bs, cr, w, data = ncl_case()

    def run():
        wf = NCLWavefunction.from_arrays(bs, cr, w["dim"], data)
        wf.check_c_projectors()
        return [[wf.spinor_projections(b, k) for b in range(wf.nband)] for k in range(wf.nwk * wf.nspin)]

    got = _with_mode(2, run)
    for h in (0, 1):
        ow = orc.OracleWavefunction(data=half(data, h), struct=bs, cr=cr, dim=w["dim"])
        ow.setup_projectors()
        for k in range(ow.nk):
            ref = ow.P[k]
            scale = np.abs(ref).max()
            for b in range(ow.nband):
                assert np.abs(got[k][b][h] - ref[b]).max() <= TOL * scale


@pytest.mark.parametrize("name", ["cfg0", "cfg2s"])
def test_tensor_core_second_pass_matches_fp64(name, workload_dirs, oracle_projectors, monkeypatch):
    """The second FFT pass on the tensor cores (PAWPY_GPU_XPICK_TC=1: the transform along the first
    axis as a split-BF16 DFT product, fused with the pick; Gamma k-points, split rows): projections
    within 1e-5 of the largest coefficient against FP64, within 5e-6 of it of the register-FFT
    form, and the overlaps of the whole projection within 1e-5 of FP64."""
    from pawpyseed_gb300.projector import Projector
    from pawpyseed_gb300.wavefunction import Wavefunction

    dirs = workload_dirs(name)
    op = oracle_projectors(name)

    def proj():
        w = Wavefunction.from_directory(dirs["defect"])
        w.check_c_projectors()
        return _projections(w)

    def overlaps():
        basis = Wavefunction.from_directory(dirs["basis"])
        wf = Wavefunction.from_directory(dirs["defect"])
        basis.check_c_projectors()
        return Projector(wf, basis).project_all()

    monkeypatch.setenv("PAWPY_GPU_XPICK_TC", "1")
    tcx = _with_mode(2, proj)
    full = _with_mode(2, overlaps)
    monkeypatch.setenv("PAWPY_GPU_XPICK_TC", "0")
    reg = _with_mode(2, proj)
    ref = np.array(op.wf.P)
    scale = np.abs(ref).max()
    assert np.abs(tcx - ref).max() <= TOL * scale
    assert np.abs(tcx - reg).max() <= 5e-6 * scale
    t = op.full()
    tv = np.array([op.band_vector(t, b) for b in range(op.wf.nband)])
    assert np.abs(full - tv).max() <= TOL

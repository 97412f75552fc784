"""PAW-corrected overlaps at the full sizes the benchmark times, against FP64.

The 64-atom workload (256 bands x 8 k-points, 60^3) and the 216-atom workload
(1024 bands, Gamma, 90^3, 206 sites in N_R and N_S, 394 N_RS pairs) run
through the C ABI exactly as the benchmark step does (host projections off, so
the first FFT pass is issued early; the resident basis held in real space).
This reaches the paths that only full sizes take: multi-tile tensor-core
contractions on real coefficients, contraction launches of thousands of
(k-point, band) rows, whole-k-point FFT sub-batches, the 90^3 register FFT.
A seeded sample of defect and basis bands at every k-point is compared with
the oracle's FP64 evaluation of the same inputs (pseudo overlap in double
precision plus the PAW terms), within the metric's 1e-5; the per-band drop-in
entry points (pseudoprojection + compensation_terms) must agree with the
batched matrix on sampled bands.
"""

import os
import sys

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _bench():
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    import bench

    return bench


@pytest.mark.parametrize("cfg", [1, 2])
def test_full_size_overlaps_match_fp64(cfg):
    import torch

    from pawpyseed_gb300 import _lib
    from pawpyseed_gb300.wavefunction import Wavefunction, pack_species

    bench = _bench()
    torch.cuda.set_device(0)
    work = bench.make_workload(cfg, None, None)
    w, basis_s, defect_s, cr, bd, dd = work
    lists = bench.site_lists(basis_s, defect_s, cr)
    work = work + (lists,)
    L = _lib.lib()
    prec0 = _lib.get_precision()
    _lib.set_precision("bf16x3")
    L.pawpy_gpu_set_host_projections(0)
    try:
        basis = Wavefunction.from_arrays(basis_s, cr, w["dim"], bd)
        wf = Wavefunction.from_arrays(defect_s, cr, w["dim"], dd)
        basis.check_c_projectors()
        assert L.pawpy_gpu_prepare_basis(basis.wf_ptr, 1) >= 0
        _lib.check()
        M_R, M_S, N_R, N_S, NRS_R, NRS_S = lists
        P = _lib.ptr
        nk = wf.nwk * wf.nspin
        pps = L.get_projector_list(len(cr.pps), *pack_species(cr), wf.grid_encut())
        dimv = np.ascontiguousarray(wf.dim, dtype=np.int32)
        L.setup_projections(wf.wf_ptr, pps, len(cr.pps), len(defect_s), dimv, wf.nums, wf.coords)
        L.overlap_setup_real(basis.wf_ptr, wf.wf_ptr, basis.nums, wf.nums, basis.coords, wf.coords,
                             P(N_R), P(N_S), P(NRS_R), P(NRS_S), len(N_R), len(N_S), len(NRS_R))
        out = np.zeros((wf.nband, basis.nband * nk), np.complex128)
        L.pawpy_gpu_project_all(out.reshape(-1), basis.wf_ptr, wf.wf_ptr, len(M_R), len(N_R), len(N_S),
                                len(NRS_R), P(M_R), P(M_S), P(N_R), P(N_S), P(NRS_R), P(NRS_S), 0)
        _lib.check()
        assert np.all(np.isfinite(out))
        # the per-band drop-in path on two sampled bands equals the batched rows
        for b in (0, wf.nband - 1):
            res = np.zeros(basis.nband * nk, np.complex128)
            L.pseudoprojection(res, basis.wf_ptr, wf.wf_ptr, b, 0)
            L.compensation_terms(res, b, wf.wf_ptr, basis.wf_ptr, len(M_R), len(N_R), len(N_S), len(NRS_R),
                                 P(M_R), P(M_S), P(N_R), P(N_S), P(NRS_R), P(NRS_S), wf.nums, wf.coords,
                                 basis.nums, basis.coords, dimv, 0)
            _lib.check()
            assert np.abs(res - out[b]).max() <= 1e-6
    finally:
        # process-wide switches back to their defaults for the tests that follow
        L.pawpy_gpu_set_host_projections(1)
        _lib.set_precision(prec0)
    smp = bench.OracleSample(work, 8, 32, seed=11 + cfg)
    smp.run()
    acc = bench.accuracy(smp, out, nk)
    print("workload %d: %s" % (cfg, acc))
    assert acc["max_abs_err_vs_fp64"] <= TOL
    L.pawpy_gpu_release(wf.wf_ptr)
    L.pawpy_gpu_release(basis.wf_ptr)

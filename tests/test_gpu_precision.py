"""Precision forms of the overlap contraction on the GPU.

Tolerances, for rows of unit norm (as the bands are):
  FP32 (CUDA cores) and split-BF16 3-term (tensor cores, FP32 accumulation):
      |S - S_FP64| <= 1e-5 for every overlap;
  TF32 (tensor cores): a reported variant, |S - S_FP64| <= 5e-3.
"""

import numpy as np
import pytest

from conftest import CASES

pytestmark = pytest.mark.gpu

TOL = {"fp32": 1e-5, "bf16x3": 1e-5, "tf32": 5e-3}


def unit_rows(rng, n, k, scale_tail=False):
    x = rng.standard_normal((n, k)) + 1j * rng.standard_normal((n, k))
    if scale_tail:  # plane-wave-like decay along K
        x *= np.exp(-np.linspace(0, 4, k))[None, :]
    x /= np.linalg.norm(x, axis=1, keepdims=True)
    return x.astype(np.complex64)


def truth(As, Bs):
    return np.stack([b.astype(np.complex128) @ np.conj(a.astype(np.complex128)).T for a, b in zip(As, Bs)])


SHAPES = [
    (200, 300, [1000, 777, 1500]),  # partial tiles in M and N, uneven K per batch
    (32, 32, [1900]),
    (129, 257, [64]),               # one row / column past a tile, two K blocks
    (256, 512, [4096, 4000]),       # whole tiles
]


@pytest.mark.parametrize("prec", ["fp32", "bf16x3", "tf32"])
@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: "%dx%dx%d" % (s[0], s[1], len(s[2])))
def test_overlap_matrix_against_fp64(prec, shape):
    from pawpyseed_gb300 import _lib

    M, N, Ks = shape
    rng = np.random.default_rng(M * 7 + N)
    As = [unit_rows(rng, M, k, True) for k in Ks]
    Bs = [unit_rows(rng, N, k, True) for k in Ks]
    ref = truth(As, Bs)
    out = _lib.overlap_matrix(As, Bs, prec)
    err = np.abs(out - ref).max()
    assert err <= TOL[prec], (prec, shape, err)
    if prec == "bf16x3":
        # the dropped lo*lo products and FP32 accumulation stay below 2^-16 sum|a||b|
        bound = 2.0 ** -16 * max((np.abs(b) @ np.abs(a).T).max() for a, b in zip(As, Bs))
        assert err <= bound, (err, bound)
        assert np.abs(out).max() > 0.05


def test_tensor_core_split_k_independent_of_split_count():
    from pawpyseed_gb300 import _lib

    rng = np.random.default_rng(5)
    As = [unit_rows(rng, 160, 6000), unit_rows(rng, 160, 5000)]
    Bs = [unit_rows(rng, 300, 6000), unit_rows(rng, 300, 5000)]
    ref = truth(As, Bs)
    L = _lib.lib()
    res = {}
    try:
        for s in (1, 3, 7, 40):
            L.pawpy_gpu_set_tc_splits(s)
            a = _lib.overlap_matrix(As, Bs, "bf16x3")
            b = _lib.overlap_matrix(As, Bs, "bf16x3")
            assert np.array_equal(a, b)  # fixed reduction order: bitwise repeatable
            assert np.abs(a - ref).max() < 5e-6
            res[s] = a
    finally:
        L.pawpy_gpu_set_tc_splits(0)
    for s in (3, 7, 40):
        assert np.abs(res[s] - res[1]).max() < 2e-6


@pytest.mark.parametrize("splits", [1, 0])
def test_coherent_sums_stay_within_target(splits):
    """Overlaps near 1 (a band with itself) accumulate a long coherent sum: the
    tensor core's truncated accumulation must not bias them beyond 1e-5."""
    from pawpyseed_gb300 import _lib

    rng = np.random.default_rng(11)
    a = unit_rows(rng, 128, 24000)
    ref = a.astype(np.complex128) @ np.conj(a.astype(np.complex128)).T
    L = _lib.lib()
    try:
        L.pawpy_gpu_set_tc_splits(splits)
        out = _lib.overlap_matrix([a], [a], "bf16x3")[0]
    finally:
        L.pawpy_gpu_set_tc_splits(0)
    assert np.abs(np.diag(out) - np.diag(ref)).max() <= 5e-6
    assert np.abs(out - ref).max() <= 5e-6


def test_split_bf16_keeps_the_cross_terms():
    """Inputs that bf16 alone cannot represent: hi*lo terms carry the answer."""
    from pawpyseed_gb300 import _lib

    k = 512
    a = np.full((128, k), 1.0 + 2.0 ** -12, np.float32).astype(np.complex64)
    b = np.full((256, k), 1.0 + 2.0 ** -11, np.float32) * (1 + 1j)
    b = b.astype(np.complex64)
    out = _lib.overlap_matrix([a], [b], "bf16x3")[0]
    ref = (b.astype(np.complex128) @ np.conj(a.astype(np.complex128)).T)
    assert np.abs(out - ref).max() <= 1e-6 * np.abs(ref).max()
    plain = (1.0 * k) * (1 + 1j)
    assert np.abs(out - plain).max() > 100 * np.abs(out - ref).max()


@pytest.mark.parametrize("name", list(CASES))
def test_projections_in_each_precision(name, workload_dirs, oracle_projectors):
    """project_all (pseudo overlap + PAW terms) per precision against the FP64 truth."""
    from pawpyseed_gb300 import _lib
    from pawpyseed_gb300.projector import Projector
    from pawpyseed_gb300.wavefunction import Wavefunction

    dirs = workload_dirs(name)
    basis = Wavefunction.from_directory(dirs["basis"])
    wf = Wavefunction.from_directory(dirs["defect"])
    op = oracle_projectors(name)
    t = op.full()
    tv = np.array([op.band_vector(t, b) for b in range(wf.nband)])
    try:
        for prec in ("bf16x3", "tf32", "fp32"):
            _lib.set_precision(prec)
            pr = Projector(wf, basis)
            full = pr.project_all()
            err = np.abs(full - tv).max()
            assert err <= TOL[prec], (name, prec, err)
            if prec == "bf16x3":
                again = pr.project_all()
                assert np.array_equal(full, again)
                one = pr.single_band_projection(wf.nband - 1)
                assert np.abs(one - tv[-1]).max() <= TOL[prec]
    finally:
        _lib.set_precision("fp32")


@pytest.mark.parametrize("tile", [64, 128, 0])
@pytest.mark.parametrize("prec", ["bf16x3", "tf32"])
@pytest.mark.parametrize("shape", SHAPES + [(300, 40, [5000, 4100]), (16, 100, [2048])],
                         ids=lambda s: "%dx%dx%d" % (s[0], s[1], len(s[2])))
def test_tensor_core_tile_widths(tile, prec, shape):
    """Both tile widths of the tensor-core contraction (64 and 128 defect bands per tile, the
    64-band tiles two CTAs per SM) and the tuner's choice (0) against FP64, on partial tiles and
    uneven K; the tuner times every candidate once per shape, each computing the full result."""
    from pawpyseed_gb300 import _lib

    M, N, Ks = shape
    rng = np.random.default_rng(M * 31 + N + 7 * tile)
    As = [unit_rows(rng, M, k, scale_tail=True) for k in Ks]
    Bs = [unit_rows(rng, N, k, scale_tail=True) for k in Ks]
    L = _lib.lib()
    L.pawpy_gpu_set_tc_tile(tile)
    try:
        s = _lib.overlap_matrix(As, Bs, prec)
        s2 = _lib.overlap_matrix(As, Bs, prec)  # the tuned or cached choice again
    finally:
        L.pawpy_gpu_set_tc_tile(0)
    t = truth(As, Bs)
    assert np.abs(s - t).max() <= TOL[prec]
    assert np.abs(s2 - t).max() <= TOL[prec]

"""The allocation-free overlap entry point against the regular one.

pawpy_gpu_overlap_noalloc serves callers that cannot allocate device memory
(their device memory belongs to another allocator or to a fixed budget, or
they must not pay the device synchronisation of cudaMalloc). It keeps its
split-K partial sums in a static device array, so this test checks two
calls in a row: the second reuses the scratch the first one left behind.
The device buffers here come from torch; the test itself is not such a caller.
"""

import ctypes as C
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _lib():
    from pawpyseed_gb300 import _lib

    L = _lib.lib()
    L.pawpy_gpu_overlap_noalloc.restype = C.c_int
    L.pawpy_gpu_overlap_noalloc.argtypes = [C.c_void_p, C.c_longlong, C.c_void_p, C.c_longlong,
                                            C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    return _lib, L


def _padded(c, kpad):
    out = np.zeros((c.shape[0], kpad), np.complex64)
    out[:, : c.shape[1]] = c
    return out


def test_noalloc_overlap_matches_pseudoprojection(workload_dirs):
    import torch

    from pawpyseed_gb300 import vaspio
    from pawpyseed_gb300.wavefunction import Wavefunction

    _l, L = _lib()
    d = workload_dirs("cfg0")
    basis = Wavefunction.from_directory(d["basis"])
    wf = Wavefunction.from_directory(d["defect"])
    nk = basis.nwk * basis.nspin
    # the regular entry point: every defect band through pseudoprojection
    ref = np.array([wf.pseudoprojection(b, basis) for b in range(wf.nband)])  # [bS][bR*nk + k]
    ref = ref.reshape(wf.nband, basis.nband, nk)
    rb = vaspio.read_wavecar_numpy(os.path.join(d["basis"], "WAVECAR"))
    rw = vaspio.read_wavecar_numpy(os.path.join(d["defect"], "WAVECAR"))
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream()
    for k in range(nk):
        W = rb["coeffs"][k].shape[1]
        K = (W + 15) // 16 * 16
        A = torch.from_numpy(_padded(rb["coeffs"][k], K)).to(dev)
        B = torch.from_numpy(_padded(rw["coeffs"][k], K)).to(dev)
        M, N = A.shape[0], B.shape[0]
        outs = []
        for _ in range(2):  # two calls in a row share the static scratch
            out = torch.full((N, M), float("nan"), dtype=torch.complex64, device=dev)
            splits = L.pawpy_gpu_overlap_noalloc(A.data_ptr(), K, B.data_ptr(), K, M, N, K,
                                                 out.data_ptr(), C.c_void_p(stream.cuda_stream))
            _l.check()
            assert splits >= 2, "the split-K scratch path was not exercised"
            torch.cuda.synchronize()
            outs.append(out.cpu().numpy())
        for o in outs:
            assert np.all(np.isfinite(o))
            assert np.abs(o - ref[:, :, k]).max() <= TOL
        assert np.array_equal(outs[0], outs[1])


def _random_rows(rng, n, k):
    c = (rng.standard_normal((n, k)) + 1j * rng.standard_normal((n, k))).astype(np.complex64)
    return (c / np.linalg.norm(c, axis=1, keepdims=True)).astype(np.complex64)


@pytest.mark.parametrize("M,N,K,use_lib_stream", [
    (2048, 2040, 64, False),   # 4,177,920 output values, just under the limit: one split, direct write
    (40, 24, 8192, False),     # a small output over a long K: many splits through the scratch
    (96, 80, 1024, True),      # NULL stream: the library's own stream
])
def test_noalloc_overlap_matches_fp64_contraction(M, N, K, use_lib_stream):
    """Shapes the workload case above does not reach, each against conj(A) B^T in FP64, two calls
    in a row. With the split heuristic (two waves of 64 x 64 tiles) no output fits fewer
    splits than it asks for, so the capacity clamp never binds; the largest output goes
    through the direct-write path."""
    import torch

    _l, L = _lib()
    rng = np.random.default_rng(M * 7 + N + K)
    a = _random_rows(rng, M, K)
    b = _random_rows(rng, N, K)
    truth = b.astype(np.complex128) @ a.astype(np.complex128).conj().T  # [N][M]
    dev = torch.device("cuda:0")
    A = torch.from_numpy(a).to(dev)
    B = torch.from_numpy(b).to(dev)
    stream = None if use_lib_stream else C.c_void_p(torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    outs = []
    for _ in range(2):
        out = torch.full((N, M), float("nan"), dtype=torch.complex64, device=dev)
        splits = L.pawpy_gpu_overlap_noalloc(A.data_ptr(), K, B.data_ptr(), K, M, N, K, out.data_ptr(), stream)
        _l.check()
        if M * N > 4_000_000:
            assert splits == 1
        elif K >= 8192:
            assert splits >= 2
        if use_lib_stream:
            L.pawpy_gpu_synchronize()
        torch.cuda.synchronize()
        outs.append(out.cpu().numpy())
    for o in outs:
        assert np.all(np.isfinite(o))
        assert np.abs(o - truth).max() <= TOL
    assert np.array_equal(outs[0], outs[1])


def test_noalloc_overlap_rejects_oversized_output():
    _l, L = _lib()
    # 4096 x 4096 outputs exceed the 4,194,304-value scratch limit; rejected before any launch
    fake = C.c_void_p(256)
    r = L.pawpy_gpu_overlap_noalloc(fake, 16, fake, 16, 4096, 4096, 16, fake, None)
    assert r < 0
    with pytest.raises(_l.PAWpyGPUError, match="scratch limit"):
        _l.check()
    r = L.pawpy_gpu_overlap_noalloc(fake, 16, fake, 16, 32, 32, 24, fake, None)
    assert r < 0
    with pytest.raises(_l.PAWpyGPUError, match="multiple of 16"):
        _l.check()

"""Serving form: resident bases, continuous batching, admission by memory budget.

A request's result is the same alone and in a mix of concurrent requests
(every reduction of the path has a fixed order; requests share only read-only
basis data), and equals the FP64 truth within the path's 1e-5 bar.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5


def small_bases():
    from pawpyseed_gb300 import serve, synth

    out = []
    for cfg, nb, nk in ((0, 32, None), (1, 8, 2)):
        w = synth.small_workload(cfg, nband=nb, nk=nk)
        bs, _ = synth.structures(cfg)
        out.append((bs, w, synth.wavefunction_data(bs, w, 100 + cfg)))
    return out


def requests(bases, n, seed):
    from pawpyseed_gb300 import serve, synth

    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(n):
        b = i % len(bases)
        bs, w, _ = bases[b]
        ds = serve.point_defects(bs, rng, int(rng.integers(1, 4)))
        nb = int(rng.integers(4, 12))
        reqs.append((b, ds, synth.wavefunction_data(ds, dict(w, nband=nb), 300 + i)))
    return reqs


def run(bases, reqs, slots, together):
    from pawpyseed_gb300 import _lib, serve
    from pawpyseed_gb300.wavefunction import Wavefunction

    _lib.set_precision("bf16x3")
    cr = serve.core_region()
    srv = serve.ProjectionServer(8 << 30, slots)
    try:
        bw = []
        for bs, w, data in bases:
            b = Wavefunction.from_arrays(bs, cr, w["dim"], data)
            srv.add_basis(b)
            bw.append(b)
        outs = []
        if together:
            ids = [srv.submit(b, Wavefunction.from_arrays(ds, cr, bases[b][1]["dim"], data)) for b, ds, data in reqs]
            outs = [srv.wait(i)[0] for i in ids]
        else:
            for b, ds, data in reqs:
                outs.append(srv.wait(srv.submit(b, Wavefunction.from_arrays(ds, cr, bases[b][1]["dim"], data)))[0])
        counts = srv.counts()
    finally:
        srv.close()
        _lib.set_precision("fp32")
    return outs, counts


def test_results_are_the_same_alone_and_in_the_mix():
    bases = small_bases()
    reqs = requests(bases, 8, 7)
    alone, _ = run(bases, reqs, 1, False)
    mixed, counts = run(bases, reqs, 4, True)
    assert counts["done"] == len(reqs)
    for a, m in zip(alone, mixed):
        assert a.shape == m.shape
        assert np.isfinite(a).all()
        assert np.abs(a - m).max() <= 1e-7


def test_served_request_matches_fp64_truth(workload_dirs, oracle_projectors):
    from pawpyseed_gb300 import _lib, serve
    from pawpyseed_gb300.wavefunction import Wavefunction

    d = workload_dirs("cfg0")
    op = oracle_projectors("cfg0")
    truth = op.full()
    _lib.set_precision("bf16x3")
    srv = serve.ProjectionServer(8 << 30, 2)
    try:
        basis = Wavefunction.from_directory(d["basis"])
        bid = srv.add_basis(basis)
        ids = [srv.submit(bid, Wavefunction.from_directory(d["defect"])) for _ in range(3)]
        outs = [srv.wait(i) for i in ids]
    finally:
        srv.close()
        _lib.set_precision("fp32")
    tv = np.array([op.band_vector(truth, b) for b in range(outs[0][0].shape[0])])
    for out, info in outs:
        assert np.abs(out - tv).max() <= TOL
        assert info["latency_ms"] >= info["run_ms"] > 0


def test_admission_keeps_estimates_within_budget():
    from pawpyseed_gb300 import _lib, serve
    from pawpyseed_gb300.wavefunction import Wavefunction

    bases = small_bases()[:1]
    reqs = requests(bases, 4, 11)
    cr = serve.core_region()
    # room for about one request at a time: the server must hold the others back
    probe = serve.ProjectionServer(64 << 30, 1)
    b = Wavefunction.from_arrays(*bases[0][:1], cr, bases[0][1]["dim"], bases[0][2])
    probe.add_basis(b)
    _, info = probe.wait(probe.submit(0, Wavefunction.from_arrays(reqs[0][1], cr, bases[0][1]["dim"], reqs[0][2])))
    probe.close()
    est = info["est_bytes"]
    srv = serve.ProjectionServer(int(est * 1.9), 4)
    try:
        b = Wavefunction.from_arrays(*bases[0][:1], cr, bases[0][1]["dim"], bases[0][2])
        srv.add_basis(b)
        ids = [srv.submit(0, Wavefunction.from_arrays(ds, cr, bases[0][1]["dim"], data)) for _, ds, data in reqs]
        for i in ids:
            srv.wait(i)
        counts = srv.counts()
        assert counts["done"] == len(reqs)
        assert counts["peak_est_bytes"] <= int(est * 1.9)
        tiny = serve.ProjectionServer(1 << 20, 1)
        tiny.add_basis(Wavefunction.from_arrays(*bases[0][:1], cr, bases[0][1]["dim"], bases[0][2]))
        with pytest.raises(_lib.PAWpyGPUError):
            tiny.submit(0, Wavefunction.from_arrays(reqs[0][1], cr, bases[0][1]["dim"], reqs[0][2]))
        tiny.close()
    finally:
        srv.close()

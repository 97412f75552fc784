import hashlib
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

GOLDEN = os.path.join(ROOT, "tests", "golden")

# name -> (workload, nband, nk): the reduced workloads the golden fixtures were made from
CASES = {
    "cfg0": (0, 32, None),
    "cfg1s": (1, 8, 2),
    "cfg2s": (2, 4, None),
    "cfg3s": (3, 4, 2),
}


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs the library's kernels)")


class GoldenInputsDiffer(UserWarning):
    """The regenerated synthetic inputs are not byte-identical to the ones the golden fixtures
    were made from, so the fixture comparisons run at the tolerance of the FP64 truth instead
    of at rounding level."""


def same_golden_inputs(dirs, g, name):
    """Whether the regenerated workload has the fixture's bytes; warns (loudly) when not."""
    import warnings

    same = fingerprint(dirs["basis"]) == str(g["fp_basis"]) and fingerprint(dirs["defect"]) == str(g["fp_defect"])
    if not same:
        warnings.warn(GoldenInputsDiffer("%s: regenerated inputs differ in bytes from the golden fixture's; "
                                         "comparing at the FP64-truth tolerance instead" % name))
    return same


def fingerprint(path):
    h = hashlib.sha256()
    for name in ("WAVECAR", "POTCAR", "CONTCAR", "vasprun.xml"):
        with open(os.path.join(path, name), "rb") as fh:
            h.update(fh.read())
    return h.hexdigest()


@pytest.fixture(scope="session")
def workload_dirs(tmp_path_factory):
    """Lazily written synthetic workloads: name -> {'basis': dir, 'defect': dir}."""
    from pawpyseed_gb300 import synth

    root = tmp_path_factory.mktemp("workloads")
    cache = {}

    def get(name):
        if name not in cache:
            cfg, nb, nk = CASES[name]
            cache[name] = synth.write_workload(str(root / name), cfg, nband=nb, nk=nk)
        return cache[name]

    return get


@pytest.fixture(scope="session")
def realspace_dirs(tmp_path_factory):
    """The 8-atom workload reduced to 4 bands and 2 k-points (the real-space golden fixture's)."""
    from pawpyseed_gb300 import synth

    return synth.write_workload(str(tmp_path_factory.mktemp("realspace")), 0, nband=4, nk=2)


@pytest.fixture(scope="session")
def golden():
    def get(name):
        return np.load(os.path.join(GOLDEN, name + ".npz"))

    return get


@pytest.fixture(scope="session")
def oracle_projectors(workload_dirs):
    """Oracle (FP64 restatement) projector per case, built once per session."""
    import oracle as orc

    cache = {}

    def get(name):
        if name not in cache:
            d = workload_dirs(name)
            b = orc.OracleWavefunction(d["basis"])
            w = orc.OracleWavefunction(d["defect"])
            cache[name] = orc.OracleProjector(w, b)
        return cache[name]

    return get


def have_gpu():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session", autouse=True)
def _build_lib():
    """Make sure the in-tree library and the oracle exist before tests import them."""
    from pawpyseed_gb300 import build as B

    if not os.path.exists(B.LIB):
        B.build()
    import oracle as orc

    if not os.path.exists(orc.LIB_PATH):
        orc.build()

"""The real-space functions of density.c on the device against the reference's golden vectors and
the oracle's FP64 evaluation: realspace_state (with and without remove_phase), ae_chg_density,
project_realspace_state and the batched projection of every defect band, and the VASP volumetric
files written from them.

Tolerances: states and densities within 1e-5 of their largest magnitude (single-precision
transforms and sphere sums on the device, FP64 accumulation of the density); projections within
1e-5 absolute (the accuracy target of the band-pair metric); the batched projection equal to the
per-band entry point within 1e-6.
"""

import os

import numpy as np
import pytest

from conftest import same_golden_inputs

pytestmark = pytest.mark.gpu

TOL = 1e-5


@pytest.fixture(scope="module")
def rs_case(realspace_dirs, golden):
    import oracle as orc

    from pawpyseed_gb300.wavefunction import Wavefunction

    g = golden("realspace_cfg0")
    same = same_golden_inputs(realspace_dirs, g, "realspace_cfg0")
    basis = Wavefunction.from_directory(realspace_dirs["basis"])
    wf = Wavefunction.from_directory(realspace_dirs["defect"])
    ow = orc.OracleWavefunction(realspace_dirs["defect"])
    ob = orc.OracleWavefunction(realspace_dirs["basis"])
    ow.setup_projectors()
    ob.setup_projectors()
    return dict(g=g, same=same, basis=basis, wf=wf, ow=ow, ob=ob)


def test_realspace_state_density_and_projection_match_reference(rs_case):
    from pawpyseed_gb300.projector import Projector

    g, wf, basis, ow, ob = rs_case["g"], rs_case["wf"], rs_case["basis"], rs_case["ow"], rs_case["ob"]
    N = np.asarray(g["fftg"], dtype=np.int32)
    # one state: band 1 at k-point 1
    x = wf.get_state_realspace(1, 1, 0, dim=N)
    truth = ow.realspace_state(1, 1, N)
    scale = np.abs(truth).max()
    assert np.abs(x - truth).max() <= TOL * scale
    if rs_case["same"]:
        assert np.abs(x - g["state_b1_k1"]).max() <= TOL * scale
    # remove_phase divides out exp(2 pi i k.r)
    xr = wf.get_state_realspace(1, 1, 0, dim=N, remove_phase=True)
    kf = ow.kpts[1]
    fr = [np.arange(N[a]) / N[a] for a in range(3)]
    kdotr = kf[0] * fr[0][:, None, None] + kf[1] * fr[1][None, :, None] + kf[2] * fr[2][None, None, :]
    assert np.abs(xr - truth * np.exp(-2j * np.pi * kdotr)).max() <= TOL * scale
    # charge density of the occupied bands
    rho = wf.get_realspace_density(dim=N)
    rtruth = ow.ae_chg_density(N)
    assert np.abs(rho - rtruth).max() <= TOL * np.abs(rtruth).max()
    if rs_case["same"]:
        assert np.abs(rho - g["rho"]).max() <= TOL * np.abs(rtruth).max()
    # projections of every defect band onto the basis on the same grid
    pr = Projector(wf, basis, method="realspace")
    mine = np.array([pr._single_band_projection_realspace(b, dim=N) for b in range(wf.nband)])
    nk = ow.nk
    vol = abs(np.linalg.det(ow.lattice))
    n3 = int(np.prod(N))
    ptruth = np.zeros_like(mine)
    for k in range(nk):
        S = np.array([ow.realspace_state(b, k, N).ravel() for b in range(ow.nband)])
        R = np.array([ob.realspace_state(b, k, N).ravel() for b in range(ob.nband)])
        ptruth[:, k::nk] = S @ R.conj().T * vol / n3
    assert np.abs(mine - ptruth).max() <= TOL
    if rs_case["same"]:
        assert np.abs(mine - g["proj"]).max() <= TOL


def test_realspace_projector_batched_equals_per_band(rs_case):
    """project_all (all defect bands through the grouped contraction) against the per-band entry
    point on the default grid (twice the defect's), and the per-band density sum against the
    band-selected density."""
    from pawpyseed_gb300.projector import Projector

    wf, basis = rs_case["wf"], rs_case["basis"]
    pr = Projector(wf, basis, method="realspace")
    per_band = np.array([pr.single_band_projection(b) for b in range(wf.nband)])
    allb = pr.project_all()
    assert np.all(np.isfinite(allb))
    assert np.abs(allb - per_band).max() <= 1e-6
    sel = wf.get_realspace_density(bands=[0])
    acc = np.zeros_like(sel)
    for s in range(wf.nspin):
        for k in range(wf.nwk):
            acc += wf.get_state_realspace_density(0, k, s) * wf.kws[k] / wf.nspin
    assert np.abs(sel - acc).max() <= 1e-12 * np.abs(acc).max()
    with pytest.raises(ValueError):
        wf.get_state_realspace(wf.nband, 0, 0)


def test_volumetric_files_have_the_reference_layout(rs_case, tmp_path):
    """write_state_realspace / write_density_realspace: POSCAR-style header, the grid line, then
    the values with the first index fastest, five per line."""
    wf = rs_case["wf"]
    N = np.asarray(rs_case["g"]["fftg"], dtype=np.int32)
    prefix = str(tmp_path / "st_")
    res = wf.write_state_realspace(0, 0, 0, fileprefix=prefix, dim=N, scale=2.0)
    fn = prefix + "B0K0S0_REAL.vasp"
    assert os.path.exists(fn) and os.path.exists(prefix + "B0K0S0_IMAG.vasp")
    lines = open(fn).read().splitlines()
    n_atoms = len(wf.structure.species)
    grid_line = 8 + n_atoms + 1
    assert [int(v) for v in lines[grid_line].split()] == list(N)
    vals = np.array(" ".join(lines[grid_line + 1:]).split(), dtype=np.float64)
    assert vals.size == int(np.prod(N))
    want = np.real(res).transpose(2, 1, 0).ravel() * 2.0
    assert np.abs(vals - want).max() <= 1e-6 * np.abs(want).max()
    dn = str(tmp_path / "AECCAR.vasp")
    rho = wf.write_density_realspace(dn, dim=N)
    dl = open(dn).read().splitlines()
    dv = np.array(" ".join(dl[grid_line + 1:]).split(), dtype=np.float64)
    assert np.abs(dv - rho.transpose(2, 1, 0).ravel()).max() <= 1e-6 * np.abs(rho).max()

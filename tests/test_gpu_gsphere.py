"""Plane-wave spheres enumerated on the device (the WAVECAR reader's G loop,
reader.c:230-271) and the reader that uses them.

The device list must equal the reference's list bit for bit: the same points in
the same (VASP) order. The check is an exact restatement of the reference's
arithmetic in Python floats (IEEE double, no fused multiply-add): the reciprocal
lattice as the reader builds it (cross products times 2 pi / det, reader.c:58-65),
sumkg_j = (k1+g1) b1_j + (k2+g2) b2_j + (k3+g3) b3_j, |s| = pow(s.s, 0.5),
pow(|s|, 2.0) / c <= ENCUT — decided this way for every point within 1e-9 of the
cutoff, by the cheaper numpy form elsewhere. Cases: the reference's Ga4 WAVECAR
fixture (945 plane waves at its first k-point), random triclinic cells and
k-points, and plane waves placed exactly on the cutoff (ENCUT equal to a point's
energy, and one ulp below it) — the points that the device leaves to the host.
"""

import ctypes as C
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CEV = 0.262465831


def _cross(a, b):
    return [a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]]


def _rec(lattice):
    a = [list(map(float, r)) for r in np.asarray(lattice, dtype=np.float64).reshape(3, 3)]
    m = [x for r in a for x in r]
    v = (m[0] * m[4] * m[8] + m[1] * m[5] * m[6] + m[2] * m[3] * m[7] - m[2] * m[4] * m[6]
         - m[1] * m[3] * m[8] - m[0] * m[5] * m[7])
    f = 2.0 * math.pi / v
    return [[x * f for x in _cross(a[1], a[2])], [x * f for x in _cross(a[2], a[0])],
            [x * f for x in _cross(a[0], a[1])]]


def _etot(b, k, g):
    s = [(k[0] + g[0]) * b[0][j] + (k[1] + g[1]) * b[1][j] + (k[2] + g[2]) * b[2][j] for j in range(3)]
    gt = math.pow(s[0] * s[0] + s[1] * s[1] + s[2] * s[2], 0.5)
    return math.pow(gt, 2.0) / CEV


def reference_gvectors(lattice, kpt, encut):
    from pawpyseed_gb300 import vaspio

    b = _rec(lattice)
    nb = vaspio.nbmax(lattice, encut)
    ax = [vaspio._wrap_axis(n) for n in nb]
    g3, g2, g1 = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    g = np.stack([g1.ravel(), g2.ravel(), g3.ravel()], axis=1)
    B = np.array(b)
    kg = (kpt[0] + g[:, 0:1]) * B[0] + (kpt[1] + g[:, 1:2]) * B[1] + (kpt[2] + g[:, 2:3]) * B[2]
    e = (kg * kg).sum(1) / CEV
    keep = e <= encut
    near = np.nonzero(np.abs(e - encut) <= 1e-9 * encut)[0]
    for i in near:
        keep[i] = _etot(b, [float(x) for x in kpt], [int(x) for x in g[i]]) <= encut
    return g[keep].astype(np.int32)


def device_gvectors(lattice, kpt, encut):
    from pawpyseed_gb300 import _lib

    L = _lib.lib()
    lat = np.ascontiguousarray(np.asarray(lattice, dtype=np.float64).reshape(-1))
    k = np.ascontiguousarray(np.asarray(kpt, dtype=np.float64))
    n = L.pawpy_gpu_gvectors(lat, k, float(encut), None, 0)
    _lib.check()
    out = np.zeros((max(n, 1), 3), dtype=np.int32)
    m = L.pawpy_gpu_gvectors(lat, k, float(encut), out.ctypes.data, n)
    _lib.check()
    assert m == n
    return out[:n]


def test_device_sphere_matches_reference_wavecar_fixture(golden):
    g = golden("fft_ga4")
    gs = device_gvectors(g["lattice"], g["kpt"], 320.0)
    assert gs.shape[0] == 945
    assert np.array_equal(gs, g["gs"])


@pytest.mark.parametrize("seed", range(8))
def test_device_sphere_matches_reference_on_triclinic_cells(seed):
    rng = np.random.default_rng(100 + seed)
    lat = np.diag(rng.uniform(4.0, 9.0, 3)) + rng.uniform(-1.5, 1.5, (3, 3)) * (1 - np.eye(3))
    for _ in range(3):
        k = rng.uniform(-0.5, 0.5, 3)
        encut = float(rng.uniform(150.0, 450.0))
        ref = reference_gvectors(lat, k, encut)
        dev = device_gvectors(lat, k, encut)
        assert np.array_equal(dev, ref)


@pytest.mark.parametrize("lattice,kpt,g0", [
    (np.diag([5.0, 5.0, 5.0]), [0.0, 0.0, 0.0], (3, 0, 0)),
    (np.diag([5.43, 5.43, 5.43]), [0.25, 0.25, 0.25], (2, -1, 1)),
    (np.array([[4.0, 0.3, 0.0], [0.1, 5.0, 0.2], [0.0, 0.4, 6.0]]), [0.5, 0.0, -0.25], (-2, 1, 3)),
])
def test_device_sphere_decides_points_on_the_cutoff(lattice, kpt, g0):
    """ENCUT set to a plane wave's own energy keeps it (<=); one ulp below drops it."""
    b = _rec(lattice)
    e0 = _etot(b, kpt, g0)
    for encut, kept in ((e0, True), (math.nextafter(e0, 0.0), False)):
        ref = reference_gvectors(lattice, kpt, encut)
        dev = device_gvectors(lattice, kpt, encut)
        assert np.array_equal(dev, ref)
        assert bool((dev == np.array(g0, dtype=np.int32)).all(1).any()) == kept


def _read(path, kws):
    from pawpyseed_gb300 import _lib

    p = _lib.lib().pawpy_gpu_read_wavefunctions(path.encode(), kws)
    _lib.check()
    return p


def test_reader_with_device_spheres_matches_numpy_reader(workload_dirs):
    """Two spins, four k-points: the reader's G lists (device spheres) and coefficients equal the
    numpy restatement of reader.c:129-299."""
    from pawpyseed_gb300 import _lib, vaspio

    d = workload_dirs("cfg3s")["basis"]
    ref = vaspio.read_wavecar_numpy(os.path.join(d, "WAVECAR"))
    p = _read(os.path.join(d, "WAVECAR"), np.full(ref["nwk"], 1.0 / ref["nwk"]))
    try:
        w = p.contents
        assert (w.nspin, w.nwk, w.nband, w.is_ncl) == (ref["nspin"], ref["nwk"], ref["nband"], 0)
        for k in range(w.nspin * w.nwk):
            kp = w.kpts[k].contents
            g = np.ctypeslib.as_array(kp.Gs, shape=(3 * kp.num_waves,)).reshape(-1, 3)
            assert np.array_equal(g, ref["gs"][k])
            for b in range(w.nband):
                c = np.ctypeslib.as_array(C.cast(kp.bands[b].contents.Cs, C.POINTER(C.c_float)),
                                          shape=(2 * kp.num_waves,)).view(np.complex64)
                assert np.array_equal(c, ref["coeffs"][k][b])
    finally:
        _lib.lib().pawpy_gpu_free_pswf(p)


def test_reader_with_device_spheres_detects_noncollinear_files(tmp_path):
    """A spinor WAVECAR (twice the sphere's count per record) is marked noncollinear and its G
    list stored twice (reader.c:274-284)."""
    from pawpyseed_gb300 import _lib, synth, vaspio

    w = synth.small_workload(0, nband=4, nk=2)
    bs, _ = synth.structures(0)
    data = synth.wavefunction_data(bs, w, 5, ncl=True)
    path = str(tmp_path / "WAVECAR")
    vaspio.write_wavecar(path, data["lattice"], data["encut"], data["kpts"], data["coeffs"],
                         data["energies"], data["occs"])
    p = _read(path, np.full(data["nwk"], 1.0 / data["nwk"]))
    try:
        wv = p.contents
        assert wv.is_ncl == 1
        for k in range(wv.nwk):
            kp = wv.kpts[k].contents
            ng = data["gs"][k].shape[0]
            assert kp.num_waves == 2 * ng
            g = np.ctypeslib.as_array(kp.Gs, shape=(3 * kp.num_waves,)).reshape(-1, 3)
            assert np.array_equal(g[:ng], data["gs"][k]) and np.array_equal(g[ng:], data["gs"][k])
            c = np.ctypeslib.as_array(C.cast(kp.bands[3].contents.Cs, C.POINTER(C.c_float)),
                                      shape=(2 * kp.num_waves,)).view(np.complex64)
            assert np.array_equal(c, data["coeffs"][k][3])
    finally:
        _lib.lib().pawpy_gpu_free_pswf(p)

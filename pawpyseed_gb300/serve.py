"""Serving form of the band-projection path: resident bases, continuous
batching of projection requests, latency statistics.

``ProjectionServer`` wraps the library's server (``pawpy_gpu_server_*`` in
include/pawpy_gpu.h): bases stay resident on the device; each request (a
defect wavefunction against one basis) runs setup_projections,
overlap_setup_real and pawpy_gpu_project_all on a worker thread with a CUDA
stream of its own, so the work of requests in flight overlaps on the device.
Requests are admitted first in, first out, when a worker is free and their
estimated device memory fits the budget.

``poisson_workload`` and ``run_stream`` generate and replay the serving
workload: a Poisson stream of requests against resident 8-, 64- and 216-atom
bases, each a seeded defect cell with 1-3 point defects and a log-uniform band
count, with throughput and p50/p99 latency.
"""

import ctypes as C
import time

import numpy as np

from . import _lib, structs, synth, vaspio
from .wavefunction import Wavefunction, pack_species


def site_lists(basis, defect):
    """M_R, M_S, N_R, N_S, N_RS_R, N_RS_S of a basis/defect pair.

    The classification of Projector.make_site_lists (projector.py:115-160), with the
    defect-side radius of an N_RS candidate read from the defect's own site j: the
    reference reads it from sites[i] with the basis index i, which fails for defect
    cells with vacancies (fewer sites than the basis)."""
    ref, cur = basis.structure, defect.structure
    D = ref.distance_matrix(cur)
    same = (D <= 0.02) & (np.array(ref.species)[:, None] == np.array(cur.species)[None, :])
    Mi, Mj = np.nonzero(same)
    M_R, M_S = [int(x) for x in Mi], [int(x) for x in Mj]
    in_M_R, in_M_S = set(M_R), set(M_S)
    N_R = [i for i in range(len(ref)) if i not in in_M_R]
    N_S = [j for j in range(len(cur)) if j not in in_M_S]
    N_RS = []
    if N_R and N_S:
        r1 = np.array([basis.cr.pps[ref.species[i]].rmax for i in N_R])
        r2 = np.array([defect.cr.pps[cur.species[j]].rmax for j in N_S])
        close = D[np.ix_(N_R, N_S)] < r1[:, None] + r2[None, :]
        N_RS = [(N_R[a], N_S[b]) for a, b in zip(*np.nonzero(close))]
    a = lambda x: np.ascontiguousarray(np.array(x, dtype=np.int32))  # noqa: E731
    return [a(M_R), a(M_S), a(N_R), a(N_S), a([x for x, _ in N_RS]), a([y for _, y in N_RS])]


class ProjectionServer:
    """Continuous-batching server over the library (see the module docstring)."""

    def __init__(self, hbm_budget_bytes=100 << 30, slots=4, keep_real_space=True):
        self._keep = 1 if keep_real_space else 0
        self._L = _lib.lib()
        self._h = self._L.pawpy_gpu_server_create(int(hbm_budget_bytes), int(slots))
        _lib.check()
        self._bases = []
        self._pending = {}

    def add_basis(self, basis):
        """Make a basis Wavefunction resident; returns its index."""
        basis.check_c_projectors()
        idx = self._L.pawpy_gpu_server_add_basis(self._h, basis.wf_ptr, basis.nums, basis.coords,
                                                 len(basis.structure), self._keep)
        _lib.check()
        self._bases.append(basis)
        return idx

    def submit(self, basis_id, defect, lists=None):
        """Queue defect (a Wavefunction whose projectors are not set up) against basis basis_id.

        The server takes over the defect's device and host data; returns a request id."""
        basis = self._bases[basis_id]
        L = self._L
        if lists is None:
            lists = site_lists(basis, defect)
        labels, ls, wg, pr, ae, ps, rm = pack_species(defect.cr)
        pps = L.get_projector_list(len(defect.cr.pps), labels, ls, wg, pr, ae, ps, rm, defect.grid_encut())
        _lib.check()
        nk = basis.nwk * basis.nspin
        out = np.zeros((defect.nband, basis.nband * nk), np.complex128)
        keep = dict(fftg=np.ascontiguousarray(defect.dim, dtype=np.int32), labels=defect.nums,
                    coords=defect.coords, lists=lists, out=out, pairs=defect.nband * basis.nband * nk)
        ptr = lambda a: a.ctypes.data if a is not None and len(a) else None  # noqa: E731
        req = structs.pawpy_gpu_request_t(
            basis=basis_id, wf=defect.wf_ptr, pps=pps, num_elems=len(defect.cr.pps),
            num_sites=len(defect.structure), fftg=keep["fftg"].ctypes.data, labels=keep["labels"].ctypes.data,
            coords=keep["coords"].ctypes.data, num_M=len(lists[0]), num_N_R=len(lists[2]),
            num_N_S=len(lists[3]), num_N_RS=len(lists[4]), M_R=ptr(lists[0]), M_S=ptr(lists[1]),
            N_R=ptr(lists[2]), N_S=ptr(lists[3]), N_RS_R=ptr(lists[4]), N_RS_S=ptr(lists[5]),
            out=out.ctypes.data)
        rid = L.pawpy_gpu_server_submit(self._h, C.byref(req))
        if rid < 0:
            L.pawpy_gpu_free_ppot_list(pps, len(defect.cr.pps))
            _lib.check()
        defect.detach()  # the server frees the wavefunction
        self._pending[rid] = keep
        return rid

    def wait(self, rid):
        """(result nband_S x (nband_R nk), dict of queue/run/latency ms, estimate bytes, pairs)."""
        times = (C.c_double * 7)()
        est = C.c_longlong(0)
        msg = C.create_string_buffer(1024)
        st = self._L.pawpy_gpu_server_wait(self._h, int(rid), times, C.byref(est), msg, len(msg))
        keep = self._pending.pop(rid)
        if st:
            raise _lib.PAWpyGPUError(st, msg.value.decode(errors="replace"))
        return keep["out"], dict(queue_ms=times[0], run_ms=times[1], latency_ms=times[2], setup_ms=times[3],
                                 overlap_ms=times[4], project_ms=times[5], release_ms=times[6], est_bytes=est.value,
                                 pairs=keep["pairs"])

    def counts(self):
        done, run, q, peak = C.c_longlong(), C.c_int(), C.c_int(), C.c_longlong()
        self._L.pawpy_gpu_server_counts(self._h, C.byref(done), C.byref(run), C.byref(q), C.byref(peak))
        return dict(done=done.value, running=run.value, queued=q.value, peak_est_bytes=peak.value)

    def close(self):
        if self._h:
            self._L.pawpy_gpu_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------------ workload

SERVE_BASES = (0, 1, 2)  # the 8-, 64- and 216-atom cells


def point_defects(struct, rng, n):
    """A copy of struct with n point defects (vacancy, A<->B substitution or a 0.1 A displacement)."""
    species = list(struct.species)
    coords = struct.frac_coords.copy()
    keep = np.ones(len(species), bool)
    for i in rng.choice(len(species), size=n, replace=False):
        kind = rng.integers(3)
        if kind == 0 and keep.sum() > 1:
            keep[i] = False
        elif kind == 1:
            species[i] = "B" if species[i] == "A" else "A"
        else:
            d = rng.normal(size=3)
            coords[i] += 0.1 * d / np.linalg.norm(d) / struct.abc
    species = [s for s, k in zip(species, keep) if k]
    coords = coords[keep]
    order = sorted(range(len(species)), key=lambda i: ({"A": 0, "B": 1}[species[i]], i))
    return vaspio.Structure(struct.lattice, [species[i] for i in order], coords[order])


def poisson_workload(n_requests=64, rate=200.0, seed=4, max_bands=512, pool=2):
    """Resident bases and a seeded Poisson request stream.

    Returns (bases, requests): bases[i] = (structure, workload, data) of the 8-, 64- and
    216-atom cells; requests = list of dict(t, basis, defect, data, nband) with arrival time t
    (s). Defect coefficient sets are drawn from a small pool per basis (the first nband bands
    of a pool entry); every request is still a separate wavefunction to the library. Requests
    use their basis's k-points (overlaps need the basis and the defect on the same k-set)."""
    rng = np.random.default_rng(seed)
    bases, pools = [], []
    for cfg in SERVE_BASES:
        w = dict(synth.workload(cfg))
        bs, _ = synth.structures(cfg)
        bases.append((bs, w, synth.wavefunction_data(bs, w, 100 + cfg)))
        entries = []
        for j in range(pool):
            ds = point_defects(bs, rng, int(rng.integers(1, 4)))
            wd = dict(w, nband=max_bands)
            entries.append((ds, synth.wavefunction_data(ds, wd, 200 + 10 * cfg + j)))
        pools.append(entries)
    t = 0.0
    reqs = []
    for _ in range(n_requests):
        t += rng.exponential(1.0 / rate)
        b = int(rng.integers(len(SERVE_BASES)))
        ds, data = pools[b][int(rng.integers(pool))]
        nb = int(min(max_bands, round(np.exp(rng.uniform(np.log(16), np.log(512))))))
        reqs.append(dict(t=t, basis=b, defect=ds, data=data, nband=nb))
    return bases, reqs


def band_subset(data, nb):
    """The first nb bands of in-memory WAVECAR content."""
    return dict(data, nband=nb, coeffs=[c[:nb] for c in data["coeffs"]],
                energies=np.asarray(data["energies"])[:, :nb], occs=np.asarray(data["occs"])[:, :nb])


def core_region():
    return vaspio.CoreRegion(synth.potcar_text(["A", "B"]))


def run_stream(bases, reqs, slots=4, budget=100 << 30, precision="bf16x3", keep_real_space=True):
    """Replays the request stream in real time; returns per-request records and totals."""
    _lib.set_precision(precision)
    L = _lib.lib()
    L.pawpy_gpu_set_host_projections(0)
    cr = core_region()
    srv = ProjectionServer(budget, slots, keep_real_space)
    try:
        bwf = []
        for bs, w, data in bases:
            b = Wavefunction.from_arrays(bs, cr, w["dim"], data)
            srv.add_basis(b)
            bwf.append(b)
        # host-side request objects before the clock starts (their construction is client work)
        prepared = []
        for r in reqs:
            bs, w, _ = bases[r["basis"]]
            d = Wavefunction.from_arrays(r["defect"], cr, w["dim"], band_subset(r["data"], r["nband"]))
            prepared.append((r, d, site_lists(bwf[r["basis"]], d)))
        t0 = time.monotonic()
        ids = []
        for r, d, lists in prepared:
            delay = t0 + r["t"] - time.monotonic()
            if delay > 0:
                time.sleep(delay)
            ids.append((srv.submit(r["basis"], d, lists), r))
        recs = []
        for rid, r in ids:
            out, info = srv.wait(rid)
            info.update(basis=r["basis"], nband=r["nband"])
            recs.append(info)
        t1 = time.monotonic()
        counts = srv.counts()
    finally:
        srv.close()
    lat = np.array([x["latency_ms"] for x in recs])
    pairs = sum(x["pairs"] for x in recs)
    return dict(records=recs, wall_s=t1 - t0, pairs=pairs, pairs_per_s=pairs / (t1 - t0),
                p50_ms=float(np.percentile(lat, 50)), p99_ms=float(np.percentile(lat, 99)),
                mean_ms=float(lat.mean()), peak_est_bytes=counts["peak_est_bytes"])

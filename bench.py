"""Band-pair projection throughput on one GB300 (pawpyseed aug_real path).

A step is the defect-side work of BasisExpansion-style analysis against a
resident basis: element setup (get_projector_list, run in full every step:
its per-input cache is switched off while timing), <p|psi> of every defect
band (setup_projections: batched scatter + 3D FFT + sphere gather), the
overlap setup (overlap_setup_real: smoothed partial waves on both sides, N_RS
pair matrices) and the full PAW overlap matrix of every defect band against
every basis band (pseudo overlap + O_M + O_R + O_S + O_N). The metric counts
band pairs NB_R * NB_S * NK per step. The basis is resident: its coefficients,
projector coefficients and real-space wavefunctions stay in HBM (not timed).

Headline workload (--workload 2, the largest configuration): the 216-atom cubic
16.29 A cell (species A:B = 3:1 on diamond sites), defect = two A->B
substitutions plus seeded displacements within +-0.05 A, Gamma only, 1024
bands, ENCUT 400 eV (78,517 plane waves), FFT grid 90^3. The 64-atom cell (8
k-points, 256 bands, 60^3) is measured the same way and reported in the same
line under "secondary". Synthetic seeded coefficients (no dataset exists for
this path).

Every timed result is checked: after timing, the overlaps of a seeded sample
of defect and basis bands at every k-point are compared with an FP64
evaluation of the same inputs by the oracle, and the line is printed only when
the largest error is within 1e-5 (the metric's accuracy bar).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

TOL = 1e-5  # max |overlap error| vs FP64 of the metric


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", type=int, default=2)
    ap.add_argument("--secondary", type=int, default=1, help="second workload in the same line (-1: none)")
    ap.add_argument("--bands", type=int, default=None, help="reduced band count (testing only)")
    ap.add_argument("--nk", type=int, default=None, help="reduced k-point count (testing only)")
    ap.add_argument("--precision", default="bf16x3", choices=["fp32", "bf16x3", "tf32"])
    ap.add_argument("--sample-defect-bands", type=int, default=8,
                    help="defect bands of the CPU sample and of the FP64 check")
    ap.add_argument("--sample-basis-bands", type=int, default=32,
                    help="basis bands of the CPU sample and of the FP64 check")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-serve", action="store_true", help="leave the serving streams out of the line")
    ap.add_argument("--serve", action="store_true",
                    help="replay only the serving stream (Poisson requests against resident bases)")
    ap.add_argument("--requests", type=int, default=64)
    ap.add_argument("--rate", type=float, default=200.0, help="mean request arrival rate (1/s)")
    ap.add_argument("--slots", type=int, default=4, help="requests in flight at once")
    ap.add_argument("--budget-gb", type=float, default=100.0, help="device-memory admission budget")
    ap.add_argument("--cpu-report", action="store_true",
                    help="the reference algorithm's CPU port per workload (0, 1, 2): defect setup, overlaps, "
                         "pairs/s and its error against FP64, one JSON line each (no GPU work)")
    ap.add_argument("--ingest-report", action="store_true",
                    help="WAVECAR reading: the library reader (device plane-wave spheres, parallel record "
                         "reads), the same without a device, and the serial numpy restatement")
    ap.add_argument("--ingest-child", default=None, help=argparse.SUPPRESS)
    ap.add_argument("--precision-report", action="store_true",
                    help="overlap matrix of the workload in every precision against FP64 (error and time)")
    return ap.parse_args()


# ---------------------------------------------------------------- distributed

def dist_init(n):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as td

        td.init_process_group("gloo")
        pg = td
    return rank, world, local, pg


from pawpyseed_gb300.replicas import barrier, max_over_ranks, sum_over_ranks  # noqa: E402


# ---------------------------------------------------------------- clocks

class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "50"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            out, _ = self.p.communicate(timeout=5)
        except Exception:
            self.p.kill()
            return None
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------- workload

WORKLOAD_NAMES = {
    0: "8-atom cubic 5.43 A cell, atom 0 moved 0.1 A, 4 k-points, {nb} bands, ENCUT 300 eV, FFT {g}, aug_real",
    1: "64-atom cubic 10.86 A A/B cell minus one A, 8 k-points (2x2x2 MP), {nb} bands, ENCUT 400 eV, FFT {g}, "
       "aug_real",
    2: "216-atom cubic 16.29 A A/B (3:1) cell, two A->B substitutions and displacements within 0.05 A, "
       "Gamma only, {nb} bands, ENCUT 400 eV, FFT {g}, aug_real",
    3: "96-atom orthorhombic 10x12x14 A A/B cell, 2 spins x 24 irregular k-points, {nb} bands, ENCUT 450 eV, "
       "FFT {g}, aug_real",
}


def make_workload(cfg, bands, nk):
    from pawpyseed_gb300 import synth, vaspio

    w = synth.small_workload(cfg, nband=bands, nk=nk)
    basis_s, defect_s = synth.structures(cfg)
    syms = [s for s in ("A", "B") if s in basis_s.species or s in defect_s.species]
    cr = vaspio.CoreRegion(synth.potcar_text(syms))
    bd = synth.wavefunction_data(basis_s, w, 11 + 7 * cfg)
    dd = synth.wavefunction_data(defect_s, w, 22 + 7 * cfg)
    return w, basis_s, defect_s, cr, bd, dd


def site_lists(basis_s, defect_s, cr):
    from pawpyseed_gb300.projector import Projector

    class P:
        pass

    p = P()
    p.basis = type("W", (), {"structure": basis_s, "cr": cr})()
    p.wf = type("W", (), {"structure": defect_s, "cr": cr})()
    M_R, M_S, N_R, N_S, N_RS = Projector.make_site_lists(p)
    a = lambda x: np.array(x, dtype=np.int32)  # noqa: E731
    return [a(M_R), a(M_S), a(N_R), a(N_S), a([x for x, _ in N_RS]), a([y for _, y in N_RS])]


def workload_name(cfg, w):
    g = "x".join(str(int(x)) for x in w["dim"])
    return WORKLOAD_NAMES.get(cfg, "workload %d" % cfg).format(nb=w["nband"], g=g)


# ---------------------------------------------------------------- our arm

def run_ours(args, cfg, rank, world, local, pg, work=None):
    """Times one workload: device-resident steps, the plain FP32 form, end-to-end steps and one
    profiled step. Returns (result dict, work tuple, out matrix of the last bf16x3 step)."""
    import torch

    torch.cuda.set_device(local)
    from pawpyseed_gb300 import _lib
    from pawpyseed_gb300.wavefunction import Wavefunction, pack_species

    if work is None:
        work = make_workload(cfg, args.bands, args.nk)
        work = work + (site_lists(work[1], work[2], work[3]),)
    w, basis_s, defect_s, cr, bd, dd, lists = work
    L = _lib.lib()
    _lib.set_precision(args.precision)
    L.pawpy_gpu_set_host_projections(0)
    basis = Wavefunction.from_arrays(basis_s, cr, w["dim"], bd)
    wf = Wavefunction.from_arrays(defect_s, cr, w["dim"], dd)
    # resident basis (not timed): coefficients, projections and real-space wavefunctions in HBM
    basis.check_c_projectors()
    grids = L.pawpy_gpu_prepare_basis(basis.wf_ptr, 1)
    _lib.check()
    M_R, M_S, N_R, N_S, NRS_R, NRS_S = lists
    P = _lib.ptr
    species = pack_species(cr)
    ge = wf.grid_encut()
    dimv = np.ascontiguousarray(wf.dim, dtype=np.int32)
    nk = wf.nwk * wf.nspin
    out = np.zeros((wf.nband, basis.nband * nk), np.complex128)
    pairs = basis.nband * wf.nband * nk
    # every step runs the whole element setup, as the reference does per structure
    L.pawpy_gpu_set_element_cache(0)

    def step():
        pps = L.get_projector_list(len(cr.pps), *species, ge)
        L.setup_projections(wf.wf_ptr, pps, len(cr.pps), len(defect_s), dimv, wf.nums, wf.coords)
        L.overlap_setup_real(basis.wf_ptr, wf.wf_ptr, basis.nums, wf.nums, basis.coords, wf.coords,
                             P(N_R), P(N_S), P(NRS_R), P(NRS_S), len(N_R), len(N_S), len(NRS_R))
        L.pawpy_gpu_project_all(out.reshape(-1), basis.wf_ptr, wf.wf_ptr, len(M_R), len(N_R), len(N_S),
                                len(NRS_R), P(M_R), P(M_S), P(N_R), P(N_S), P(NRS_R), P(NRS_S), 0)
        _lib.check()

    def timed(n):
        L.pawpy_gpu_synchronize()
        barrier(pg)
        L.pawpy_gpu_timer_start()
        for _ in range(n):
            step()
        ms = L.pawpy_gpu_timer_stop_ms()
        barrier(pg)
        return max_over_ranks(pg, ms / n)

    # ---- device-resident: the defect's coefficients already in HBM
    wf.upload()
    for _ in range(args.warmup):
        step()
    L.pawpy_gpu_synchronize()
    clocks = Clocks(local)
    clocks.start()
    L.pawpy_gpu_launch_count(1)
    ms_step = timed(args.steps)
    launches = L.pawpy_gpu_launch_count(0)
    clk = clocks.stop()
    value = sum_over_ranks(pg, pairs) / (ms_step / 1e3)

    # ---- the plain FP32 form (CUDA-core contraction) on the same resident inputs, warmed as the headline
    plain = None
    if args.precision != "fp32":
        _lib.set_precision("fp32")
        for _ in range(args.warmup):
            step()
        ms_fp32 = timed(args.steps)
        plain = dict(value=sum_over_ranks(pg, pairs) / (ms_fp32 / 1e3), ms_per_step=ms_fp32)
        _lib.set_precision(args.precision)
        for _ in range(args.warmup):
            step()

    # ---- end to end: host pswf_t, the defect's coefficients read from host memory and the
    # matrix written to host memory inside every step
    h2d = sum(c.nbytes for c in dd["coeffs"])
    d2h = out.nbytes
    L.pawpy_gpu_release(wf.wf_ptr)
    step()
    L.pawpy_gpu_synchronize()
    barrier(pg)
    L.pawpy_gpu_timer_start()
    for _ in range(args.steps):
        L.pawpy_gpu_release(wf.wf_ptr)
        step()
    ms_e2e = L.pawpy_gpu_timer_stop_ms()
    barrier(pg)
    e2e_step = max_over_ranks(pg, ms_e2e / args.steps)
    e2e_value = sum_over_ranks(pg, pairs) / (e2e_step / 1e3)

    # ---- one profiled step (per kernel family device time) for the roofline
    wf.upload()
    step()
    L.pawpy_gpu_synchronize()
    _lib.kernel_stats(reset=True)
    L.pawpy_gpu_profile(1)
    step()
    L.pawpy_gpu_profile(0)
    stats = _lib.kernel_stats(reset=True, work=True)
    L.pawpy_gpu_set_element_cache(1)
    roof = roofline(stats, w, basis, wf, lists, cr)
    if not np.all(np.isfinite(out)):
        raise RuntimeError("non-finite overlaps")
    result = dict(pairs_per_step=pairs, ms=ms_step, value=value, e2e_ms=e2e_step, e2e_value=e2e_value,
                  plain=plain, h2d=h2d, d2h=d2h, launches=launches // args.steps, clocks=clk, roofline=roof,
                  resident_real_space_basis=bool(grids == 1),
                  kernel_ms={k: v[0] for k, v in stats.items() if not k.startswith("host.")},
                  host_ms={k[5:]: v[0] for k, v in stats.items() if k.startswith("host.")})
    L.pawpy_gpu_release(wf.wf_ptr)
    L.pawpy_gpu_release(basis.wf_ptr)
    del basis, wf
    return result, work, out


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), float(p["bf16_tflops"]), "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


# DRAM bytes per band-FFT of both passes (ncu dram__bytes_read.sum + dram__bytes_write.sum of the
# pass-A and pass-B launches of one k-point, divided by its band count), per FFT grid
FFT_TRAFFIC = {
    (60, 60, 60): (47.9e6 + 195.0e6 + 261.2e6 + 99.1e6) / 256.0,
    # the 216-atom defect's step: k_planes_pipe 81.5 MB read + 375.5 MB written, k_xpick_direct
    # 456.6 MB read + 1,385 MB written per 128 bands (the picked values of every sphere)
    (90, 90, 90): (81.5e6 + 375.5e6 + 456.6e6 + 1385.0e6) / 128.0,
}


def roofline(stats, w, basis, wf, lists, cr):
    """Dominant kernel family of one profiled step: achieved algorithmic rate against the measured peak.

    The library's launches declare their algorithmic work while profiling: per band, the first
    FFT pass reads the coefficients and writes the occupied planes of H (8 (W + n1 N2 N3) bytes),
    the second reads those planes and writes the picked values (8 (n1 N2 N3 + picked points)
    bytes: complex64, or BF16 hi and lo words); 8 bytes per picked value the sphere contraction
    reads; 8 M N K useful flops of the overlap contraction per k-point (K: plane waves plus
    augmentation columns). achieved = the family's declared work in the step / its device time in
    the step (CUDA events around every launch, on the stream it runs on).
    """
    hbm, tc, src = peaks()
    if not stats:
        return None
    fams = {}
    for name, (ms, n, work) in stats.items():
        if name.startswith("host."):
            continue
        key = "fft" if name in ("fft_planes", "fft_x_pick") else (
            "sphere_contract" if name.startswith("sphere_contract") else name)
        a = fams.setdefault(key, [0.0, 0, 0.0, []])
        a[0] += ms
        a[1] += n
        a[2] += work
        a[3].append(name)
    by_family = {}
    for key, (ms, n, work, members) in fams.items():
        if work <= 0 or ms <= 0:
            continue
        if key.startswith("gemm"):
            by_family[key] = dict(ms=ms, achieved=work / (ms / 1e3) / 1e12, unit="TFLOP/s",
                                  frac=work / (ms / 1e3) / 1e12 / tc, bound="tensor")
        else:
            by_family[key] = dict(ms=ms, achieved=work / (ms / 1e3) / 1e9, unit="GB/s",
                                  frac=work / (ms / 1e3) / 1e9 / hbm, bound="hbm")
    fam = max(fams, key=lambda k: fams[k][0])
    ms, n, work, members = fams[fam]
    out = dict(kernel="+".join(members), launches=n, ms_per_launch=ms / max(n, 1), peak_source=src,
               traffic=None, by_family=by_family)
    if fam in by_family:
        f = by_family[fam]
        out.update(bound=f["bound"], achieved=f["achieved"], unit=f["unit"], frac=f["frac"],
                   peak=tc if f["bound"] == "tensor" else hbm, algorithmic_work_per_launch=work / max(n, 1))
    else:
        out.update(bound="hbm", achieved=None, peak=hbm, unit="GB/s", frac=None)
    if fam == "fft":
        out.update(algorithmic_bytes_per_band_fft=work / (wf.nband * wf.nwk * wf.nspin))
        t = FFT_TRAFFIC.get(tuple(int(x) for x in w["dim"]))
        if t is not None:
            out.update(traffic=t, traffic_unit="bytes per band-FFT (ncu dram__bytes_read+write, both passes)")
    return out


# ---------------------------------------------------------------- oracle sample (CPU arm and FP64 check)

def sample_bands(n, m, seed):
    rng = np.random.default_rng(seed)
    return np.sort(rng.choice(n, size=min(n, m), replace=False))


class OracleSample:
    """The oracle (the reference algorithm in C + OpenMP, FP64) on a band sample of a workload:
    nsb defect bands against nrb basis bands at every k-point. Phases are timed separately so the
    full workload's CPU time can be extrapolated by the band count each phase scales with:

      band-independent: element setup, sphere tables, smoothed-wave tables, pair matrices
      per defect band:  FFT + gather of <p|psi> and of the smoothed-wave projections (N_R)
      per basis band:   FFT + gather of the smoothed-wave projections onto N_S sites
      per band pair:    pseudo overlap (FP32 accumulation, as cblas_cdotc_sub) + PAW terms

    The basis's own setup (its projections) is resident and not counted. fixed_once reuses the
    band-independent parts of the first run (timed once) in later runs."""

    def __init__(self, work, nsb, nrb, seed=7):
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as orc

        self.orc = orc
        self.work = work
        w, basis_s, defect_s, cr, bd, dd, lists = work
        self.sb = sample_bands(dd["nband"], nsb, seed)
        self.rb = sample_bands(bd["nband"], nrb, seed + 1)
        self.ob = orc.OracleWavefunction(data=orc.band_subset(bd, self.rb), struct=basis_s, cr=cr, dim=w["dim"])
        self.ob.setup_projectors()  # resident basis, not timed
        M_R, M_S, N_R, N_S, NRS_R, NRS_S = [list(map(int, x)) for x in lists]
        self.lists = (M_R, M_S, N_R, N_S, list(zip(NRS_R, NRS_S)))
        self.fixed = None
        self._prev = None

    def run(self, fixed_once=False):
        orc = self.orc
        w, basis_s, defect_s, cr, bd, dd, lists = self.work
        tm = {}
        reuse = self._prev if (fixed_once and self._prev is not None) else None
        t0 = time.perf_counter()
        ow = orc.OracleWavefunction(data=orc.band_subset(dd, self.sb), struct=defect_s, cr=cr, dim=w["dim"])
        ow.setup_projectors(timer=tm, reuse=reuse.wf if reuse is not None else None)
        op = orc.OracleProjector(ow, self.ob, lists=self.lists, timer=tm, reuse=reuse)
        t1 = time.perf_counter()
        p32 = op.pseudo_full(fp32=True)
        comp = op.comp_full()
        t2 = time.perf_counter()
        tm["pairs"] = t2 - t1
        self.total_s = t2 - t0
        if reuse is None:
            self.fixed = {k: tm.get(k, 0.0) for k in ("element", "tables", "smooth_tables", "pair_matrices")}
            self._prev = op
        self.timings = tm
        self.op = op
        self.p32, self.comp = p32, comp
        return tm

    def truth(self):
        """FP64 overlaps of the sample: [nk, nsb, nrb] (pseudo in double precision + PAW terms)."""
        return self.op.pseudo_full(fp32=False) + self.comp

    def extrapolate(self):
        """(pairs/s of the full workload, seconds) from the last run's per-band phases and the
        band-independent phases of the first run."""
        w, basis_s, defect_s, cr, bd, dd, lists = self.work
        NS, NR = dd["nband"], bd["nband"]
        ns, nr = len(self.sb), len(self.rb)
        tm = self.timings
        fixed = sum(self.fixed.values())
        per_def = tm.get("project", 0.0) + tm.get("wp_defect", 0.0)
        per_bas = tm.get("wp_basis", 0.0)
        secs = fixed + per_def * NS / ns + per_bas * NR / nr + tm["pairs"] * (NS * NR) / (ns * nr)
        pairs = NS * NR * len(bd["coeffs"])
        return pairs / secs, secs

    def describe(self):
        w = self.work[0]
        return ("oracle port on %d defect x %d basis bands at all %d k-point(s) (seeded sample), phases timed "
                "and extrapolated to the full %d x %d bands by the band count each scales with; "
                "band-independent setup (element, sphere and smoothed-wave tables, pair matrices) timed once"
                % (len(self.sb), len(self.rb), len(w["kpts"]) * w["nspin"], self.work[5]["nband"],
                   self.work[4]["nband"]))


def accuracy(sample, out, nk):
    """max and RMS |S - S_FP64| of our matrix on the oracle's sample (every k-point)."""
    truth = sample.truth()  # [nk, nsb, nrb]
    mine = np.empty_like(truth)
    for k in range(nk):
        mine[k] = out[np.ix_(sample.sb, sample.rb * nk + k)]
    err = np.abs(mine - truth)
    return dict(max_abs_err_vs_fp64=float(err.max()), rms_abs_err_vs_fp64=float(np.sqrt((err ** 2).mean())),
                max_abs_overlap=float(np.abs(truth).max()), tolerance=TOL,
                sample="%d defect x %d basis bands (seeded) at all %d k-point(s): %d overlaps"
                       % (len(sample.sb), len(sample.rb), nk, err.size))


def cores():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def threads_used():
    """OpenMP threads of the oracle: OMP_NUM_THREADS when set, else every host core."""
    try:
        return int(os.environ["OMP_NUM_THREADS"])
    except (KeyError, ValueError):
        return cores()


def run_reference(args, rank, world, pg):
    """The reference algorithm's CPU implementation (oracle port), all host threads, on the same
    workload: every step times the per-band work of a band sample; the band-independent setup is
    timed once (first warm-up) and counted in every step's extrapolated value."""
    if rank != 0:
        return
    os.environ.setdefault("OMP_NUM_THREADS", str(cores()))
    work = make_workload(args.workload, args.bands, args.nk)
    work = work + (site_lists(work[1], work[2], work[3]),)
    w = work[0]
    smp = OracleSample(work, args.sample_defect_bands, args.sample_basis_bands)
    smp.run()
    for _ in range(max(0, args.warmup - 1)):
        smp.run(fixed_once=True)
    rates, secs, walls = [], [], []
    for _ in range(args.steps):
        smp.run(fixed_once=True)
        r, s = smp.extrapolate()
        rates.append(r)
        secs.append(s)
        walls.append(smp.total_s)
    value = float(np.median(rates))
    line = dict(metric="band-pair projections/sec", value=value, unit="pairs/s", n_gpus=args.gpus,
                steps=args.steps, warmup=args.warmup, ms_per_step=float(np.median(secs)) * 1e3,
                higher_is_better=True, scaling="weak", vs_baseline=None, dtype="c64 / f64", data="synthetic",
                impl="reference", config=config(args, args.workload, w, work),
                cpu_baseline=dict(value=value, unit="pairs/s", cores=threads_used(), kind="port", sample=smp.describe(),
                                  sample_wall_s=float(np.median(walls))),
                e2e=dict(value=value, unit="pairs/s", h2d_bytes_per_step=0, d2h_bytes_per_step=0))
    print(json.dumps(line))


def config(args, cfg, w, work=None):
    l2 = None
    if work is not None:
        mb = [sum(c.nbytes for c in d["coeffs"]) / 1e6 for d in (work[4], work[5])]
        l2 = ("inputs larger than L2" if min(mb) > 129 else "inputs smaller than L2") + \
            " (basis coefficients %.0f MB, defect coefficients %.0f MB; no flush between steps)" % tuple(mb)
    return {"workload": workload_name(cfg, w), "nband": w["nband"], "nk": len(w["kpts"]) * w["nspin"],
            "fft_grid": [int(x) for x in w["dim"]], "precision": args.precision, "l2": l2}


# ---------------------------------------------------------------- serving

def run_serve_streams(args, rank, local, rates=(20.0, 200.0), n=24):
    """Seeded Poisson streams against the resident 8-, 64- and 216-atom bases: one at a rate the
    device sustains (latency is service time) and one at 200 requests/s (latency includes queueing)."""
    import torch

    torch.cuda.set_device(local)
    from pawpyseed_gb300 import serve

    res = []
    for rate in rates:
        bases, reqs = serve.poisson_workload(n_requests=n, rate=rate, seed=4 + rank)
        r = serve.run_stream(bases, reqs, slots=args.slots, budget=int(args.budget_gb * (1 << 30)),
                             precision=args.precision)
        res.append(dict(rate_per_s=rate, requests=len(reqs), value=r["pairs_per_s"], unit="pairs/s",
                        p50_ms=r["p50_ms"], p99_ms=r["p99_ms"], mean_ms=r["mean_ms"], wall_s=r["wall_s"],
                        slots=args.slots, budget_gb=args.budget_gb,
                        peak_admitted_gb=r["peak_est_bytes"] / (1 << 30)))
    return res


def run_serve(args, rank, world, local):
    """Serving form: a seeded Poisson stream against resident 8-, 64- and 216-atom bases.

    Every rank replays its own stream (replicas; seeds differ by rank); rank 0 prints."""
    import torch

    torch.cuda.set_device(local)
    from pawpyseed_gb300 import serve

    bases, reqs = serve.poisson_workload(n_requests=args.requests, rate=args.rate, seed=4 + rank)
    res = serve.run_stream(bases, reqs, slots=args.slots, budget=int(args.budget_gb * (1 << 30)),
                           precision=args.precision)
    per_basis = {}
    for r in res["records"]:
        per_basis.setdefault(r["basis"], []).append(r["latency_ms"])
    if rank == 0:
        line = dict(metric="band-pair projections/sec (served stream)", value=res["pairs_per_s"], unit="pairs/s",
                    higher_is_better=True, n_gpus=world, p50_ms=res["p50_ms"], p99_ms=res["p99_ms"],
                    mean_ms=res["mean_ms"], requests=len(reqs), wall_s=res["wall_s"], pairs=res["pairs"],
                    dtype="c64 (fp32 accumulate) / f64 setup", precision=args.precision,
                    data="synthetic (seeded VASP-format content)",
                    config=dict(workload="Poisson %.0f req/s against resident 8-, 64- and 216-atom bases; "
                                         "1-3 point defects, log-uniform 16-512 bands, the basis k-points"
                                % args.rate, slots=args.slots, budget_gb=args.budget_gb,
                                peak_admitted_gb=res["peak_est_bytes"] / (1 << 30)),
                    p50_ms_by_basis={str(k): float(np.percentile(v, 50)) for k, v in per_basis.items()},
                    p99_ms_by_basis={str(k): float(np.percentile(v, 99)) for k, v in per_basis.items()})
        print(json.dumps(line))


def run_precision_report(args, local):
    """Pseudo-overlap matrix <C_R|C_S> of the workload (every k-point) in FP32 (CUDA cores), TF32 and
    split-BF16 (tensor cores) through pawpy_gpu_overlap_matrix, each against an FP64 evaluation of the
    same complex64 coefficients (torch complex128 matmul on the device, the checker only)."""
    import torch

    torch.cuda.set_device(local)
    from pawpyseed_gb300 import _lib

    w, basis_s, defect_s, cr, bd, dd = make_workload(args.workload, args.bands, args.nk)
    nk = len(bd["coeffs"])
    As = [np.ascontiguousarray(c) for c in bd["coeffs"]]
    Bs = [np.ascontiguousarray(c) for c in dd["coeffs"]]
    truth = []
    for a, b in zip(As, Bs):
        ta = torch.from_numpy(a).to("cuda", torch.complex128)
        tb = torch.from_numpy(b).to("cuda", torch.complex128)
        truth.append((tb @ ta.conj().T).cpu().numpy())
    truth = np.stack(truth)
    L = _lib.lib()
    out = {}
    for prec in ("fp32", "tf32", "bf16x3"):
        _lib.overlap_matrix(As, Bs, prec)  # warm-up (tuning, allocations)
        t0 = time.perf_counter()
        L.pawpy_gpu_timer_start()
        s = _lib.overlap_matrix(As, Bs, prec)
        ms = L.pawpy_gpu_timer_stop_ms()
        err = np.abs(s - truth)
        out[prec] = dict(max_abs_err=float(err.max()), rms_abs_err=float(np.sqrt((err ** 2).mean())),
                         call_ms=ms, wall_ms=(time.perf_counter() - t0) * 1e3)
    # worst case for accumulation bias: the basis against itself (diagonal = 1)
    self_truth = np.stack([np.ones(a.shape[0]) for a in As])
    for prec in ("fp32", "tf32", "bf16x3"):
        s = _lib.overlap_matrix(As, As, prec)
        d = np.abs(np.stack([np.diag(x) for x in s]) - self_truth)
        out[prec]["self_diag_max_err"] = float(d.max())
    W = [a.shape[1] for a in As]
    print(json.dumps(dict(metric="pseudo-overlap error vs FP64 per precision", workload=args.workload,
                          nband_R=As[0].shape[0], nband_S=Bs[0].shape[0], nk=nk, W=W, max_abs_overlap=float(
                              np.abs(truth).max()), variants=out,
                          note="call_ms includes the host-to-device copy of both coefficient sets")))


# ---------------------------------------------------------------- main

def measure(args, cfg, rank, world, local, pg, with_cpu):
    """One workload through our arm, checked against FP64 on the oracle's sample; on rank 0 also the
    CPU baseline from the same oracle run."""
    res, work, out = run_ours(args, cfg, rank, world, local, pg)
    w = work[0]
    acc, cpu = None, None
    if rank == 0:
        os.environ.setdefault("OMP_NUM_THREADS", str(cores()))
        smp = OracleSample(work, args.sample_defect_bands, args.sample_basis_bands)
        smp.run()
        nk = len(w["kpts"]) * w["nspin"]
        acc = accuracy(smp, out, nk)
        if not acc["max_abs_err_vs_fp64"] <= TOL:
            raise RuntimeError("workload %d: max |overlap error| vs FP64 %.3e exceeds %.0e on the sample"
                               % (cfg, acc["max_abs_err_vs_fp64"], TOL))
        if with_cpu:
            r, secs = smp.extrapolate()
            cpu = dict(value=r, unit="pairs/s", cores=threads_used(), kind="port", sample=smp.describe(),
                       sample_wall_s=smp.total_s, extrapolated_s=secs)
    return res, work, acc, cpu


def run_cpu_report(args):
    """Per workload: the oracle port (the reference's algorithm, all host threads) on a band sample
    (the whole 8-atom workload; 8 defect x 32 basis bands at every k-point of the others), the
    band-independent setup timed once and the per-band phases extrapolated to the full workload,
    and the error of its overlaps (single-precision pseudo overlap as the reference computes it,
    FP64 PAW terms) against the FP64 evaluation of the same sample."""
    for cfg in (0, 1, 2):
        work = make_workload(cfg, None, None)
        work = work + (site_lists(work[1], work[2], work[3]),)
        w, basis_s, defect_s, cr, bd, dd, lists = work
        full = cfg == 0
        smp = OracleSample(work, dd["nband"] if full else 8, bd["nband"] if full else 32, seed=31 + cfg)
        smp.run()
        smp.run(fixed_once=True)
        pps, secs = smp.extrapolate()
        w_, NS, NR = smp.timings, dd["nband"], bd["nband"]
        ns, nr = len(smp.sb), len(smp.rb)
        setup = (sum(smp.fixed.values()) + (w_.get("project", 0.0) + w_.get("wp_defect", 0.0)) * NS / ns
                 + w_.get("wp_basis", 0.0) * NR / nr)
        overlaps = w_["pairs"] * (NS * NR) / (ns * nr)
        err = np.abs(smp.p32 + smp.comp - smp.truth())
        print(json.dumps(dict(workload=cfg, pairs=NS * NR * len(bd["coeffs"]), cores=threads_used(),
                              defect_setup_s=setup, overlaps_s=overlaps, pairs_per_s=pps, extrapolated_s=secs,
                              max_abs_err_vs_fp64=float(err.max()), rms_abs_err_vs_fp64=float(np.sqrt((err ** 2).mean())),
                              sample=smp.describe())), flush=True)


def copy_rates(nbytes):
    """Host-to-device copy rates of nbytes (cudaMemcpyAsync through torch, CUDA events, best of
    three): from pinned and from pageable host memory."""
    import torch

    dev = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    out = {}
    for kind, pin in (("pinned_copy_gb_s", True), ("pageable_copy_gb_s", False)):
        host = torch.empty(nbytes, dtype=torch.uint8, pin_memory=pin)
        host.fill_(1)
        best = float("inf")
        for _ in range(3):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            a.record()
            dev.copy_(host, non_blocking=pin)
            b.record()
            torch.cuda.synchronize()
            best = min(best, a.elapsed_time(b))
        out[kind] = nbytes / best / 1e6
        del host
    del dev
    return out


def _time_reader(path, nwk, reps):
    from pawpyseed_gb300 import _lib

    L = _lib.lib()
    kws = np.full(nwk, 1.0 / nwk)
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        p = L.pawpy_gpu_read_wavefunctions(path.encode(), kws)
        _lib.check()
        ts.append(time.perf_counter() - t0)
        L.pawpy_gpu_free_pswf(p)
    return float(np.median(ts)) * 1e3


def run_ingest_report(args):
    """Per workload (64-atom, 216-atom): the defect WAVECAR written to a temporary directory (in the
    page cache), then read by pawpy_gpu_read_wavefunctions with the plane-wave spheres on the
    device, by the same reader in a process that sees no CUDA device (spheres on the host threads),
    and by the serial numpy restatement of reader.c; and the spheres alone (device, numpy)."""
    import tempfile

    from pawpyseed_gb300 import _lib, synth, vaspio

    if args.ingest_child:
        path, nwk = args.ingest_child.rsplit(":", 1)
        print(json.dumps(dict(ms=_time_reader(path, int(nwk), 5))), flush=True)
        return
    L = _lib.lib()
    for cfg in (1, 2):
        w = synth.small_workload(cfg)
        _, defect_s = synth.structures(cfg)
        data = synth.wavefunction_data(defect_s, w, 22 + 7 * cfg)
        with tempfile.TemporaryDirectory() as tmp:
            path = os.path.join(tmp, "WAVECAR")
            vaspio.write_wavecar(path, data["lattice"], data["encut"], data["kpts"], data["coeffs"],
                                 data["energies"], data["occs"], nspin=data["nspin"])
            size = os.path.getsize(path)
            nwk = data["nwk"]
            dev_ms = _time_reader(path, nwk, 5)
            env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
            r = subprocess.run([sys.executable, os.path.abspath(__file__), "--ingest-child", "%s:%d" % (path, nwk)],
                               env=env, capture_output=True, text=True, check=True)
            host_ms = json.loads(r.stdout.strip().splitlines()[-1])["ms"]
            t0 = time.perf_counter()
            vaspio.read_wavecar_numpy(path)
            numpy_ms = (time.perf_counter() - t0) * 1e3
            # the device's in-place read of the host band arrays (the end-to-end step's upload):
            # device time of its launches against plain host-to-device copies of the same bytes
            p = L.pawpy_gpu_read_wavefunctions(path.encode(), np.full(nwk, 1.0 / nwk))
            _lib.check()
            L.pawpy_gpu_upload(p)
            L.pawpy_gpu_synchronize()
            L.pawpy_gpu_release(p)
            _lib.kernel_stats(reset=True)
            L.pawpy_gpu_profile(1)
            L.pawpy_gpu_upload(p)
            L.pawpy_gpu_synchronize()
            L.pawpy_gpu_profile(0)
            st = _lib.kernel_stats(reset=True)
            L.pawpy_gpu_release(p)
            L.pawpy_gpu_free_pswf(p)
            coef_bytes = sum(int(c.nbytes) for c in data["coeffs"])
            read_ms = st.get("load_host", (float("nan"), 0))[0]
            link = dict(in_place_read_gb_s=coef_bytes / read_ms / 1e6, in_place_read_ms=read_ms)
            link.update(copy_rates(coef_bytes))
        lat = np.ascontiguousarray(np.asarray(data["lattice"], dtype=np.float64).reshape(-1))
        ks = [np.ascontiguousarray(k, dtype=np.float64) for k in np.asarray(data["kpts"]).reshape(-1, 3)]
        L.pawpy_gpu_gvectors(lat, ks[0], float(data["encut"]), None, 0)
        _lib.check()
        t0 = time.perf_counter()
        for k in ks:
            L.pawpy_gpu_gvectors(lat, k, float(data["encut"]), None, 0)
        sph_dev_ms = (time.perf_counter() - t0) * 1e3
        t0 = time.perf_counter()
        for k in ks:
            vaspio.gvectors(data["lattice"], k, data["encut"])
        sph_np_ms = (time.perf_counter() - t0) * 1e3
        print(json.dumps(dict(workload=cfg, wavecar_bytes=size, kpoints=len(ks), bands=data["nband"],
                              plane_waves=[int(g.shape[0]) for g in data["gs"]][:1],
                              reader_ms=dev_ms, reader_gb_s=size / dev_ms / 1e6,
                              reader_no_device_ms=host_ms, numpy_reader_ms=numpy_ms,
                              spheres_device_ms=sph_dev_ms, spheres_numpy_ms=sph_np_ms,
                              host_link=link, host_threads=threads_used())), flush=True)


def main():
    args = parse()
    if args.ingest_report or args.ingest_child:
        run_ingest_report(args)
        return
    if args.cpu_report:
        run_cpu_report(args)
        return
    rank, world, local, pg = dist_init(args.gpus)
    if args.precision_report:
        run_precision_report(args, local)
        return
    if args.impl == "reference":
        run_reference(args, rank, world, pg)
        return
    if args.serve:
        run_serve(args, rank, world, local)
        return
    res, work, acc, cpu = measure(args, args.workload, rank, world, local, pg, not args.no_cpu_baseline)
    w = work[0]
    del work
    secondary = None
    if args.secondary >= 0 and args.secondary != args.workload and args.bands is None and args.nk is None:
        r2, work2, acc2, cpu2 = measure(args, args.secondary, rank, world, local, pg, not args.no_cpu_baseline)
        if rank == 0:
            secondary = dict(config=config(args, args.secondary, work2[0], work2), value=r2["value"],
                             ms_per_step=r2["ms"], e2e=dict(value=r2["e2e_value"], ms_per_step=r2["e2e_ms"],
                                                            h2d_bytes_per_step=r2["h2d"],
                                                            d2h_bytes_per_step=r2["d2h"]),
                             accuracy=acc2, roofline=r2["roofline"], cpu_baseline=cpu2,
                             plain_fp32_form=r2["plain"], gpu_launches=r2["launches"],
                             kernel_ms=r2["kernel_ms"])
        del work2
    serve_res = None
    if not args.no_serve and args.bands is None and args.nk is None:
        serve_res = run_serve_streams(args, rank, local)
    if rank == 0:
        plain = res["plain"]
        if plain is not None:
            plain = dict(plain, bf16x3_over_fp32=res["value"] / plain["value"])
        line = dict(metric="band-pair projections/sec", value=res["value"], unit="pairs/s", n_gpus=world,
                    steps=args.steps, warmup=args.warmup, ms_per_step=res["ms"], higher_is_better=True,
                    scaling="weak", vs_baseline=None, dtype="c64 (fp32 accumulate) / f64 setup",
                    data="synthetic (seeded VASP-format WAVECAR/POTCAR content)",
                    config=config(args, args.workload, w, None) | {
                        "l2": "inputs larger than L2 (defect coefficients %.0f MB per step)" % (res["h2d"] / 1e6)},
                    e2e=dict(value=res["e2e_value"], unit="pairs/s", ms_per_step=res["e2e_ms"],
                             h2d_bytes_per_step=res["h2d"], d2h_bytes_per_step=res["d2h"]),
                    accuracy=acc, gpu_launches=res["launches"], roofline=res["roofline"], cpu_baseline=cpu,
                    clocks=res["clocks"], plain_fp32_form=plain,
                    resident_real_space_basis=res["resident_real_space_basis"],
                    kernel_ms=res["kernel_ms"], host_ms=res["host_ms"], secondary=secondary, serve=serve_res)
        print(json.dumps(line))


if __name__ == "__main__":
    main()

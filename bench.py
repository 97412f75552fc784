"""Band-pair projection throughput on one GB300 (pawpyseed aug_real path).

A step is the defect-side work of BasisExpansion-style analysis against a
resident basis: element setup (get_projector_list), <p|psi> of every defect
band (setup_projections: batched scatter + 3D FFT + sphere gather), the
overlap setup (overlap_setup_real: smoothed partial waves, N_RS pairs) and the
full PAW overlap matrix of every defect band against every basis band
(pseudo overlap + O_M + O_R + O_S + O_N). The metric counts band pairs
NB_R * NB_S * NK per step.

Workload (default): the 64-atom cubic 10.86 A cell, two species (A: l=0,0,1,1;
B: l=0,0,1,1,2,2), one A atom removed in the defect, 8 k-points (2x2x2 MP),
256 bands, ENCUT 400 eV (23,234 plane waves), FFT grid 60^3; synthetic seeded
coefficients (no dataset exists for this path).

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


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", type=int, default=1)
    ap.add_argument("--bands", type=int, default=None, help="reduced band count (testing only)")
    ap.add_argument("--nk", type=int, default=None, help="reduced k-point count (testing only)")
    ap.add_argument("--precision", default="bf16x3", choices=["fp32", "bf16x3", "tf32"])
    ap.add_argument("--cpu-sample-bands", type=int, default=16)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--serve", action="store_true",
                    help="replay the serving stream (Poisson requests against resident bases) instead")
    ap.add_argument("--requests", type=int, default=64)
    ap.add_argument("--rate", type=float, default=200.0, help="mean request arrival rate (1/s)")
    ap.add_argument("--slots", type=int, default=4, help="requests in flight at once")
    ap.add_argument("--budget-gb", type=float, default=100.0, help="device-memory admission budget")
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
                                       "--format=csv,noheader,nounits", "-lms", "100"],
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


# ---------------------------------------------------------------- our arm

def run_ours(args, rank, world, local, pg):
    import torch

    torch.cuda.set_device(local)
    from pawpyseed_gb300 import _lib
    from pawpyseed_gb300.wavefunction import Wavefunction, pack_species

    _lib.set_precision(args.precision)
    w, basis_s, defect_s, cr, bd, dd = make_workload(args.workload, args.bands, args.nk)
    L = _lib.lib()
    L.pawpy_gpu_set_host_projections(0)
    basis = Wavefunction.from_arrays(basis_s, cr, w["dim"], bd)
    wf = Wavefunction.from_arrays(defect_s, cr, w["dim"], dd)
    basis.check_c_projectors()  # resident basis (not timed)
    lists = site_lists(basis_s, defect_s, cr)
    M_R, M_S, N_R, N_S, NRS_R, NRS_S = lists
    P = _lib.ptr
    species = pack_species(cr)
    ge = wf.grid_encut()
    dimv = np.ascontiguousarray(wf.dim, dtype=np.int32)
    nk = wf.nwk * wf.nspin
    out = np.zeros((wf.nband, basis.nband * nk), np.complex128)
    pairs = basis.nband * wf.nband * nk

    def step():
        pps = L.get_projector_list(len(cr.pps), *species, ge)
        L.setup_projections(wf.wf_ptr, pps, len(cr.pps), len(defect_s), dimv, wf.nums, wf.coords)
        L.overlap_setup_real(basis.wf_ptr, wf.wf_ptr, basis.nums, wf.nums, basis.coords, wf.coords,
                             P(N_R), P(N_S), P(NRS_R), P(NRS_S), len(N_R), len(N_S), len(NRS_R))
        L.pawpy_gpu_project_all(out.reshape(-1), basis.wf_ptr, wf.wf_ptr, len(M_R), len(N_R), len(N_S),
                                len(NRS_R), P(M_R), P(M_S), P(N_R), P(N_S), P(NRS_R), P(NRS_S), 0)
        _lib.check()

    # ---- device-resident: coefficients already in HBM
    wf.upload()
    for _ in range(args.warmup):
        step()
    L.pawpy_gpu_synchronize()
    clocks = Clocks(local)
    barrier(pg)
    clocks.start()
    L.pawpy_gpu_launch_count(1)
    L.pawpy_gpu_timer_start()
    for _ in range(args.steps):
        step()
    ms = L.pawpy_gpu_timer_stop_ms()
    launches = L.pawpy_gpu_launch_count(0)
    clk = clocks.stop()
    _lib.check()
    barrier(pg)
    ms_step = max_over_ranks(pg, ms / args.steps)
    value = sum_over_ranks(pg, pairs) / (ms_step / 1e3)

    # ---- the plain FP32 form (CUDA-core contraction) on the same resident inputs, for comparison
    plain = None
    if args.precision != "fp32":
        _lib.set_precision("fp32")
        step()
        L.pawpy_gpu_synchronize()
        barrier(pg)
        L.pawpy_gpu_timer_start()
        for _ in range(args.steps):
            step()
        ms_fp32 = max_over_ranks(pg, L.pawpy_gpu_timer_stop_ms() / args.steps)
        plain = dict(value=sum_over_ranks(pg, pairs) / (ms_fp32 / 1e3), ms_per_step=ms_fp32)
        _lib.set_precision(args.precision)
        step()

    # ---- end to end: host pswf_t, H2D of the defect's coefficients and D2H of the matrix every step
    h2d = sum(c.nbytes for c in dd["coeffs"])
    d2h = out.nbytes
    L.pawpy_gpu_release(wf.wf_ptr)
    step()
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
    stats = _lib.kernel_stats(reset=True)
    roof = roofline(stats, w, basis, wf, lists, cr)

    result = dict(pairs_per_step=pairs, ms=ms_step, value=value, e2e_ms=e2e_step, e2e_value=e2e_value, plain=plain,
                  h2d=h2d, d2h=d2h, launches=launches // args.steps, clocks=clk, roofline=roof,
                  kernel_ms={k: v[0] for k, v in stats.items() if not k.startswith("host.")},
                  host_ms={k[5:]: v[0] for k, v in stats.items() if k.startswith("host.")})
    # correctness spot check of this run against itself being finite
    if not np.all(np.isfinite(out)):
        raise RuntimeError("non-finite overlaps")
    return result, (w, basis_s, defect_s, cr, bd, dd, lists)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), float(p["bf16_tflops"]), "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


def roofline(stats, w, basis, wf, lists, cr):
    """Dominant kernel family of one step: achieved algorithmic rate against the measured peak.

    Per-launch work is uniform within a family, so achieved = (units of the step x
    algorithmic bytes or flops per unit) / (device time of the family in the step).
    The FFT family is the two passes of the transform (fft_planes + fft_x_pick) with
    16 N^3 bytes per band-FFT (one complex64 read and write of the grid); the overlap
    GEMM counts 8 NB_R NB_S (W + K_aug) useful flops per k-point.
    """
    from pawpyseed_gb300 import vaspio

    hbm, tc, src = peaks()
    if not stats:
        return None
    fams = {}
    for name, (ms, n) in stats.items():
        if name.startswith("host."):
            continue
        key = "fft" if name.startswith("fft") else name
        a = fams.setdefault(key, [0.0, 0, []])
        a[0] += ms
        a[1] += n
        a[2].append(name)
    fam = max(fams, key=lambda k: fams[k][0])
    ms, n, members = fams[fam]
    secs = ms / 1e3
    nk = wf.nwk * wf.nspin
    N3 = int(np.prod(w["dim"]))
    W = float(vaspio.gvectors(wf.structure.lattice, w["kpts"][0], w["encut"]).shape[0])
    out = dict(kernel="+".join(members), launches=n, ms_per_launch=ms / max(n, 1), peak_source=src,
               traffic=None)
    if fam.startswith("gemm"):
        kc = comp_columns(cr, lists, basis, wf)
        flops = 8.0 * basis.nband * wf.nband * (W + kc) * nk
        ach = flops / secs / 1e12
        out.update(bound="tensor", achieved=ach, peak=tc, unit="TFLOP/s", frac=ach / tc)
    elif fam == "fft":
        nbytes = 16.0 * N3 * wf.nband * nk
        ach = nbytes / secs / 1e9
        out.update(bound="hbm", achieved=ach, peak=hbm, unit="GB/s", frac=ach / hbm,
                   algorithmic_bytes_per_band_fft=16.0 * N3)
        if tuple(w["dim"]) == (60, 60, 60):
            # DRAM bytes of both passes per band-FFT from one ncu capture of this workload's
            # launches (profiles/fft_passes_traffic_60cubed.md, launches of 256 bands, one
            # k-point): pass A 47.9 MB read + 195.0 MB written, pass B 261.2 MB read + 99.1 MB
            # written
            out.update(traffic=(47.9e6 + 195.0e6 + 261.2e6 + 99.1e6) / 256.0,
                       traffic_unit="bytes per band-FFT (ncu dram__bytes_read+write, both passes)")
    else:
        out.update(bound="hbm", achieved=None, peak=hbm, unit="GB/s", frac=None)
    return out


def comp_columns(cr, lists, basis, wf):
    tot = {e: sum(2 * l + 1 for l in cr.pps[e].ls) for e in cr.pps}
    M_R, M_S, N_R, N_S, NRS_R, NRS_S = lists
    kc = sum(tot[basis.structure.species[i]] for i in M_R)
    kc += sum(tot[basis.structure.species[i]] for i in N_R)
    kc += sum(tot[wf.structure.species[i]] for i in N_S)
    kc += sum(tot[basis.structure.species[i]] for i in NRS_R)
    return kc


# ---------------------------------------------------------------- CPU arm (oracle port)

def cpu_sample(work, nbands_s, repeat=1):
    """Oracle port (the reference algorithm in C+OpenMP) on k-point 0 and the first
    nbands_s defect bands against the full basis at that k-point. Returns
    (pairs/s, seconds per sample, pairs per sample)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc

    w, basis_s, defect_s, cr, bd, dd, lists = work

    def sub(d, nb):
        return dict(d, nwk=1, nspin=1, kpts=d["kpts"][:1], gs=d["gs"][:1],
                    coeffs=[d["coeffs"][0][:nb]], energies=d["energies"][:1, :nb], occs=d["occs"][:1, :nb],
                    nband=nb, weights=np.ones(1))

    ob = orc.OracleWavefunction(data=sub(bd, bd["nband"]), struct=basis_s, cr=cr, dim=w["dim"])
    ob.setup_projectors()  # resident basis, not timed
    M_R, M_S, N_R, N_S, NRS_R, NRS_S = [list(x) for x in lists]
    N_RS = list(zip(NRS_R, NRS_S))
    times = []
    for _ in range(repeat):
        t0 = time.perf_counter()
        ow = orc.OracleWavefunction(data=sub(dd, nbands_s), struct=defect_s, cr=cr, dim=w["dim"])
        ow.setup_projectors()
        op = orc.OracleProjector(ow, ob, lists=(M_R, M_S, N_R, N_S, N_RS))
        op.pseudo_full(fp32=True)
        op.comp_full()
        times.append(time.perf_counter() - t0)
    pairs = bd["nband"] * nbands_s
    t = float(np.median(times))
    return pairs / t, t, pairs


def cores():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def run_reference(args, rank, world, pg):
    """The reference algorithm's CPU implementation (oracle port), all host threads."""
    if rank != 0:
        return
    os.environ.setdefault("OMP_NUM_THREADS", str(cores()))
    work = make_workload(args.workload, args.bands, args.nk)
    w, basis_s, defect_s, cr = work[:4]
    work = work + (site_lists(basis_s, defect_s, cr),)
    nb_s = args.cpu_sample_bands
    for _ in range(args.warmup):
        cpu_sample(work, nb_s)
    rates, ts = [], []
    for _ in range(args.steps):
        r, t, pairs = cpu_sample(work, nb_s)
        rates.append(r)
        ts.append(t)
    value = float(np.median(rates))
    sample = ("k-point 0 of %d, %d of %d defect bands against all %d basis bands (%d pairs per step); "
              "defect setup + overlap setup + pseudo overlaps (FP32 accumulate) + PAW terms"
              % (len(w["kpts"]), nb_s, w["nband"], w["nband"], pairs))
    line = dict(metric="band-pair projections/sec", value=value, unit="pairs/s", n_gpus=args.gpus,
                steps=args.steps, warmup=args.warmup, ms_per_step=float(np.median(ts)) * 1e3,
                higher_is_better=True, scaling="weak", vs_baseline=None, dtype="c64/f64", data="synthetic",
                impl="reference",
                config=config(args, w, work),
                cpu_baseline=dict(value=value, unit="pairs/s", cores=cores(), kind="port", sample=sample),
                e2e=dict(value=value, unit="pairs/s", h2d_bytes_per_step=0, d2h_bytes_per_step=0))
    print(json.dumps(line))


def config(args, w, work=None):
    l2 = "inputs larger than L2"
    if work is not None:
        mb = [sum(c.nbytes for c in d["coeffs"]) / 1e6 for d in (work[4], work[5])]
        l2 += " (basis coefficients %.0f MB, defect coefficients %.0f MB)" % tuple(mb)
    return {"workload": "64-atom cubic 10.86 A A/B cell minus one A, 8 k-points (2x2x2 MP), %d bands, "
                        "ENCUT %g eV, FFT %dx%dx%d, aug_real" % (w["nband"], w["encut"], *w["dim"])
            if args.workload == 1 else "workload %d" % args.workload,
            "nband": w["nband"], "nk": len(w["kpts"]) * w["nspin"], "fft_grid": list(w["dim"]),
            "precision": args.precision, "l2": l2}


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


def main():
    args = parse()
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
    res, work = run_ours(args, rank, world, local, pg)
    w = work[0]
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        os.environ.setdefault("OMP_NUM_THREADS", str(cores()))
        r, t, pairs = cpu_sample(work, args.cpu_sample_bands)
        cpu = dict(value=r, unit="pairs/s", cores=cores(), kind="port",
                   sample="k-point 0, %d defect bands x %d basis bands (%d pairs) of the same workload, "
                          "%.1f s" % (args.cpu_sample_bands, w["nband"], pairs, t))
    if rank == 0:
        line = dict(metric="band-pair projections/sec", value=res["value"], unit="pairs/s", n_gpus=world,
                    steps=args.steps, warmup=args.warmup, ms_per_step=res["ms"], higher_is_better=True,
                    scaling="weak", vs_baseline=None, dtype="c64 (fp32 accumulate) / f64 setup",
                    data="synthetic (seeded VASP-format WAVECAR/POTCAR content)", config=config(args, w, work),
                    e2e=dict(value=res["e2e_value"], unit="pairs/s", ms_per_step=res["e2e_ms"],
                             h2d_bytes_per_step=res["h2d"], d2h_bytes_per_step=res["d2h"]),
                    gpu_launches=res["launches"], roofline=res["roofline"], cpu_baseline=cpu,
                    clocks=res["clocks"], kernel_ms=res["kernel_ms"], host_ms=res["host_ms"],
                    plain_fp32_form=res["plain"])
        print(json.dumps(line))


if __name__ == "__main__":
    main()

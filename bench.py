#!/usr/bin/env python
"""Benchmark of the mock-generation path: 256^3 realisations per second.

One step = one realisation of the single-box workload: Gaussian field
(nd = 256, Lc = 2 Mpc/h, L = 512 Mpc/h, synthetic BBKS P(k)), halo finding
with the ellipsoidal barrier (a = 1, beta = 0.12, alpha = 0), the top-hat
smoothing ladder of 50 log-spaced radii from one cell to 30 Mpc/h with its
per-cell first-crossing map, 2LPT displacement of the halos, CIC of the halo positions on a 256^3 grid and the
power spectrum in 128 bins.  Every step takes the next seed of the reference's own field stream (GSL taus, polar
deviates in its loop order), so both arms compute the same realisations.

  value   device-resident: C ABI calls with device buffers (k, P are the only
          inputs, 8 KB), halo positions and the grid stay in HBM
  e2e     the public Python API (mock.Generate_Halos_Box_from_Pk,
          lib.exshalos.smoothing_ladder, simulation.Compute_Density_Grid,
          simulation.Compute_Power_Spectrum)
          with host numpy arrays, copies in both directions inside the timing
  --impl reference
          the reference's CPU algorithm (the oracle's C restatement in the
          reference's float precision, GSL-taus field stream) on all host
          cores, one full 256^3 realisation per step

Multi-GPU: one process per GPU (torchrun); realisations are independent, so
every rank runs its own seeds (weak scaling) and value sums all ranks.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time
from concurrent.futures import ThreadPoolExecutor

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

ND, LC, NK_PK = 256, 2.0, 128
BARRIER = dict(a=1.0, beta=0.12, alpha=0.0)
# kernel classes whose time is set by dependent loads rather than bandwidth
LATENCY_NOTES = {
    "sort": "latency-bound: exact Lomuto order, dependent L2 loads along the > chains of each level "
            "(eight steps per load through per-level jump tables)",
    "grow": "latency-bound: per-peak shell gathers and reservation rounds",
    "mass": "per halo: one taus draw by jump-ahead, count-only tables, inverse-spline knot search and Horner step (FP64)",
    "halo_disp": "per-halo gathers over member cells",
}
N_RADII, R_LADDER = 50, 30.0
LADDER_SAMPLE = 5          # radii of the ladder timed on the host (each radius is the same work)
METRIC = "256^3 realisations/s (halos+P(k))"


def dist_init(backend="nccl"):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def aggregate_value(ws, steps, t_max):
    """Whole-job realisations per second: every rank runs `steps` of its own
    realisations, the job takes the slowest rank's time."""
    return ws * steps / t_max


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    INTERVAL_MS = 50

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []          # (monotonic time, csv line)
        self.windows = []

    def start(self):
        """Start nvidia-smi and wait (at most 5 s) for its first sample, so
        that the sampler is live when the timed region opens."""
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", str(self.INTERVAL_MS)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
            return
        t_end = time.monotonic() + 5.0
        while not self.lines and time.monotonic() < t_end and self.proc.poll() is None:
            time.sleep(0.01)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.monotonic(), line.strip()))

    def open_window(self):
        self.windows.append([time.monotonic(), None])

    def close_window(self):
        if self.windows and self.windows[-1][1] is None:
            self.windows[-1][1] = time.monotonic()

    def stop(self):
        """Median SM clock and the throttle reasons seen.  With windows
        (timed regions) marked, only the samples taken inside them count, and
        the sample before the first window is added when a window is shorter
        than the sampling interval and caught none."""
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        lines = self.lines
        if self.windows:
            inside = [(t, ln) for t, ln in lines
                      if any(a <= t <= (b if b is not None else float("inf")) for a, b in self.windows)]
            if not inside:
                before = [(t, ln) for t, ln in lines if t < self.windows[0][0]]
                inside = before[-1:]
            lines = inside
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for _, ln in lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 6:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[2:6]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        v = d.get("hbm_gbs") or d.get("hbm_GBs") or d.get("hbm")
        if isinstance(v, dict):
            v = v.get("value") or v.get("burst")
        return float(v), "measured"
    except (OSError, ValueError, TypeError):
        return 6800.0, "fallback"


def committed_traffic():
    """DRAM bytes per launch of the dominant kernel class from the committed
    ncu summary (profiles/*.txt lines 'traffic_per_launch <class> <bytes>')."""
    out = {}
    pdir = os.path.join(ROOT, "profiles")
    if not os.path.isdir(pdir):
        return out
    for fn in sorted(os.listdir(pdir)):
        if not fn.endswith(".txt"):
            continue
        with open(os.path.join(pdir, fn)) as f:
            for line in f:
                p = line.split()
                if len(p) == 3 and p[0] == "traffic_per_launch":
                    try:
                        out[p[1]] = float(p[2])
                    except ValueError:
                        pass
    return out


def cpu_baseline_sample(k, P, seed=1):
    """The reference algorithm on the host: one full 256^3 realisation (Lc = 2)
    with the GSL-taus field stream in float precision, all host threads."""
    from oracle import orc
    nthr = os.cpu_count() or 1
    orc.set_threads(nthr, prec="f32")
    nd = ND
    t0 = time.perf_counter()
    r = orc.halos_box_from_pk(k, P, nd=nd, Lc=LC, seed=seed, stream=0, do_2lpt=1, prec="f32", **BARRIER)
    g = orc.cic(r["posh"], nd, nd * LC, prec="f32")
    orc.power(g, nd * LC, window=2, Nk=NK_PK, prec="f32")
    dt = time.perf_counter() - t0
    # smoothing ladder: LADDER_SAMPLE of the N_RADII radii on the same modes,
    # scaled to the full ladder (a constant barrier; the cost is the transforms)
    p = orc.make_params(nd, LC, seed=seed)
    modes = orc.field_modes(p, k, P, stream=0, prec="f32")
    R = np.geomspace(LC, R_LADDER, N_RADII).astype(np.float32)[-LADDER_SAMPLE:]
    t1 = time.perf_counter()
    orc.ladder(p, modes, R, np.full(LADDER_SAMPLE, 1.686, dtype=np.float32), prec="f32")
    dt += (time.perf_counter() - t1) * N_RADII / LADDER_SAMPLE
    equiv = (nd / ND) ** 3
    return dt, equiv, nthr


MAX_SKIPPED = 16            # realisations skipped at most (range errors) before a run gives up


def run_seeds(fn, steps, first_seed, range_error, max_skipped=MAX_SKIPPED):
    """Call fn(seed) on seeds first_seed, first_seed + 1, ... until `steps`
    calls have completed.  A seed whose realisation raises `range_error` (a
    halo mass outside the mass-function splines, where the reference's
    gsl_spline_eval aborts, find_halos.c:472-474) is skipped, recorded and
    not counted; both arms of the benchmark use this policy on the same seed
    list.  Returns (results of the completed calls, completed seeds, skipped
    seeds)."""
    out, done, skipped = [], [], []
    s = first_seed
    while len(done) < steps:
        if len(skipped) > max_skipped:
            raise RuntimeError(f"more than {max_skipped} realisations failed with range errors")
        try:
            out.append(fn(s))
            done.append(s)
        except range_error:
            skipped.append(s)
        s += 1
    return out, done, skipped


def run_reference(args, ws, rank):
    from exshalos_gb300.workloads import synthetic_pk
    from oracle import orc
    if rank != 0:
        return
    k, P = synthetic_pk()
    k, P = k.astype(np.float32), P.astype(np.float32)
    run_seeds(lambda s: cpu_baseline_sample(k, P, seed=s), args.warmup, 100, orc.RangeError)
    res, done, skipped = run_seeds(lambda s: cpu_baseline_sample(k, P, seed=s), args.steps, 1, orc.RangeError)
    tot = sum(r[0] for r in res)
    eq = sum(r[1] for r in res)
    nthr = res[-1][2] if res else 1
    v = eq / tot
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "realisations/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * tot / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "box_256 (nd=256, Lc=2, L=512, 2LPT, barrier a=1 beta=0.12 alpha=0, CIC 256^3, "
                                   "P(k) 128 bins, 50-radius ladder)", "sample": "one full 256^3 realisation per step",
                       "field_stream": "the reference's (GSL taus seeded with the step's seed)",
                       "seeds": [done[0], done[-1]] if done else None, "skipped_seeds": skipped,
                       "skip_policy": "realisations whose halo masses leave the mass-function splines (the "
                                      "reference's GSL spline aborts there) are skipped and not timed"},
            "cpu_baseline": {"value": v, "unit": "realisations/s", "cores": nthr, "kind": "port",
                             "sample": "one 256^3 realisation (field, halos, 2LPT, CIC, P(k)) per step; ladder timed on "
                                       f"{LADDER_SAMPLE} of {N_RADII} radii and scaled"},
            "e2e": {"value": v, "unit": "realisations/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def step_algorithmic_bytes(nd, n_radii, nh):
    """Compulsory HBM bytes of one realisation (each 3-D FFT one read of its
    input and one write of its output, each fused stage once): field 8Nc,
    c2r 8Nc + 4N, ladder R (8Nc + 2N), peaks + growth 8N, 1LPT 8Nc + 20N,
    2LPT 52N + 16Nc, CIC + r2c + bins 12 nh + 8N + 16Nc."""
    N = float(nd) ** 3
    Nc = float(nd) * nd * (nd // 2 + 1)
    return (8 * Nc + (8 * Nc + 4 * N) + n_radii * (8 * Nc + 2 * N) + 8 * N + (8 * Nc + 20 * N) +
            (52 * N + 16 * Nc) + (12 * nh + 8 * N + 16 * Nc))


def _rel_rms(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.sqrt(np.mean((a - b) ** 2) / np.mean(b ** 2)))


def accuracy_summary(k, P, seed):
    """Error figures of one box_256 realisation (a timed seed), computed
    after the timed region: the catalogue against the oracle's Find_Halos on
    the GPU's float field (bit-exact or not), the field, the halo
    displacements, the CIC grid and the 128-bin P(k) against the FP64
    oracle (same positions / same grid), the whole chain's P(k) against the
    FP64 chain on the same catalogue, and the fraction of cells whose
    first-crossing radius in the 50-radius ladder differs from the FP64
    ladder's."""
    from exshalos_gb300 import simulation
    from exshalos_gb300.lib import exshalos as exl
    from oracle import orc
    nthr = os.cpu_count() or 1
    orc.set_threads(nthr, prec="f64")
    Lbox = ND * LC
    r = exl.halos_box_from_pk(k, P, 1e5, ND, ND, ND, LC, seed, 1e4, 0.31, 0.0, -1.0, 1, BARRIER["a"],
                              BARRIER["beta"], BARRIER["alpha"], 0, 0.0, 1, 0, 0, 1, 1, 0, 0, 1, _catalogue=True)
    r = {kk: np.array(v) for kk, v in r.items()}
    p = orc.make_params(ND, LC, seed=seed, **BARRIER)
    ref = orc.find_halos(p, r["grid"], orc.sigma_tables(p, k, P))
    same = bool(r["Mh"].size == ref["nh"] and np.array_equal(r["x"], ref["x"]) and
                np.array_equal(r["count"], ref["count"]) and
                np.array_equal(r["Mh"].view(np.uint32), ref["Mh"].view(np.uint32)) and
                np.array_equal(r["flag"].reshape(-1), ref["flag"]))
    modes = orc.field_modes(p, k, P, stream=0)
    e_field = _rel_rms(r["grid"], orc.field_real(p, modes))
    lp = orc.lpt_posh(p, k, P, ref["flag"], ref["x"], ref["count"], do_2lpt=1, modes=modes)
    centre = LC * (ref["x"] + 0.5)
    wrap = lambda d: (d + Lbox / 2) % Lbox - Lbox / 2          # noqa: E731
    dD = wrap(r["posh"].astype(np.float64) - lp["posh"])
    e_disp = float(np.sqrt(np.mean(dD ** 2) / np.mean(wrap(lp["posh"] - centre) ** 2)))
    grid = simulation.Compute_Density_Grid(r["posh"], nd=ND, L=Lbox, window="CIC")
    e_grid = _rel_rms(grid, orc.cic(r["posh"].astype(np.float64), ND, Lbox))
    pk = simulation.Compute_Power_Spectrum(grid, L=Lbox, window="CIC", Nk=NK_PK)
    kmin, kmax = np.float32(2 * np.pi / Lbox), np.float32(np.pi / Lbox * ND)
    want = orc.power(np.asarray(grid, dtype=np.float64), Lbox, window=2, Nk=NK_PK, kmin=kmin, kmax=kmax)
    m = want["Nk"] > 0
    chain = orc.power(orc.cic(lp["posh"], ND, Lbox), Lbox, window=2, Nk=NK_PK, kmin=kmin, kmax=kmax)
    cr = exl.smoothing_ladder(k, P, R_LADDER, ND, ND, ND, LC, seed=seed, n_radii=N_RADII, **BARRIER)
    want_cross = orc.ladder(orc.make_params(ND, LC, seed=seed), modes, cr["R"], cr["B"])
    return {"seed": int(seed), "halos": int(ref["nh"]), "catalogue_identical": same,
            "field_rel_rms_vs_fp64": e_field, "halo_displacement_rel_rms_vs_fp64": e_disp,
            "cic_rel_rms_vs_fp64": e_grid,
            "pk_counts_identical": bool(np.array_equal(pk["Nk"], want["Nk"])),
            "pk_max_rel_err_vs_fp64": float(np.max(np.abs(pk["Pk"][m] / want["Pk"][m] - 1))),
            "pk_chain_max_rel_err_vs_fp64": float(np.max(np.abs(pk["Pk"][m] / chain["Pk"][m] - 1))),
            "ladder_flip_fraction": float(np.mean(cr["cross"] != want_cross)),
            "ladder_crossed_fraction": float(np.mean(want_cross != 255)),
            "how": "one timed seed after the timed region; catalogue vs the oracle's Find_Halos on the GPU field; "
                   "field, halo displacements (same labelling), CIC (same positions), P(k) (same grid) and the "
                   "chain's P(k) (FP64 LPT -> CIC -> P(k) on the same catalogue) vs the FP64 oracle; flips vs the "
                   "FP64 ladder of the same modes"}


def field_stream_summary(k, P, reps=5):
    """The 256^3 Gaussian field alone (exh_density_grid_compute, device
    output) with each random stream: Philox (one counter-based block per
    mode, generated inside the first transform pass) and the reference's
    taus stream (deviates drawn in its loop order beforehand, then read by
    the same pass).  A new seed per call; CUDA events, median of reps."""
    import torch
    from exshalos_gb300 import _capi
    L_ = _capi.load()
    ctx = _capi.context()
    out = torch.empty(ND ** 3, dtype=torch.float32, device="cuda")
    res = {}
    for name in ("philox", "taus"):
        times = []
        for r in range(reps + 2):
            prm = _capi.default_params(ndx=ND, ndy=ND, ndz=ND, Lc=LC, seed=7000 + r,
                                       field_stream=_capi.field_stream_code(name))
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            _capi.check(L_.exh_density_grid_compute(ctx, _capi.ptr(k), _capi.ptr(P), k.size, prm, _capi.ptr(out),
                                                    _capi.EXH_MEM_DEVICE, None))
            e1.record()
            torch.cuda.synchronize()
            if r >= 2:
                times.append(e0.elapsed_time(e1))
        res[name + "_ms"] = round(float(np.median(times)), 4)
    res["workload"] = "field_256: the 256^3 Gaussian field (modes + inverse FFT), device output, new seed per call"
    return res


def fft_comparator_summary(sizes=(256, 512), reps=5):
    """The library's 3-D real FFT beside cuFFT (through torch.fft, which
    calls it), as a timing and accuracy comparator only: the same seeded
    float32 field, forward r2c and the r2c + c2r round trip, CUDA events
    (median of reps after two warm-ups), and both forward transforms
    against a cuFFT FP64 transform of the same field (relative rms over the
    half-complex modes).  The library's path uses its own kernels; nothing
    here feeds it."""
    import torch
    from exshalos_gb300 import _capi
    L_ = _capi.load()
    ctx = _capi.context()
    out = {}
    for nd in sizes:
        g = torch.Generator(device="cuda").manual_seed(11)
        x = torch.randn(nd, nd, nd, device="cuda", dtype=torch.float32, generator=g)
        y = torch.empty(nd, nd, nd, device="cuda", dtype=torch.float32)
        c = torch.empty(nd, nd, nd // 2 + 1, device="cuda", dtype=torch.complex64)

        def ours_fwd():
            _capi.check(L_.exh_fft_r2c_3d(ctx, nd, nd, nd, _capi.ptr(x), _capi.ptr(c), None))

        def ours_rt():
            ours_fwd()
            _capi.check(L_.exh_fft_c2r_3d(ctx, nd, nd, nd, _capi.ptr(c), _capi.ptr(y), None))

        def cufft_fwd():
            return torch.fft.rfftn(x)

        def cufft_rt():
            return torch.fft.irfftn(torch.fft.rfftn(x), s=(nd, nd, nd), norm="forward")

        def timed(f):
            ts = []
            for r in range(reps + 2):
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                f()
                e1.record()
                torch.cuda.synchronize()
                if r >= 2:
                    ts.append(e0.elapsed_time(e1))
            return round(float(np.median(ts)), 4)

        res = {"ours_r2c_ms": timed(ours_fwd), "cufft_r2c_ms": timed(cufft_fwd),
               "ours_roundtrip_ms": timed(ours_rt), "cufft_roundtrip_ms": timed(cufft_rt)}
        ref = torch.fft.rfftn(x.double())
        den = float(torch.sqrt(torch.mean(torch.abs(ref) ** 2)))
        ours_fwd()
        res["ours_r2c_rel_rms_vs_fp64"] = float(torch.sqrt(torch.mean(torch.abs(c.to(torch.complex128) - ref) ** 2))) / den
        res["cufft_r2c_rel_rms_vs_fp64"] = float(torch.sqrt(torch.mean(torch.abs(cufft_fwd().to(torch.complex128) - ref) ** 2))) / den
        del ref
        ours_rt()
        xs = float(torch.sqrt(torch.mean(x.double() ** 2)))
        res["ours_roundtrip_rel_rms"] = float(torch.sqrt(torch.mean((y.double() / nd ** 3 - x.double()) ** 2))) / xs
        res["cufft_roundtrip_rel_rms"] = float(torch.sqrt(torch.mean((cufft_rt().double() / nd ** 3 - x.double()) ** 2))) / xs
        out[f"fft_{nd}"] = res
        del x, y, c
        torch.cuda.empty_cache()
    out["how"] = ("seeded N(0,1) float32 field; library exh_fft_r2c_3d / exh_fft_c2r_3d (unnormalised, FFTW layout) "
                  "beside torch.fft.rfftn / irfftn(norm='forward') = cuFFT; forward transforms against cuFFT FP64")
    return out


def batched_summary(k, P, lanes, ws=1, rank=0):
    """Batched workload: 256 realisations with Philox seeds 0..255 and box
    sizes drawn uniformly from {64, 96, 128, 192, 256} (fixed draw), cell
    size 2 Mpc/h, halos (2LPT, barrier a=1 beta=0.12 alpha=0) and the 64-bin
    CIC P(k) of each; the lanes runner against the plain loop (one lane) on
    the same items.  Throughput in 256^3 equivalents (sum nd^3 / 256^3).
    With several ranks the box list is split by cell-count-balanced greedy
    bin packing (exshalos_gb300.shard), each rank runs its share on its own
    GPU and the slowest rank's time counts (weak scaling of the list)."""
    import torch
    from exshalos_gb300 import shard
    from exshalos_gb300.lib import exshalos as exl
    rng = np.random.default_rng(2024)
    nds_all = rng.choice([64, 96, 128, 192, 256], size=256)
    seeds_all = np.arange(256)
    parts, loads = shard.partition(nds_all, ws)
    mine = np.asarray(parts[rank], dtype=np.int64)
    nds, seeds = nds_all[mine], seeds_all[mine]
    eq = float(np.sum(nds_all.astype(np.float64) ** 3) / 256.0 ** 3)
    kw = dict(Lc=LC, Nk_pk=64, DO_2LPT=1, **BARRIER)
    exl.batch_run(k, P, nds, seeds + 1000, lanes=lanes, **kw)       # warm-up: buffers and plans of every lane
    exl.batch_run(k, P, nds[:8], seeds[:8] + 2000, lanes=1, **kw)
    out = {}
    res = {}
    for name, nl in (("plain", 1), ("batched", lanes)):
        barrier(ws)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res[name] = exl.batch_run(k, P, nds, seeds, lanes=nl, **kw)
        torch.cuda.synchronize()
        out[name] = eq / max_over_ranks(time.perf_counter() - t0, ws)
    same = all(np.array_equal(res["plain"][x], res["batched"][x]) for x in ("nh", "Pk", "Nk", "status"))
    same = max_over_ranks(0.0 if same else 1.0, ws) == 0.0
    failed = int(sum_over_ranks(float((res["batched"]["status"] != 0).sum()), ws))
    return {"workload": "batch_256: 256 boxes, nd ~ U{64,96,128,192,256} (seeded draw), Lc=2, Philox seeds 0..255, "
                        "2LPT, barrier a=1 beta=0.12, halos + CIC + 64-bin P(k) each",
            "unit": "256^3-equivalent realisations/s", "equivalents": round(eq, 3), "lanes": lanes,
            "value": out["batched"], "plain_loop_value": out["plain"], "speedup_vs_plain": out["batched"] / out["plain"],
            "identical_to_plain": bool(same), "failed_items": failed,
            "ranks": ws, "cells_per_rank": loads,
            "timing": "host wall clock around the synchronous batch call, slowest rank"}


def diff_summary(k, P, reps=3):
    """Differentiable workload: white noise 256^3 (unit Gaussian, seed 7)
    scaled by 20 log-spaced P(k) knots, 2LPT, CIC 256^3, 64-bin P(k), chi^2
    against the seed-8 spectrum; forward and hand-written adjoint timed with
    CUDA events (median of reps)."""
    import torch
    from exshalos_gb300 import diff
    nd, L = 256, 512.0
    knot_k, knot_P = diff.knots_from_spectrum(k, P, 20, 2 * np.pi / L, np.sqrt(3) * np.pi * nd / L * 1.01)
    model = diff.pk_chi2_model(nd, L, knot_k, Nk=64)
    g8 = torch.Generator(device="cuda").manual_seed(8)
    w8 = torch.randn((nd, nd, nd), generator=g8, device="cuda", dtype=torch.float32)
    _, target, _, _ = model.forward(w8, knot_P, np.ones(64, dtype=np.float32))
    g7 = torch.Generator(device="cuda").manual_seed(7)
    w = torch.randn((nd, nd, nd), generator=g7, device="cuda", dtype=torch.float32)
    gw = torch.empty_like(w)
    fw, bw = [], []
    for r in range(reps + 1):
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        torch.cuda.synchronize()
        e0.record()
        loss, _, _, _ = model.forward(w, knot_P, target)
        e1.record()
        model.backward(1.0, gw)
        e2.record()
        torch.cuda.synchronize()
        if r:
            fw.append(e0.elapsed_time(e1))
            bw.append(e1.elapsed_time(e2))
    f, b = float(np.median(fw)), float(np.median(bw))
    return {"workload": "diff_256: noise 256^3 seed 7, 20 knots, 2LPT, CIC 256^3, P(k) 64 bins, chi^2 vs seed 8",
            "forward_ms": round(f, 3), "adjoint_ms": round(b, 3), "adjoint_over_forward": round(b / f, 3),
            "loss": loss}


def galaxies_summary(k, P, reps=3, cpu=True):
    """Galaxy population of one 256^3 halo catalogue (seed 1, 2LPT, barrier
    a=1 beta=0.12, Lc=2; about 1e6 halos) with the reference's default HOD
    (Zheng 2005 parameters, sigma=0.5, taus seed 12345, nd=256 so satellites
    wrap): the device-resident C-ABI call timed with CUDA events (median of
    reps), the public host-array call and the colour split by wall clock, and
    the sequential oracle (the reference's algorithm, one thread) on the same
    catalogue."""
    import ctypes as C

    import torch
    from exshalos_gb300 import _capi, mock
    r = mock.Generate_Halos_Box_from_Pk(k, P, nd=ND, Lc=LC, seed=1, DO_2LPT=True, OUT_VEL=True, **BARRIER)
    posh, velh, Mh = r["posh"], r["velh"], r["Mh"]
    nh = Mh.size
    L_ = _capi.load()
    ctx = _capi.context()
    dpos, dvel, dM = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (posh, velh, Mh))
    prm = _capi.HodParams(LC, 0.31, 0.0, ND, ND, ND, 13.25424743, 0.26461332, 13.28383025, 14.32465146,
                          1.00811277, 0.5, -1.0, 12345)
    ng = C.c_int64(0)
    out_pos = out_vel = out_flag = None
    times = []
    for rep in range(reps + 1):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        _capi.check(L_.exh_hod_populate(ctx, dpos.data_ptr(), dvel.data_ptr(), dM.data_ptr(), None, nh,
                                        C.byref(prm), 1, C.byref(ng), _capi.EXH_MEM_DEVICE, None))
        if out_pos is None:
            n = int(ng.value)
            out_pos = torch.empty((n, 3), dtype=torch.float32, device="cuda")
            out_vel = torch.empty((n, 3), dtype=torch.float32, device="cuda")
            out_flag = torch.empty(n, dtype=torch.int64, device="cuda")
        _capi.check(L_.exh_hod_fetch(ctx, out_pos.data_ptr(), out_vel.data_ptr(), out_flag.data_ptr(),
                                     _capi.EXH_MEM_DEVICE, None))
        e1.record()
        torch.cuda.synchronize()
        if rep:
            times.append(e0.elapsed_time(e1))
    t_dev = float(np.median(times))
    n = int(ng.value)
    kw = dict(ndx=ND, ndy=ND, ndz=ND, Lc=LC, OUT_VEL=True, OUT_FLAG=True)
    mock.Generate_Galaxies_from_Halos(posh, Mh, velh=velh, **kw)
    t0 = time.perf_counter()
    g = mock.Generate_Galaxies_from_Halos(posh, Mh, velh=velh, **kw)
    t_e2e = time.perf_counter() - t0
    mock.Split_Galaxies(Mh, g["flag"])
    t0 = time.perf_counter()
    mock.Split_Galaxies(Mh, g["flag"])
    t_split = time.perf_counter() - t0
    base = None
    if cpu:
        from oracle import orc
        t0 = time.perf_counter()
        want = orc.populate_halos(posh, Mh, velh=velh, Lc=LC, nd=(ND, ND, ND), out_vel=True)
        t_cpu = time.perf_counter() - t0
        same = bool(np.array_equal(want["flag"], g["flag"]) and
                    np.max(np.abs(want["posg"] - g["posg"]), initial=0.0) < 1e-4)
        base = {"value": want["posg"].shape[0] / t_cpu, "unit": "galaxies/s", "cores": 1, "kind": "port",
                "ms": round(1000.0 * t_cpu, 3), "sample": "the whole catalogue, the reference's sequential algorithm",
                "speedup_device": round(t_cpu / (t_dev / 1000.0), 2), "speedup_e2e": round(t_cpu / t_e2e, 2),
                "identical_catalogue": same}
    return {"workload": "galaxies_256: halos of one 256^3 box (seed 1) populated with the default HOD, "
                        "positions + velocities + flags",
            "halos": int(nh), "galaxies": n, "random_satellite_draws": int(np.sum(Mh >= 10 ** 13.28383025)),
            "device_ms": round(t_dev, 3), "galaxies_per_s": n / (t_dev / 1000.0),
            "e2e_ms": round(1000.0 * t_e2e, 3), "split_e2e_ms": round(1000.0 * t_split, 3),
            "cpu_baseline": base,
            "timing": "device: CUDA events around exh_hod_populate + exh_hod_fetch on device arrays; "
                      "e2e/split/cpu: host wall clock"}


def run_ours(args, ws, rank, local):
    os.environ["EXH_DEVICE"] = str(local)
    import ctypes as C

    import torch
    torch.cuda.set_device(local)
    from exshalos_gb300 import _capi
    from exshalos_gb300 import mock, simulation
    from exshalos_gb300.lib import exshalos as exl
    from exshalos_gb300.workloads import synthetic_pk
    k, P = synthetic_pk()
    k, P = k.astype(np.float32), P.astype(np.float32)
    L_ = _capi.load()
    ctx = _capi.context()
    ng = ND ** 3
    Lbox = np.float32(ND * LC)
    kmin, kmax = np.float32(2 * np.pi / Lbox), np.float32(np.pi / Lbox * ND)
    posh_dev = torch.empty(3 * ng // 2, dtype=torch.float32, device="cuda")
    grid_dev = torch.empty(ng, dtype=torch.float32, device="cuda")
    k_out = np.zeros(NK_PK, dtype=np.float32)
    P_out = np.zeros(NK_PK, dtype=np.float32)
    c_out = np.zeros(NK_PK, dtype=np.int64)
    cross_dev = torch.empty(ng, dtype=torch.uint8, device="cuda")
    nh = C.c_int64(0)
    nh_seen = []
    # the ladder does not depend on the halo chain: it runs on its own library
    # context (own buffers) and stream, beside the halo finder, whose sort and
    # growth are latency-bound
    ctx_lad = C.c_void_p()
    _capi.check(L_.exh_ctx_create(local, C.byref(ctx_lad)))
    s_lad = torch.cuda.Stream()
    # the halo chain is the critical path: its stream gets the higher priority
    s_halo = torch.cuda.Stream(priority=-1)
    hs = C.c_void_p(s_halo.cuda_stream)

    def step(seed, serial=False):
        # serial: the ladder on the halo chain's stream (the per-class timing
        # pass, where each class's event time must cover its own kernels only)
        prm = _capi.default_params(ndx=ND, ndy=ND, ndz=ND, Lc=LC, seed=seed, DO_2LPT=1, **BARRIER)
        _capi.check(L_.exh_smoothing_ladder(ctx_lad, _capi.ptr(k), _capi.ptr(P), k.size, prm, N_RADII, R_LADDER,
                                            _capi.ptr(cross_dev), None, None, _capi.EXH_MEM_DEVICE,
                                            hs if serial else C.c_void_p(s_lad.cuda_stream)))
        _capi.check(L_.exh_halos_box_from_pk(ctx, _capi.ptr(k), _capi.ptr(P), k.size, prm, C.byref(nh), hs))
        _capi.check(L_.exh_halos_fetch(ctx, _capi.ptr(posh_dev), None, None, None, None, None, None, None, None,
                                       _capi.EXH_MEM_DEVICE, hs))
        _capi.check(L_.exh_grid_compute(ctx, _capi.ptr(posh_dev), nh.value, ND, float(Lbox), 2, 1,
                                        _capi.ptr(grid_dev), _capi.EXH_MEM_DEVICE, hs))
        _capi.check(L_.exh_power_compute(ctx, _capi.ptr(grid_dev), ND, float(Lbox), 2, NK_PK, float(kmin),
                                         float(kmax), _capi.ptr(k_out), _capi.ptr(P_out), _capi.ptr(c_out),
                                         _capi.EXH_MEM_DEVICE, hs))
        nh_seen.append(nh.value)

    # the same seed policy as the reference arm: a realisation whose halo
    # masses leave the mass-function splines is skipped (run_seeds)
    seed0 = 1000 * rank + 1
    # the timed seeds are screened in an untimed pass: the timed region then
    # holds exactly `steps` completed realisations, as the reference arm
    # counts them.  The warm-up seeds run after it, so that no context enters
    # the timed region holding the field draws of a timed seed
    _, done_seeds, skipped_seeds = run_seeds(step, args.steps, seed0, _capi.HaloRangeError)
    run_seeds(step, args.warmup, seed0 + 500, _capi.HaloRangeError)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    l0 = _capi.launch_count()
    barrier(ws)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks.open_window()
    ev0.record()
    s_lad.wait_stream(torch.cuda.current_stream())
    s_halo.wait_stream(torch.cuda.current_stream())
    for s in done_seeds:
        step(s)
    torch.cuda.current_stream().wait_stream(s_lad)
    torch.cuda.current_stream().wait_stream(s_halo)
    ev1.record()
    torch.cuda.synchronize()
    clocks.close_window()
    barrier(ws)
    launches = _capi.launch_count() - l0
    # per-kernel-class times come from a second pass of the same steps with
    # CUDA events around every launch (they add host work, so the headline
    # is timed without them); in that pass every stage runs on one stream
    # (the ladder on the halo chain's, the library's LPT without its fork)
    # and the ladder launches its kernels one by one
    _capi.timing_enable(True)
    clocks.open_window()
    for s in done_seeds:
        step(s, serial=True)
    torch.cuda.synchronize()
    clocks.close_window()
    clk = clocks.stop()
    clk["windows"] = "the timed steps and the per-class pass"
    rep = _capi.timing_report()
    _capi.timing_enable(False)
    t_dev = ev0.elapsed_time(ev1) / 1000.0
    t_max = max_over_ranks(t_dev, ws)
    value = aggregate_value(ws, args.steps, t_max)

    # end to end through the public API with host arrays, arranged as the
    # device-timed step: the ladder call in a worker thread on its own stream
    # (its own per-thread library context), the halo chain (halo box, CIC of
    # the halos, P(k)) on a high-priority stream in this thread; each step's
    # host outputs are consumed (byte counts) and dropped before the next, so
    # the library's host-buffer pool hands the same buffers out again
    e2e_steps = max(1, min(args.steps, 5))
    lad_pool = ThreadPoolExecutor(max_workers=1)
    s_lad_e2e = torch.cuda.Stream()
    s_halo_e2e = torch.cuda.Stream(priority=-1)
    sh_e2e = s_halo_e2e.cuda_stream

    def e2e_step(s):
        fut = lad_pool.submit(exl.smoothing_ladder, k, P, R_LADDER, ND, ND, ND, LC, seed=s, n_radii=N_RADII,
                              stream=s_lad_e2e.cuda_stream, **BARRIER)
        try:
            r = mock.Generate_Halos_Box_from_Pk(k, P, nd=ND, Lc=LC, seed=s, DO_2LPT=True, stream=sh_e2e, **BARRIER)
            grid = simulation.Compute_Density_Grid(r["posh"], nd=ND, L=float(Lbox), window="CIC", stream=sh_e2e)
            pk = simulation.Compute_Power_Spectrum(grid, L=float(Lbox), window="CIC", Nk=NK_PK, stream=sh_e2e)
        finally:
            cr = fut.result()
        n = r["posh"].shape[0]
        return (k.nbytes + P.nbytes + 12 * n + 4 * ng,
                cr["cross"].nbytes + 16 * n + 4 * ng + pk["k"].nbytes + pk["Pk"].nbytes + pk["Nk"].nbytes)

    run_seeds(e2e_step, min(args.warmup, 2), seed0 + 150, _capi.HaloRangeError)   # untimed: host buffers settle
    barrier(ws)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_bytes = run_seeds(e2e_step, e2e_steps, seed0 + 200, _capi.HaloRangeError)[0]
    torch.cuda.synchronize()
    t_e2e = max_over_ranks(time.perf_counter() - t0, ws)
    lad_pool.shutdown()
    e2e = ws * e2e_steps / t_e2e
    h2d = sum(b[0] for b in e2e_bytes)
    d2h = sum(b[1] for b in e2e_bytes)

    # roofline of the dominant kernel class (live CUDA-event timing); the
    # achieved figure is its algorithmic bytes over its event time
    dom = max(rep.items(), key=lambda kv: kv[1][0])
    name, (ms, nl, by) = dom
    peak, peak_kind = measured_peak()
    achieved = by / (ms / 1000.0) / 1e9 if nl and ms > 0 and by > 0 else None
    by_class = {}
    for kk, (cms, cnl, cby) in rep.items():
        if cnl and cms > 0 and cby > 0:
            gbs = cby / (cms / 1000.0) / 1e9
            by_class[kk] = {"gbs": round(gbs, 1), "frac": round(gbs / peak, 4), "launches": cnl,
                            "ms_per_launch": round(cms / cnl, 4)}
    traffic = committed_traffic().get(name)
    mean_nh = float(np.mean(nh_seen[-args.steps:])) if nh_seen else 0.0
    step_bytes = step_algorithmic_bytes(ND, N_RADII, mean_nh)
    step_gbs = step_bytes / (t_max / args.steps) / 1e9
    step_rf = {"algorithmic_bytes": step_bytes, "achieved": step_gbs, "peak": peak, "unit": "GB/s",
               "frac": step_gbs / peak,
               "note": "whole realisation: compulsory bytes of every stage over the step time; the sort and the "
                       "growth are latency-bound, so this stays far below the streaming passes' fractions"}
    accuracy = None
    if rank == 0 and not args.no_accuracy:
        accuracy = accuracy_summary(k, P, done_seeds[0])
    fields = field_stream_summary(k, P) if rank == 0 else None
    fft_cmp = fft_comparator_summary() if (rank == 0 and not args.no_batched) else None
    batched = None if args.no_batched else batched_summary(k, P, args.lanes, ws=ws, rank=rank)
    differentiable = None if args.no_batched else diff_summary(k, P)
    galaxies = None if args.no_batched else galaxies_summary(k, P, reps=5, cpu=not args.no_cpu_baseline)
    if rank != 0:
        return
    cpu = None
    if not args.no_cpu_baseline:
        dt, eq, nthr = cpu_baseline_sample(k, P)
        cpu = {"value": eq / dt, "unit": "realisations/s", "cores": nthr, "kind": "port",
               "sample": "one 256^3 realisation (field, halos, 2LPT, CIC, P(k)) in the reference's float "
                         f"arithmetic and GSL-taus field stream; ladder timed on {LADDER_SAMPLE} of {N_RADII} "
                         "radii and scaled"}
    line = {
        "metric": METRIC, "value": value, "unit": "realisations/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * t_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "box_256: nd=256, Lc=2 Mpc/h (L=512), synthetic BBKS P(k) sigma8=0.81, 2LPT, barrier "
                               "a=1 beta=0.12 alpha=0, 50-radius top-hat ladder + crossing map, CIC 256^3 of the halos, "
                               "P(k) 128 bins; new seed per step",
                   "field_stream": "the reference's (GSL taus seeded with the step's seed): the reference arm's "
                                   "realisations",
                   "l2": "inputs and intermediates (>1 GB per realisation) exceed L2",
                   "smoothing_ladder": f"{N_RADII} radii, Lc..{R_LADDER} Mpc/h, u8 first-crossing map",
                   "class_timing": "stage_ms_per_step, roofline_by_class and roofline from a second pass of the "
                                   "same number of steps with CUDA events around every launch, all stages on one stream "
                                   "(no overlap, so each class's time is its own kernels')",
                   "mean_halos": float(np.mean(nh_seen[-args.steps:])) if nh_seen else None,
                   "seeds": [done_seeds[0], done_seeds[-1]], "skipped_seeds": skipped_seeds},
        "e2e": {"value": e2e, "unit": "realisations/s", "h2d_bytes_per_step": int(h2d / e2e_steps),
                "d2h_bytes_per_step": int(d2h / e2e_steps), "steps": e2e_steps,
                "arrangement": "host wall clock around the public Python calls with host arrays: smoothing_ladder "
                               "in a worker thread on its own stream, Generate_Halos_Box_from_Pk -> "
                               "Compute_Density_Grid -> Compute_Power_Spectrum on a high-priority stream"},
        "gpu_launches": int(launches),
        "step_roofline": step_rf,
        "roofline": {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "peak_source": peak_kind,
                     "traffic": traffic, "launches": nl, "ms_total": ms,
                     "note": LATENCY_NOTES.get(name, "streaming passes against the HBM copy peak")},
        "stage_ms_per_step": {kk: round(v[0] / args.steps, 4) for kk, v in rep.items() if v[1]},
        "roofline_by_class": by_class,
        "clocks": clk,
        "cpu_baseline": cpu,
        "accuracy": accuracy,
        "field_streams": fields,
        "fft_comparator": fft_cmp,
        "batched": batched,
        "differentiable": differentiable,
        "galaxies": galaxies,
    }
    print(json.dumps(line), flush=True)


def run_box512(args, ws, rank, local):
    """Large box: nd = 512, L = 1024 Mpc/h, 2LPT, ~8e6 halos plus the 512^3
    particle catalogue, CIC of the 512^3 particles on 512^3 and P(k) in 256
    bins.  Reports realisations/s and the algorithmic-byte GB/s of every
    kernel class (FFT passes, stencils, CIC, binning) from CUDA events."""
    import ctypes as C

    import torch
    torch.cuda.set_device(local)
    from exshalos_gb300 import _capi
    from exshalos_gb300.workloads import synthetic_pk
    k, P = synthetic_pk()
    k, P = k.astype(np.float32), P.astype(np.float32)
    L_ = _capi.load()
    ctx = _capi.context()
    nd, nk_pk = 512, 256
    ng = nd ** 3
    Lbox = float(nd * LC)
    kmin, kmax = np.float32(2 * np.pi / Lbox), np.float32(np.pi / Lbox * nd)
    pos = torch.empty(3 * ng, dtype=torch.float32, device="cuda")
    grid = torch.empty(ng, dtype=torch.float32, device="cuda")
    k_out = np.zeros(nk_pk, dtype=np.float32)
    P_out = np.zeros(nk_pk, dtype=np.float32)
    c_out = np.zeros(nk_pk, dtype=np.int64)
    nh = C.c_int64(0)
    seen = []

    def step(seed):
        prm = _capi.default_params(ndx=nd, ndy=nd, ndz=nd, Lc=LC, seed=seed, DO_2LPT=1, OUT_LPT=1, **BARRIER)
        _capi.check(L_.exh_halos_box_from_pk(ctx, _capi.ptr(k), _capi.ptr(P), k.size, prm, C.byref(nh), None))
        _capi.check(L_.exh_halos_fetch(ctx, None, None, None, None, None, None, _capi.ptr(pos), None, None,
                                       _capi.EXH_MEM_DEVICE, None))
        _capi.check(L_.exh_grid_compute(ctx, _capi.ptr(pos), ng, nd, Lbox, 2, 1, _capi.ptr(grid),
                                        _capi.EXH_MEM_DEVICE, None))
        _capi.check(L_.exh_power_compute(ctx, _capi.ptr(grid), nd, Lbox, 2, nk_pk, float(kmin), float(kmax),
                                         _capi.ptr(k_out), _capi.ptr(P_out), _capi.ptr(c_out),
                                         _capi.EXH_MEM_DEVICE, None))
        seen.append(nh.value)

    for w in range(args.warmup):
        step(500 + w)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    _capi.timing_enable(True)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks.open_window()
    ev0.record()
    for s in range(args.steps):
        step(1 + s)
    ev1.record()
    torch.cuda.synchronize()
    clocks.close_window()
    rep = _capi.timing_report()
    _capi.timing_enable(False)
    clk = clocks.stop()
    t = ev0.elapsed_time(ev1) / 1000.0
    peak, peak_kind = measured_peak()
    by_class = {}
    for kk, (cms, cnl, cby) in rep.items():
        if cnl and cms > 0:
            gbs = cby / (cms / 1000.0) / 1e9 if cby > 0 else None
            by_class[kk] = {"ms_per_step": round(cms / args.steps, 3), "launches_per_step": cnl / args.steps,
                            "gbs": round(gbs, 1) if gbs else None,
                            "frac": round(gbs / peak, 4) if gbs else None,
                            "note": LATENCY_NOTES.get(kk, "streaming passes against the HBM copy peak")}
    line = {"metric": "512^3 realisations/s (halos + 512^3 particles + CIC + P(k))", "value": args.steps / t,
            "unit": "realisations/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * t / args.steps, "higher_is_better": True, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "box_512: nd=512, Lc=2 Mpc/h (L=1024), 2LPT, barrier a=1 beta=0.12 alpha=0, "
                                   "OUT_LPT 512^3 particles, CIC 512^3, P(k) 256 bins; new seed per step",
                       "mean_halos": float(np.mean(seen[-args.steps:]))},
            "peak_gbs": peak, "peak_source": peak_kind, "kernel_classes": by_class, "clocks": clk}
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_fft512(args, local):
    """Kernel workload: a 512^3 real-to-complex transform and its inverse,
    device-resident (1.1 GB: the real grid and the half-complex modes), each
    direction three passes (row pass, y pass, x pass).  Reports ms per
    transform and per kernel class with algorithmic GB/s (each pass one read
    of its input and one write of its output) against the HBM copy peak."""
    import torch
    torch.cuda.set_device(local)
    from exshalos_gb300 import _capi
    L_ = _capi.load()
    ctx = _capi.context()
    nd = 512
    nc = nd // 2 + 1
    g = torch.Generator(device="cuda").manual_seed(5)
    x = torch.randn(nd ** 3, device="cuda", generator=g)
    kx = torch.empty(nd * nd * nc * 2, device="cuda")

    def step():
        _capi.check(L_.exh_fft_r2c_3d(ctx, nd, nd, nd, _capi.ptr(x), _capi.ptr(kx), None))
        _capi.check(L_.exh_fft_c2r_3d(ctx, nd, nd, nd, _capi.ptr(kx), _capi.ptr(x), None))
        x.mul_(1.0 / nd ** 3)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    _capi.timing_enable(True)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(args.steps):
        step()
    ev1.record()
    torch.cuda.synchronize()
    rep = _capi.timing_report()
    _capi.timing_enable(False)
    peak, peak_kind = measured_peak()
    classes = {}
    for kk, (cms, cnl, cby) in rep.items():
        if cnl and cms > 0:
            gbs = cby / (cms / 1000.0) / 1e9 if cby > 0 else None
            classes[kk] = {"ms_per_launch": round(cms / cnl, 4), "launches": cnl,
                           "gbs": round(gbs, 1) if gbs else None, "frac": round(gbs / peak, 4) if gbs else None}
    print(json.dumps({"workload": "fft_512: r2c + c2r of a 512^3 grid, device-resident",
                      "ms_per_roundtrip": ev0.elapsed_time(ev1) / args.steps, "peak_gbs": peak,
                      "peak_source": peak_kind, "kernel_classes": classes}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-workload summary")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the error figures against the FP64 oracle")
    ap.add_argument("--lanes", type=int, default=12, help="lanes of the batched runner")
    ap.add_argument("--workload", default="box_256", choices=["box_256", "box_512", "galaxies_256", "fft_512"],
                    help="box_256: the headline line; box_512: the large-box kernel-class report; "
                         "galaxies_256: the galaxy-population summary alone; fft_512: a 512^3 FFT round trip "
                         "per kernel class")
    args = ap.parse_args()
    ws, rank, local = dist_init()
    if args.impl == "reference":
        run_reference(args, ws, rank)
    elif args.workload == "box_512":
        run_box512(args, ws, rank, local)
    elif args.workload == "fft_512":
        if rank == 0:
            run_fft512(args, local)
    elif args.workload == "galaxies_256":
        if rank == 0:
            os.environ["EXH_DEVICE"] = str(local)
            import torch
            torch.cuda.set_device(local)
            from exshalos_gb300.workloads import synthetic_pk
            k, P = synthetic_pk()
            print(json.dumps(galaxies_summary(k.astype(np.float32), P.astype(np.float32), reps=5,
                                              cpu=not args.no_cpu_baseline)), flush=True)
    else:
        run_ours(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

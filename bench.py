"""Benchmark: batched 2-D IM spectra/s on one GB300.

Workload: 4096 independent Demographics2D.IM integrations (parameters drawn
from numpy default_rng(0): s ~ U(.05,.95); nu1, nu2 log-uniform on [.01,100];
T log-uniform on [.01,2]; m12, m21 ~ U(0,10)), each on the default grids
pts [80, 90, 100], from_phi at ns (40,40), quadratic Richardson extrapolation
and the Poisson log-likelihood against synthetic data
Poisson(5e4 * model(first parameter set)).  A step is one pass of the batched
engine over the whole 4096-instance batch.  Synthetic data stands in for an
observed spectrum (none is used by the reference's benchmark).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--serve R] [--no-adjoint] [--no-config2]

`value` times the engine with the parameters already on the device; `e2e`
times the public API call (host parameter and data arrays in, host spectra and
likelihoods out).  --impl reference times the CPU integrator restatement
(the reference's algorithm: Python time loop over C sweeps) on all host
cores over a bounded stratified sample and scales it to the workload by
point-sweeps; it imports nothing of the GPU package.  `parity` compares the
GPU batch's spectra with the oracle's on the stratified 64-instance sample
that the CPU baseline integrates.  `serving` reports p50/p99 latency and
spectra/s of a served mixed request stream; `adjoint` the time of 256 IM and
32 three-population likelihood gradients; `config2` the three-population
growth model at pts [70,80,90].
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

# the serving leg keeps ~26 streams busy at once: give each its own hardware
# queue (must be set before CUDA starts)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))

METRIC = ("2D IM spectra/s batched vs plain on GB300 @≤1e-9 rel err; "
          "served p50/p99 latency")
PTS_L = (80, 90, 100)
NS = (40, 40)
NINST = 4096
BYTES_PER_PS = 16      # algorithmic HBM bytes per point-sweep (phi read + write)
FLOPS_PER_PS = 30      # algorithmic FP64 flops per point-sweep (reference formulation)
# FP64 thread instructions per point-sweep in k_integrate2d, from ncu
# counters (sm__sass_thread_inst_executed_op_fp64_pred_on.sum over the
# point-sweeps of 1024 seed-0 instances, all three grids): 10.40 (the
# recurrence's 10 per point plus the per-step vector builds)
FP64_INSTR_PER_PS = 10.4
# ncu dram__bytes_read.sum + dram__bytes_write.sum of the integration of one
# full step of this workload, by launch mode: one mixed launch, or the three
# launches of per_grid (L = 100 and L = 80 with two items per CTA: 1.061 +
# 0.319 GB and 0.997 + 0.176 GB; L = 90 one item per CTA: 1.033 + 0.245 GB)
K2_TRAFFIC_BYTES = {"persistent": 2.89e9 + 0.886e9,
                    "per_grid": (1.0611 + 1.0325 + 0.9971) * 1e9 + (318.70 + 244.73 + 175.57) * 1e6}


def im_draws(n, seed):
    rng = np.random.default_rng(seed)
    s = rng.uniform(0.05, 0.95, n)
    nu1 = np.exp(rng.uniform(np.log(0.01), np.log(100), n))
    nu2 = np.exp(rng.uniform(np.log(0.01), np.log(100), n))
    T = np.exp(rng.uniform(np.log(0.01), np.log(2), n))
    m12 = rng.uniform(0, 10, n)
    m21 = rng.uniform(0, 10, n)
    return np.stack([s, nu1, nu2, T, m12, m21], axis=1)


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"




class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0, period_ms=500):
        self.index = index
        self.period_ms = max(int(period_ms), 100)
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", str(self.period_ms)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        busy = [s for s in sm if s > 0.5 * max(sm)] or sm
        return {"sm_mhz": float(np.median(busy)), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("BENCH_BACKEND") != "gloo" else "gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(torch, world, x):
    """The largest x over the ranks (the job's time is its slowest rank's)."""
    if world == 1:
        return x
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_draws(rank):
    """Rank r integrates its own 4096 instances, drawn like the workload's
    with seed r (weak scaling: per-GPU work is fixed as ranks are added;
    ranks exchange nothing but the timing)."""
    return im_draws(NINST, rank)


def _cand_name(c):
    """Autotuner candidate (mode, gam placement, threads) as a JSON key."""
    mode, gam, threads = c
    return "%s/%s/%s" % (mode, "shared" if gam == 1 else "workspace",
                         "auto" if threads == 0 else "%d threads" % threads)


def job_value(world, ms_per_step):
    """Whole-job spectra/s: every rank's instances over the slowest rank's
    step time."""
    return world * NINST / (ms_per_step / 1e3)


def point_sweeps(steps, pts_l):
    return int(np.sum(steps)) * int(sum(2 * L * L for L in pts_l))


# ------------------------------------------------------------------ CPU arm

WORKLOAD = ("batched 2-D IM, 4096 instances, pts [80,90,100], ns (40,40), "
            "extrapolated + Poisson and multinomial ll")


def workload_config(world, ps):
    """The `config` of both arms' lines (identical, so the two are the same
    workload)."""
    return {"workload": WORKLOAD, "global_batch": NINST * world, "pts_l": list(PTS_L),
            "ns": list(NS), "point_sweeps_per_step": int(ps),
            "parallelism": "replicas x%d" % world,
            "l2": "flushed between iterations (256 MB write); phi outputs 803 MB > L2"}


def _cpu_one(args):
    """One extrapolated IM spectrum and its Poisson and multinomial
    log-likelihoods on the CPU restatement (Python time loop over the C
    sweeps, as the reference runs).  Returns (index, seconds, spectrum)."""
    i, p, pts_l, ns, obs = args
    from oracle import numerics as onum
    t = time.perf_counter()
    fs = onum.extrap_model(onum.IM, p, ns, pts_l)
    mask = onum.corner_mask(fs.shape)
    onum.ll(5e4 * fs, obs, mask)
    onum.ll_multinom(fs, obs, mask)
    return i, time.perf_counter() - t, np.asarray(fs)


def oracle_steps(draws):
    """Steps of each instance's schedule, walked by the oracle (the
    reference's loop restated in C)."""
    from oracle import clib
    clib.build()
    return clib.im_steps(draws)


def oracle_obs(draws):
    """The observed spectrum as both arms make it: Poisson(5e4 * model(set 0))."""
    from oracle import numerics as onum
    fs0 = onum.extrap_model(onum.IM, draws[0], NS, PTS_L)
    return np.random.default_rng(0).poisson(5e4 * fs0).astype(np.float64)


def parity_sample(draws, steps):
    """The stratified 64-instance sample (draws 0-5, the longest and shortest
    schedules, each parameter's extremes, step-count quantiles)."""
    import cases
    return cases.im_parity_sample(draws, steps, 64)


def cpu_rate(draws, steps, idx, cores, obs, pool=None):
    """Spectra/s of the CPU restatement on `cores` processes for the sample
    idx, scaled to the workload by point-sweeps: cores x (sample point-sweeps
    / summed per-instance seconds) -- the throughput of the cores kept busy,
    as the whole workload would keep them.  Returns (value, info, spectra by
    instance)."""
    import multiprocessing as mp
    ps_per_inst = steps * sum(2 * L * L for L in PTS_L)
    total_ps = float(np.sum(ps_per_inst))
    order = sorted(idx, key=lambda i: -steps[i])  # longest first packs best
    own = pool is None
    if own:
        pool = mp.get_context("spawn").Pool(cores)
    try:
        t0 = time.perf_counter()
        res = list(pool.imap_unordered(_cpu_one, [(int(i), draws[i], PTS_L, NS, obs)
                                                  for i in order], chunksize=1))
        wall = time.perf_counter() - t0
    finally:
        if own:
            pool.close()
            pool.join()
    task_s = float(sum(r[1] for r in res))
    sample_ps = float(np.sum(ps_per_inst[list(idx)]))
    value = len(draws) * (cores * sample_ps / task_s) / total_ps
    info = {"instances": len(idx), "point_sweeps": sample_ps, "task_s": task_s, "wall_s": wall}
    return value, info, {r[0]: r[2] for r in res}


def parity_of(fs_gpu, fs_cpu):
    """Spectrum parity of the GPU batch's spectra against the oracle's over
    the instances in fs_cpu: entries >= 1e-12 of a spectrum's largest
    compared relatively, smaller ones absolutely relative to the largest
    (the tests' spectrum bar)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import util
    worst, worst_small, n_small, worst_i = 0.0, 0.0, 0, None
    for i, ref in fs_cpu.items():
        rel, ab, ns = util.fs_parity(fs_gpu[i], ref)
        if rel > worst:
            worst, worst_i = rel, int(i)
        worst_small = max(worst_small, ab)
        n_small += ns
    return {"n_checked": len(fs_cpu), "max_rel": worst, "worst_instance": worst_i,
            "n_small": n_small, "max_abs_small_over_max": worst_small,
            "bar": "max_rel <= %g over entries >= %g x max; smaller entries <= %g x max "
                   "absolutely (the reference's own rounding noise sets the level)"
                   % (util.FS_REL, util.TINY_FRAC, util.FS_REL * util.TINY_FRAC),
            "pass": bool(worst <= util.FS_REL and worst_small <= util.FS_REL * util.TINY_FRAC),
            "against": "the oracle (the reference's algorithm, bit-identical to dadi's "
                       "golden vectors) on the stratified 64-instance sample"}


def run_reference(a, world, rank):
    """The reference's algorithm (the oracle port: Python time loop over the
    C sweeps, as dadi runs) on all host cores.  Each step integrates one
    quarter of the stratified 64-instance sample (16 instances spread over the
    step-count quantiles), scaled to the workload by point-sweeps.  Nothing
    of the GPU package is imported."""
    if rank != 0:
        return 0
    import multiprocessing as mp
    draws = im_draws(NINST, 0)
    steps = oracle_steps(draws)
    ps = point_sweeps(steps, PTS_L)
    obs = oracle_obs(draws)
    idx = parity_sample(draws, steps)
    by_cost = sorted(idx, key=lambda i: steps[i])
    slices = [by_cost[r::4] for r in range(4)]
    cores = os.cpu_count() or 1
    vals = []
    with mp.get_context("spawn").Pool(cores) as pool:
        for it in range(a.warmup + a.steps):
            v, info, _ = cpu_rate(draws, steps, slices[it % 4], cores, obs, pool)
            if it >= a.warmup:
                vals.append((v, info))
    v = float(np.mean([x[0] for x in vals]))
    info = vals[-1][1]
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "spectra/s", "n_gpus": a.gpus,
        "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": float(np.mean([x[1]["wall_s"] for x in vals])) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seed-0 IM parameter draws; observed spectrum Poisson(5e4*model))",
        "config": workload_config(world, ps),
        "cpu_baseline": {"value": v, "unit": "spectra/s", "cores": cores, "kind": "port",
                         "sample": "per step 16 of the stratified 64 seed-0 instances "
                                   "(%.3g point-sweeps, %.1f s of CPU on %d processes), "
                                   "scaled to the 4096-instance workload by point-sweeps"
                                   % (info["point_sweeps"], info["task_s"], cores)},
        "e2e": {"value": v, "unit": "spectra/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------ GPU arm

def run_ours(a, world, rank, local):
    import torch
    torch.cuda.set_device(local)
    from dadi_gb300 import batch, build
    build.build()
    draws = replica_draws(rank)
    rec = batch.im_instances(draws)
    steps = batch.count_steps(rec)   # host walk of the same schedules: point-sweep count
    ps = point_sweeps(steps, PTS_L)
    eng = batch.Batch2D(PTS_L, NS, gam_placement=a.gam)
    tuned = None
    if a.launch:
        eng.launch_mode = a.launch
    elif a.gam == 0 and not a.no_tune:
        # launch configuration chosen by timing the candidates on a sample
        from dadi_gb300 import autotune
        tuned = autotune.tune_batch2d(eng, rec)
    # synthetic observed data: Poisson(5e4 * model(set 0)), as a device tensor
    fs0, _, _ = eng.run(im_draws(1, 0))
    obs = np.random.default_rng(0).poisson(5e4 * fs0.cpu().numpy()[0]).astype(np.float64)
    d_obs = torch.from_numpy(obs).cuda()
    flush = torch.empty(256 * 1024 * 1024 // 8, dtype=torch.float64, device="cuda")
    def step_device():
        # one pass of the engine over the batch with the parameters prepared
        # on the device side of the API: device schedules, the integration,
        # and the epilogue (from_phi, extrapolation, likelihood) all run on
        # the GPU, in 5 launches
        phis, status = eng.integrate(rec)
        fs, ll, llm = eng.spectra_ll(phis, d_obs, 5e4, multinom=True)
        return fs, ll, status

    # warm-up
    warm_ms = []
    for _ in range(a.warmup):
        w0 = torch.cuda.Event(enable_timing=True)
        w1 = torch.cuda.Event(enable_timing=True)
        w0.record()
        step_device()
        w1.record()
        torch.cuda.synchronize()
        warm_ms.append(w0.elapsed_time(w1))

    # timed region: per-kernel events around the integration for the roofline
    clocks = ClockSampler(local, a.clock_ms)
    if a.clock_ms > 0:
        clocks.start()
    kern_ms = []
    barrier(world)
    torch.cuda.synchronize()
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    total_ms = 0.0
    for _ in range(a.steps):
        flush.fill_(1.0)  # L2 flush between iterations (256 MB > 129 MB L2)
        torch.cuda.synchronize()
        k0 = torch.cuda.Event(enable_timing=True)
        k1 = torch.cuda.Event(enable_timing=True)
        t_start.record()
        phis, status = eng.integrate(rec, timer=(k0, k1))
        fs, ll, llm = eng.spectra_ll(phis, d_obs, 5e4, multinom=True)
        t_end.record()
        torch.cuda.synchronize()
        total_ms += t_start.elapsed_time(t_end)
        kern_ms.append(k0.elapsed_time(k1))
    barrier(world)
    clk = clocks.stop()
    total_ms = max_over_ranks(torch, world, total_ms)
    ms_per_step = total_ms / a.steps
    value = job_value(world, ms_per_step)
    bad = int((status != 0).sum())
    # the scores of the workload: Poisson ll of 5e4 * model and the
    # multinomial ll (optimal scaling) against the observed spectrum
    ll_h, llm_h = ll.cpu().numpy(), llm.cpu().numpy()
    fs_last = fs.cpu().numpy()
    scores = {"ll_set0": float(ll_h[0]), "ll_multinom_set0": float(llm_h[0]),
              "ll_best": float(np.nanmax(ll_h)), "ll_multinom_best": float(np.nanmax(llm_h))}

    # end to end through the public API (host arrays in and out)
    e2e_ms = 0.0
    h2d = draws.nbytes + obs.nbytes
    d2h = 0
    for _ in range(max(1, a.steps)):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fs_d, ll_d, st_d = eng.run(draws, data=obs, scale=5e4)
        fs_h = fs_d.cpu().numpy()
        ll_h = ll_d.cpu().numpy()
        e2e_ms += (time.perf_counter() - t0) * 1e3
        d2h = fs_h.nbytes + ll_h.nbytes
    e2e_ms = max_over_ranks(torch, world, e2e_ms / max(1, a.steps))
    e2e_value = world * NINST / (e2e_ms / 1e3)

    # plain one-at-a-time drop-in path on a sample, scaled by point-sweeps
    plain = None
    if rank == 0 and not a.no_plain:
        from dadi_gb300 import models, numerics
        rng = np.random.default_rng(7)
        sample = [i for i in rng.permutation(NINST) if 500 <= steps[i] <= 3000][:3]
        sps = point_sweeps(steps[sample], PTS_L)

        def one_at_a_time(p):
            # as dadi's make_extrap_func runs it: the grids one after another
            res = [models.IM(p, NS, L) for L in PTS_L]
            return numerics.extrapolate(res, [r.extrap_x for r in res])
        concurrent = numerics.make_extrap_func(models.IM)  # the grids on three streams
        rates = {}
        for name, f in (("seq", one_at_a_time),
                        ("conc", lambda p: concurrent(p, NS, list(PTS_L)))):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for i in sample:
                f(draws[i])
            rates[name] = NINST * (sps / (time.perf_counter() - t0)) / ps
        plain = {"value": rates["seq"], "unit": "spectra/s",
                 "concurrent_grids_value": rates["conc"],
                 "sample": "%d seed-0 instances through the drop-in one at a time (two_pops "
                           "per grid, grids in sequence as dadi's make_extrap_func runs them; "
                           "concurrent_grids_value: the three grids on three streams), "
                           "scaled by point-sweeps" % len(sample)}

    # CPU baseline (oracle restatement, bounded sample) on rank 0 at N=1, and
    # the parity of the GPU batch's spectra against it on that sample
    cpu = parity = None
    if rank == 0 and world == 1 and not a.no_cpu:
        cores = os.cpu_count() or 1
        idx = parity_sample(draws, steps)
        v, info, fs_cpu = cpu_rate(draws, steps, idx, cores, obs)
        cpu = {"value": v, "unit": "spectra/s", "cores": cores, "kind": "port",
               "sample": "the stratified 64 seed-0 instances (draws 0-5, longest and shortest "
                         "schedules, each parameter's extremes, step-count quantiles; %.3g "
                         "point-sweeps, %.1f s of CPU on %d processes, %.1f s wall), scaled "
                         "to the 4096-instance workload by point-sweeps"
                         % (info["point_sweeps"], info["task_s"], cores, info["wall_s"])}
        parity = parity_of(fs_last, fs_cpu)

    serve = run_serving(a, obs) if (rank == 0 and a.serve > 0) else None
    adjoint = run_adjoint(a, obs) if (rank == 0 and not a.no_adjoint) else None
    config2 = run_config2(a) if (rank == 0 and not a.no_config2) else None

    if rank != 0:
        return 0
    from dadi_gb300 import _lib as glib
    fp64_peak_measured = glib.fp64_fma_peak_tflops(torch)
    peak, src = load_peaks()
    kmean = float(np.mean(kern_ms)) / 1e3
    achieved = ps * BYTES_PER_PS / kmean / 1e9
    # DRAM bytes (read + write) of the integration of one step on this
    # workload, from one ncu capture of the timed launches (1-pass metrics)
    traffic = K2_TRAFFIC_BYTES.get(eng.launch_mode) \
        if (NINST, PTS_L, NS) == (4096, (80, 90, 100), (40, 40)) else None
    fp64_achieved = ps * FLOPS_PER_PS / kmean / 1e12
    fp64_instr = ps * FP64_INSTR_PER_PS * 2 / kmean / 1e12
    fp64_peak = fp64_peak_measured
    line = {
        "metric": METRIC, "value": value, "unit": "spectra/s", "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seed-%d IM parameter draws; observed spectrum Poisson(5e4*model))"
                % rank,
        "config": workload_config(world, ps),
        "engine": {"gam_placement": eng.gam_placement, "launch_mode": eng.launch_mode,
                   "threads_per_cta": eng.threads or "auto"},
        "autotune": None if tuned is None else {
            "choice": list(tuned["choice"]), "sample_instances": tuned["sample"],
            "ms": {_cand_name(c): v for c, v in tuned["ms"].items()},
            "large_sample_instances": tuned["large_sample"],
            "ms_large": {_cand_name(c): v for c, v in tuned["ms_large"].items()}},
        "e2e": {"value": e2e_value, "unit": "spectra/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "peak_source": src,
                     "kernel": "k_integrate2d",
                     "launches_per_step": eng.launches_per_integrate() - 2,
                     "per": "step: achieved and traffic cover every integration launch of "
                            "one step (one per grid size with per_grid)",
                     "note": "FP64-pipe bound: phi stays in shared memory, so HBM carries "
                             "little; see fp64"},
        "fp64": {"algorithmic_tflops": fp64_achieved,
                 "pipe_tflops": fp64_instr, "peak_tflops": fp64_peak,
                 "frac": fp64_instr / fp64_peak,
                 "peak_source": "measured in this run (dgb_probe_fp64_fma: FMA chains, "
                                "4 and 8 warps/SM on every SM, ~0.1 s launches, best of 5)",
                 "note": "pipe_tflops counts %.2f FP64 thread instructions (as FMAs) per "
                         "point-sweep, measured with ncu counters; algorithmic_tflops counts "
                         "%d reference flops per point-sweep" % (FP64_INSTR_PER_PS, FLOPS_PER_PS)},
        "kernel_ms_per_step": kmean * 1e3,
        "warmup_ms": warm_ms,
        "clocks": clk,
        # per step: 2 schedule passes, the integration (one launch per grid
        # with per_grid), 2 epilogue
        "gpu_launches": (eng.launches_per_integrate() + 2) * a.steps,
        "failed_instances": bad,
        "scores": scores,
        "plain": plain,
        "batched_over_plain": (value / plain["value"]) if plain else None,
        "cpu_baseline": cpu,
        "parity": parity,
        "serving": serve,
        "adjoint": adjoint,
        "config2": config2,
    }
    print(json.dumps(line), flush=True)
    return 0


def run_serving(a, obs):
    """The serving workload: a seeded Poisson request stream (mean `rate`
    requests/s; 70% 2-D IM at pts base 40..100 with pts_l base, +10, +20 and
    ns (20,20) or (40,40); 20% DFE cache entries, IM with selection on the
    50-point gamma grid over [-2000, -1e-4]; 8% 3-D growth model at pts
    60..90; 2% four populations at pts 30..40; 10% of the IM requests with
    ns (40,40) also want gradients) served with continuous batching.  Latency
    is completion minus arrival, on the host clock."""
    from dadi_gb300 import serving
    srv = serving.Server(hbm_budget=a.serve_budget << 30)
    srv.prepare(range(40, 121), [(20, 20), (40, 40)])
    # warm-up: a stream of the same size (another seed), so that the measured
    # burst meets the server in its steady state -- worker engines built, and
    # the allocator's per-stream memory pools grown (the first burst a server
    # sees pays device allocations in its waves: p50 5.5 s against 1.1 s)
    srv.run(serving.config5_stream(a.serve, seed=1, rate=a.serve_rate, obs=obs))
    summ = _serve_stream(srv, a.serve, a.serve_rate, obs, a.serve_budget)
    summ["warmup"] = "a %d-request stream of the same mix (seed 1) served first" % a.serve
    if a.serve_sustained > 0:
        # the same mix at a rate the server keeps up with: latency without
        # the backlog of a burst
        summ["below_capacity"] = _serve_stream(srv, a.serve_sustained, a.serve_sustained_rate,
                                               obs, a.serve_budget, seed=2)
    return summ


def _serve_stream(srv, n, rate, obs, budget, seed=0):
    from dadi_gb300 import serving
    reqs = serving.config5_stream(n, seed=seed, rate=rate, obs=obs)
    out = srv.run(reqs)
    summ = serving.latency_summary(out)
    by = {}
    for kind in ("im", "im_sel", "growth3", "four"):
        lat = [r.latency for r in out if r.kind == kind and not r.want_grad and r.error is None]
        if lat:
            by[kind] = {"n": len(lat), "p50_s": float(np.percentile(lat, 50)),
                        "p99_s": float(np.percentile(lat, 99))}
    lat = [r.latency for r in out if r.want_grad and r.error is None]
    if lat:
        by["im_grad"] = {"n": len(lat), "p50_s": float(np.percentile(lat, 50)),
                         "p99_s": float(np.percentile(lat, 99))}
    summ.update({"arrival_rate_per_s": rate, "arrival_span_s": float(out[-1].arrival),
                 "hbm_budget_gib": budget, "by_class": by,
                 "failed_status": sum(1 for r in out if r.status)})
    return summ


def run_adjoint(a, obs):
    """Gradients of the Poisson log-likelihood for the first 256 seed-0 IM
    parameter sets at pts [100,110,120], ns (40,40) (forward with
    checkpoints, from_phi/extrapolation/likelihood backward through torch,
    and the discrete adjoint; CUDA-event timed), and for 32 parameter sets of
    the three-population growth model at pts 80."""
    import torch
    from dadi_gb300 import batch
    draws = im_draws(256, 0)
    eng = batch.Batch2D((100, 110, 120), NS)
    d_obs = torch.from_numpy(obs).cuda()
    eng.loglik_and_grad(draws[:4], d_obs, scale=5e4)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e2 = torch.cuda.Event(enable_timing=True)
    e0.record()
    ll, ctx = eng.forward_for_adjoint(draws, d_obs, scale=5e4)
    e1.record()
    grad = eng.adjoint(ctx, torch.ones_like(ll))
    e2.record()
    torch.cuda.synchronize()
    fwd = e0.elapsed_time(e1) / 1e3
    adj = e1.elapsed_time(e2) / 1e3
    out = {"im2d": {"sets": 256, "pts_l": [100, 110, 120], "ns": list(NS),
                    "checkpoint_every": ctx["C"], "forward_s": fwd, "adjoint_s": adj,
                    "gradients_per_s": 256 / (fwd + adj),
                    "failed_instances": int((ctx["status"] != 0).sum()),
                    "finite": bool(torch.isfinite(grad).all())}}
    del ll, ctx, grad
    # one gradient request: the longest of the first 4096 seed-0 draws
    # (19,546 steps), each grid's forward and backward walk on a cluster of 8
    # CTAs (the default for a few items), then on one CTA per grid
    d4 = im_draws(NINST, 0)
    i = int(np.argmax(batch.count_steps(batch.im_instances(d4))))
    single = {}
    for name, cf, ca in (("clusters", True, 8), ("one_cta", False, 0)):
        eng.cluster_forward, eng.cluster_adjoint = cf, ca
        e0.record()
        ll, ctx = eng.forward_for_adjoint(d4[i:i + 1], d_obs, scale=5e4)
        e1.record()
        g1 = eng.adjoint(ctx, torch.ones_like(ll))
        e2.record()
        torch.cuda.synchronize()
        single[name] = {"forward_s": e0.elapsed_time(e1) / 1e3,
                        "adjoint_s": e1.elapsed_time(e2) / 1e3,
                        "finite": bool(torch.isfinite(g1).all())}
        del ll, ctx
    eng.cluster_forward, eng.cluster_adjoint = batch.Batch2D.cluster_forward, \
        batch.Batch2D.cluster_adjoint
    single["steps"] = int(batch.count_steps(batch.im_instances(d4[i:i + 1]))[0])
    out["im2d"]["single_request"] = single
    # three populations: 32 sets of the growth model's parameters, each
    # scaled by exp(U(log .5, log 2)) (seed 0), at pts 80, ns (20,20,20)
    from dadi_gb300 import adjoint_nd, models
    th0 = adjoint_nd.Growth3.from_model_params(models.GROWTH3_DEFAULT)
    sets = th0 * np.exp(np.random.default_rng(0).uniform(np.log(.5), np.log(2), (32, 10)))
    m3 = adjoint_nd.Growth3((80,), (20, 20, 20))
    fs3, _ = m3.spectrum_ll(th0)
    obs3 = np.random.default_rng(0).poisson(1e4 * np.abs(fs3.cpu().numpy())).astype(float)
    d3 = torch.from_numpy(obs3).cuda()
    m3.loglik_and_grad_batch(sets[:2], d3, 1e4)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res = m3.loglik_and_grad_batch(sets, d3, 1e4)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    finite = all(bool(torch.isfinite(g).all()) for _, g, _ in res)
    t0 = time.perf_counter()
    res4 = m3.loglik_and_grad_many(sets, d3, 1e4, workers=4)
    torch.cuda.synchronize()
    wall4 = time.perf_counter() - t0
    same = all(torch.equal(a[1], b[1]) for a, b in zip(res, res4))
    out["growth3"] = {"sets": 32, "pts": 80, "ns": [20, 20, 20], "wall_s": wall,
                      "gradients_per_s": 32 / wall, "finite": finite,
                      "streams_wall_s": wall4, "streams_gradients_per_s": 32 / wall4,
                      "bitwise_equal": same,
                      "note": "host wall clock of loglik_and_grad_batch: the sets in groups "
                              "whose recorded densities fit half the free device memory "
                              "(here one group), every sweep launch over "
                              "all the sets of a group (forward recording every step's "
                              "density, the loss tails, the adjoint, the table derivatives); "
                              "streams_*: loglik_and_grad_many, four sets at a time on their "
                              "own streams"}
    return out


def run_config2(a):
    """The three-population growth model at pts [70,80,90], ns (20,20,20),
    extrapolated (T = 0.15, 675 steps per grid), through the drop-in public
    call (make_extrap_func: the three grids on their own streams; host
    parameters in, host spectrum out): host wall clock, median of 3 after a
    warm-up."""
    import torch
    from dadi_gb300 import models, numerics
    f = numerics.make_extrap_func(models.growth3)
    args = (models.GROWTH3_DEFAULT, (20, 20, 20), [70, 80, 90])
    f(*args)
    times = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fs = f(*args)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    ps = 675 * 3 * (70 ** 3 + 80 ** 3 + 90 ** 3)
    t = float(np.median(times))
    out = {"model": "three populations, exponential growth, pts [70,80,90], ns (20,20,20)",
           "seconds": t, "times_s": times, "point_sweeps": ps,
           "point_sweeps_per_s": ps / t, "finite": bool(np.all(np.isfinite(np.asarray(fs))))}
    # 32 parameter sets of the model (each parameter scaled by exp(U(log .5,
    # log 2)), seed 0) as one batch per grid through batchnd.ModelBatch
    from dadi_gb300 import batchnd
    sets = growth3_sets(32)
    mb = batchnd.ModelBatch("growth3", [70, 80, 90], (20, 20, 20))
    mb.run(sets[:2])
    tabs, _ = mb.tables(sets)
    ps32 = sum(len(tb) for tb in tabs[0]) * 3 * (70 ** 3 + 80 ** 3 + 90 ** 3)
    bt = []
    for _ in range(2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fsb, _, st = mb.run(sets)
        fsb.cpu()
        bt.append(time.perf_counter() - t0)
    tb = float(min(bt))
    out["batch32"] = {"sets": 32, "seconds": tb, "spectra_per_s": 32 / tb,
                      "point_sweeps": ps32, "point_sweeps_per_s": ps32 / tb,
                      "failed_sets": int(np.count_nonzero(st)),
                      "note": "host wall clock of ModelBatch.run (schedules walked in C, the "
                              "three grids batched on their own streams, N-D from_phi and "
                              "extrapolation on the device, spectra copied back); best of 2"}
    return out


def run_line_solvers(a):
    """The line solvers of the batched N-D engine on the growth model's
    grids (pts 70, 80, 90): Thomas per thread, warp PCR and the partitioned
    Thomas with 2, 4 and 8 segments per line, for one parameter set alone
    (a single 3-D integration: one grid's lines per launch) and for 32 sets
    batched.  CUDA events around dgb_batchnd_integrate, best of 3 after a
    warm-up; prints one JSON line."""
    import torch
    from dadi_gb300 import batchnd, models
    sets = growth3_sets(32)
    tabs, st = batchnd.schedules([batchnd.growth3_instance(p) for p in sets])
    assert not st.any()
    one, _ = batchnd.schedules([batchnd.growth3_instance(models.GROWTH3_DEFAULT)])
    solvers = [("thomas", 0, 0), ("pcr", 1, 0), ("part2", 2, 2), ("part4", 2, 4),
               ("part8", 2, 8)]
    out = {}
    for L in (70, 80, 90):
        phi0 = torch.from_numpy(batchnd.initial_density("growth3", L)).cuda()
        row = {}
        for name, ls, seg in solvers:
            eng = batchnd.BatchND(3, L, line_solver=ls, segments=seg)
            res = {}
            for label, tb in (("one_ms", one), ("batch32_ms", tabs)):
                ts = []
                for _ in range(4):
                    ev = (torch.cuda.Event(enable_timing=True),
                          torch.cuda.Event(enable_timing=True))
                    eng.integrate(phi0, tb, timer=ev)
                    torch.cuda.synchronize()
                    ts.append(ev[0].elapsed_time(ev[1]))
                res[label] = float(min(ts[1:]))
            steps = [len(t) for t in tabs]
            res["batch32_point_sweeps_per_s"] = 3 * sum(steps) * L ** 3 / (res["batch32_ms"] / 1e3)
            res["one_point_sweeps_per_s"] = 3 * len(one[0]) * L ** 3 / (res["one_ms"] / 1e3)
            row[name] = res
        out["pts%d" % L] = row
    # single integrations of other shapes: 3-D grids of 40, 60 and 120
    # points, and the four-population model at 20, 30 and 40 points
    four, _ = batchnd.schedules([batchnd.four_split_instance(models.FOUR_DEFAULT)])
    alone = {}
    for P, L, tb, kind in [(3, 40, one, "growth3"), (3, 60, one, "growth3"),
                           (3, 120, one, "growth3"), (4, 20, four, "four"),
                           (4, 30, four, "four"), (4, 40, four, "four")]:
        phi0 = torch.from_numpy(batchnd.initial_density(kind, L)).cuda()
        row = {}
        for name, ls, seg in [("thomas", 0, 0), ("part2", 2, 2), ("part4", 2, 4),
                              ("part8", 2, 8)]:
            if ls and L < 3 * seg:
                continue
            eng = batchnd.BatchND(P, L, line_solver=ls, segments=seg)
            ts = []
            for _ in range(4):
                ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                eng.integrate(phi0, tb, timer=ev)
                torch.cuda.synchronize()
                ts.append(ev[0].elapsed_time(ev[1]))
            row[name + "_ms"] = float(min(ts[1:]))
        alone["%dD_pts%d" % (P, L)] = row
    # the drop-in on config 2: make_extrap_func (the grids on their own
    # streams) and the grids one after another as dadi's make_extrap_func
    # runs them, with the Thomas solve and with the automatic choice
    from dadi_gb300 import integration, numerics
    f = numerics.make_extrap_func(models.growth3)
    args = (models.GROWTH3_DEFAULT, (20, 20, 20), [70, 80, 90])
    dropin = {}
    saved = integration.nd_line_solver
    try:
        for mode in ("thomas", "auto"):
            integration.nd_line_solver = mode
            for label, fn in (("concurrent_grids_s", lambda: f(*args)),
                              ("sequential_grids_s",
                               lambda: [models.growth3(args[0], args[1], L) for L in args[2]])):
                fn()
                ts = []
                for _ in range(3):
                    torch.cuda.synchronize()
                    t0 = time.perf_counter()
                    fn()
                    torch.cuda.synchronize()
                    ts.append(time.perf_counter() - t0)
                dropin["%s_%s" % (mode, label)] = float(np.median(ts))
    finally:
        integration.nd_line_solver = saved
    print(json.dumps({"line_solvers": out, "alone": alone, "dropin_config2": dropin,
                      "model": "three-population growth model (models.growth3): one set = "
                      "the default parameters, 675 steps; 32 sets as run_config2's batch; "
                      "four populations: models.four_split at its defaults",
                      "timing": "CUDA events around the integration, best of 3 after one "
                      "warm-up; dropin_config2: host wall clock, median of 3"}))
    return 0


def growth3_sets(n, seed=0):
    """n parameter sets of the three-population growth model: each of (nu0 x3,
    nuF x3, m12, m13, m23, T) scaled by exp(U(log .5, log 2)), seed 0."""
    from dadi_gb300 import models
    nu0, nuF, m, g, T = models.GROWTH3_DEFAULT
    th0 = np.array(list(nu0) + list(nuF) + list(m) + [T])
    th = th0 * np.exp(np.random.default_rng(seed).uniform(np.log(.5), np.log(2), (n, 10)))
    return [(tuple(r[0:3]), tuple(r[3:6]), tuple(r[6:9]), g, float(r[9])) for r in th]


def run_profile_case(a):
    """A small batch for ncu captures: each launch of the integration kernel
    lasts ~0.1 s and holds ~100 MB on the device."""
    import torch
    from dadi_gb300 import batch, build
    build.build()
    draws = im_draws(NINST, 0)
    rec = batch.im_instances(draws)
    steps = batch.count_steps(rec)
    sel = np.where((steps >= 200) & (steps <= 800))[0][:a.profile_items]
    eng = batch.Batch2D(PTS_L, NS, gam_placement=a.gam)
    eng.launch_mode = a.launch or "persistent"
    for _ in range(2):
        t = time.perf_counter()
        phis, st = eng.integrate(rec[sel])
        torch.cuda.synchronize()
        dt = time.perf_counter() - t
    ps = point_sweeps(steps[sel], PTS_L)
    print(json.dumps({"mode": "profile", "launch_mode": eng.launch_mode,
                      "instances": int(len(sel)), "point_sweeps": ps,
                      "seconds": dt, "status_nonzero": int((st != 0).sum())}))
    return 0


def run_profile_kernel(a):
    """Small cases of the other kernels for ncu captures (each launch well
    under 0.1 s, a few hundred MB on the device at most), run twice --
    except grad_request, a full-size gradient request (launches up to 1.5
    s, 11 GB of trajectory) for the one-pass launch list only."""
    import torch
    from dadi_gb300 import adjoint_nd, batch, build, epilogue, models
    build.build()
    for _ in range(2):
        t = time.perf_counter()
        if a.profile == "epilogue":
            # the epilogue of the full 4096-instance batch: 12288 densities
            eng = batch.Batch2D(PTS_L, NS)
            phis = [torch.rand(NINST, L, L, dtype=torch.float64, device="cuda")
                    for L in PTS_L]
            fs, ll = epilogue.spectra_2d_batch(torch, phis, eng.xxs, NS,
                                               torch.ones(41, 41, dtype=torch.float64,
                                                          device="cuda"), 1.0)
        elif a.profile == "sweep3d":
            # the 3-population growth model at pts 70 (675 steps x 3 sweeps)
            m = adjoint_nd.Growth3((70,), (20, 20, 20))
            m.spectrum_ll(adjoint_nd.Growth3.from_model_params(models.GROWTH3_DEFAULT))
        elif a.profile == "adjoint2d":
            draws = im_draws(NINST, 0)
            steps = batch.count_steps(batch.im_instances(draws))
            sel = np.where((steps >= 200) & (steps <= 400))[0][:16]
            eng = batch.Batch2D(PTS_L, NS)
            eng.loglik_and_grad(draws[sel], torch.ones(41, 41, dtype=torch.float64,
                                                       device="cuda"), 1.0)
        elif a.profile == "batchnd":
            # 48 sets of the three-population growth model at pts 70 as one
            # batch (132 MB of densities, more than L2)
            from dadi_gb300 import batchnd
            sets = growth3_sets(48)
            tabs, _ = batchnd.schedules([batchnd.growth3_instance(p) for p in sets])
            eng = batchnd.BatchND(3, 70)
            eng.integrate(torch.from_numpy(batchnd.initial_density("growth3", 70)).cuda(),
                          tabs)
        elif a.profile in ("thomas3d", "part3d"):
            # one set of the three-population growth model at pts 70 as a
            # batch of one: Thomas, or the partitioned solve with 8 segments
            from dadi_gb300 import batchnd
            tabs, _ = batchnd.schedules([batchnd.growth3_instance(models.GROWTH3_DEFAULT)])
            part = a.profile == "part3d"
            eng = batchnd.BatchND(3, 70, line_solver=2 if part else 0, segments=8 if part else 0)
            eng.integrate(torch.from_numpy(batchnd.initial_density("growth3", 70)).cuda(),
                          tabs)
        elif a.profile == "fromphind":
            # spectra (20,20,20) of 32 three-population densities at pts 90
            from dadi_gb300 import numerics, spectrum
            phis = torch.rand(32, 90, 90, 90, dtype=torch.float64, device="cuda")
            spectrum.from_phi_nd_batch(torch, phis, (20, 20, 20), numerics.default_grid(90))
        elif a.profile == "cluster2d":
            # one IM integration (seed-0 draw 1, 2648 steps) at L = 120 through
            # the drop-in on a cluster of 8 CTAs, then of 16
            from dadi_gb300 import integration, models
            saved = integration.line_solver_2d, integration.cluster_ctas
            try:
                for c in (8, 16):
                    integration.line_solver_2d, integration.cluster_ctas = "cluster", c
                    models.IM(im_draws(2, 0)[1], (40, 40), 120)
            finally:
                integration.line_solver_2d, integration.cluster_ctas = saved
        elif a.profile == "adjoint2d_cluster":
            # one IM gradient (seed-0 draw 1, 2648 steps) at pts 120: the
            # backward walk on a cluster of 8 CTAs from its stored trajectory
            # (0.6 GB)
            draws = im_draws(2, 0)
            eng = batch.Batch2D((120,), NS)
            eng.loglik_and_grad(draws[1:2], torch.ones(41, 41, dtype=torch.float64,
                                                       device="cuda"), 1.0)
        elif a.profile == "grad_request":
            # one gradient request: the longest of the first 4096 seed-0
            # draws (19,546 steps) at pts [100,110,120] (forward and adjoint
            # on clusters, trajectory 11 GB)
            d4 = im_draws(NINST, 0)
            i = int(np.argmax(batch.count_steps(batch.im_instances(d4))))
            eng = batch.Batch2D((100, 110, 120), NS)
            eng.loglik_and_grad(d4[i:i + 1], torch.ones(41, 41, dtype=torch.float64,
                                                         device="cuda"), 5e4)
        elif a.profile == "adjointnd_batch":
            # 8 three-population gradients at pts 32 as one batch (every
            # step's density recorded: about 1.5 GB), every sweep launch over
            # the lines of all 8 sets
            m = adjoint_nd.Growth3((32,), (10, 10, 10))
            sets = [adjoint_nd.Growth3.from_model_params(p) for p in growth3_sets(8)]
            m.loglik_and_grad_batch(sets, torch.ones(11, 11, 11, dtype=torch.float64,
                                                     device="cuda"), 1.0)
        elif a.profile == "adjointnd":
            m = adjoint_nd.Growth3((40,), (10, 10, 10))
            th = adjoint_nd.Growth3.from_model_params(models.GROWTH3_DEFAULT)
            m.loglik_and_grad(th, torch.ones(11, 11, 11, dtype=torch.float64,
                                             device="cuda"), 1.0)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t
    print(json.dumps({"mode": "profile", "case": a.profile, "seconds": dt}))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-budget", type=float, default=15.0,
                    help="seconds of CPU work per CPU measurement")
    ap.add_argument("--gam", type=int, default=0, help="0 auto, 1 shared, 2 workspace")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-tune", action="store_true",
                    help="skip the launch-configuration autotuner (use --gam's placement)")
    ap.add_argument("--launch", default=None, choices=["persistent", "one_per_cta", "per_grid"],
                    help="launch mode instead of the autotuner's choice (with --gam)")
    ap.add_argument("--clock-ms", type=int, default=500,
                    help="nvidia-smi sampling period during the timed region (0: off)")
    ap.add_argument("--serve", type=int, default=600,
                    help="requests in the served stream (0: skip serving)")
    ap.add_argument("--serve-rate", type=float, default=2000.0)
    ap.add_argument("--serve-budget", type=int, default=32, help="GiB the server may hold")
    ap.add_argument("--serve-sustained", type=int, default=200,
                    help="requests of a second, below-capacity stream (0: skip)")
    ap.add_argument("--serve-sustained-rate", type=float, default=20.0)
    ap.add_argument("--no-adjoint", action="store_true",
                    help="skip timing 256 IM gradients at pts [100,110,120] and 32 "
                         "three-population gradients at pts 80")
    ap.add_argument("--no-config2", action="store_true",
                    help="skip timing the three-population growth model at pts [70,80,90]")
    ap.add_argument("--profile-items", type=int, default=0,
                    help="run only a small batch (this many seed-0 instances with 200-800 "
                         "steps, twice) for profiler captures, then exit")
    ap.add_argument("--profile", default=None,
                    choices=["epilogue", "sweep3d", "adjoint2d", "adjointnd", "batchnd",
                             "fromphind", "thomas3d", "part3d", "adjointnd_batch",
                             "cluster2d", "adjoint2d_cluster", "grad_request"],
                    help="run a small case of another kernel for profiler captures, then exit")
    ap.add_argument("--line-solvers", action="store_true",
                    help="time the batched N-D engine's line solvers on the growth model's "
                         "grids, one set and 32 sets, then exit")
    a = ap.parse_args()
    if a.line_solvers:
        return run_line_solvers(a)
    if a.profile_items:
        return run_profile_case(a)
    if a.profile:
        return run_profile_kernel(a)
    world, rank, local = dist_init()
    if a.impl == "reference":
        rc = run_reference(a, world, rank)
    else:
        rc = run_ours(a, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return rc


if __name__ == "__main__":
    sys.exit(main())

"""Benchmark: histories/s of the 8-group two-zone k-eigenvalue problem.

Workload (the GPU-scale plain-method configuration): 8 groups, a 30 cm fuel
cube inside a 60 cm reflector cube, vacuum outside, seeded cross sections,
1e6 histories per cycle, FP64 tracking.  ``--workload ce`` runs the
continuous-energy plain method instead: three synthetic nuclides on 5e4-point
log grids (1/v capture, 200 SLBW resonances, potential scattering), free-gas
scattering at 293.6 K, a homogeneous mixture in a reflected 40 cm box,
1e6 histories per cycle.  A step is one active k-eigenvalue
cycle: transport of 1e6 source particles (each drawn from the previous
cycle's bank), fission-bank sites and their prefix sum, k of the cycle.
``value`` times the K steps with CUDA events on the engine's stream around
one mc_keig_cycles call (one host synchronisation, k per cycle returned),
with the bank resident in HBM; ``e2e`` times the
same workload through the C ABI's host-buffer call (mc_transport_bank), with
the source copied in from pinned host memory and the fission bank copied
back every step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

``--impl reference`` times the reference path on the host cores: the CPU
oracle (a restatement of the reference's transport loop, all host threads)
on the same problem.  N>1 (torchrun) runs independent replicas, one per GPU.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

METRIC = "histories/s on 1 GB300, plain vs surrogate-TSL at matched k_eff sigma/spectrum chi2"
UNIT = "histories/s"
WORKLOADS = {
    "two_zone": "8-group two-zone k-eigenvalue (fuel cube 30 cm in reflector cube 60 cm), 1e6 histories/cycle",
    "ce": "continuous-energy k-eigenvalue (3 synthetic SLBW nuclides, 5e4-point grids, free gas at 293.6 K, "
          "reflected 40 cm box), 1e6 histories/cycle",
}
BYTES_PER_EVENT = 128  # minimal SoA particle state read + write per event


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


class Replicas:
    """The N>1 path: one process per GPU, each running an independent replica
    of the workload (its own seed), with no collective on the data path.
    The process group serves only the timing contract: a barrier on both
    sides of the timed region and the whole-job figure, i.e. the units all
    ranks processed divided by the slowest rank's time.  ``backend`` is
    "nccl" under torchrun on GPUs ("gloo" runs the same logic on the CPU)."""

    def __init__(self, backend: str = "nccl"):
        self.ws, self.rank = _dist()
        self.backend = backend
        self.dist = None
        if self.ws > 1:
            import torch.distributed as dist

            dist.init_process_group(backend)
            self.dist = dist

    def _device(self):
        return "cuda" if self.backend == "nccl" else "cpu"

    def barrier(self) -> None:
        if self.dist is not None:
            self.dist.barrier()

    def total_rate(self, units: float, ms: float) -> tuple[float, float]:
        """(units of all ranks per second over the slowest rank's time, that
        time in ms).  With one rank: units / ms."""
        if self.dist is None:
            return units / (ms / 1e3), ms
        import torch

        t = torch.tensor([ms], dtype=torch.float64, device=self._device())
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        u = torch.tensor([units], dtype=torch.float64, device=self._device())
        self.dist.all_reduce(u, op=self.dist.ReduceOp.SUM)
        ms_max = float(t.item())
        return float(u.item()) / (ms_max / 1e3), ms_max

    def close(self) -> None:
        if self.dist is not None:
            self.dist.destroy_process_group()
            self.dist = None


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed
    region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.samples: list[list[str]] = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return

        def read():
            for line in self.proc.stdout:
                self.samples.append([x.strip() for x in line.split(",")])

        self.thread = threading.Thread(target=read, daemon=True)
        self.thread.start()

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)
        sm = [float(s[0]) for s in self.samples if len(s) >= 8 and s[0].replace(".", "").isdigit()]
        smax = [float(s[1]) for s in self.samples if len(s) >= 8 and s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples if len(s) >= 8 for i in range(4)
                          if s[4 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(self.samples)}


def peaks() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def problem(workload: str, histories: int, seed: int = 1) -> dict:
    """The workload's XML, the directory its data files live in, and the
    fields of the JSON line that describe it."""
    if workload == "ce":
        import atexit
        import shutil
        import tempfile

        from minimc_gb300 import synth_ce

        base = Path(tempfile.mkdtemp(prefix="mc_ce_"))
        atexit.register(shutil.rmtree, base, True)
        files = synth_ce.write_nuclides(base, seed=2027, n_grid=50_000)
        xml = synth_ce.ce_problem_xml(files, histories=histories, inactive=20, active=50)
        xml = xml.replace("<seed>1</seed>", f"<seed>{seed}</seed>")
        return {"xml": xml, "base": str(base), "kernel": "k_history_ce", "site_energy": 2.0,
                "config": {"nuclides": 3, "grid_points": 50_000, "temperature_K": 293.6}}
    from minimc_gb300 import synth

    p = synth.two_zone_cubes(histories=histories, inactive=20, active=50)
    p.seed = seed
    return {"xml": p.xml(), "base": "", "kernel": "k_history_mg", "site_energy": 1.0, "config": {"groups": 8}}


def cpu_baseline(xml: str, base: str, histories: int, threads: int, cycles: int) -> dict:
    """Times the CPU oracle (reference algorithm, minstd streams) on the host
    cores: `cycles` cycles of `histories` histories from the initial source."""
    from oracle.build import Oracle

    o = Oracle(xml, base)
    r = o.run_keigenvalue(histories, 1, 1, cycles - 1, threads=threads)
    hps = histories * cycles / r["seconds"]
    return {"value": hps, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{cycles} cycles x {histories} histories of the same problem (CPU oracle, "
                      f"{threads} threads), {r['seconds']:.1f} s",
            "k_cycles": [round(float(k), 6) for k in r["k_cycle"]],
            "reference_code_speed": "the restatement is 1.5-2.4x faster than the reference's own code at equal "
                                    "threads (oracle/ref/calibrate.py), so speed-ups against it are conservative"}


def run_reference(args) -> None:
    ws, rank = _dist()
    if rank != 0:
        return
    hist = args.histories
    wl = problem(args.workload, hist)
    xml, base = wl["xml"], wl["base"]
    threads = os.cpu_count() or 1
    # warm-up: one short cycle
    from oracle.build import Oracle

    Oracle(xml, base).run_keigenvalue(min(hist, 100_000), 1, 1, 0, threads=threads)
    o = Oracle(xml, base)
    # each step: one cycle of the workload on all host threads (the first
    # cycle starts from the point source; the bank converges in a few cycles)
    r = o.run_keigenvalue(hist, 1, args.warmup, args.steps, threads=threads)
    secs = r["seconds"]
    cycles = args.warmup + args.steps
    value = hist * cycles / secs
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / cycles,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOADS[args.workload], "histories_per_cycle": hist,
                   "rng": "minstd (reference streams)", **wl["config"]},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{cycles} cycles x {hist} histories (CPU oracle restating the reference path)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_gpu(args) -> None:
    import torch

    ws, rank = _dist()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    rep = Replicas("nccl")
    from minimc_gb300 import RNG_PHILOX, SITE_DTYPE, Context

    hist = args.histories
    wl = problem(args.workload, hist, seed=1 + rank)
    xml, base = wl["xml"], wl["base"]
    ctx = Context(local)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)
    ctx.load_xml(xml, base)
    opts = dict(rng=RNG_PHILOX, fast_math=int(args.fast), block_size=args.block, schedule=args.schedule,
                variant=args.variant)
    if args.mode == "kernel":
        # profiling mode: warm-up cycles (the first runs the autotuner unless
        # --variant is given) then `steps` active cycles; nothing else
        ctx.keig_begin(**opts)
        for i in range(args.warmup + args.steps):
            k = ctx.keig_cycle(i >= args.warmup)
        torch.cuda.synchronize()
        print(json.dumps({"mode": "kernel", "k_last": k, "schedule": ctx.schedule_info()}), flush=True)
        ctx.keig_end()
        rep.close()
        return

    def barrier():
        rep.barrier()
        torch.cuda.synchronize()

    # ---- device-resident cycles
    ctx.keig_begin(**opts)
    # warm-up through the same call as the timed cycles (the first cycle and
    # the autotuner's cycle run on their own inside it)
    k_warm = [float(k) for k in ctx.keig_cycles(args.warmup, False)]
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")  # > L2 (129 MB)
    st0 = ctx.keig_status()
    clocks = ClockSampler(local)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    flush.zero_()  # L2 flushed before the timed cycles (outside the event pair)
    barrier()
    t_wall = time.perf_counter()
    # the K active cycles in one call: each cycle transports the sources it
    # draws from the previous cycle's bank, with one host synchronisation
    # at the end (mc_keig_cycles); a cycle streams its ~310 MB working set
    # (source bank 64 MB, fission records 64 MB, per-history scores 128 MB,
    # bank written 57 MB) through the 129 MB L2
    e0.record(stream)
    k_steps = [float(k) for k in ctx.keig_cycles(args.steps, True)]
    e1.record(stream)
    barrier()
    wall = time.perf_counter() - t_wall
    clk = clocks.stop()
    st1 = ctx.keig_status()
    total_ms = e0.elapsed_time(e1)
    sched = ctx.schedule_info()
    k_out = ctx.keig_end()
    events = st1.events - st0.events
    kernel_ms = st1.kernel_ms - st0.kernel_ms
    launches = st1.launches - st0.launches
    # histories of all ranks over the slowest rank's time
    value, total_ms = rep.total_rate(hist * args.steps, total_ms)
    e_h = events / (hist * args.steps)
    peak, peak_kind = peaks()
    alg_bytes = e_h * BYTES_PER_EVENT * hist  # per transport launch (one per step)
    launch_ms = kernel_ms / args.steps        # the transport kernel alone, CUDA events
    achieved = alg_bytes / (launch_ms / 1e3) / 1e9
    traffic = fp64 = None
    tf = ROOT / "profiles" / "traffic.json"
    if tf.exists():
        prof = json.loads(tf.read_text())
        traffic = prof.get(f"{wl['kernel']}_dram_bytes_per_launch")
        fp64 = prof.get(f"{wl['kernel']}_fp64_pipe_active")

    # ---- end to end through the host-buffer ABI call
    n_sites = hist
    host_src = torch.empty(n_sites * SITE_DTYPE.itemsize, dtype=torch.uint8, pin_memory=True)
    src = host_src.numpy().view(SITE_DTYPE)
    cap = n_sites * max(1, ctx.info.max_yield)
    host_bank = torch.empty(cap * SITE_DTYPE.itemsize, dtype=torch.uint8, pin_memory=True)
    bank = host_bank.numpy().view(SITE_DTYPE)
    rng = np.random.default_rng(1234 + rank)
    # converged starting source: the last device bank is not exposed, so start
    # from isotropic sites at the origin and let the warm-up steps spread them
    src["x"] = src["y"] = src["z"] = 0.0
    mu = rng.uniform(-1, 1, n_sites)
    ph = rng.uniform(0, 2 * np.pi, n_sites)
    st = np.sqrt(1 - mu * mu)
    src["u"], src["v"], src["w"] = mu, st * np.cos(ph), st * np.sin(ph)
    src["energy"] = wl["site_energy"]
    src["key"] = np.arange(n_sites, dtype=np.uint64)
    e2e_times = []
    h2d = n_sites * SITE_DTYPE.itemsize
    d2h_total = 0
    for i in range(args.warmup + args.steps):
        barrier()
        t0 = time.perf_counter()
        m = ctx.transport_bank_into(src, bank, **opts)
        t1 = time.perf_counter()
        if i >= args.warmup:
            e2e_times.append(t1 - t0)
            d2h_total += m * SITE_DTYPE.itemsize
        # caller-side resampling of the next source (outside the timed call)
        idx = rng.integers(0, m, n_sites)
        nxt = bank[idx]
        src[:] = nxt
        src["key"] = np.arange(n_sites, dtype=np.uint64) + (i + 1) * n_sites
    e2e_value, _ = rep.total_rate(hist * args.steps, 1e3 * sum(e2e_times))

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        cpu = cpu_baseline(xml, base, args.cpu_histories, os.cpu_count() or 1, args.cpu_cycles)

    # the surrogate half of the metric: the thermal broomstick with the POD
    # sampler and with the guided (surrogate) form, outside the timed region
    surrogate = None
    if rank == 0 and args.workload == "two_zone" and not args.no_surrogate:
        f = thermal_forms(local, 1_000_000, 3, 1)
        surrogate = {"workload": f["workload"], "histories_per_step": f["histories_per_step"],
                     "pod_histories_per_s": f["pod"]["histories_per_s"],
                     "pod_queue_histories_per_s": f["pod_queue"]["histories_per_s"],
                     "surrogate_histories_per_s": f["guided"]["histories_per_s"],
                     "surrogate_vs_pod": f["guided"]["vs_pod"],
                     "surrogate_vs_pod_queue": f["guided"]["histories_per_s"] / f["pod_queue"]["histories_per_s"],
                     "energy_chi2_vs_pod": f["guided"]["energy_chi2_vs_pod"],
                     "cosine_chi2_vs_pod": f["guided"]["cosine_chi2_vs_pod"],
                     "identical_tallies_same_seed": f["guided"]["identical_tallies_same_seed"],
                     "form": "guided: the guide network starts each SampleAlpha CDF search, POD confirms it",
                     "exact_form": {k: (v["histories_per_s"] if isinstance(v, dict) else v)
                                    for k, v in f["exact_form"].items()},
                     "train": f["train"], "timed": "engine device time of each fixed-source run"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOADS[args.workload], "histories_per_cycle": hist, **wl["config"],
                       "rng": "philox",
                       "fast_math": bool(args.fast),
                       "l2": "flushed (256 MB write) before the timed cycles; inside them each cycle's working set "
                             "(~310 MB: source bank, fission records, per-history scores, bank written) is larger "
                             "than L2",
                       "timed": "the K active cycles through one mc_keig_cycles call (one host synchronisation; "
                                "k per cycle returned)",
                       "parallelism": f"replicas{ws}" if ws > 1 else "single GPU",
                       "schedule": sched},
            "k_cycles": [round(k, 6) for k in k_steps],
            "k": {"gpu_mean": float(np.mean(k_steps)),
                  "gpu_std": float(np.std(k_steps, ddof=1) / np.sqrt(len(k_steps))) if len(k_steps) > 1 else None,
                  "gpu_first_cycles": [round(k, 6) for k in (k_warm + k_steps)[:args.cpu_cycles]],
                  "cpu_first_cycles": cpu["k_cycles"] if cpu else None,
                  "note": "both runs start from the same point source; the 3-sigma k_eff test at 1e6 histories, "
                          "30 + 30 cycles, is tests/test_gpu_c2_keff.py"},
            "events_per_history": e_h,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                         "kernel": wl["kernel"], "algorithmic_bytes_per_launch": alg_bytes,
                         "launch_ms": launch_ms, "fp64_pipe_active_ncu": fp64,
                         "note": "state lives in registers, so DRAM traffic is far below the algorithmic "
                                 "bytes; the limiter is the FP64 pipe (2 ops/clk/SM on this part)"},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": int(d2h_total / max(1, args.steps)),
                    "call": "mc_transport_bank (pinned host banks: the transport kernel reads the sites in host "
                            "memory over the chip-to-chip link; multigroup Philox fission sites are sampled "
                            "straight into the host bank, coalesced, while the score commit runs on a second "
                            "stream); the caller's resampling of the next source (numpy) is outside the timed "
                            "call"},
            "surrogate": surrogate,
            "gpu_launches": int(launches),
            "clocks": clk,
            "wall_s": wall,
        }
        print(json.dumps(line), flush=True)
    rep.close()


def tsl_problem(histories: int, seed: int = 1, energy: float = 1e-6, base: Path | None = None) -> dict:
    """Broomstick with the synthetic POD thermal library (1 eV beam, 450 K)."""
    import atexit
    import shutil
    import tempfile

    from minimc_gb300 import synth_tsl

    if base is None:
        base = Path(tempfile.mkdtemp(prefix="mc_tsl_"))
        atexit.register(shutil.rmtree, base, True)
    tsl = synth_tsl.write_tsl(base)
    nuc = synth_tsl.moderator_nuclide(base)
    xml = synth_tsl.broomstick_xml(tsl, nuc, histories=histories, energy=energy, temperature=450.0)
    return {"xml": xml.replace("<seed>1</seed>", f"<seed>{seed}</seed>"), "base": str(base)}


TSL_WORKLOAD = ("thermal broomstick fixed source (POD S(alpha,beta,T) library rank 30, 4+4 partitions; "
                "1 eV pencil beam on a 0.01 cm hydrogen-moderator cylinder at 450 K; cosine x energy leakage "
                "tally 202 x 202 bins)")
GUIDE_TRAIN = dict(E_range=(5e-9, 2e-6), T_range=(283.6, 623.6), conditions=4096, samples_per_condition=512,
                   batch=16384, steps=10000, lr=1e-3, seed=3)


def chi2_two_sample(a, b) -> dict:
    """Two-sample chi-square of two histograms (bins with >= 10 counts)."""
    from scipy import stats

    keep = (a + b) >= 10
    a, b = a[keep], b[keep]
    ka, kb = np.sqrt(b.sum() / a.sum()), np.sqrt(a.sum() / b.sum())
    chi2 = float(np.sum((ka * a - kb * b) ** 2 / (a + b)))
    dof = int(keep.sum()) - 1
    return {"chi2": chi2, "dof": dof, "p": float(stats.chi2.sf(chi2, dof))}


def _spectra(ctx, r):
    e = ctx.estimators()[0]
    t = r.sum[e.offset:e.offset + e.n_bins].reshape(int(e.cosine_bins), int(e.energy_bins))
    return t.sum(0), t.sum(1)


def thermal_forms(local: int, hist: int, steps: int, warmup: int, quantile: bool = False) -> dict:
    """The thermal broomstick (C4 shape) transported with each form of the
    thermal sampler, histories/s from the engine's device timing of each
    fixed-source run (a step = one run of `hist` histories):
      pod        -- ThermalScattering's POD sampler inside the history kernel (FP32 form);
      pod_queue  -- the same sampler as a batched launch over the thermal-scatter queue;
      guided     -- the queue with the guide network starting each CDF search (the
                    surrogate form: the POD sampler's samples, for less work);
      quantile   -- (optional) the MLP inverse-CDF surrogate on the queue (approximate).
    Spectrum chi-square of each form against the POD form at independent seeds."""
    from minimc_gb300 import (RNG_PHILOX, THERMAL_GUIDED, THERMAL_POD, THERMAL_POD_QUEUE, THERMAL_SURROGATE,
                              Context)

    wl = tsl_problem(hist)
    ctx = Context(local)
    ctx.load_xml(wl["xml"], wl["base"])
    t0 = time.perf_counter()
    g = ctx.train_surrogate_guide(0, **GUIDE_TRAIN)
    train = {"guide_s": time.perf_counter() - t0, "guide_loss": g.loss_alpha, "guide_rows": g.samples,
             "guide_data_ms": g.data_ms, "guide_train_ms": g.train_ms}
    forms = {"pod": THERMAL_POD, "pod_queue": THERMAL_POD_QUEUE, "guided": THERMAL_GUIDED}
    if quantile:
        t0 = time.perf_counter()
        tq = ctx.train_surrogate(0, E_range=(5e-9, 2e-6), T_range=(283.6, 623.6), conditions=16384,
                                 samples_per_condition=1024, batch=16384, steps=12000, lr=1e-3, seed=3)
        train.update({"quantile_s": time.perf_counter() - t0, "quantile_loss_beta": tq.loss_beta,
                      "quantile_loss_alpha": tq.loss_alpha})
        forms["quantile"] = THERMAL_SURROGATE
    base = dict(rng=RNG_PHILOX, fast_math=1, histories=hist)
    out = {}

    def timed(mode, fast_math):
        kw = dict(base, fast_math=fast_math)
        for _ in range(warmup):
            ctx.run_fixed_source(thermal=mode, **kw)
        ms = kms = 0.0
        events = launches = 0
        for i in range(steps):
            r = ctx.run_fixed_source(thermal=mode, seed=1000 + i, **kw)
            ms += r.raw.transport_ms
            kms += r.raw.kernel_ms
            events += r.raw.events
            launches += r.raw.launches
        return {"histories_per_s": hist * steps / (ms / 1e3), "ms_per_step": ms / steps,
                "events_per_history": events / (hist * steps), "launches_per_step": launches / steps}

    for name, mode in forms.items():
        out[name] = timed(mode, 1)
    # the exact (FP64) sampler throughout (fast_math off): where the
    # network's saving -- FP64 reconstructions -- is largest
    exact = {f"{k}_exact": timed(v, 0) for k, v in (("pod", THERMAL_POD), ("pod_queue", THERMAL_POD_QUEUE),
                                                      ("guided", THERMAL_GUIDED))}
    for k in exact:
        exact[k]["vs_pod_exact"] = exact[k]["histories_per_s"] / exact["pod_exact"]["histories_per_s"]
    out["exact_form"] = exact
    ref = ctx.run_fixed_source(thermal=THERMAL_POD, seed=101, **base)
    same = ctx.run_fixed_source(thermal=THERMAL_GUIDED, seed=101, **base)
    out["guided"]["identical_tallies_same_seed"] = bool(np.allclose(same.sum, ref.sum, rtol=1e-12, atol=0))
    for name, mode in forms.items():
        if name == "pod":
            continue
        r = ctx.run_fixed_source(thermal=mode, seed=202, **base)
        sp, sr = _spectra(ctx, r), _spectra(ctx, ref)
        out[name]["energy_chi2_vs_pod"] = chi2_two_sample(sp[0], sr[0])
        out[name]["cosine_chi2_vs_pod"] = chi2_two_sample(sp[1], sr[1])
    for name in forms:
        out[name]["vs_pod"] = out[name]["histories_per_s"] / out["pod"]["histories_per_s"]
    out["exact_form"]["guided_vs_pod_queue"] = (out["exact_form"]["guided_exact"]["histories_per_s"] /
                                                out["exact_form"]["pod_queue_exact"]["histories_per_s"])
    out["train"] = train
    out["workload"] = TSL_WORKLOAD
    out["histories_per_step"] = hist
    return out


def c4_scale(ctx, stream, n: int = 10_000_000, bins: int = 200) -> dict:
    """C4 at its stated scale, per incident energy (0.01, 0.1, 1 eV): n
    scatters with T uniform in 283.6-623.6 K per sample, outgoing beta and
    alpha histograms of 200 equiprobable bins (edges from one exact-POD
    sample), and the two-sample chi-square of the guided sampler (exact
    form) and of the MLP quantile surrogate against an independent
    exact-POD sample."""
    import torch

    from minimc_gb300 import TSL_GUIDED, TSL_MLP, TSL_PHILOX, TSL_POD

    out = {"samples_per_energy": n, "bins": bins, "T": "uniform 283.6-623.6 K per sample"}
    g = torch.Generator(device="cuda")
    g.manual_seed(13)
    T = 283.6 + 340.0 * torch.rand(n, dtype=torch.float64, device="cuda", generator=g)
    E = torch.empty_like(T)
    b = torch.empty_like(T)
    a = torch.empty_like(T)

    def draw(method, seed):
        ctx.sample_tsl_device(0, E.data_ptr(), T.data_ptr(), n, b.data_ptr(), a.data_ptr(), seed=seed, method=method)
        torch.cuda.synchronize()
        return b.clone(), a.clone()

    def counts(x, edges):
        x = x[~torch.isnan(x)]
        return torch.bincount(torch.bucketize(x, edges), minlength=bins + 2).cpu().numpy().astype(np.float64)

    for e_ev in (0.01, 0.1, 1.0):
        E.fill_(e_ev * 1e-6)
        ref = draw(TSL_POD | TSL_PHILOX, 101)
        pod = draw(TSL_POD | TSL_PHILOX, 202)
        res = {"guided": draw(TSL_GUIDED, 303), "mlp_quantile": draw(TSL_MLP, 404)}
        row = {}
        for v, name in ((0, "beta"), (1, "alpha")):
            x = ref[v][~torch.isnan(ref[v])].sort().values
            edges = x[torch.linspace(0, len(x) - 1, bins + 1, device="cuda").round().long()][1:-1].contiguous()
            cp = counts(pod[v], edges)
            for form, smp in res.items():
                row.setdefault(form, {})[name] = chi2_two_sample(counts(smp[v], edges), cp)
        out[f"{e_ev:g} eV"] = row
    return out


def run_gpu_tsl(args) -> None:
    """Broomstick transport (histories/s) with each thermal sampler form,
    plus the sampler-level comparison of the POD forms, the guided sampler
    and the MLP quantile surrogate on C4's incident energies with T uniform
    in 283.6-623.6 K per sample."""
    import torch

    from minimc_gb300 import TSL_FAST, TSL_GUIDED, TSL_MLP, TSL_PHILOX, TSL_POD, Context

    ws, rank = _dist()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    rep = Replicas("nccl")
    hist = args.histories
    stream = torch.cuda.current_stream()
    if args.mode == "kernel":
        # profiling mode: each sampler form on 4e6 samples, `steps` times; no transport
        wl = tsl_problem(hist)
        ctx = Context(local)
        ctx.set_stream(stream.cuda_stream)
        ctx.load_xml(wl["xml"], wl["base"])
        n = 4_000_000
        E = torch.full((n,), 1e-7, dtype=torch.float64, device="cuda")
        T = torch.full((n,), 450.0, dtype=torch.float64, device="cuda")
        b = torch.empty_like(E)
        a = torch.empty_like(E)
        ctx.train_surrogate_guide(0, **GUIDE_TRAIN)
        ctx.train_surrogate(0, E_range=(5e-9, 2e-6), T_range=(283.6, 623.6), conditions=4096,
                            samples_per_condition=512, batch=8192, steps=3000, seed=3)
        for method in (TSL_POD | TSL_PHILOX | TSL_FAST, TSL_GUIDED | TSL_FAST, TSL_POD | TSL_PHILOX, TSL_GUIDED,
                       TSL_MLP):
            for i in range(args.steps):
                ctx.sample_tsl_device(0, E.data_ptr(), T.data_ptr(), n, b.data_ptr(), a.data_ptr(), seed=1 + i,
                                      method=method)
        torch.cuda.synchronize()
        print(json.dumps({"mode": "kernel", "beta_mean": float(b.mean())}), flush=True)
        rep.close()
        return
    clocks = ClockSampler(local)
    clocks.start()
    rep.barrier()
    forms = thermal_forms(local, hist, args.steps, args.warmup, quantile=True)
    clk = clocks.stop()
    value, _ = rep.total_rate(hist * args.steps, forms["guided"]["ms_per_step"] * args.steps)

    # sampler level: POD exact, POD FP32, guided, MLP quantile surrogate
    wl = tsl_problem(hist)
    ctx = Context(local)
    ctx.set_stream(stream.cuda_stream)
    ctx.load_xml(wl["xml"], wl["base"])
    ctx.train_surrogate_guide(0, **GUIDE_TRAIN)
    tr = ctx.train_surrogate(0, E_range=(5e-9, 2e-6), T_range=(283.6, 623.6), conditions=16384,
                             samples_per_condition=1024, batch=16384, steps=12000, lr=1e-3, seed=3)
    n = 4_000_000
    g = torch.Generator(device="cuda")
    g.manual_seed(7)
    E = torch.tensor([0.01e-6, 0.1e-6, 1.0e-6], dtype=torch.float64, device="cuda")[
        torch.randint(0, 3, (n,), device="cuda", generator=g)]
    T = 283.6 + 340.0 * torch.rand(n, dtype=torch.float64, device="cuda", generator=g)
    b = torch.empty(n, dtype=torch.float64, device="cuda")
    a = torch.empty_like(b)
    rates, samples = {}, {}
    for name, method in (("pod_exact", TSL_POD | TSL_PHILOX), ("guided_exact", TSL_GUIDED),
                         ("pod_fp32", TSL_POD | TSL_PHILOX | TSL_FAST), ("guided_fp32", TSL_GUIDED | TSL_FAST),
                         ("mlp_quantile", TSL_MLP)):
        for _ in range(2):
            ctx.sample_tsl_device(0, E.data_ptr(), T.data_ptr(), n, b.data_ptr(), a.data_ptr(), seed=11, method=method)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        reps = 3
        e0.record(stream)
        for i in range(reps):
            ctx.sample_tsl_device(0, E.data_ptr(), T.data_ptr(), n, b.data_ptr(), a.data_ptr(), seed=11 + i,
                                  method=method)
        e1.record(stream)
        torch.cuda.synchronize()
        rates[name] = n * reps / (e0.elapsed_time(e1) / 1e3)
        samples[name] = (b.cpu().numpy().copy(), a.cpu().numpy().copy())
    from scipy import stats

    ks = {k: {"beta": float(stats.ks_2samp(samples[k][0][:200_000], samples["pod_exact"][0][:200_000]).statistic),
              "alpha": float(stats.ks_2samp(samples[k][1][:200_000], samples["pod_exact"][1][:200_000]).statistic)}
          for k in ("pod_fp32", "mlp_quantile")}
    same = {form: bool(np.array_equal(samples[f"guided_{form}"][0], samples[f"pod_{form}"][0], equal_nan=True) and
                       np.array_equal(samples[f"guided_{form}"][1], samples[f"pod_{form}"][1], equal_nan=True))
            for form in ("exact", "fp32")}
    c4 = c4_scale(ctx, stream, n=10_000_000)
    flops = 2 * 2 * (16 * 128 + 2 * 128 * 128 + 128)  # two network rows per sample, multiply-adds x 2
    bf16_peak = None
    pk = ROOT / "MEASURED_PEAKS.json"
    if pk.exists():
        bf16_peak = json.loads(pk.read_text()).get("bf16_tflops")
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        from oracle.build import Oracle

        o = Oracle(wl["xml"], wl["base"])
        nc = min(hist, 2_000_000)
        thr = os.cpu_count() or 1
        rc = o.run_fixed_source(nc, 1, threads=thr)
        cpu = {"value": nc / rc["seconds"], "unit": UNIT, "cores": thr, "kind": "port",
               "sample": f"{nc} histories of the same broomstick (CPU oracle, {thr} threads), {rc['seconds']:.1f} s"}
    if rank == 0:
        peak, peak_kind = peaks()
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": forms["guided"]["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": TSL_WORKLOAD, "histories_per_step": hist, "rng": "philox", "fast_math": True,
                       "form": "guided (surrogate-started CDF searches, POD-exact samples)",
                       "l2": "inputs generated on device; tallies 0.65 MB"},
            "thermal_forms": forms,
            "c4_scale": c4,
            "sampler": {"samples_per_s": rates, "ks_vs_pod_exact": ks, "guided_equals_pod": same,
                        "guided_exact_vs_pod_exact": rates["guided_exact"] / rates["pod_exact"],
                        "guided_fp32_vs_pod_fp32": rates["guided_fp32"] / rates["pod_fp32"],
                        "quantile_train": {"loss_beta": tr.loss_beta, "loss_alpha": tr.loss_alpha,
                                           "samples": tr.samples, "data_ms": tr.data_ms, "train_ms": tr.train_ms},
                        "mlp_quantile_tflops": rates["mlp_quantile"] * flops / 1e12,
                        "guided_tflops": rates["guided_fp32"] * flops / 1e12, "bf16_peak_tflops": bf16_peak,
                        "sample_n": n},
            "roofline": {"bound": "hbm", "achieved": None, "peak": peak, "unit": "GB/s", "frac": None,
                         "traffic": None, "peak_kind": peak_kind, "kernel": "k_history_ce",
                         "note": "see the default two-zone line; this workload is latency-bound"},
            "cpu_baseline": cpu,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 2 * 8 * 40804,
                    "call": "mc_run_fixed_source (tallies read back every step)"},
            "gpu_launches": int(forms["guided"]["launches_per_step"] * args.steps), "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    rep.close()


BATCH_WORKLOAD = ("64 independent 8-group two-zone k-eigenvalue problems (seeds 0..63, cube sides log-uniform "
                  "10-80 cm, 1e4-1e6 histories/cycle log-uniform, material temperatures uniform 300-600 K with "
                  "the two thermal groups' scatter transfer sampled from the MLP surrogate at each problem's "
                  "temperature) in one batch: one persistent transport launch per cycle, per-cycle CUDA graph")
QUANT_TRAIN = dict(E_range=(5e-9, 2e-6), T_range=(283.6, 623.6), conditions=16384, samples_per_condition=1024,
                   batch=16384, steps=12000, lr=1e-3, seed=3)


def batch_cpu_baseline(probs, rows, temps, threads: int, subset: int = 16, cycles: int = 6, seed: int = 21) -> dict:
    """The CPU oracle (reference algorithm, minstd streams) on a seeded
    subset of the batch's problems, each run alone for `cycles` cycles of
    its own histories per cycle (capped at 2e5): total histories over total
    time."""
    from minimc_gb300 import thermal_groups
    from oracle.build import Oracle

    pick = sorted(np.random.default_rng(seed).choice(len(probs), size=min(subset, len(probs)), replace=False))
    hist = secs = 0.0
    for i in pick:
        p, h = probs[i]
        n = min(int(h), 200_000)
        q = thermal_groups.with_thermal_rows(p, temps[i], rows[i])
        r = Oracle(q.xml()).run_keigenvalue(n, p.seed, 1, cycles - 1, threads=threads)
        hist += n * cycles
        secs += r["seconds"]
    return {"value": hist / secs, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"problems {[int(i) for i in pick]} of the batch (seeded subset), each alone on the CPU "
                      f"oracle: {cycles} cycles x min(its histories, 2e5), {threads} threads, {secs:.1f} s"}


def run_gpu_batch(args) -> None:
    """C5: 64 uneven problems whose thermal groups scatter by transfer rows
    sampled from the MLP surrogate at each problem's temperature, in one
    batch; against (a) the same problems with the POD sampler's rows
    (per-problem k within sigma: the plain form), (b) the same problems run
    one after another through the single-problem path (identical k; the
    batching gain) and (c) the CPU oracle on a seeded subset."""
    import torch
    from scipy import stats

    from minimc_gb300 import RNG_PHILOX, TSL_MLP, TSL_PHILOX, TSL_POD, Batch, Context, synth, thermal_groups

    ws, rank = _dist()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    rep = Replicas("nccl")
    probs = synth.batch_problems(count=64, seed=7 + rank)
    if args.mode == "kernel":
        # profiling mode: the batch's cycles only (no thermal rows, no
        # surrogate training, no comparisons)
        b = Batch(local)
        for p, h in probs:
            b.add(p.xml(), histories=h, seed=p.seed)
        r = b.run(inactive=args.warmup, active=args.steps, fast_math=int(args.fast))
        print(json.dumps({"mode": "kernel", "variant": r["variant"], "active_ms": r["active_ms"]}), flush=True)
        rep.close()
        return
    temps = thermal_groups.problem_temperatures(len(probs), seed=11 + rank)
    # transfer rows of the thermal groups: surrogate and POD sampler
    wl = tsl_problem(10)
    tctx = Context(local)
    tctx.load_xml(wl["xml"], wl["base"])
    t0 = time.perf_counter()
    tr = tctx.train_surrogate(0, **QUANT_TRAIN)
    train_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    rows_s, fail_s = thermal_groups.transfer_rows(tctx, 0, temps, seed=3, method=TSL_MLP)
    rows_ms = 1e3 * (time.perf_counter() - t0)
    rows_p, fail_p = thermal_groups.transfer_rows(tctx, 0, temps, seed=4, method=TSL_POD | TSL_PHILOX)
    thermal = [thermal_groups.with_thermal_rows(p, T, r) for (p, _), T, r in zip(probs, temps, rows_s)]
    plain = [thermal_groups.with_thermal_rows(p, T, r) for (p, _), T, r in zip(probs, temps, rows_p)]

    def make(problems, seed_offset=0):
        b = Batch(local)
        for q, (p, h) in zip(problems, probs):
            b.add(q.xml(), histories=h, seed=p.seed + seed_offset)
        return b

    clocks = ClockSampler(local)
    clocks.start()
    rep.barrier()
    r = make(thermal).run(inactive=args.warmup, active=args.steps, fast_math=int(args.fast))
    clk = clocks.stop()
    cycles = args.warmup + args.steps
    n_cycle = int(sum(h for _, h in probs))
    value, _ = rep.total_rate(n_cycle * args.steps, r["active_ms"])
    rp = make(plain, 1000).run(inactive=args.warmup, active=args.steps, fast_math=int(args.fast))
    z = (r["k_mean"] - rp["k_mean"]) / np.hypot(r["k_std"], rp["k_std"])
    chi2 = float(np.sum(z ** 2))
    # the plain path: each problem alone, the same cycles
    seq_ms = 0.0
    agree = True
    for i, (q, (p, h)) in enumerate(zip(thermal, probs)):
        ctx = Context(local)
        ctx.load_xml(q.xml())
        s = ctx.run_keigenvalue(rng=RNG_PHILOX, fast_math=int(args.fast), histories=h, seed=p.seed,
                                inactive=args.warmup, active=args.steps, variant=r["variant"] + 1)
        seq_ms += s.raw.transport_ms
        agree &= bool(np.array_equal(s.k_cycle, r["k_cycle"][i]))
    seq_value = n_cycle * cycles / (seq_ms / 1e3)
    all_value = n_cycle * cycles / (r["transport_ms"] / 1e3)
    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = batch_cpu_baseline(probs, rows_s, temps, os.cpu_count() or 1)
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": r["active_ms"] / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": BATCH_WORKLOAD, "problems": len(probs), "histories_per_cycle": n_cycle,
                       "rng": "philox", "fast_math": bool(args.fast),
                       "timed": "the active cycles (a step = one cycle of all problems); the warm-up cycles "
                                "and the autotuner's runs before them are outside",
                       "l2": "working set (sources, banks, records of 1.4e7 histories) far above L2"},
            "batch": {"variant": r["variant"], "graph": bool(r["graph"]), "launches": r["launches"],
                      "tune_ms": [round(x, 3) for x in r["tune_ms"] if x > 0],
                      "all_cycles_histories_per_s": all_value,
                      "sequential_histories_per_s": seq_value, "speedup_vs_sequential": all_value / seq_value,
                      "k_identical_to_single_runs": agree,
                      "k_mean_range": [float(r["k_mean"].min()), float(r["k_mean"].max())]},
            "thermal_groups": {
                "temperatures_K": [round(float(t), 1) for t in temps],
                "rows": "surrogate (MLP quantile networks, tcgen05) at each temperature, 2^20 scatters per "
                        "thermal group, binned on the device",
                "rows_ms": rows_ms, "train_s": train_s, "train_loss": [tr.loss_beta, tr.loss_alpha],
                "sampler_failures": [int(fail_s), int(fail_p)],
                "max_row_diff_vs_pod": float(np.abs(rows_s - rows_p).max()),
                "k_vs_pod_rows": {"chi2": chi2, "dof": len(z), "p": float(stats.chi2.sf(chi2, len(z))),
                                  "max_abs_z": float(np.abs(z).max()),
                                  "within_3_sigma": int((np.abs(z) < 3).sum()),
                                  "k_surrogate": [round(float(k), 6) for k in r["k_mean"]],
                                  "k_pod": [round(float(k), 6) for k in rp["k_mean"]],
                                  "note": "independent seeds; z = dk / combined standard error"}},
            "cpu_baseline": cpu,
            "e2e": {"value": all_value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0,
                    "call": "mc_batch_run over all cycles, warm-up included (problems loaded before; k read back "
                            "once at the end)"},
            "gpu_launches": int(r["launches"]), "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    rep.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--workload", default="two_zone", choices=sorted(WORKLOADS) + ["tsl", "batch"])
    ap.add_argument("--histories", type=int, default=1_000_000)
    ap.add_argument("--block", type=int, default=0, help="0: autotuned")
    ap.add_argument("--fast", type=int, default=1,
                    help="FP32 sampling arithmetic (geometry, positions, k and tallies stay FP64)")
    ap.add_argument("--schedule", type=int, default=0, help="0 auto, 1 history, 2 event")
    ap.add_argument("--cpu-histories", type=int, default=1_000_000)
    ap.add_argument("--cpu-cycles", type=int, default=6)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-surrogate", action="store_true", help="skip the thermal surrogate leg of the default line")
    ap.add_argument("--variant", type=int, default=0, help="history-kernel variant + 1 (0: autotuned)")
    ap.add_argument("--mode", default="full", choices=["full", "kernel"],
                    help="kernel: only the k-eigenvalue cycles (for profiler captures)")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "tsl":
        run_gpu_tsl(args)
    elif args.workload == "batch":
        run_gpu_batch(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()

"""Benchmark of the checkerboard PT hot path (one JSON line on rank 0).

Workload: batched 3D Ising parallel tempering — L = 8, 16, 32, 64, 128, 32
replicas per size on a linear T grid over [4.40, 4.62], int8 spins hot-started
from seed 42, exchange every 10 sweeps, measure every 5 (integer E/M fused into
the sweep).  One step = one exchange period: 10 sweeps of all 160 lattices,
2 measurements and 1 replica-exchange pass, replayed as one CUDA graph.

value      spin flips/ns (attempted site updates of all lattices / device time),
           inputs resident in HBM, L2 flushed (256 MiB write) before every step.
e2e        the same metric through the C-ABI entry point isg_ising_pt_run with
           host record arrays: each step returns its (slot, E, M) records to the
           host inside the timed region.
roofline   the half-sweep kernel: 3 algorithmic bytes per site update
           (read own + neighbour colour plane, write own plane) x sites per
           launch / mean launch time (CUDA events on the kernel's stream).
cpu_baseline / --impl reference: the reference CPU path (random-site
           Metropolis, src/metropolis.rs:8-27) restated in C (oracle/), one
           replica of every size per host thread, on all host threads.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import re
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
SIZES = [8, 16, 32, 64, 128]
REPLICAS = 32
TMIN, TMAX = 4.40, 4.62
EXCHANGE_EVERY, MEASURE_EVERY = 10, 5
SWEEPS_PER_STEP = 10
SEED = 42
BYTES_PER_UPDATE = 3  # int8 colour-split: read 1 B own + 1 B neighbour plane, write 1 B
WORKLOAD = "3D Ising PT L=8,16,32,64,128 x 32 replicas, T in [4.40,4.62], exchange 10, measure 5"
METRIC = "spin flips/ns (site-update attempts per ns), batched checkerboard PT"
TC_3D = 4.5115


def _load(name, path):
    import importlib.util
    if name in sys.modules:
        return sys.modules[name]
    spec = importlib.util.spec_from_file_location(
        name, path, submodule_search_locations=[str(path.parent)] if path.name == "__init__.py"
        else None)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def temps():
    return [TMIN + (TMAX - TMIN) * i / (REPLICAS - 1) for i in range(REPLICAS)]


def sites_per_sweep():
    return sum(L ** 3 for L in SIZES) * REPLICAS


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


HEADLINE_PROFILE = "ising_halfsweep_L8-128x32.txt"
HBM_PROFILE = "ising_halfsweep_L128x128.txt"
HBM_REPLICAS = 128
ESS_SWEEPS = 100000
ESS_WARMUP = 10000


def ncu_traffic(name: str):
    """DRAM bytes per half-sweep launch from a committed ncu summary, if any."""
    p = ROOT / "profiles" / name
    if p.exists():
        m = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", p.read_text())
        if m:
            return float(m.group(1))
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.dev}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = []
        for line in (self.out or "").splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, f in rows for i, v in enumerate(f) if v == "Active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows),
                "sm_max_mhz": max(r[1] for r in rows), "reasons": reasons,
                "samples": len(rows)}


def cpu_sample(threads: int, sweeps: float = 1.0):
    """Bounded sample of the reference CPU path: `threads` host threads, each
    `sweeps` sweeps of one replica of every workload size."""
    oracle = _load("isg_oracle", ROOT / "oracle" / "oracle.py")
    rb = oracle.RefBench(SIZES, 3, TMIN, TMAX, threads, seed=SEED)
    rb.step(0.05)
    sec, flips = rb.step(sweeps)
    rb.close()
    return flips / sec * 1e-9, sec, flips


def cpu_replay(threads: int) -> dict:
    """The checkerboard/Philox update of this path restated in C (the oracle's
    replay: same random stream, thresholds and colour order) on the host threads,
    one L=64 replica per thread, 20 sweeps each: what the GPU algorithm itself
    costs on the CPU, beside the reference's random-site path."""
    oracle = _load("isg_oracle", ROOT / "oracle" / "oracle.py")
    oracle.replay_bench(64, 3, 4.5, 1, threads)
    sec, flips = oracle.replay_bench(64, 3, 4.5, 20, threads)
    return {"value": flips / sec * 1e-9, "unit": "flips/ns", "cores": threads,
            "sample": f"{threads} threads x 20 checkerboard sweeps of L=64 ({flips:.3g} flips, "
                      f"{sec:.2f} s)"}


def host_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def tau_int(x) -> float:
    x = np.asarray(x, float)
    x = x - x.mean()
    n = len(x)
    max_lag = n // 4
    var = np.var(x)
    if var < 1e-15 or max_lag < 2:
        return 0.5
    f = np.fft.rfft(x, 2 * n)
    acf = np.fft.irfft(f * np.conj(f))[:max_lag] / (var * np.arange(n, n - max_lag, -1))
    tau = 0.5
    for t in range(1, len(acf)):
        tau += acf[t]
        if t >= 6 * tau:
            break
    return float(tau)


def tau_blocking(x, nb=20) -> float:
    """tau_int from the spread of nb block means: var(block mean) = 2 tau
    var(x) / B for blocks of B samples much longer than tau.  Unlike the
    windowed sum it sees rare long excursions (a sticky independence chain)."""
    x = np.asarray(x, float)
    B = len(x) // nb
    var = np.var(x)
    if B < 2 or var < 1e-15:
        return 0.5
    bm = x[:B * nb].reshape(nb, B).mean(1)
    return float(max(0.5, B * np.var(bm, ddof=1) / (2 * var)))


def max_over_ranks(value: float, device="cpu") -> float:
    """The slowest rank's value (the job's timed region ends with the last rank);
    the value itself on a single process."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_flips_per_ns(sites_per_sweep_per_rank: int, sweeps: int, world: int,
                     max_ms: float) -> float:
    """Whole-job throughput: every rank advances its own replicas (replicas only,
    no data exchange), so the job does world x the per-rank work in the slowest
    rank's time."""
    return sites_per_sweep_per_rank * sweeps * world / (max_ms * 1e6)


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def run_reference(args):
    ws, rank, _ = dist_info()
    if rank != 0:
        return 0
    threads = host_threads()
    oracle = _load("isg_oracle", ROOT / "oracle" / "oracle.py")
    rb = oracle.RefBench(SIZES, 3, TMIN, TMAX, threads, seed=SEED)
    # calibrate: each step is a fraction of a sweep of every size per thread,
    # sized so the whole --steps/--warmup run takes about args.ref_seconds
    s0, _ = rb.step(0.05)
    frac = min(1.0, 0.05 * args.ref_seconds / max(s0, 1e-6) / (args.steps + args.warmup))
    frac = max(frac, 1e-4)
    for _ in range(args.warmup):
        rb.step(frac)
    tot_s = tot_f = 0.0
    for _ in range(args.steps):
        s, f = rb.step(frac)
        tot_s += s
        tot_f += f
    rb.close()
    v = tot_f / tot_s * 1e-9
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "flips/ns",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": tot_s / max(args.steps, 1) * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int8", "data": "synthetic",
        "config": {"workload": WORKLOAD,
                   "step": f"{frac:.4g} random-site sweeps of every size per host thread",
                   "l2": "n/a (host CPU)"},
        "cpu_baseline": {"value": v, "unit": "flips/ns", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} steps x {threads} threads x {frac:.4g} sweeps "
                                   f"of each of L=8..128 (reference CPU path restated in C; the "
                                   f"Rust original cannot be built here)"},
        "e2e": {"value": v, "unit": "flips/ns", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def _timed_pt_steps(b, stream, flush, steps):
    """Per-step device ms of `steps` PT steps (one exchange period each, one CUDA
    graph replay), L2 flushed before every step, events on the library's stream."""
    import torch
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    with torch.cuda.stream(stream):
        for i in range(steps):
            flush.fill_(i & 0xFF)
            starts[i].record(stream)
            # 10 sweeps, 2 fused measures, 1 exchange; records stay in the
            # device ring (read after the timed region)
            b.pt_launch(SWEEPS_PER_STEP, EXCHANGE_EVERY, MEASURE_EVERY)
            ends[i].record(stream)
    torch.cuda.synchronize()
    return [s.elapsed_time(e) for s, e in zip(starts, ends)]


def _roofline(b, launch_ms, peak, peak_kind, traffic, kernel, residency):
    sites_launch = b.sites_per_halfsweep()
    alg_bytes = sites_launch * BYTES_PER_UPDATE
    achieved = alg_bytes / (launch_ms * 1e-3) / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": traffic, "kernel": kernel,
            "bytes_per_launch": alg_bytes, "launch_ms": launch_ms, "residency": residency,
            "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs, copy bandwidth)"}


def hbm_case(pkg, stream, flush, steps, peak, peak_kind):
    """3D Ising L = 128 alone, 128 replicas on the same T grid width (268 MB of
    spins, twice the L2): the spec roofline configuration.  Same step and
    timing as the headline; the half-sweep is timed inside a graph of 20 launches
    with L2 flushed before each replay."""
    R = HBM_REPLICAS
    T = [TMIN + (TMAX - TMIN) * i / (R - 1) for i in range(R)]
    b = pkg.IsingBatch([128], R, seed=SEED + 7)
    b.set_stream(stream)
    b.set_temperatures(T)
    b.step(20)
    b.reset_sampling()
    for _ in range(3):
        b.pt_launch(SWEEPS_PER_STEP, EXCHANGE_EVERY, MEASURE_EVERY)
    step_ms = _timed_pt_steps(b, stream, flush, steps)
    dev_ms = float(sum(step_ms))
    sites = R * 128 ** 3
    value = sites * SWEEPS_PER_STEP * steps / (dev_ms * 1e6)
    launch_ms = b.time_halfsweep_graph(2 * SWEEPS_PER_STEP, 256 << 20, 5)
    roof = _roofline(b, launch_ms, peak, peak_kind, ncu_traffic(HBM_PROFILE),
                     "k_ising_words<3,0,3,4,2,1> (one half-sweep of 128 L=128 lattices; four words per lane through the shared-memory ring)",
                     f"HBM: {R * 128 ** 3 / 2 ** 20:.0f} MiB of spins, twice the L2; "
                     f"graph of {2 * SWEEPS_PER_STEP} half-sweeps, L2 flushed before each replay")
    b.close()
    return {"workload": f"3D Ising PT L=128 x {R} replicas, T in [{TMIN},{TMAX}], exchange 10, "
                        f"measure 5", "value": value, "unit": "flips/ns",
            "ms_per_step": dev_ms / steps, "steps": steps,
            "sweeps_per_s": SWEEPS_PER_STEP * steps / (dev_ms * 1e-3), "roofline": roof}


UNEVEN_SIZES = [8, 12, 16, 24, 32, 48, 64, 96, 128]


def uneven_case(pkg, stream, flush, steps):
    """Sizes from 8 to 128 that are not all powers of two, 32 replicas each, in
    one launch per half-sweep: rolling tasks (32, 64, 128), flat word tasks
    (8, 16, and 24, 48, 96 with rows that are not a power of two words long)
    and site-block tasks (12).  The same PT step and timing as the headline."""
    R = REPLICAS
    T = [TMIN + (TMAX - TMIN) * i / (R - 1) for i in range(R)]
    b = pkg.IsingBatch(UNEVEN_SIZES, R, seed=SEED + 5)
    b.set_stream(stream)
    b.set_temperatures(T)
    b.step(10)
    b.reset_sampling()
    for _ in range(3):
        b.pt_launch(SWEEPS_PER_STEP, EXCHANGE_EVERY, MEASURE_EVERY)
    step_ms = _timed_pt_steps(b, stream, flush, steps)
    dev_ms = float(sum(step_ms))
    sites = R * sum(L ** 3 for L in UNEVEN_SIZES)
    launch_ms = b.time_halfsweep_graph(2 * SWEEPS_PER_STEP, 256 << 20, 5)
    b.close()
    return {"workload": f"3D Ising PT L={','.join(map(str, UNEVEN_SIZES))} x {R} replicas, "
                        f"T in [{TMIN},{TMAX}], exchange 10, measure 5",
            "value": sites * SWEEPS_PER_STEP * steps / (dev_ms * 1e6), "unit": "flips/ns",
            "ms_per_step": dev_ms / steps, "steps": steps,
            "halfsweep_launches_per_sweep": 2, "halfsweep_ms": launch_ms,
            "halfsweep_flips_per_ns": sites / 2 / (launch_ms * 1e6)}


def ess_case(pkg, stream, sweeps_per_s):
    """ESS/s of |M| on the headline batch from a run of its own: ESS_WARMUP
    warm-up sweeps, then ESS_SWEEPS sweeps with a record every 5 (at L = 128
    near Tc, tau_int has come out between about 800 and 1700 sweeps, so the
    run covers 60-125 tau).  tau is the
    larger of the windowed estimate (reproduce_validation.py:157-163) and the
    20-block estimate, per size at the slot nearest Tc.  ESS/s follows the
    spec definition: sweeps/s of the timed batch / tau_int(|M|) in sweeps,
    with tau_int = 1/2 + sum of the autocorrelation (1/2 for independent samples;
    N / (2 tau_int) is the other common convention and is half of it)."""
    T = temps()
    b = pkg.IsingBatch(SIZES, REPLICAS, seed=SEED + 11)
    b.set_stream(stream)
    b.set_temperatures(T)
    b.step(ESS_WARMUP)
    b.reset_sampling()
    rt, rb, rm = b.pt_run(ESS_SWEEPS, EXCHANGE_EVERY, MEASURE_EVERY)
    b.close()
    slot = int(np.argmin([abs(t - TC_3D) for t in T]))
    per = {}
    for s, L in enumerate(SIZES):
        sl = slice(s * REPLICAS, (s + 1) * REPLICAS)
        mask = rt[:, sl] == slot
        series = np.abs(rm[:, sl][mask].astype(float)) / L ** 3
        tw, tb = tau_int(series), tau_blocking(series)
        tau_s = max(tw, tb) * MEASURE_EVERY
        per[str(L)] = {"tau_int_sweeps": tau_s, "tau_windowed_sweeps": tw * MEASURE_EVERY,
                       "tau_blocking_sweeps": tb * MEASURE_EVERY, "records": int(len(series)),
                       "records_per_tau": len(series) * MEASURE_EVERY / tau_s,
                       "ess_per_s": sweeps_per_s / tau_s}
    h = per["128"]
    return {"value": h["ess_per_s"], "unit": "ESS/s", "observable": "|M|", "L": 128,
            "T": T[slot], "tau_int_sweeps": h["tau_int_sweeps"], "records": h["records"],
            "sweeps": ESS_SWEEPS, "warmup_sweeps": ESS_WARMUP,
            "convention": "sweeps/s / tau_int(|M|) in sweeps, tau_int = 1/2 + sum rho(t) "
                          "(max of windowed and 20-block estimates); N/(2 tau) is half of it",
            "per_size": per}


def config1_case(pkg):
    """3D cubic Ising L = 16, single T = 4.5115, seed 42, 1000 warm-up + 1000
    measured sweeps with E and |M| every sweep (the reference's plain sweep
    binary).  One synchronous C-ABI call (isg_ising_run_schedule) runs all 2000
    sweeps in one launch of the cluster-resident kernel; timed end to end
    (host record arrays included).  Beside it, the reference CPU path (random-site
    Metropolis, src/metropolis.rs:8-27, restated in C) on one host thread."""
    L, T, n = 16, TC_3D, 16 ** 3
    b = pkg.IsingBatch([L], 1, seed=SEED)
    b.set_temperatures([T])
    b.run_schedule(None, 2000, 1)        # warm the code path (module load, first launch)
    times, recs = [], None
    for rep in range(5):
        c = pkg.IsingBatch([L], 1, seed=SEED)
        c.set_temperatures([T])
        t0 = time.perf_counter()
        bond, mag = c.run_schedule(None, 2000, 1)
        times.append(time.perf_counter() - t0)
        recs = (bond, mag)
        c.close()
    b.close()
    wall = statistics.median(times)
    m = np.abs(recs[1][1000:, 0].astype(float)) / n
    e = -recs[0][1000:, 0].astype(float) / n
    tau = max(tau_int(m), tau_blocking(m))
    oracle = _load("isg_oracle", ROOT / "oracle" / "oracle.py")
    t0 = time.perf_counter()
    oracle.ref_run(L, 3, T, SEED, 1000, 1000)
    cpu_s = time.perf_counter() - t0
    return {"workload": "3D Ising L=16, T=4.5115, 1000 warm-up + 1000 measured sweeps, E and |M| "
                        "every sweep (one lattice)",
            "value": 2000 * n / (wall * 1e9), "unit": "flips/ns", "wall_ms": wall * 1e3,
            "sweeps_per_s": 2000 / wall, "E": float(e.mean()), "M": float(m.mean()),
            "tau_int_sweeps": tau, "ess_per_s": 1000 / tau / wall,
            "path": "isg_ising_run_schedule (C ABI), one resident-kernel launch, host records",
            "cpu_baseline": {"value": 2000 * n / (cpu_s * 1e9), "unit": "flips/ns", "cores": 1,
                             "kind": "port", "wall_ms": cpu_s * 1e3,
                             "sample": "the same 2000 sweeps on one host thread (reference CPU "
                                       "path restated in C)"}}


def run_gpu(args):
    import torch
    ws, rank, local = dist_info()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    pkg = _load("ising_gb300", ROOT / "ising-rs_gb300" / "__init__.py")

    stream = torch.cuda.Stream(device=dev)
    T = temps()
    b = pkg.IsingBatch(SIZES, REPLICAS, seed=SEED + rank)
    b.set_stream(stream)
    b.set_temperatures(T)
    if args.autotune:
        b.autotune()
    b.step(100)
    b.reset_sampling()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    nsweep_sites = sites_per_sweep()
    for _ in range(args.warmup):
        b.pt_run(SWEEPS_PER_STEP, EXCHANGE_EVERY, MEASURE_EVERY)
    b.reset_sampling()
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    with clocks:
        wall0 = time.perf_counter()
        step_ms = _timed_pt_steps(b, stream, flush, args.steps)
        wall = time.perf_counter() - wall0
    if ws > 1:
        torch.distributed.barrier()
    dev_ms = max_over_ranks(float(sum(step_ms)), dev)
    value = job_flips_per_ns(nsweep_sites, SWEEPS_PER_STEP * args.steps, ws, dev_ms)
    sweeps_per_s = SWEEPS_PER_STEP * args.steps / (dev_ms * 1e-3)

    # e2e: the C-ABI call with host record buffers, records copied back each step
    b2 = pkg.IsingBatch(SIZES, REPLICAS, seed=SEED + 1000 + rank)
    b2.set_stream(stream)
    b2.set_temperatures(T)
    b2.step(100)
    b2.reset_sampling()
    e2e_steps = max(1, args.steps // 2)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    d2h = 0
    for i in range(e2e_steps):
        rt, rb, rm = b2.pt_run(SWEEPS_PER_STEP, EXCHANGE_EVERY, MEASURE_EVERY)
        d2h += rt.nbytes + rb.nbytes + rm.nbytes
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e_value = nsweep_sites * SWEEPS_PER_STEP * e2e_steps * ws / (e2e_s * 1e9)
    b2.close()

    # roofline of the half-sweep kernel as it runs in the timed step: a graph of
    # the step's 20 half-sweeps, L2 flushed before each replay
    peak, peak_kind = measured_peaks()
    launch_ms = b.time_halfsweep_graph(2 * SWEEPS_PER_STEP, 256 << 20, 5)
    roof = _roofline(b, launch_ms, peak, peak_kind, ncu_traffic(HEADLINE_PROFILE),
                     "k_ising_words<3,0,3,4,2,1> (one half-sweep, all 160 lattices)",
                     "L2: the 73 MiB batch fits in L2, which is flushed once per 20 "
                     "half-sweeps (before every step), so most launches read L2; the HBM "
                     "figure is roofline_hbm")
    roof["share_of_step"] = 2 * SWEEPS_PER_STEP * launch_ms / (dev_ms / args.steps)
    b.close()

    if rank != 0:
        return 0
    hbm = hbm_case(pkg, stream, flush, max(3, min(args.steps, 100)), peak, peak_kind)
    ess = ess_case(pkg, stream, sweeps_per_s)
    cfg1 = config1_case(pkg)
    uneven = uneven_case(pkg, stream, flush, args.steps)
    learned = learned_summary(pkg, args) if args.learned_seconds > 0 else None
    threads = host_threads()
    cpu_v, cpu_s, cpu_f = cpu_sample(threads, sweeps=args.cpu_sweeps)
    launches_per_step = 2 * SWEEPS_PER_STEP + (SWEEPS_PER_STEP // MEASURE_EVERY)
    line = {
        "metric": METRIC, "value": value, "unit": "flips/ns", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dev_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int8",
        "data": "synthetic (seeded Philox hot start)",
        "config": {"workload": WORKLOAD, "step": "10 sweeps + 2 fused measures + 1 exchange "
                                                 "(one CUDA graph)",
                   "sites_per_sweep": nsweep_sites, "l2": "flushed (256 MiB write) before "
                                                          "every timed step",
                   "launch": "persistent word kernel, grid = SMs x occupancy"},
        "sweeps_per_s": sweeps_per_s,
        "hbm_gbs_algorithmic": value * BYTES_PER_UPDATE,
        "ess_per_s": ess,
        "e2e": {"value": e2e_value, "unit": "flips/ns", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": d2h // e2e_steps,
                "path": "isg_ising_pt_run (C ABI) per step, (slot,E,M) records copied to host "
                        "arrays in the timed region; a PT step consumes no host input "
                        "(lattices and temperature tables stay resident in HBM)"},
        "roofline": roof,
        "roofline_hbm": hbm,
        "config1": cfg1,
        "uneven": uneven,
        "learned": learned,
        "cpu_baseline": {"value": cpu_v, "unit": "flips/ns", "cores": threads, "kind": "port",
                         "sample": f"{threads} threads x {args.cpu_sweeps:g} random-site sweeps "
                                   f"of L=8..128 each ({cpu_f:.3g} flips, {cpu_s:.1f} s); "
                                   f"reference CPU path restated in C"},
        "cpu_replay": cpu_replay(threads),
        "gpu_launches": launches_per_step * args.steps,
        "clocks": clocks.summary(),
        "wall_s": wall,
    }
    print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def jackknife_mean_err(x, nb=20):
    x = np.asarray(x, float)
    n = len(x) // nb * nb
    if n < nb:
        return float("nan")
    x = x[:n]
    full = x.mean()
    jk = np.array([(x.sum() - x[b * (n // nb):(b + 1) * (n // nb)].sum()) / (n - n // nb)
                   for b in range(nb)])
    return float(np.sqrt((nb - 1) / nb * ((jk - full) ** 2).sum()))


def learned_case(pkg, L, dim, T, train_seconds, chain_batches, pt_sweeps):
    """Learned-proposal workload (2D L=16/32 at T=2.269, 3D L=8 at T=4.51): ESS/s
    of |M| and E of one chain at T, plain checkerboard PT vs the
    learned independence proposal (+ interleaved sweeps)."""
    import torch
    import importlib
    lrn = importlib.import_module(pkg.__name__ + ".learned")
    n = L ** dim
    H, W = (L, L) if dim == 2 else (L * L, L)
    # plain PT: 17 replicas on a linear grid with T at the middle slot
    R = 17
    width = 0.20 if dim == 2 else 0.10
    temps = [T - width + 2 * width * i / (R - 1) for i in range(R)]
    b = pkg.IsingBatch([L], R, seed=SEED, dim=dim)
    b.set_temperatures(temps)
    b.step(5000)
    b.reset_sampling()
    b.pt_run(2000, 10, 1)
    b.sync()
    t0 = time.perf_counter()
    rt, rb, rm = b.pt_run(pt_sweeps, 10, 1)
    pt_s = time.perf_counter() - t0
    mid = R // 2
    series = np.array([abs(rm[i][rt[i] == mid][0]) / n for i in range(rt.shape[0])], float)
    eseries = np.array([-float(rb[i][rt[i] == mid][0]) / n for i in range(rt.shape[0])], float)
    # the larger of the windowed and the blocking estimate, on both sides
    tau_pt_w, tau_pt_b = tau_int(series), tau_blocking(series)
    tau_pt = max(tau_pt_w, tau_pt_b)
    ess_pt = len(series) / (2 * tau_pt) / pt_s
    tau_pt_e = max(tau_int(eseries), tau_blocking(eseries))
    ess_pt_e = len(eseries) / (2 * tau_pt_e) / pt_s
    # training data from the plain sampler at T, with Z2 partners
    t1 = time.perf_counter()
    # streaming maximum-likelihood training: every step sees fresh
    # configurations of the plain sampler at T (256 chains, a snapshot every 10
    # sweeps, with negations), so the network cannot memorise a fixed set
    stream = lrn.TrainingStream(L, dim, T, chains=256, gap=10, warmup=2000)
    q = lrn.LearnedProposal(H, W, layers=6, seed=SEED, zrow=L if dim == 3 else 0)
    steps = 0
    tt = time.perf_counter()
    while time.perf_counter() - tt < train_seconds:
        q.train(stream.next(), batch=128, steps=4, lr=1e-3)
        steps += 4
    train_s = time.perf_counter() - t1
    nll = -q.train(stream.next(), batch=128, steps=1, lr=1e-4) / n  # held-out batch
    stream.close()
    # 20 checkerboard sweeps between batches: with a single sweep the
    # independence chain at L = 32 had not left the ordered states the network
    # over-represents after 10M proposals; 20 cost under 5% of a batch
    ch = lrn.LearnedChain(q, L, dim, T, K=None, sweeps=20, fallback_sweeps=50, min_accept=0.002)
    ch.start(1000)
    ch.batch()
    t2 = time.perf_counter()
    for _ in range(chain_batches):
        ch.batch()
    torch.cuda.synchronize()
    ch_s = time.perf_counter() - t2
    m = ch.m_series()[ch.K:]
    tau_l_w, tau_l_b = tau_int(m), tau_blocking(m)
    tau_l = max(tau_l_w, tau_l_b)
    ess_l = len(m) / (2 * tau_l) / ch_s
    m_err_l, m_err_pt = jackknife_mean_err(m), jackknife_mean_err(series)
    e = ch.e_series()[ch.K:]
    tau_l_e = max(tau_int(e), tau_blocking(e))
    ess_l_e = len(e) / (2 * tau_l_e) / ch_s
    e_err_l, e_err_pt = jackknife_mean_err(e), jackknife_mean_err(eseries)
    out = {"case": f"{dim}D L={L} T={T}", "plain_pt": {
        "replicas": R, "T_grid": [temps[0], temps[-1]], "sweeps": pt_sweeps,
        "seconds": pt_s, "sweeps_per_s": pt_sweeps / pt_s, "tau_int_sweeps": tau_pt,
        "tau_windowed": tau_pt_w, "tau_blocking": tau_pt_b,
        "ess_per_s": ess_pt, "M": float(series.mean()), "M_err": m_err_pt,
        "tau_E_sweeps": tau_pt_e, "ess_E_per_s": ess_pt_e, "E": float(eseries.mean()),
        "E_err": e_err_pt},
        "learned": {"layers": 6, "channels": 32, "train_steps": steps, "train_s": train_s,
                    "nll_per_site": nll, "batch_K": ch.K, "sweeps_per_batch": ch.sweeps,
                    "proposals": len(m), "seconds": ch_s,
                    "acceptance": float(np.mean(ch.batch_accept[1:])),
                    "tau_int_proposals": tau_l, "tau_windowed": tau_l_w, "tau_blocking": tau_l_b,
                    "ess_per_s": ess_l, "M": float(m.mean()), "M_err": m_err_l,
                    "tau_E_proposals": tau_l_e, "ess_E_per_s": ess_l_e, "E": float(e.mean()),
                    "E_err": e_err_l},
        # both chains sample the same distribution: their |M| and E must agree
        "M_diff_sigma": float((m.mean() - series.mean()) / np.hypot(m_err_l, m_err_pt)),
        "E_diff_sigma": float((e.mean() - eseries.mean()) / np.hypot(e_err_l, e_err_pt)),
        "ratio_learned_over_plain": ess_l / ess_pt,
        "ratio_E_learned_over_plain": ess_l_e / ess_pt_e}
    ch.close()
    return out


CONT_WORKLOADS = {
    # Heisenberg PT: O(3), L=32,64,96 x 24 replicas on [1.40,1.48], 1 Metropolis (cone) + 4 OR
    "heisenberg": dict(nc=3, sizes=[32, 64, 96], R=24, tmin=1.40, tmax=1.48, n_or=4, delta=0.5,
                       bytes_per_update=36),
    # XY PT: O(2), L=32,64,128 x 16 replicas on [2.18,2.22], uniform-angle Metropolis + 2 OR
    "xy": dict(nc=2, sizes=[32, 64, 128], R=16, tmin=2.18, tmax=2.22, n_or=2, delta=math.pi,
               bytes_per_update=24),
}


def run_continuous(args):
    """Configs 3/4: one step = 10 sweeps (each n_or overrelaxation sweeps + one
    Metropolis sweep), 2 measurements (E, M, helicity sums), 1 exchange."""
    import torch
    w = CONT_WORKLOADS[args.workload]
    torch.cuda.set_device(0)
    pkg = _load("ising_gb300", ROOT / "ising-rs_gb300" / "__init__.py")
    stream = torch.cuda.Stream()
    R = w["R"]
    T = [w["tmin"] + (w["tmax"] - w["tmin"]) * i / (R - 1) for i in range(R)]
    b = pkg.ContinuousBatch(w["sizes"], R, w["nc"], seed=SEED)
    b.set_stream(stream)
    b.set_temperatures(T)
    if args.workload == "heisenberg":
        # Heisenberg: cone width tuned for about 50% acceptance during warm-up
        w = dict(w, delta=pkg.tune_delta(b, w["delta"], w["n_or"], 0.5))
    b.sweep(50, w["delta"], w["n_or"])
    b.reset_sampling()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    for _ in range(args.warmup):
        b.pt_run(10, 10, 5, w["delta"], w["n_or"], 100)
    b.reset_sampling()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    torch.cuda.synchronize()
    clocks = ClockSampler(0)
    with clocks:
        with torch.cuda.stream(stream):
            for i in range(args.steps):
                flush.fill_(i & 0xFF)
                starts[i].record(stream)
                _ck = pkg.lib().isg_cont_pt_run(b._h, 10, 10, 5, float(w["delta"]), w["n_or"], 100,
                                                None, None, None, None, 0, None)
                pkg._check(_ck)
                ends[i].record(stream)
        torch.cuda.synchronize()
    dev_ms = sum(s_.elapsed_time(e_) for s_, e_ in zip(starts, ends))
    sites = b.sites_per_sweep()                     # site updates of one full sweep
    updates = sites * (1 + w["n_or"]) * 10 * args.steps
    value = updates / (dev_ms * 1e6)
    kt = [float(x) for x in b.time_kernels(20)]     # OR half, Metropolis half, measure,
                                                    # Metropolis half + fused measure (ms)
    half = sites // 2
    peak, peak_kind = measured_peaks()
    roof = {}
    for name, ms in (("overrelax", kt[0]), ("metropolis", kt[1])):
        ach = half * w["bytes_per_update"] / (ms * 1e-3) / 1e9
        roof[name] = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                      "frac": ach / peak, "launch_ms": float(ms),
                      "bytes_per_launch": half * w["bytes_per_update"]}
    meas_bytes = sites * w["nc"] * 4
    roof["measure"] = {"achieved": meas_bytes / (kt[2] * 1e-3) / 1e9, "launch_ms": float(kt[2]),
                       "bytes_per_launch": meas_bytes, "unit": "GB/s",
                       "note": "separate pass (isg_cont_measure); the PT step fuses it"}
    fb = half * w["bytes_per_update"]
    roof["metropolis_fused_measure"] = {
        "bound": "hbm", "achieved": fb / (kt[3] * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
        "frac": fb / (kt[3] * 1e-3) / 1e9 / peak, "launch_ms": float(kt[3]),
        "bytes_per_launch": fb,
        "note": "colour-1 Metropolis half-sweep of a measured sweep with the 10 sums fused; "
                "extra time over a Metropolis half-sweep: %.4f ms" % (kt[3] - kt[1])}
    acc = b.metropolis_accepted().sum() / (sites * 10 * args.steps)
    line = {"metric": f"site updates/ns ({args.workload} PT, Metropolis + {w['n_or']} OR per sweep)",
            "value": value, "unit": "updates/ns", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True,
            "dtype": "f32", "data": "synthetic (seeded Philox start)",
            "config": {"workload": f"{args.workload}: L={w['sizes']} x {R} replicas, T in "
                                   f"[{w['tmin']},{w['tmax']}], delta {w['delta']:.4g}",
                       "l2": "flushed (256 MiB write) before every timed step"},
            "metropolis_acceptance": float(acc), "roofline": roof,
            "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
            "clocks": clocks.summary()}
    print(json.dumps(line), flush=True)
    return 0


ANNEAL = dict(sizes=[8, 12, 16, 20, 24, 28], t_min=3.5, t_max=5.5, t_steps=41, warmup=500,
              samples=200)


def run_anneal(args):
    """`fss --gpu` (src/cuda/fss_gpu.rs:7-39) at the reference's FssConfig defaults
    (src/fss.rs:20-36): every size anneals from 5.5 down to 3.5 over 41 temperatures,
    500 warm-up + 200 measured sweeps at each.  One step = the whole schedule
    through the synchronous C-ABI call isg_fss_anneal (host arrays in and out), so
    value and e2e are the same wall-clock measurement."""
    import ctypes as C
    import torch
    torch.cuda.set_device(0)
    pkg = _load("ising_gb300", ROOT / "ising-rs_gb300" / "__init__.py")
    a = ANNEAL
    sz = np.ascontiguousarray(a["sizes"], np.int32)
    out = np.zeros((len(a["sizes"]), a["t_steps"], 7), np.float64)

    def once():
        pkg._check(pkg.lib().isg_fss_anneal(
            sz.ctypes.data_as(C.c_void_p), len(sz), 3, a["t_min"], a["t_max"], a["t_steps"], 1.0,
            0.0, a["warmup"], a["samples"], SEED, out.ctypes.data_as(C.c_void_p)))

    steps, warm = max(1, min(args.steps, 10)), max(1, min(args.warmup, 3))
    for _ in range(warm):
        once()
    torch.cuda.synchronize()
    clocks = ClockSampler(0)
    with clocks:
        t0 = time.perf_counter()
        for _ in range(steps):
            once()
        wall = time.perf_counter() - t0
    updates = sum(L ** 3 for L in a["sizes"]) * a["t_steps"] * (a["warmup"] + a["samples"])
    value = updates * steps / wall * 1e-9
    threads = host_threads()
    oracle = _load("isg_oracle", ROOT / "oracle" / "oracle.py")
    rb = oracle.RefBench(a["sizes"], 3, 4.5, 4.5 + 1e-9, threads, seed=SEED)
    rb.step(0.5)
    sec, flips = rb.step(200.0)
    rb.close()
    cpu = flips / sec * 1e-9
    d2h = len(a["sizes"]) * a["t_steps"] * a["samples"] * (4 + 8 + 8)
    h2d = a["t_steps"] * len(a["sizes"]) * (16 * 4 + 8 + 2 * 4)
    line = {"metric": "spin flips/ns, annealing FSS schedule (fss --gpu defaults)",
            "value": value, "unit": "flips/ns", "n_gpus": 1, "steps": steps, "warmup": warm,
            "ms_per_step": wall / steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int8", "data": "synthetic (seeded Philox start)",
            "config": {"workload": f"fss --gpu: L={a['sizes']}, {a['t_steps']} T from "
                                   f"{a['t_max']} down to {a['t_min']}, {a['warmup']}+"
                                   f"{a['samples']} sweeps per T",
                       "timing": "wall clock around the synchronous isg_fss_anneal call",
                       "l2": "all lattices together (50 KB) stay in L2; the schedule is "
                             "launch-bound"},
            "e2e": {"value": value, "unit": "flips/ns", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "cpu_baseline": {"value": cpu, "unit": "flips/ns", "cores": threads, "kind": "port",
                             "sample": f"200 random-site sweeps of each of L={a['sizes']} per "
                                       f"host thread at T=4.5 (reference CPU Metropolis path "
                                       f"restated in C)"},
            "clocks": clocks.summary()}
    print(json.dumps(line), flush=True)
    return 0


KZ = dict(n=20, t_start=6.0, t_end=1.0, tau_min=100, tau_max=100000, tau_steps=20, trials=5,
          warmup=200)
COARSEN = dict(n=30, t_high=10.0, t_quench=0.5, warmup=200, steps=50000, every=100)


def _quench_line(metric, workload, value, steps, warm, wall, h2d, d2h, cpu, sample, clocks):
    return {"metric": metric, "value": value, "unit": "flips/ns", "n_gpus": 1, "steps": steps,
            "warmup": warm, "ms_per_step": wall / steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int8",
            "data": "synthetic (seeded Philox start)",
            "config": {"workload": workload,
                       "timing": "wall clock around the synchronous C-ABI call",
                       "l2": "lattices (<= 27 KB each) stay on chip (distributed shared memory)"},
            "e2e": {"value": value, "unit": "flips/ns", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "cpu_baseline": {"value": cpu, "unit": "flips/ns", "cores": host_threads(),
                             "kind": "port", "sample": sample},
            "clocks": clocks}


def run_quench(args):
    """`kz --gpu` and `coarsening --gpu` at the reference CLIs' defaults
    (src/bin/kz.rs:63-75, src/coarsening.rs:36-50).  One step = the whole protocol
    through isg_kz_sweep / isg_coarsening (host arrays in and out)."""
    import ctypes as C
    import torch
    torch.cuda.set_device(0)
    pkg = _load("ising_gb300", ROOT / "ising-rs_gb300" / "__init__.py")
    oracle = _load("isg_oracle", ROOT / "oracle" / "oracle.py")
    L = pkg.lib()
    steps, warm = max(1, min(args.steps, 5)), max(1, min(args.warmup, 2))
    threads = host_threads()
    if args.workload == "kz":
        k = KZ
        lmin, lmax = math.log(k["tau_min"]), math.log(k["tau_max"])
        taus = np.array([round(math.exp(lmin + (lmax - lmin) * i / (k["tau_steps"] - 1)))
                         for i in range(k["tau_steps"])], np.int64)
        out = np.zeros((len(taus), 2))

        def once():
            pkg._check(L.isg_kz_sweep(k["n"], 1.0, k["t_start"], k["t_end"],
                                      taus.ctypes.data_as(C.c_void_p), len(taus), k["trials"],
                                      k["warmup"], 0, 0.01, SEED, out.ctypes.data_as(C.c_void_p)))
        updates = int((taus + k["warmup"]).sum()) * k["trials"] * k["n"] ** 3
        workload = (f"kz --gpu: N={k['n']}, {k['tau_steps']} tau_q log-spaced in "
                    f"[{k['tau_min']},{k['tau_max']}], {k['trials']} trials, warm-up "
                    f"{k['warmup']}, ramp {k['t_start']} -> {k['t_end']}")
        h2d = int((taus + k["warmup"]).sum()) * 4 + len(taus) * 64
        d2h = len(taus) * k["trials"] * 16
        metric = "spin flips/ns, Kibble-Zurek quench sweep (kz --gpu defaults)"
        size = [k["n"]]
    else:
        k = COARSEN
        pts = (k["steps"] - 1) // k["every"] + 1
        st = np.zeros(pts, np.int64)
        rho = np.zeros(pts)
        npt = C.c_int64()

        def once():
            pkg._check(L.isg_coarsening(k["n"], 1.0, k["t_high"], k["t_quench"], k["warmup"],
                                        k["steps"], k["every"], SEED,
                                        st.ctypes.data_as(C.c_void_p),
                                        rho.ctypes.data_as(C.c_void_p), pts, C.byref(npt)))
        updates = (k["warmup"] + k["steps"]) * k["n"] ** 3
        workload = (f"coarsening --gpu: N={k['n']}, warm-up {k['warmup']} at T={k['t_high']}, "
                    f"{k['steps']} sweeps at T={k['t_quench']}, rho every {k['every']}")
        h2d = 2 * (16 * 4 + 8)
        d2h = pts * 16
        metric = "spin flips/ns, coarsening after a quench (coarsening --gpu defaults)"
        size = [k["n"]]
    for _ in range(warm):
        once()
    clocks = ClockSampler(0)
    with clocks:
        t0 = time.perf_counter()
        for _ in range(steps):
            once()
        wall = time.perf_counter() - t0
    value = updates * steps / wall * 1e-9
    rb = oracle.RefBench(size, 3, 3.5, 3.5 + 1e-9, threads, seed=SEED)
    rb.step(0.5)
    sec, flips = rb.step(200.0)
    rb.close()
    sample = (f"200 random-site sweeps of L={size[0]} per host thread at T=3.5 (reference CPU "
              f"Metropolis path restated in C)")
    line = _quench_line(metric, workload, value, steps, warm, wall, h2d, d2h,
                        flips / sec * 1e-9, sample, clocks.summary())
    print(json.dumps(line), flush=True)
    return 0


JFIT = dict(graph_n=8, replicas=20, warmup=5000, samples=50000, exchange_every=10,
            temps={"ising": (6.0, 6.7), "heisenberg": (1.5, 3.0), "xy": (1.5, 3.0)})


def run_jfit(args):
    """`gpu_jfit --model ising|heisenberg|xy` at the reference CLI's defaults
    (src/bin/gpu_jfit.rs:25-35: 20 replicas, 5000 + 50000 samples, exchange
    every 10) on a BCC graph of 8^3 cells (1024 nodes, coordination 8).  One
    step = the whole protocol through the C ABI: create, warm-up, sampling with
    the (slot, E, M) records of every replica and sample copied to the host.
    The unit is the reference's unit of work, one replica sample (a sweep of N
    attempts, or one Wolff cluster for xy, followed by a measurement)."""
    import torch
    torch.cuda.set_device(0)
    pkg = _load("ising_gb300", ROOT / "ising-rs_gb300" / "__init__.py")
    oracle = _load("isg_oracle", ROOT / "oracle" / "oracle.py")
    model = args.workload.split("-", 1)[1] if "-" in args.workload else "ising"
    k = JFIT
    g = pkg.GraphDef.bcc(k["graph_n"])
    R, warmup, samples, ee = k["replicas"], k["warmup"], k["samples"], k["exchange_every"]
    tmin, tmax = k["temps"][model]
    temps = pkg.linspace_temperatures(tmin, tmax, R)
    nc = {"ising": 1, "heisenberg": 3, "xy": 2}[model]
    chunk = 10000

    def once():
        if model == "ising":
            b = pkg.GraphBatch(g.n_nodes, g.edges, R, seed=SEED)
        else:
            b = pkg.ContinuousGraphBatch(g.n_nodes, g.edges, R, nc, seed=SEED)
        b.set_temperatures(temps)
        b.step(warmup)
        b.reset_sampling()
        done = 0
        while done < samples:
            n = min(chunk, samples - done)
            b.pt_run(n, ee, 1)
            done += n
        b.close()

    steps, warm = max(1, min(args.steps, 5)), max(1, min(args.warmup, 2))
    for _ in range(warm):
        once()
    clocks = ClockSampler(0)
    with clocks:
        t0 = time.perf_counter()
        for _ in range(steps):
            once()
        wall = time.perf_counter() - t0
    per_step = R * (warmup + samples)
    value = per_step * steps / wall * 1e-3
    h2d = g.edges.size * 4 + R * 8
    rec = 4 + 8 + 8 * max(nc, 1)
    d2h = samples * R * rec
    # reference CPU algorithm (one thread, one shared generator), bounded sample
    cpu_samples = {"ising": 6000, "heisenberg": 2000, "xy": 8000}[model]
    t0 = time.perf_counter()
    if model == "ising":
        oracle.graph_ref_pt(g.n_nodes, g.edges, temps, 1.0, SEED, 0, cpu_samples, ee)
    else:
        oracle.cgraph_ref_pt(g.n_nodes, g.edges, nc, temps, 1.0, SEED, 0, cpu_samples, ee)
    cpu = R * cpu_samples / (time.perf_counter() - t0) * 1e-3
    line = {"metric": f"replica samples/ms, gpu_jfit --model {model} defaults on BCC N="
                      f"{k['graph_n']} ({g.n_nodes} nodes)",
            "value": value, "unit": "samples/ms", "n_gpus": 1, "steps": steps, "warmup": warm,
            "ms_per_step": wall / steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int8" if model == "ising" else "f32 (f64 sums)",
            "data": "synthetic (seeded Philox start)",
            "config": {"workload": f"gpu_jfit --model {model}: BCC {k['graph_n']}^3 cells, "
                                   f"{R} replicas, T in [{tmin}, {tmax}], warm-up {warmup}, "
                                   f"{samples} samples, exchange every {ee}",
                       "timing": "wall clock around the whole protocol (C ABI, host records)",
                       "l2": "the graph and the replicas' spins (< 1 MB) stay on chip"},
            "e2e": {"value": value, "unit": "samples/ms", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "cpu_baseline": {"value": cpu, "unit": "samples/ms", "cores": 1, "kind": "port",
                             "sample": f"{cpu_samples} samples of all {R} replicas, the "
                                       "reference's CPU algorithm restated in C "
                                       "(gpu_jfit.rs run loop, one shared Xoshiro256++)"},
            "clocks": clocks.summary()}
    print(json.dumps(line), flush=True)
    return 0


RW = dict(sims=20, samples=100000, targets=200, n=16, cpu_fraction=0.05)


def run_reweight(args):
    """The reweighting consumer of a gpu_fss run (analysis/scripts/
    analyze_gpu_fss.py:160-243, wham_reweight_fine): WHAM over 20 simulations
    x 100,000 samples (the gpu_fss default sample count) and the observables
    with their jackknife errors on a 200-point temperature grid.  One step =
    one call through the Python mirror with host arrays in and out (the
    samples are uploaded in the timed region).  The samples are synthetic
    overlapping Gaussian energies and |m| of an N = 16^3 lattice."""
    import torch
    torch.cuda.set_device(0)
    pkg = _load("ising_gb300", ROOT / "ising-rs_gb300" / "__init__.py")
    oracle = _load("isg_oracle", ROOT / "oracle" / "oracle.py")
    k = RW
    V = k["n"] ** 3
    rng = np.random.default_rng(SEED)
    betas = np.linspace(1 / 4.60, 1 / 4.40, k["sims"])
    el, ml = [], []
    for b in betas:
        el.append(rng.normal(-1.0 * V - 60000.0 * (b - betas[0]), 90.0, k["samples"]))
        ml.append(np.clip(rng.normal(0.3 + 30.0 * (b - betas[0]), 0.05, k["samples"]), 0, 1))
    T = np.linspace(4.40, 4.60, k["targets"])
    steps, warm = max(1, min(args.steps, 5)), max(1, min(args.warmup, 2))
    for _ in range(warm):
        pkg.wham_reweight_fine(el, ml, betas, T, k["n"])
    clocks = ClockSampler(0)
    with clocks:
        t0 = time.perf_counter()
        for _ in range(steps):
            pkg.wham_reweight_fine(el, ml, betas, T, k["n"])
        wall = time.perf_counter() - t0
    ms = wall / steps * 1e3
    # the reference algorithm in numpy on a bounded sample (every 20th sample
    # of each simulation); its cost is linear in the sample count
    frac = k["cpu_fraction"]
    sub = max(1, int(round(1 / frac)))
    t0 = time.perf_counter()
    oracle.rw_wham_fine([x[::sub] for x in el], [x[::sub] for x in ml], betas, T, k["n"])
    cpu_ms = (time.perf_counter() - t0) * 1e3 * sub
    P = k["sims"] * k["samples"]
    line = {"metric": "ms per WHAM reweighting of a gpu_fss run (wham_reweight_fine)",
            "value": ms, "unit": "ms", "n_gpus": 1, "steps": steps, "warmup": warm,
            "ms_per_step": ms, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Gaussian samples)",
            "config": {"workload": f"wham_reweight_fine: {k['sims']} simulations x "
                                   f"{k['samples']} samples (N = {k['n']}^3), "
                                   f"{k['targets']} target temperatures, 20 jackknife blocks",
                       "timing": "wall clock through the Python mirror (host arrays)"},
            "e2e": {"value": ms, "unit": "ms", "h2d_bytes_per_step": P * 8 * 5,
                    "d2h_bytes_per_step": k["targets"] * 21 * 6 * 8},
            "cpu_baseline": {"value": cpu_ms, "unit": "ms", "cores": 1, "kind": "port",
                             "sample": f"the reference's numpy algorithm (restated) on every "
                                       f"{sub}th sample, time scaled by {sub} (linear in the "
                                       "sample count)"},
            "clocks": clocks.summary()}
    print(json.dumps(line), flush=True)
    return 0


def ncu_case_resident():
    """No timing: one schedule of 2000 sweeps of one L=30 lattice (the coarsening
    default size) for an ncu capture of the cluster-resident kernel."""
    pkg = _load("ising_gb300", ROOT / "ising-rs_gb300" / "__init__.py")
    b = pkg.IsingBatch([30], 1, seed=SEED)
    b.set_temperatures([0.5])
    b.run_schedule(None, 2000)
    b.sync()
    print("ncu case done")
    return 0


def learned_summary(pkg, args):
    """The learned proposal against plain checkerboard PT, bounded for the
    default run: 2D L = 16 and L = 32 at T = 2.269, args.learned_seconds of
    streaming training each, 150 chain batches, 50,000 plain PT sweeps; ESS/s
    of |M| and E on both sides with the same estimator (learned_case).
    The full comparison is `bench.py --learned` (60 s of training, 800 batches)."""
    out = {"target": "learned / plain ESS/s of |M| >= 3 at 2D L=32, T=2.269", "cases": []}
    for L in (16, 32):
        c = learned_case(pkg, L, 2, 2.269, args.learned_seconds, 150, 50000)
        out["cases"].append({
            "case": c["case"], "ratio_M": c["ratio_learned_over_plain"],
            "ratio_E": c["ratio_E_learned_over_plain"],
            "plain_ess_M_per_s": c["plain_pt"]["ess_per_s"],
            "learned_ess_M_per_s": c["learned"]["ess_per_s"],
            "acceptance": c["learned"]["acceptance"], "train_s": c["learned"]["train_s"],
            "nll_per_site": c["learned"]["nll_per_site"], "M_diff_sigma": c["M_diff_sigma"]})
    return out


def run_learned(args):
    import torch
    torch.cuda.set_device(0)
    pkg = _load("ising_gb300", ROOT / "ising-rs_gb300" / "__init__.py")
    cases = [(16, 2, 2.269), (32, 2, 2.269), (8, 3, 4.51)]
    for L, dim, T in cases:
        out = learned_case(pkg, L, dim, T, args.train_seconds, args.chain_batches, args.pt_sweeps)
        print(json.dumps({"metric": "ESS/s of |M| and E at T (learned vs plain PT)", **out}),
              flush=True)
    return 0


def ncu_case_graph(kind: str):
    """No timing: cases for ncu captures of the graph, reweighting and learned
    kernels.  graph / cgraph3 / cgraph2: one 100-sweep launch on every replica
    of a BCC 8^3 graph (1024 nodes, 20 replicas) with a record every sweep;
    reweight: one WHAM analysis of 20 x 100,000 samples; learned: one chain
    batch (4096 rounded up to whole waves of the sampler) of the untrained 2D
    L=32 network (sampling, then the flipped scores); train: three training
    steps of that network on 128 seeded configurations."""
    pkg = _load("ising_gb300", ROOT / "ising-rs_gb300" / "__init__.py")
    if kind == "learned":
        import importlib
        import torch
        torch.cuda.set_device(0)
        lrn = importlib.import_module(pkg.__name__ + ".learned")
        q = lrn.LearnedProposal(32, 32, layers=6, seed=SEED)
        qn = q.batch_quantum()
        q.sample(-(-4096 // qn) * qn, 1)
        q.sync()
        print("ncu case done")
        return 0
    if kind == "train":
        # three training steps of the 2D L = 32 network on 128 configurations
        # (seeded +-1 bytes): the tensor-core forward, input and weight gradients
        import importlib
        import torch
        torch.cuda.set_device(0)
        lrn = importlib.import_module(pkg.__name__ + ".learned")
        q = lrn.LearnedProposal(32, 32, layers=6, seed=SEED)
        g = torch.Generator(device="cuda").manual_seed(SEED)
        d = (torch.randint(0, 2, (128, 1024), device="cuda", generator=g, dtype=torch.int8) * 2 - 1)
        q.train(d, batch=128, steps=3, lr=1e-3)
        q.sync()
        print("ncu case done")
        return 0
    if kind == "reweight":
        V = 16 ** 3
        rng = np.random.default_rng(SEED)
        betas = np.linspace(1 / 4.60, 1 / 4.40, 20)
        el = [rng.normal(-1.0 * V - 60000.0 * (b - betas[0]), 90.0, 100000) for b in betas]
        ml = [np.clip(rng.normal(0.3 + 30.0 * (b - betas[0]), 0.05, 100000), 0, 1) for b in betas]
        pkg.wham_reweight_fine(el, ml, betas, np.linspace(4.40, 4.60, 200), 16)
        print("ncu case done")
        return 0
    g = pkg.GraphDef.bcc(8)
    R = 20
    if kind == "graph":
        b = pkg.GraphBatch(g.n_nodes, g.edges, R, seed=SEED)
        b.set_temperatures(pkg.linspace_temperatures(6.0, 6.7, R))
    else:
        b = pkg.ContinuousGraphBatch(g.n_nodes, g.edges, R, 3 if kind == "cgraph3" else 2,
                                     seed=SEED)
        b.set_temperatures(pkg.linspace_temperatures(1.5, 3.0, R))
    b.step(50)
    b.reset_sampling()
    b.pt_run(100, 100, 1)
    print("ncu case done")
    return 0


def ncu_case_pt():
    """No timing: the headline PT workload (L = 8..128 x 32 replicas) for ncu:
    100 plain sweeps, then 10 PT steps (10 sweeps, 2 fused measurements, 1
    exchange each), L2 flushed (256 MiB write) before every step as in the
    timed region."""
    import torch
    torch.cuda.set_device(0)
    pkg = _load("ising_gb300", ROOT / "ising-rs_gb300" / "__init__.py")
    stream = torch.cuda.Stream()
    b = pkg.IsingBatch(SIZES, REPLICAS, seed=SEED)
    b.set_stream(stream)
    b.set_temperatures(temps())
    b.step(100)
    b.reset_sampling()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    _timed_pt_steps(b, stream, flush, 10)
    print("ncu case done")
    return 0


def ncu_case():
    """No timing: a few half-sweeps of the L=128 roofline case (128 replicas,
    268 MB of spins) for ncu captures of the half-sweep kernel."""
    pkg = _load("ising_gb300", ROOT / "ising-rs_gb300" / "__init__.py")
    R = HBM_REPLICAS
    b = pkg.IsingBatch([128], R, seed=SEED + 7)
    b.set_temperatures([TMIN + (TMAX - TMIN) * i / (R - 1) for i in range(R)])
    b.step(3)
    b.sync()
    print("ncu case done")
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--autotune", action="store_true")
    ap.add_argument("--cpu-sweeps", type=float, default=1.0)
    ap.add_argument("--ref-seconds", type=float, default=90.0)
    ap.add_argument("--workload", default="ising",
                    choices=["ising", "heisenberg", "xy", "anneal", "kz", "coarsening",
                             "jfit", "jfit-heisenberg", "jfit-xy", "reweight"])
    ap.add_argument("--learned", action="store_true",
                    help="learned proposal vs plain PT ESS/s on 2D L=16/32 and 3D L=8 "
                         "(separate JSON lines)")
    ap.add_argument("--train-seconds", type=float, default=60.0)
    ap.add_argument("--learned-seconds", type=float, default=20.0,
                    help="training seconds per case of the learned comparison carried by the "
                         "default line (0: leave it out)")
    ap.add_argument("--chain-batches", type=int, default=800)
    ap.add_argument("--pt-sweeps", type=int, default=200000)
    ap.add_argument("--ncu-case", nargs="?", const="words",
                    choices=["words", "pt", "resident", "graph", "cgraph3", "cgraph2",
                             "reweight", "learned", "train"],
                    help="no timing: 'words' = a few half-sweeps of L=128 x 128 replicas (268 MB, "
                         "larger than L2) for an ncu capture of the half-sweep kernel; "
                         "'pt' = 10 steps of the headline PT workload (launch list, traffic); "
                         "'resident' = one 2000-sweep schedule of an L=30 lattice; "
                         "'graph'/'cgraph3'/'cgraph2' = one 100-sweep launch of the graph "
                         "kernels (BCC 8^3, 20 replicas); 'reweight' = one WHAM analysis; "
                         "'learned' = 4096 proposals of the L=32 network (sample + score); "
                         "'train' = three training steps of that network")
    args = ap.parse_args()
    if args.ncu_case == "resident":
        return ncu_case_resident()
    if args.ncu_case == "pt":
        return ncu_case_pt()
    if args.ncu_case in ("graph", "cgraph3", "cgraph2", "reweight", "learned", "train"):
        return ncu_case_graph(args.ncu_case)
    if args.ncu_case:
        return ncu_case()
    if args.learned:
        return run_learned(args)
    if args.workload == "anneal":
        return run_anneal(args)
    if args.workload in ("kz", "coarsening"):
        return run_quench(args)
    if args.workload.startswith("jfit"):
        return run_jfit(args)
    if args.workload == "reweight":
        return run_reweight(args)
    if args.workload != "ising":
        return run_continuous(args)
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())

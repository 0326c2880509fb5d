"""Throughput of the lattice Monte Carlo hot path: attempted spin updates/ns.

Workload (one GPU): the XY parallel-tempering ladder -- L=128 periodic
square lattice, J=1, 32 temperatures geometric in [0.70, 1.20], angles drawn
uniformly in [0, 2pi) from a seed (wrapped to [-pi, pi)), Gaussian Metropolis
proposals with per-temperature widths tuned to ~50% acceptance during warm-up,
a replica exchange every 10 sweeps and a sample of (E, mx, my, twist cos/sin)
every 10 sweeps.  One step = 100 sweeps of all 32 replicas
(52,428,800 attempted updates).

Arms:
  default           the batched mixed-precision engine (mcgb.batch.LadderBatch),
                    one launch per 10 sweeps (sweeps, sample, exchange), CUDA-graph
                    replay;
  --impl reference  the reference algorithm on the host cores: the C
                    restatement of its kernels (the reference has no CPU sweep
                    of its own), OpenMP over replicas, a bounded sample;
  --api dropin      the same ladder through the reference's entry points,
                    Simulation(ParallelTempering(Runtime(XYModel()))), with
                    the reference's update rule (per-colour kernels, uniform
                    proposal), its schedule replayed as CUDA graphs.

`value` is the production mode (updates + exchange + sampling); `modes` adds
the same ladder with updates only and with updates + exchange.

Under torchrun each rank runs its own independent ladder (seeded by rank):
ladders share nothing, so the work shards with no data-path collective
(weak scaling); the timing takes the max over ranks.
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
for _p in (ROOT, ROOT / "gpu-monte-carlo_gb300"):
    if str(_p) not in sys.path:
        sys.path.insert(0, str(_p))

L = 128
N_TEMPS = 32
T_MIN, T_MAX = 0.70, 1.20
EXCHANGE_INTERVAL = 10
SAMPLE_INTERVAL = 10
SWEEPS_PER_STEP = 100
BYTES_PER_UPDATE = 40      # XY: 4+4 B angle read+write, 32 B RNG stream read+write
METRIC = "attempted spin updates/ns"
WORKLOAD = "XY PT ladder L=128 x 32 temperatures geometric [0.70, 1.20], Gaussian MH (sigma tuned to ~50%)"
REFERENCE_WORKLOAD = ("XY PT ladder L=128 x 32 temperatures geometric [0.70, 1.20], the reference's uniform "
                      "proposal theta + 1.5 (2u - 1) (models/xy/update.py:6-54)")


def temperatures():
    return np.geomspace(T_MIN, T_MAX, N_TEMPS)


def initial_angles(seed):
    rng = np.random.default_rng(seed)
    theta = rng.uniform(0.0, 2 * np.pi, (N_TEMPS, L, L))
    theta = np.where(theta >= np.pi, theta - 2 * np.pi, theta).astype(np.float32)
    return np.clip(theta, np.float32(-np.pi), np.nextafter(np.float32(np.pi), np.float32(0)))


PROFILE = {"xy-pt-l128": "window_kernel_xy_L128x32.md", "he3-ragged": "window_kernel_he3_ragged.md",
           "kawamura-l96x64": "window_kernel_kawamura_L96x3072.md", "fss-ising": "window_kernel_fss_ising.md",
           "fss-xy": "window_kernel_fss_xy.md"}


def profile_figures(name):
    """Figures of a committed ncu summary under profiles/ (one capture of the
    workload's window kernel): {metric: value} for the rows whose metric name
    is given in backticks, in base units, or {} if there is none."""
    path = ROOT / "profiles" / name if name else None
    if path is None or not path.exists():
        return {}
    scale = {"byte": 1, "Kbyte": 1e3, "Mbyte": 1e6, "Gbyte": 1e9, "inst": 1, "us": 1e-6, "ms": 1e-3}
    out = {}
    for line in path.read_text().splitlines():
        cells = line.split("|")
        if len(cells) < 4 or "(`" not in cells[1]:
            continue
        key = cells[1].split("(`")[1].split("`)")[0]
        fields = cells[2].split()
        try:
            out[key] = float(fields[0].replace(",", "")) * scale.get(fields[1] if len(fields) > 1 else "", 1)
        except (ValueError, IndexError):
            continue
    return out


def roofline_line(figs, source, updates_per_launch, launch_ms, bytes_per_update, sm_mhz, kernel,
                  scale_traffic=False):
    """The window kernel against the bound that binds it.

    Two bounds are evaluated.  Instruction issue: warp instructions per
    launch (per attempted update from the ncu capture, smsp__inst_executed.sum
    over the captured launch's updates) / the launch's event-timed duration,
    against SMs x 4 schedulers x 1 warp instruction per cycle x the SM clock
    sampled during the timed region.  HBM: the capture's DRAM bytes
    (dram__bytes_read.sum + write.sum, per launch; with ``scale_traffic``
    scaled from the captured case to this launch by the updates each
    processes) over the duration, against the measured copy bandwidth.  The
    larger fraction names the bound.  With "issue", "achieved"/"peak" are
    warp instructions per second; with "hbm" they are the model's
    algorithmic bytes (state r+w + 32 B of RNG stream per update) per
    second, as the roofline of a bandwidth-bound kernel counts them; both
    figures appear under "issue" and "hbm"."""
    import torch
    peak_hbm, peak_kind = load_peaks()
    alg = bytes_per_update * updates_per_launch / (launch_ms * 1e-3) / 1e9
    n_sm = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    issue_peak = n_sm * 4 * sm_mhz * 1e6 / 1e9
    traffic = None
    if "dram__bytes_read.sum" in figs and "dram__bytes_write.sum" in figs:
        traffic = figs["dram__bytes_read.sum"] + figs["dram__bytes_write.sum"]
        if scale_traffic and figs.get("updates"):
            traffic *= updates_per_launch / figs["updates"]
    dram_frac = None if traffic is None else traffic / (launch_ms * 1e-3) / 1e9 / peak_hbm
    hbm = {"achieved": alg, "peak": peak_hbm, "unit": "GB/s", "frac": alg / peak_hbm,
           "bytes_per_update": bytes_per_update, "peak_source": peak_kind,
           "dram_frac": dram_frac,
           "note": "achieved: algorithmic bytes (state r+w + 32 B of RNG stream per update) over the kernel time; "
                   "dram_frac: the DRAM bytes actually moved (traffic) over the kernel time"}
    issue = {"achieved": None, "peak": issue_peak, "unit": "G warp-instructions/s", "frac": None,
             "peak_source": f"{n_sm} SMs x 4 schedulers x {sm_mhz:.0f} MHz (sampled)"}
    if "smsp__inst_executed.sum" in figs and figs.get("updates"):
        per_update = figs["smsp__inst_executed.sum"] / figs["updates"]
        achieved = per_update * updates_per_launch / (launch_ms * 1e-3) / 1e9
        issue.update({"achieved": achieved, "frac": achieved / issue_peak, "warp_instructions_per_update": per_update})
    line = {"traffic": traffic, "kernel": kernel, "kernel_ms": launch_ms, "issue": issue, "hbm": hbm,
            "source": f"profiles/{source}" if figs else None}
    if dram_frac is not None and (issue["frac"] is None or dram_frac > issue["frac"]):
        line.update({"bound": "hbm", "achieved": alg, "peak": peak_hbm, "unit": "GB/s", "frac": alg / peak_hbm})
    else:
        line.update({"bound": "issue", "achieved": issue["achieved"], "peak": issue_peak,
                     "unit": "G warp-instructions/s", "frac": issue["frac"]})
    return line


def load_peaks():
    path = ROOT / "MEASURED_PEAKS.json"
    if path.exists():
        d = json.loads(path.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, ValueError):
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
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ CPU arms


def cpu_sample(n_threads, sweeps, seed=7):
    """Time the oracle (the reference algorithm restated in C: uniform
    delta = 1.5 proposals, models/xy/update.py:6-54) on the host cores for
    `sweeps` sweeps of the ladder with exchanges and samples; updates/ns."""
    import oracle

    temps = temperatures()
    R = N_TEMPS
    theta = initial_angles(seed)
    rng = oracle.rng_states(R * L * L, seed)
    betas = (1.0 / temps).astype(np.float32)
    w2t = np.arange(R, dtype=np.int32)
    t2w = np.arange(R, dtype=np.int32)
    pair_rng = oracle.rng_states(R - 1, seed + 1)
    counts = np.zeros((3, R - 1), np.int64)
    trips = oracle.pt_initial_trips(R)
    done, parity = 0, 0
    t0 = time.perf_counter()
    while done < sweeps:
        n = min(EXCHANGE_INTERVAL, sweeps - done)
        oracle.xy_sweeps(theta, rng, betas, np.float32(1.0), np.float32(1.5), n, n_threads=n_threads)
        done += n
        if n == EXCHANGE_INTERVAL:
            e = oracle.xy_energy(theta, np.float32(1.0))
            oracle.pt_exchange(e, betas, w2t, t2w, pair_rng, counts, trips, parity, done)
            parity ^= 1
            oracle.xy_measure(theta, np.float32(1.0), temperature_indices=w2t, cached=e)
    dt = time.perf_counter() - t0
    return R * L * L * sweeps / (dt * 1e9), dt


def ladder_seed(rank):
    """Seed of rank `rank`'s ladder: the 42 + L convention, offset per rank so
    that every rank samples an independent chain."""
    return 42 + L + 1000 * rank


def max_over_ranks(x, dist, device):
    """The job's time is the slowest rank's: all-reduce MAX (identity on one rank)."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(world, updates_per_step, steps, total_ms):
    """Whole-job updates/ns: every rank did `steps` steps within `total_ms`."""
    return world * updates_per_step * steps / (total_ms * 1e6)


def run_reference(args, rank, world):
    if rank != 0:
        return None
    cores = os.cpu_count() or 1
    # A bounded sample of the workload per step (two exchange windows, about
    # 0.1 s on 16 cores), so K steps end within minutes for any usual K.
    sweeps = 2 * EXCHANGE_INTERVAL
    cpu_sample(cores, 10)  # warm-up pages and threads
    vals = []
    t_start = time.perf_counter()
    for _ in range(args.warmup):
        cpu_sample(cores, sweeps)
    for _ in range(args.steps):
        v, _ = cpu_sample(cores, sweeps)
        vals.append(v)
    total = time.perf_counter() - t_start
    value = float(np.median(vals))
    ms = N_TEMPS * L * L * sweeps / (value * 1e6)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "updates/ns",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded uniform angles)",
        "config": {"workload": REFERENCE_WORKLOAD, "sweeps_per_step": sweeps, "parallelism": "host threads",
                   "step": f"a bounded sample: {sweeps} of the workload's {SWEEPS_PER_STEP} sweeps per step"},
        "cpu_baseline": {"value": value, "unit": "updates/ns", "cores": cores, "kind": "port",
                         "sample": f"{sweeps} sweeps of the 32-replica L=128 ladder per step, exchange "
                                   f"every 10 sweeps, {cores} OpenMP threads (the reference has no CPU "
                                   f"sweep; this is its kernels restated in C)"},
        "e2e": {"value": value, "unit": "updates/ns", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "wall_s": total,
    }
    return line


# ------------------------------------------------------------------ GPU arm


def run_mcgb(args, rank, world):
    import torch

    import mcgb
    from mcgb import device
    from mcgb.batch import LadderBatch
    from mcgb.models.xy.model import XYModel

    local = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        if dist is not None:
            dist.barrier()

    temps = temperatures()
    seed = ladder_seed(rank)
    batch = LadderBatch(XYModel(J=1.0), [(L, temps)], seeds=[seed], exchange_interval=EXCHANGE_INTERVAL,
                        proposal="gaussian", sigma0=1.0, initial_states=[initial_angles(seed)],
                        resident=not args.no_resident)
    if args.shape:
        batch.configure(*(int(x) for x in args.shape.split(",")))
    else:
        batch.autotune(sample_interval=SAMPLE_INTERVAL)
    # Warm-up: thermalise and tune the proposal widths (adaptation stops here).
    batch.run(max(args.warmup, 3) * SWEEPS_PER_STEP, tune=True)
    sigma = batch.sigma_t.copy_to_host()
    n_slots = (args.steps + 2) * SWEEPS_PER_STEP // SAMPLE_INTERVAL
    batch.allocate_samples(batch.sweeps + SAMPLE_INTERVAL, SAMPLE_INTERVAL, n_slots)
    batch.run(SWEEPS_PER_STEP)  # captures the replay graphs outside the timed region
    torch.cuda.synchronize()

    # L2 flush buffer (larger than the 129 MB L2), written between timed steps.
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    updates_per_step = N_TEMPS * L * L * SWEEPS_PER_STEP
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    step_ms = []
    barrier()
    torch.cuda.synchronize()
    for _ in range(args.steps):
        flush.fill_(1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        batch.run(SWEEPS_PER_STEP)
        e1.record(stream)
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    total_ms = max_over_ranks(np.sum(step_ms), dist, "cuda")
    value = aggregate_rate(world, updates_per_step, args.steps, total_ms)

    # The same ladder in the profiler's three modes (profiling/profile_he3.py):
    # updates only (no exchange, no samples), + replica exchange, + sampling
    # (the timed steps above).  Bounded to 50 steps each.
    def mode_rate(b):
        n = min(args.steps, 50)
        b.run(SWEEPS_PER_STEP)
        ms = []
        for _ in range(n):
            flush.fill_(1)
            m0, m1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            m0.record(stream)
            b.run(SWEEPS_PER_STEP)
            m1.record(stream)
            m1.synchronize()
            ms.append(m0.elapsed_time(m1))
        return aggregate_rate(world, updates_per_step, n, max_over_ranks(np.sum(ms), dist, "cuda"))

    saved_samples = batch.samples
    batch.samples = None
    pt_rate = mode_rate(batch)
    batch.samples = saved_samples
    plain_ladder = LadderBatch(XYModel(J=1.0), [(L, temps)], seeds=[seed], exchange_interval=None,
                               proposal="gaussian", cluster_size=batch.cluster_size, threads=batch.threads,
                               initial_states=[batch.ladder_state(0)])
    plain_ladder.sigma_t.copy_to_device(sigma)
    updates_rate = mode_rate(plain_ladder)
    del plain_ladder

    # Dominant kernel, timed alone on the same stream: the resident launch
    # (a whole 100-sweep step: ten windows with their exchanges) when the
    # batch runs resident, else one window launch.
    from mcgb import _lib
    import ctypes
    windows = SWEEPS_PER_STEP // EXCHANGE_INTERVAL if batch.resident else 1

    def kernel_once():
        if batch.resident:
            batch._enqueue_resident(EXCHANGE_INTERVAL, windows)
            batch._advance(EXCHANGE_INTERVAL, True, windows)
        else:
            w = batch._window(EXCHANGE_INTERVAL)
            _lib.call("mcgb_batch_window_run", batch.model_id, ctypes.byref(w), _lib.stream_handle())

    kernel_once()
    torch.cuda.synchronize()
    reps = 10
    k0, k1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    k0.record(stream)
    for _ in range(reps):
        kernel_once()
    k1.record(stream)
    torch.cuda.synchronize()
    launch_ms = k0.elapsed_time(k1) / reps
    window_ms = launch_ms / windows
    sm_mhz = clk.get("sm_mhz") or clk.get("sm_max_mhz") or 2070.0
    roofline = roofline_line(profile_figures(PROFILE["xy-pt-l128"]), PROFILE["xy-pt-l128"],
                             N_TEMPS * L * L * EXCHANGE_INTERVAL * windows, launch_ms, BYTES_PER_UPDATE, sm_mhz,
                             "window_kernel<XYPolicy>" + (" (resident, %d windows)" % windows
                                                          if batch.resident else ""))
    roofline["window_ms"] = window_ms
    roofline["traffic_note"] = ("DRAM bytes of one ncu capture of a one-window launch: the strip is loaded and "
                                "written back once per launch, resident or not")

    # End to end through the public API with host buffers: every step uploads
    # the chain state (angles, RNG streams, (cos, sin) cache, running
    # energies) from pinned memory, runs 100 sweeps and reads back the chain
    # state and the step's samples.
    host = batch.pinned_state_buffers()
    out = batch.pinned_state_buffers()
    n_s = SWEEPS_PER_STEP // SAMPLE_INTERVAL
    batch.download_state(host)
    torch.cuda.synchronize()
    batch.allocate_samples(batch.sweeps + SAMPLE_INTERVAL, SAMPLE_INTERVAL, n_s)
    out_samples = torch.empty(batch.samples.nbytes, dtype=torch.uint8, pin_memory=True)
    e2e_ms = []
    for i in range(args.steps + 1):  # the first iteration captures graphs, untimed
        flush.fill_(1)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        batch.upload_state(host)
        batch.run(SWEEPS_PER_STEP)
        batch.download_state(out)
        out_samples.copy_(batch.samples.raw(), non_blocking=True)
        e1.record(stream)
        e1.synchronize()
        if i > 0:
            e2e_ms.append(e0.elapsed_time(e1))
    h2d = sum(t.numel() for t in host.values())
    d2h = sum(t.numel() for t in out.values()) + out_samples.numel()
    e2e_total = max_over_ranks(np.sum(e2e_ms), dist, "cuda")
    e2e_value = aggregate_rate(world, updates_per_step, args.steps, e2e_total)

    drift = energy_drift(batch)
    # Plain FP64 form on the same ladder (one lattice per launch), bounded.
    plain = plain_fp64_rate(batch, sigma, seed) if rank == 0 and not args.skip_plain else None
    # The reference-facing entry points on the same ladder, bounded.
    dropin = dropin_rate(20 * SWEEPS_PER_STEP, seed)[0] if rank == 0 and not args.skip_dropin else None
    # A resident launch runs a whole step (10 windows with their exchanges);
    # otherwise one fused launch per window.
    launches = args.steps * batch.launches_per_step(SWEEPS_PER_STEP // EXCHANGE_INTERVAL)

    line = None
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "updates/ns", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded uniform angles, reference has no dataset)",
            "config": {"workload": WORKLOAD, "L": L, "replicas_per_gpu": N_TEMPS,
                       "sweeps_per_step": SWEEPS_PER_STEP, "exchange_interval": EXCHANGE_INTERVAL,
                       "sample_interval": SAMPLE_INTERVAL, "cluster_size": batch.cluster_size,
                       "threads": batch.threads, "resident_launch": bool(batch.resident),
                       "l2": "flushed (256 MB write) between timed steps",
                       "parallelism": f"independent ladders x{world}"},
            "e2e": {"value": e2e_value, "unit": "updates/ns", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h)},
            "modes": {"updates": updates_rate, "pt": pt_rate, "production": value,
                      "unit": "updates/ns", "note": "updates only / + exchange every 10 / + sample every 10"},
            "roofline": roofline,
            "clocks": clk,
            "gpu_launches": launches,
            "energy_drift": drift,
            "tuned_sigma_range": [float(sigma.min()), float(sigma.max())],
        }
        if plain is not None:
            line["plain_fp64"] = {"value": plain, "unit": "updates/ns",
                                  "form": "one lattice per launch, float64 state and arithmetic, each "
                                          "exchange interval's launches replayed from a CUDA graph"}
            line["speedup_vs_plain_fp64"] = value / plain
        if dropin is not None:
            line["dropin"] = {"value": dropin, "unit": "updates/ns",
                              "form": "Simulation(ParallelTempering(Runtime(XYModel()))).run(), the reference's "
                                      "uniform proposal and per-colour kernels, schedule replayed as CUDA "
                                      "graphs, 2000 sweeps (bench.py --api dropin times it alone)"}
    return line


def dropin_rate(sweeps, seed, host_inputs=False):
    """The reference-facing entry points on the same ladder:
    ``Simulation(ParallelTempering(Runtime(XYModel(), 128, T, seed),
    exchange_interval=10), 0, sweeps, 10).run()`` with the reference's update
    rule (uniform proposal, per-colour kernels), timed with CUDA events
    around run() -- the schedule replayed as CUDA graphs, the samples
    returned to the host.  ``host_inputs``: the initial angles and the RNG
    streams are also copied up from host memory inside the timed region.
    Returns (updates/ns, bytes up, bytes down)."""
    import torch

    from mcgb.core.parallel_tempering import ParallelTempering
    from mcgb.core.runtime import Runtime
    from mcgb.core.simulation import Simulation
    from mcgb.models.xy.model import XYModel

    rt = Runtime(XYModel(J=1.0, delta=1.5), L, temperatures(), seed=seed)
    angles = initial_angles(seed)
    streams = rt.rng_states.copy_to_host()
    rt.state.copy_to_device(angles)
    pt = ParallelTempering(rt, exchange_interval=EXCHANGE_INTERVAL)
    Simulation(pt, 0, 2 * EXCHANGE_INTERVAL, SAMPLE_INTERVAL).run()  # loads the kernels
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    if host_inputs:
        rt.state.copy_to_device(angles)
        rt.rng_states.copy_to_device(streams)
        rt.invalidate_energy_cache()
    res = Simulation(pt, 0, sweeps, SAMPLE_INTERVAL).run()
    e1.record()
    torch.cuda.synchronize()
    up = angles.nbytes + streams.nbytes if host_inputs else 0
    down = sum(v.nbytes for v in res["samples"].values())
    return N_TEMPS * L * L * sweeps / (e0.elapsed_time(e1) * 1e6), up, down


def run_dropin(args, rank, world):
    """``--api dropin``: the headline ladder through the reference's entry
    points (see dropin_rate); one timed run of ``steps`` x 100 sweeps."""
    import torch
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    if rank != 0:
        return None
    seed = ladder_seed(rank)
    sweeps = args.steps * SWEEPS_PER_STEP
    dropin_rate(max(args.warmup, 3) * SWEEPS_PER_STEP, seed)
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", 0)))
    clocks.start()
    time.sleep(0.3)
    value, _, _ = dropin_rate(sweeps, seed)
    e2e, up, down = dropin_rate(sweeps, seed, host_inputs=True)
    clk = clocks.stop()
    return {
        "metric": METRIC, "value": value, "unit": "updates/ns", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": N_TEMPS * L * L * SWEEPS_PER_STEP / (value * 1e6),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded uniform angles)", "api": "dropin",
        "config": {"workload": REFERENCE_WORKLOAD, "entry": "Simulation(ParallelTempering(Runtime(XYModel())))",
                   "sweeps": sweeps, "exchange_interval": EXCHANGE_INTERVAL, "sample_interval": SAMPLE_INTERVAL,
                   "l2": "inputs (2 MB angles, 8 MB streams) are L2-resident: one long run, no flush",
                   "timed": "one Simulation.run() of all steps, samples returned to the host"},
        "e2e": {"value": e2e, "unit": "updates/ns", "h2d_bytes_per_step": int(up / args.steps),
                "d2h_bytes_per_step": int(down / args.steps)},
        "clocks": clk,
        "gpu_launches": args.steps * (SWEEPS_PER_STEP * 4 + SWEEPS_PER_STEP // EXCHANGE_INTERVAL * 4),
    }


def plain_fp64_rate(batch, sigma, seed):
    """The plain form (mcgb.plain64.PlainXYLadder): every replica in its own
    launches (4 colours), float64 angles, float64 Gaussian proposals and
    exponentials, the exchange energies from a float64 reduction per lattice,
    each exchange interval replayed from a CUDA graph.  Times 100 sweeps with
    10 exchanges."""
    import torch

    from mcgb.plain64 import PlainXYLadder

    ladder = PlainXYLadder(L, temperatures(), seed, sigmas=sigma.astype(np.float64),
                           exchange_interval=EXCHANGE_INTERVAL, initial_state=initial_angles(seed))
    ladder.sweep(2 * EXCHANGE_INTERVAL)  # captures the interval's graph
    torch.cuda.synchronize()
    n = 10 * EXCHANGE_INTERVAL
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    ladder.sweep(n)
    e1.record()
    torch.cuda.synchronize()
    return N_TEMPS * L * L * n / (e0.elapsed_time(e1) * 1e6)


# ------------------------------------------------------------------ other workloads
#
# `--workload NAME` times another configuration of the study through the same
# engine: a step is 100 sweeps of every replica with the configuration's
# exchange and sampling schedule; the line keeps the default's keys (value,
# e2e, roofline with the model's algorithmic bytes per update, clocks,
# gpu_launches, cpu_baseline on a bounded sample of its first ladder).

BYTES = {"ising": 34, "xy": 40, "kawamura": 72, "kawamura-gauss": 72, "he3": 128}  # state r+w + 32 B RNG


def workload_spec(name):
    """(model kind, ladders, exchange_interval, sample_interval, description)."""
    fss = (16, 32, 64, 128, 256, 512)
    if name == "ising-l64":
        return ("ising", [(64, [T]) for T in (1.5, 2.269, 3.0)], None, 1,
                "Ising L=64 at T in {1.5, 2.269, 3.0}, single-temperature runs, E/N and |m| every sweep")
    if name == "kawamura-l96x64":
        return ("kawamura-gauss", [(96, np.linspace(0.65, 0.80, 48))] * 64, 10, 10,
                "Kawamura L=96, 64 ladders x 48 temperatures linear in [0.65, 0.80] (3072 replicas), "
                "Gaussian MH (theta and d, widths tuned to ~50%), exchange and sample every 10")
    if name == "kawamura-l96x64-reference-proposals":
        return ("kawamura", [(96, np.linspace(0.65, 0.80, 48))] * 64, 10, 10,
                "Kawamura L=96, 64 ladders x 48 temperatures linear in [0.65, 0.80] (3072 replicas), "
                "the reference's uniform/flip/sphere proposals, exchange and sample every 10")
    if name == "he3-ragged":
        return ("he3", [(Lh, np.geomspace(0.33, 0.47, 24)) for Lh in (32, 48, 64, 96, 128)], 10, 10,
                "He3 (class defaults) ragged L in {32,48,64,96,128} x 24 temperatures geometric in "
                "[0.33, 0.47], conditional-Gaussian sampler, exchange and sample every 10")
    if name == "fss-ising":
        return ("ising", [(Lf, np.geomspace(2.0, 2.5, 64)) for Lf in fss for _ in range(8)], 10, 10,
                "Ising FSS L in {16..512} x 8 ladders x 64 temperatures geometric in [2.0, 2.5] (3072 replicas)")
    if name == "fss-xy":
        return ("xy", [(Lf, np.geomspace(0.78, 1.02, 64)) for Lf in fss for _ in range(8)], 10, 10,
                "XY FSS L in {16..512} x 8 ladders x 64 temperatures geometric in [0.78, 1.02] (3072 "
                "replicas), Gaussian MH")
    raise ValueError(f"unknown workload {name}")


def seeded_state(kind, L_, R, seed):
    """Seeded initial states in the reference layout."""
    r = np.random.default_rng(seed)
    kind = kind.split("-")[0]
    if kind == "ising":
        return r.choice(np.array([-1, 1], np.int8), (R, L_, L_))
    if kind == "xy":
        return r.uniform(-np.pi, np.pi, (R, L_, L_)).astype(np.float32)
    if kind == "kawamura":
        st = np.zeros((R, L_, L_, 5), np.float32)
        st[..., 0] = r.uniform(-np.pi, np.pi, (R, L_, L_))
        st[..., 1] = r.choice([-1.0, 1.0], (R, L_, L_))
        d = r.normal(size=(R, L_, L_, 3))
        st[..., 2:] = d / np.linalg.norm(d, axis=-1, keepdims=True)
        return st
    a = 0.3 * np.sqrt(2)
    return (r.uniform(-a, a, (R, L_, L_, 3, 2)) + 1j * r.uniform(-a, a, (R, L_, L_, 3, 2))).astype(np.complex64)


def cpu_sample_model(kind, L_, T, state, seed, n_threads, sweeps):
    """The oracle (reference kernels restated in C, reference proposals) on
    one ladder, no exchange."""
    import oracle
    kind = kind.split("-")[0]
    R = len(T)
    betas = (1.0 / np.asarray(T)).astype(np.float32)
    st = state.copy()
    rng = oracle.rng_states(R * L_ * L_, seed)
    t0 = time.perf_counter()
    if kind == "ising":
        oracle.ising_sweeps(st, rng, betas, np.float32(1), sweeps, n_threads=n_threads)
    elif kind == "xy":
        oracle.xy_sweeps(st, rng, betas, np.float32(1), np.float32(1.5), sweeps, n_threads=n_threads)
    elif kind == "kawamura":
        oracle.kawamura_sweeps(st, rng, betas, np.float32(1), np.float32(1.5), sweeps, n_threads=n_threads)
    else:
        coeff = np.array([-0.5, 1.0, 1.0, 1.0, -1.0], np.float32)
        oracle.he3_sweeps(st, rng, betas, coeff, np.float32(1), np.float32(0.15), np.float32(0), sweeps,
                          n_threads=n_threads)
    dt = time.perf_counter() - t0
    return R * L_ * L_ * sweeps / (dt * 1e9), dt


def run_workload(args, rank, world):
    import ctypes

    import torch

    from mcgb import _lib
    from mcgb.batch import LadderBatch
    from mcgb.models.he3.model import He3Model
    from mcgb.models.ising.model import IsingModel
    from mcgb.models.kawamura.model import KawamuraModel
    from mcgb.models.xy.model import XYModel

    local = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    kind, ladders, ex, si, desc = workload_spec(args.workload)
    seeds = [42 + L_ + 100003 * k + 1000 * rank for k, (L_, _) in enumerate(ladders)]
    inits = [seeded_state(kind, L_, len(T), sd) for (L_, T), sd in zip(ladders, seeds)]
    gauss = kind in ("xy", "kawamura-gauss")
    model = {"ising": IsingModel(), "xy": XYModel(J=1.0), "kawamura": KawamuraModel(),
             "kawamura-gauss": KawamuraModel(), "he3": He3Model()}[kind]
    batch = LadderBatch(model, ladders, seeds=seeds, exchange_interval=ex,
                        proposal="gaussian" if gauss else "uniform", gaussian=kind == "he3",
                        sigma0=0.5 if kind == "kawamura-gauss" else 1.0, initial_states=inits)
    if args.shape:
        batch.configure(*(int(x) for x in args.shape.split(",")))
    else:
        batch.autotune(sample_interval=si)
    tune = gauss
    batch.run(max(args.warmup, 3) * SWEEPS_PER_STEP, tune=tune)
    batch.allocate_samples(batch.sweeps + si, si, (args.steps + 2) * SWEEPS_PER_STEP // si)
    batch.run(SWEEPS_PER_STEP)
    torch.cuda.synchronize()

    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    n_sites = int(batch.n_sites)
    updates_per_step = n_sites * SWEEPS_PER_STEP
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    step_ms = []
    for _ in range(args.steps):
        flush.fill_(1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        batch.run(SWEEPS_PER_STEP)
        e1.record(stream)
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    clk = clocks.stop()
    total_ms = max_over_ranks(np.sum(step_ms), dist, "cuda")
    value = aggregate_rate(world, updates_per_step, args.steps, total_ms)

    # The window kernel alone (one window of the schedule, samples on).
    from mcgb.batch import NO_EXCHANGE_WINDOW
    win = ex or NO_EXCHANGE_WINDOW
    # One launch per size group, side by side when the batch runs its groups so.
    batch.enqueue_plain_windows(win)
    torch.cuda.synchronize()
    k0, k1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    k0.record(stream)
    for _ in range(10):
        batch.enqueue_plain_windows(win)
    k1.record(stream)
    torch.cuda.synchronize()
    window_ms = k0.elapsed_time(k1) / 10
    sm_mhz = clk.get("sm_mhz") or clk.get("sm_max_mhz") or 2070.0
    prof = PROFILE.get(args.workload)
    roofline = roofline_line(profile_figures(prof), prof, n_sites * win, window_ms, BYTES[kind], sm_mhz,
                             f"window_kernel ({kind})" + (
                                 f", {len(batch.groups)} launches (size groups"
                                 + (", side by side)" if batch.concurrent else ")") if len(batch.groups) > 1
                                 else ""), scale_traffic=True)

    # End to end: the chain state up from pinned memory, 100 sweeps, the
    # chain state and the step's samples back.
    host, out = batch.pinned_state_buffers(), batch.pinned_state_buffers()
    batch.download_state(host)
    batch.allocate_samples(batch.sweeps + si, si, SWEEPS_PER_STEP // si)
    out_samples = torch.empty(batch.samples.nbytes, dtype=torch.uint8, pin_memory=True)
    e2e_ms = []
    n_e2e = min(args.steps, 20)
    for i in range(n_e2e + 1):
        flush.fill_(1)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        batch.upload_state(host)
        batch.run(SWEEPS_PER_STEP)
        batch.download_state(out)
        out_samples.copy_(batch.samples.raw(), non_blocking=True)
        e1.record(stream)
        e1.synchronize()
        if i > 0:
            e2e_ms.append(e0.elapsed_time(e1))
    e2e_value = aggregate_rate(world, updates_per_step, n_e2e, max_over_ranks(np.sum(e2e_ms), dist, "cuda"))
    h2d = sum(t.numel() for t in host.values())
    d2h = sum(t.numel() for t in out.values()) + out_samples.numel()
    drift = energy_drift(batch)
    if rank != 0:
        return None
    windows_per_step = SWEEPS_PER_STEP // win
    line = {
        "metric": METRIC, "value": value, "unit": "updates/ns", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": {"ising": "int8+f32", "he3": "c64"}.get(kind, "f32"),
        "data": "synthetic (seeded initial states, reference has no dataset)",
        "config": {"workload": desc, "replicas_per_gpu": int(batch.R), "sites_per_sweep": n_sites,
                   "sweeps_per_step": SWEEPS_PER_STEP, "exchange_interval": ex, "sample_interval": si,
                   "cluster_size": batch.cluster_size, "threads": batch.threads,
                   "size_groups": [{"L": sizes, "cluster_size": c, "threads": t, "resident": r}
                                   for sizes, c, t, r in batch.shapes()] if len(batch.groups) > 1 else None,
                   "size_groups_side_by_side": bool(batch.concurrent) if len(batch.groups) > 1 else None,
                   "l2": "flushed (256 MB write) between timed steps",
                   "parallelism": f"independent ladders x{world}"},
        "e2e": {"value": e2e_value, "unit": "updates/ns", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "steps": n_e2e},
        "roofline": roofline,
        "clocks": clk,
        "gpu_launches": args.steps * batch.launches_per_step(windows_per_step),
        "energy_drift": drift,
    }
    if not args.no_cpu_baseline:
        cores = os.cpu_count() or 1
        L0, T0 = ladders[0]
        sweeps = {"ising": 200, "xy": 40, "kawamura": 10, "kawamura-gauss": 10, "he3": 4}[kind]
        used = min(cores, len(T0))  # the oracle parallelises over replicas
        v, dt = cpu_sample_model(kind, L0, T0, inits[0], seeds[0], used, sweeps)
        line["cpu_baseline"] = {"value": v, "unit": "updates/ns", "cores": used, "kind": "port",
                                "sample": f"{sweeps} sweeps of the first ladder (L={L0}, {len(T0)} replicas), "
                                          f"reference proposals, no exchange, {dt:.1f} s"}
    return line


def energy_drift(batch):
    """The running energies (compensated float32 sums of accepted changes)
    against an FP64 recompute of the same state, after the timed steps:
    largest |drift| per site and relative to |E| over the replicas (the
    recompute also resets the running energies)."""
    drift = batch.recompute_energy().copy_to_host()
    exact = batch.energies.copy_to_host()
    sites = batch.table_host["L"].astype(np.float64) ** 2
    return {"max_abs_per_site": float(np.max(np.abs(drift) / sites)),
            "max_rel": float(np.max(np.abs(drift) / np.maximum(np.abs(exact), 1e-300))),
            "note": "running compensated-float32 energy minus an FP64 recompute of the same state"}


def profile_windows(cluster_size=4, threads=1024, workload="xy-pt-l128"):
    """Small fixed case for ncu: the workload's batch, 3 warm windows + 3 windows."""
    import ctypes

    import torch

    from mcgb import _lib
    from mcgb.batch import LadderBatch
    from mcgb.models.he3.model import He3Model
    from mcgb.models.ising.model import IsingModel
    from mcgb.models.kawamura.model import KawamuraModel
    from mcgb.models.xy.model import XYModel

    if workload == "xy-pt-l128":
        seed = 42 + L
        b = LadderBatch(XYModel(J=1.0), [(L, temperatures())], seeds=[seed], exchange_interval=EXCHANGE_INTERVAL,
                        proposal="gaussian", sigma0=0.93, cluster_size=cluster_size, threads=threads,
                        initial_states=[initial_angles(seed)])
        win = EXCHANGE_INTERVAL
    else:
        kind, ladders, ex, _, _ = workload_spec(workload)
        fss = workload.startswith("fss-")
        if fss:
            # The reduced case: one ladder per size (384 replicas, an eighth
            # of the batch), run as the bench runs it, one launch per size.
            ladders = ladders[::8]
        seeds = [42 + L_ + 100003 * k for k, (L_, _) in enumerate(ladders)]
        inits = [seeded_state(kind, L_, len(T), sd) for (L_, T), sd in zip(ladders, seeds)]
        model = {"ising": IsingModel(), "xy": XYModel(J=1.0), "kawamura": KawamuraModel(),
                 "kawamura-gauss": KawamuraModel(), "he3": He3Model()}[kind]
        shape = {} if fss else {"cluster_size": cluster_size, "threads": threads}
        b = LadderBatch(model, ladders, seeds=seeds, exchange_interval=ex,
                        proposal="gaussian" if kind in ("xy", "kawamura-gauss") else "uniform",
                        gaussian=kind == "he3", initial_states=inits, **shape)
        if fss:
            b.split_by_size(True)
            print("groups:", b.shapes())
        from mcgb.batch import NO_EXCHANGE_WINDOW
        win = ex or NO_EXCHANGE_WINDOW
    ws = [b._window(win, group=g) for g in b.groups]
    for _ in range(6):
        for w in ws:
            _lib.call("mcgb_batch_window_run", b.model_id, ctypes.byref(w), _lib.stream_handle())
    torch.cuda.synchronize()
    print("profile windows done: %d launches per window" % len(ws))


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["mcgb", "reference"], default="mcgb")
    ap.add_argument("--skip-plain", action="store_true", help="do not time the plain FP64 form")
    ap.add_argument("--skip-dropin", action="store_true", help="do not time the drop-in entry points")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile", action="store_true",
                    help="profiling driver: set up the ladder, then launch 6 window kernels and exit")
    ap.add_argument("--profile-shape", default="4,1024", help="cluster_size,threads for --profile")
    ap.add_argument("--no-resident", action="store_true",
                    help="one launch per window instead of resident multi-window launches (for profiling)")
    ap.add_argument("--shape", default=None,
                    help="cluster_size,threads instead of autotuning (a profiler's per-launch overhead "
                         "would mislead the autotuner's timings)")
    ap.add_argument("--api", choices=["batch", "dropin"], default="batch",
                    help="batch: the batched engine (default); dropin: the headline ladder through "
                         "Simulation(ParallelTempering(Runtime(XYModel())))")
    ap.add_argument("--workload", default="xy-pt-l128",
                    choices=["xy-pt-l128", "ising-l64", "kawamura-l96x64", "kawamura-l96x64-reference-proposals",
                             "he3-ragged", "fss-ising", "fss-xy"],
                    help="configuration to time (default: the XY PT ladder the metric is quoted on)")
    args = ap.parse_args()
    if args.profile:
        c, t = (int(x) for x in args.profile_shape.split(","))
        profile_windows(c, t, args.workload)
        return
    if args.warmup < 3:
        ap.error("warm-up must be at least 3 steps")
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", args.gpus))
    if args.impl == "reference":
        line = run_reference(args, rank, world)
    elif args.api == "dropin":
        line = run_dropin(args, rank, world)
    elif args.workload != "xy-pt-l128":
        line = run_workload(args, rank, world)
    else:
        line = run_mcgb(args, rank, world)
        if line is not None and not args.no_cpu_baseline:
            cores = os.cpu_count() or 1
            v, dt = cpu_sample(cores, 500)
            v1, dt1 = cpu_sample(1, 20)
            line["cpu_baseline"] = {"value": v, "unit": "updates/ns", "cores": cores, "kind": "port",
                                    "sample": f"500 sweeps of the same ladder with 50 exchanges, {cores} OpenMP "
                                              f"threads, {dt:.1f} s (the reference has no CPU sweep; its kernels "
                                              f"restated in C)",
                                    "one_core": {"value": v1, "sample": f"20 sweeps, 1 thread, {dt1:.1f} s"}}
    if line is not None:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()

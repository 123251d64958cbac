#!/usr/bin/env python
"""Benchmark of the sea-ice step: EVP Gcell-subcycles/s on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (default): the 0.25-degree single domain, 1440 x 720 interior cells,
500 mEVP subcycles per step, dt = 1800 s, seeded synthetic fields.  One
bench step is one full sea-ice time step (dynamics preparation, 500 EVP
subcycles, ocean stress, advection, clean-up, growth, halo fills).

The headline ``value`` runs the mixed-precision step (float32 EVP and
advection, float64 thermodynamics and budgets) replayed as one CUDA graph,
with inputs resident in HBM; L2 is flushed (a 512 MiB write) before every
timed step and the flush is outside the timed events.  The metric counts
interior cells x subcycles over the whole step time.  Also reported: the
plain float64 step on the same inputs, the float32-vs-float64 errors per
field, the end-to-end rate through host buffers, the EVP kernel's roofline
and a CPU baseline (the NumPy oracle on one core, bounded sample).

``--impl reference`` times the reference's CPU algorithm (the NumPy oracle,
a restatement of the reference that is bit-identical to it on the golden
fixtures) on the host cores, each step a bounded sample extrapolated to a
full 500-subcycle step.

With ``--gpus N > 1`` (under torchrun) every rank runs an independent replica
(the workload does not shard: one domain per GPU), ``scaling`` is weak and
``value`` sums the ranks' cells over the slowest rank's time.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

BYTES_PER_CELL_SUBCYCLE = {"f32": 83, "f64": 163}
METRIC = "EVP Gcell-subcycles/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=("ours", "reference"))
    ap.add_argument("--config", default="c2_quarterdeg")
    ap.add_argument("--precision", default="f32", choices=("f32", "f64"))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true", help="skip the float64 comparison leg")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--adaptive", action="store_true", help="adaptive EVP (useAdaptiveEVP)")
    ap.add_argument("--no-routines", action="store_true",
                    help="skip the free-drift, bulk-formula and residual measurements")
    ap.add_argument("--routines-only", action="store_true",
                    help="measure only the free-drift, bulk-formula and residual routines")
    ap.add_argument("--subcycles", type=int, default=None, help="override the workload's subcycles")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--evp", default="auto", choices=("auto", "fast", "plain"))
    ap.add_argument("--f32-kernel", default="walk", choices=("tma", "walk"),
                    help="float32 EVP kernel: register-walking warps or TMA-staged tiles")
    ap.add_argument("--walk-rows", type=int, default=0, help="rows per walk (0: from the grid and the SM count)")
    ap.add_argument("--walk-variant", type=int, default=-1, help="-1: tuned on the workload")
    ap.add_argument("--adjoint", action="store_true",
                    help="time a trajectory's forward + adjoint against its forward (float64)")
    ap.add_argument("--adjoint-config", default="c3_1deg")
    ap.add_argument("--adjoint-steps", type=int, default=None)
    ap.add_argument("--adjoint-precision", default="f64", choices=("f64", "f32"))
    ap.add_argument("--snapshots", type=int, default=None, help="step snapshots (default: all)")
    ap.add_argument("--evp-checkpoint-every", type=int, default=None,
                    help="EVP subcycle checkpoint interval inside a step's adjoint "
                         "(0: keep all; default: keep all when it fits in device memory)")
    ap.add_argument("--tape", default="auto", choices=("auto", "on", "off"),
                    help="keep every EVP subcycle state during the forward")
    ap.add_argument("--adjoint-repeats", type=int, default=2)
    ap.add_argument("--no-fd", action="store_true", help="skip the centred-difference check of dL/dP*")
    ap.add_argument("--evp-alpha-beta", type=float, default=None,
                    help="override the mEVP relaxation parameters (evpAlpha = evpBeta)")
    ap.add_argument("--track-norms", action="store_true", help="record the adjoint norm after every step")
    ap.add_argument("--ensemble", action="store_true",
                    help="the batched ensemble (512 members of uneven sizes) against sequential launches")
    ap.add_argument("--members", type=int, default=512)
    ap.add_argument("--ens-shape", type=int, default=None, help="ensemble tile/walk shape (skips tuning)")
    ap.add_argument("--ens-blocks-per-sm", type=int, default=4)
    return ap.parse_args()


# ---------------------------------------------------------------- distributed

def dist_init(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
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


def replica_value(cells_per_rank, subcycles, steps, ms_max, ws):
    """Whole-job Gcell-subcycles/s of ws independent replicas (weak scaling):
    every rank's cells over the slowest rank's time."""
    return ws * cells_per_rank * subcycles * steps / (ms_max / 1e3) / 1e9


# -------------------------------------------------------------------- clocks

class ClockSampler:
    """nvidia-smi samples of SM clocks and throttle reasons while running."""

    QUERY = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
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
        self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for n, val in zip(names, parts[4:8]):
                if val.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------- peaks

def hbm_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def recorded_traffic(kernel, workload):
    """DRAM bytes per launch of ``kernel`` on ``workload`` from an ncu capture
    (profiles/roofline_traffic.json), or None."""
    path = os.path.join(ROOT, "profiles", "roofline_traffic.json")
    try:
        with open(path) as f:
            return json.load(f).get(f"{kernel}/{workload}")
    except (OSError, ValueError):
        return None


# ----------------------------------------------------------------- CPU legs

def cpu_sample(arrays, sett, n_sub_sample, n_sub_full):
    """Time the oracle (the reference's NumPy algorithm, one core) on a
    bounded sample: ``n_sub_sample`` EVP subcycles, one advection, one
    growth; extrapolated to a step of ``n_sub_full`` subcycles.  Returns
    (seconds per full step, sample description)."""
    from types import SimpleNamespace
    import copy
    from oracle import veris_oracle as O
    st = SimpleNamespace(variables=SimpleNamespace(**{k: v.copy() for k, v in arrays.items()}),
                         settings=copy.copy(sett))
    v = st.variables
    t0 = time.perf_counter()
    v.SeaIceMassC, v.SeaIceMassU, v.SeaIceMassV = O.SeaIceMass(st)
    v.AreaW, v.AreaS = O.AreaWS(st)
    v.WindForcingX, v.WindForcingY = O.WindForcingXY(st)
    v.SeaIceStrength = O.SeaIceStrength(st)
    t1 = time.perf_counter()
    c = O.evp_carry(st)
    for _ in range(n_sub_sample):
        O.evp_subcycle(st, c)
    t2 = time.perf_counter()
    v.uIce, v.vIce = c["u"], c["v"]
    v.OceanStressU, v.OceanStressV = O.OceanStressUV(st)
    v.hIceMean, v.hSnowMean, v.Area = O.Advection(st)
    out = O.clean_up_advection(st)
    v.hIceMean, v.hSnowMean, v.Area, v.TSurf, v.os_hIceMean, v.os_hSnowMean = out
    v.Area = O.ridging(st)
    O.Growth(st)
    t3 = time.perf_counter()
    per_sub = (t2 - t1) / n_sub_sample
    full = (t1 - t0) + per_sub * n_sub_full + (t3 - t2)
    desc = (f"NumPy oracle, 1 thread: {n_sub_sample} EVP subcycles + preparation + advection + "
            f"growth timed ({t3 - t0:.1f} s), extrapolated to {n_sub_full} subcycles per step")
    return full, desc


def _reference_worker(job):
    """One bounded sample of the oracle in a worker process (one core)."""
    import os as _os
    _os.environ.setdefault("OMP_NUM_THREADS", "1")
    config, seed, n_sample, n_full = job
    from veris_gb300.synthetic import CONFIGS, make_state, config_settings
    c = CONFIGS[config]
    arrays = make_state(c["nx"], c["ny"], seed=seed)
    sett = config_settings(config)
    cpu_sample(arrays, sett, n_sample, n_full)          # warm-up
    return cpu_sample(arrays, sett, n_sample, n_full)


def run_reference(args):
    """The reference's CPU algorithm (the NumPy oracle) on all host cores:
    one independent replica of the workload per core (NumPy elementwise code
    uses one core each), every replica timing a bounded sample of a step;
    value = all replicas' cells x subcycles over the slowest one's time."""
    ws, rank = int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    import multiprocessing as mp
    from veris_gb300.synthetic import CONFIGS
    c = CONFIGS[args.config]
    n_full = args.subcycles or c["n_evp"]
    cells = c["nx"] * c["ny"]
    n_sample = 2
    cores = max(1, os.cpu_count() or 1)
    ctx = mp.get_context("spawn")
    times = []
    desc = ""
    with ctx.Pool(cores) as pool:
        for k in range(args.warmup + args.steps):
            res = pool.map(_reference_worker, [(args.config, args.seed + r, n_sample, n_full) for r in range(cores)])
            if k >= args.warmup:
                times.append(max(t for t, _d in res))
                desc = res[0][1]
    sec = float(np.sum(times))
    value = cores * cells * n_full * args.steps / sec / 1e9
    sample = f"{cores} processes x ({desc})"
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Gcell-subcycles/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": sec / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": args.config, "nx": c["nx"], "ny": c["ny"], "subcycles": n_full,
                   "dt_s": c["dt"], "cells": cells, "parallelism": f"{cores} CPU replicas",
                   "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": value, "unit": "Gcell-subcycles/s", "cores": cores, "kind": "port",
                         "sample": sample, "host_cpus": os.cpu_count()},
        "e2e": {"value": value, "unit": "Gcell-subcycles/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# ----------------------------------------------------------------- our arm

def rel_errors(a, b):
    a = a.double()
    b = b.double()
    scale = float(b.abs().max())
    if scale == 0:
        scale = 1.0
    d = (a - b).abs()
    return {"max_rel": float(d.max()) / scale, "rms_rel": float(d.pow(2).mean().sqrt()) / scale}


def run_ours(args):
    import torch
    ws, rank, local = dist_init(args)
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from __graft_entry__ import build
    if rank == 0 or ws == 1:
        build()
    barrier(ws)
    from veris_gb300.engine import SeaIceStep
    from veris_gb300.state import VerisState
    from veris_gb300.synthetic import CONFIGS, make_state, config_settings

    c = CONFIGS[args.config]
    arrays = make_state(c["nx"], c["ny"], seed=args.seed + rank)
    sett = config_settings(args.config)
    if args.subcycles:
        sett.nEVPsteps = args.subcycles
    if args.evp_alpha_beta:
        sett.evpAlpha = sett.evpBeta = float(args.evp_alpha_beta)
    if args.adaptive:
        sett.useAdaptiveEVP = True
    n_sub = sett.nEVPsteps
    cells = c["nx"] * c["ny"]

    state = VerisState.from_numpy(arrays, sett, device=dev)
    eng = SeaIceStep(state, precision=args.precision, evp=args.evp, f32_kernel=args.f32_kernel,
                     walk_rows=args.walk_rows, walk_variant=max(0, args.walk_variant))
    walk_tuning = None
    if args.precision == "f32" and args.f32_kernel == "walk" and eng.evp_form == "fast" and args.walk_variant < 0:
        from veris_gb300.autotune import tune_walk
        walk_tuning = tune_walk(eng)
    eng.capture()
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    for _ in range(args.warmup):
        eng.step()
    torch.cuda.synchronize(dev)

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    barrier(ws)
    torch.cuda.synchronize(dev)
    t_wall0 = time.perf_counter()
    for k in range(args.steps):
        flush.zero_()
        starts[k].record()
        eng.step()
        ends[k].record()
    torch.cuda.synchronize(dev)
    barrier(ws)
    wall = time.perf_counter() - t_wall0
    clk = clocks.stop()
    ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends))
    ms = max_over_ranks(ms, ws)
    value = replica_value(cells, n_sub, args.steps, ms, ws)
    launches = eng.launches_per_step * args.steps

    # EVP kernel alone (eager, events around the subcycle loop on the launching stream)
    evp_ms = []
    for _ in range(3):
        flush.zero_()
        evp_ms.append(eng.timed_step())
    evp_ms = float(np.median(evp_ms))
    flush.zero_()
    phases = eng.phase_times()
    per_launch_s = evp_ms / 1e3 / n_sub
    algo_bytes = BYTES_PER_CELL_SUBCYCLE[args.precision] * cells
    achieved = algo_bytes / per_launch_s / 1e9
    peak, peak_kind = hbm_peak()
    kernel = (("evp_walk_kernel" if args.f32_kernel == "walk" else "evp_tma_kernel")
              if eng.evp_form == "fast" and args.precision == "f32" else
              ("evp_fast_kernel" if eng.evp_form == "fast" else "evp_subcycle_kernel")
              + f"<{'float' if args.precision == 'f32' else 'double'}>")
    traffic = recorded_traffic(kernel, args.config)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic, "kernel": kernel,
                "algorithmic_bytes_per_launch": algo_bytes, "avg_launch_us": per_launch_s * 1e6,
                "peak_source": f"{peak_kind} HBM copy bandwidth"}

    line = {"metric": METRIC, "value": value, "unit": "Gcell-subcycles/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": args.precision, "data": "synthetic",
            "config": {"workload": args.config, "nx": c["nx"], "ny": c["ny"], "subcycles": n_sub,
                       "evpAlpha": float(sett.evpAlpha), "evpBeta": float(sett.evpBeta),
                       "adaptive_evp": bool(sett.useAdaptiveEVP),
                       "dt_s": c["dt"], "cells": cells, "precision": args.precision,
                       "parallelism": "replicas" if ws > 1 else "single-gpu",
                       "l2": "flushed before every timed step (512 MiB write)",
                       "graph": "one CUDA graph per step", "evp_form": eng.evp_form,
                       "f32_kernel": args.f32_kernel if args.precision == "f32" else None,
                       "walk": {"rows": eng.walk_rows or "auto", "variant": eng.walk_variant,
                                "tuning": walk_tuning}
                       if args.f32_kernel == "walk" else None},
            "roofline": roofline, "gpu_launches": launches, "clocks": clk,
            "wall_s_timed_region": wall, "evp_ms_per_step": evp_ms,
            "phase_ms": {k: round(v, 4) for k, v in phases.items()}}

    # end-to-end through host buffers
    if not args.no_e2e:
        from veris_gb300.host import HostCoupledStep
        host = HostCoupledStep(eng)
        h_in, h_out = host.host_buffers()
        for _ in range(max(3, args.warmup)):   # the first call captures the exchange graph
            host.step(h_in, h_out)
        barrier(ws)
        t0 = time.perf_counter()
        ke = max(3, args.steps // 2)
        for _ in range(ke):
            host.step(h_in, h_out)
        e2e_s = time.perf_counter() - t0
        e2e_s = max_over_ranks(e2e_s, ws)
        line["e2e"] = {"value": ws * cells * n_sub * ke / e2e_s / 1e9, "unit": "Gcell-subcycles/s",
                       "h2d_bytes_per_step": host.h2d_bytes, "d2h_bytes_per_step": host.d2h_bytes,
                       "steps": ke, "api": "veris_gb300.host.HostCoupledStep.step (pinned host arrays)"}

    # float64 drop-in arithmetic on the same inputs, and the float32 error
    if not args.no_fp64 and args.precision == "f32":
        n_cmp = max(2, args.warmup + args.steps)
        names = ("uIce", "vIce", "hIceMean", "hSnowMean", "Area", "TSurf", "Qnet")
        # both precisions from the same initial state; capture() runs step 1
        st32 = VerisState.from_numpy(arrays, sett, device=dev)
        e32 = SeaIceStep(st32, precision="f32", evp=args.evp, f32_kernel=args.f32_kernel,
                         walk_rows=args.walk_rows, walk_variant=eng.walk_variant)
        e32.capture()
        st64 = VerisState.from_numpy(arrays, sett, device=dev)
        e64 = SeaIceStep(st64, precision="f64", evp=args.evp)
        e64.capture()
        torch.cuda.synchronize(dev)
        errs1 = {n: rel_errors(getattr(st32.variables, n), getattr(st64.variables, n)) for n in names}
        t64 = []
        for k in range(n_cmp - 1):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            flush.zero_()
            a.record()
            e64.step()
            b.record()
            b.synchronize()
            t64.append(a.elapsed_time(b))
            e32.step()
        torch.cuda.synchronize(dev)
        fp64_ms = float(np.median(t64[-min(len(t64), args.steps):]))
        fp64_value = cells * n_sub / (fp64_ms / 1e3) / 1e9
        line["fp64"] = {"value": fp64_value, "ms_per_step": fp64_ms, "steps_compared": n_cmp,
                        "evp_form": e64.evp_form}
        line["fp32_over_fp64_speedup"] = (value / ws) / fp64_value
        errs = {n: rel_errors(getattr(st32.variables, n), getattr(st64.variables, n)) for n in names}
        line["fp32_error_vs_fp64"] = {"after_1_step": errs1, "steps": n_cmp, "fields": errs,
                                      "definition": "max_rel = max|a-b| / max|b|, rms_rel = rms(a-b) / max|b|"}

    if not args.no_routines:
        line["routines"] = measure_routines(arrays, sett, dev, flush)

    if rank == 0 and not args.no_cpu_baseline:
        sec, desc = cpu_sample(arrays, sett, 2, n_sub)
        line["cpu_baseline"] = {"value": cells * n_sub / sec / 1e9, "unit": "Gcell-subcycles/s",
                                "cores": 1, "kind": "port", "sample": desc,
                                "host_cpus": os.cpu_count()}
    if rank == 0:
        print(json.dumps(line))
    barrier(ws)
    return 0


def _event_time(fn, repeats, flush):
    """Median CUDA-event time of ``repeats`` calls of ``fn`` (ms per call),
    each call timed alone with L2 flushed (512 MiB write) before it."""
    import torch
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(repeats)]
    fn()                                    # warm-up
    for a, b in ev:
        flush.zero_()
        a.record()
        fn()
        b.record()
    torch.cuda.synchronize()
    return float(np.median([a.elapsed_time(b) for a, b in ev]))


def measure_routines(arrays, sett, dev, flush):
    """The routines beside the step on the workload's grid: free drift and
    the bulk formula (per launch, against the HBM roofline of their
    algorithmic bytes) and the cost of the EVP residual diagnostics."""
    import ctypes
    import torch
    from veris_gb300.state import Call, VerisState
    peak, peak_kind = hbm_peak()
    out = {}
    NX, NY = arrays["hIceMean"].shape
    points = NX * NY
    for prec, dt, esz in (("f64", torch.float64, 8), ("f32", torch.float32, 4)):
        st = VerisState.from_numpy(arrays, sett, device=dev, dtype=dt)
        c = Call(st, dtype=dt)
        u, v = c.empty(2)
        fn = c.lib.veris_freedrift_solver_f64 if prec == "f64" else c.lib.veris_freedrift_solver_f32
        refs = c.refs()
        ms = _event_time(lambda: fn(*refs, u.data_ptr(), v.data_ptr(), c.stream), 20, flush)
        algo = 10 * esz * points            # 8 fields read, 2 written
        out[f"freedrift_{prec}"] = {"ms": ms, "Gpoints_per_s": points / ms / 1e6,
                                    "achieved_GBs": algo / ms / 1e6, "frac_hbm": algo / ms / 1e6 / peak,
                                    "algorithmic_bytes": algo, "points": points}
    rng = np.random.default_rng(1)
    shape = (NX, NY)
    bulk_in = [rng.normal(0, 7, shape), rng.normal(0, 7, shape), None, 0.02 * rng.random(shape),
               271 + 30 * rng.random(shape)]
    bulk_in[2] = bulk_in[4] + rng.normal(0, 5, shape)
    from veris_gb300 import _abi
    p = _abi.params_from_settings(sett)
    lib = _abi.load()
    stream = torch.cuda.current_stream(dev).cuda_stream
    for prec, dt, esz in (("f64", torch.float64, 8), ("f32", torch.float32, 4)):
        ins = [torch.as_tensor(a, dtype=dt, device=dev) for a in bulk_in]
        outs = [torch.empty(shape, dtype=dt, device=dev) for _ in range(9)]
        fn = lib.veris_bulkf_formula_lanl_f64 if prec == "f64" else lib.veris_bulkf_formula_lanl_f32
        pr = ctypes.byref(p)
        ptrs = [t.data_ptr() for t in ins] + [None] + [t.data_ptr() for t in outs]
        ms = _event_time(lambda: fn(pr, points, *ptrs, stream), 20, flush)
        algo = 14 * esz * points            # 5 inputs read, 9 outputs written
        out[f"bulkf_formula_lanl_{prec}"] = {"ms": ms, "Gpoints_per_s": points / ms / 1e6,
                                             "achieved_GBs": algo / ms / 1e6,
                                             "frac_hbm": algo / ms / 1e6 / peak,
                                             "algorithmic_bytes": algo, "points": points}
    # residual diagnostics: the float64 loop with and without them
    from veris_gb300.evp_solver import evp_solver, evp_solver_residuals
    st = VerisState.from_numpy(arrays, sett, device=dev)
    n = 20
    t_plain = _event_time(lambda: evp_solver(st, n), 3, flush)
    t_res = _event_time(lambda: evp_solver_residuals(st, n), 3, flush)
    interior = (NX - 4) * (NY - 4)
    extra_ms = max(t_res - t_plain, 1e-9) / n
    algo = 13 * 8 * interior                # both states (10 fields) and 3 masks per interior point
    out["evp_residual_f64"] = {"subcycles": n, "ms_plain_loop": t_plain, "ms_with_residuals": t_res,
                               "overhead_frac": t_res / t_plain - 1, "ms_per_residual": extra_ms,
                               "achieved_GBs": algo / extra_ms / 1e6, "frac_hbm": algo / extra_ms / 1e6 / peak,
                               "algorithmic_bytes": algo}
    out["peak_GBs"] = peak
    out["peak_source"] = f"{peak_kind} HBM copy bandwidth"
    out["l2"] = "flushed before every timed launch"
    return out


def run_routines(args):
    """Only the routines beside the step (free drift, bulk formula, EVP
    residuals) on the workload's grid: one JSON line."""
    import torch
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    from __graft_entry__ import build
    build()
    from veris_gb300.synthetic import CONFIGS, make_state, config_settings
    c = CONFIGS[args.config]
    arrays = make_state(c["nx"], c["ny"], seed=args.seed)
    sett = config_settings(args.config)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    clocks = ClockSampler(0)
    clocks.start()
    out = measure_routines(arrays, sett, dev, flush)
    line = {"metric": "routines beside the EVP step", "config": {"workload": args.config, "nx": c["nx"],
                                                                  "ny": c["ny"]},
            "data": "synthetic", "routines": out, "clocks": clocks.stop()}
    print(json.dumps(line))
    return 0


def run_adjoint(args):
    """Gradient of a tracking loss through a float64 trajectory.

    The target is the end state of the same trajectory with P* x 1.2 and the
    winds of seed + 1; the loss is the interior sum of (u - u*)^2 + (v - v*)^2
    + (A - A*)^2 at the end.  Times, with CUDA events: the forward alone
    (graph replays), and the forward with snapshots plus the adjoint sweep.
    Also checks dL/dP* against a centred difference."""
    import torch
    torch.cuda.set_device(0)
    from __graft_entry__ import build
    build()
    from veris_gb300.state import VerisState
    from veris_gb300.synthetic import CONFIGS, make_state, config_settings
    from veris_gb300.trajectory import Trajectory, tracking_loss_adjoint

    name = args.adjoint_config
    c = CONFIGS[name]
    n_steps = args.adjoint_steps or c["steps"]
    arrays = make_state(c["nx"], c["ny"], seed=args.seed)
    winds1 = make_state(c["nx"], c["ny"], seed=args.seed + 1)
    sett = config_settings(name)
    if args.subcycles:
        sett.nEVPsteps = args.subcycles
    if args.evp_alpha_beta:
        sett.evpAlpha = sett.evpBeta = float(args.evp_alpha_beta)
    st = VerisState.from_numpy(arrays, sett)
    v = st.variables
    tape = {"auto": "auto", "on": True, "off": False}[args.tape]
    torch.cuda.reset_peak_memory_stats()
    tr = Trajectory(st, n_steps, snapshots=args.snapshots, evp_checkpoint_every=args.evp_checkpoint_every,
                    tape=tape, precision=args.adjoint_precision)
    tr.track_norms = args.track_norms
    x0 = tr._save()
    p0 = float(sett.pStar)

    # target: P* x 1.2 and the other seed's winds
    wind0 = (v.uWind.clone(), v.vWind.clone())
    v.uWind.copy_(torch.as_tensor(winds1["uWind"]))
    v.vWind.copy_(torch.as_tensor(winds1["vWind"]))
    tr.set_coefficients(pStar=1.2 * p0)
    tr.forward()
    target = {k: getattr(v, k).clone() for k in ("uIce", "vIce", "Area")}
    # the loss's first call loads its torch kernels (seconds on a fresh
    # process): once here, outside the timed regions
    tracking_loss_adjoint(st, target)
    torch.cuda.synchronize()
    v.uWind.copy_(wind0[0])
    v.vWind.copy_(wind0[1])
    tr.set_coefficients(pStar=p0)
    tr._load(x0)

    def ev():
        return torch.cuda.Event(enable_timing=True)

    # forward alone: graph replays
    tr._ensure_graph()
    fw = []
    for _ in range(1 + max(1, args.adjoint_repeats)):
        tr._load(x0)
        torch.cuda.synchronize()
        a, b = ev(), ev()
        a.record()
        for _k in range(n_steps):
            tr.eng.step()
        b.record()
        b.synchronize()
        fw.append(a.elapsed_time(b))
    t_fwd = float(np.median(fw[1:]))

    # forward with snapshots, then the adjoint
    res = []
    for _ in range(max(1, args.adjoint_repeats)):
        tr._load(x0)
        torch.cuda.synchronize()
        a, m, b = ev(), ev(), ev()
        a.record()
        tr.forward()
        L, lam = tracking_loss_adjoint(st, target)
        m.record()
        grads, coeffs, _ = tr.backward(lam)
        b.record()
        b.synchronize()
        res.append((a.elapsed_time(m), m.elapsed_time(b), float(L), float(coeffs["pStar"]), dict(tr.stats)))
    t_f2, t_adj, L0, dLdP, stats = res[-1]

    peak = torch.cuda.max_memory_allocated() / 1e9
    # centred difference in P* (a wider step for the float32 forward)
    fd = None
    if not args.no_fd:
        hP = (1e-6 if args.adjoint_precision == "f64" else 1e-3) * p0
        Ls = []
        for pv in (p0 + hP, p0 - hP):
            tr.set_coefficients(pStar=pv)
            tr._load(x0)
            tr.forward()
            Ls.append(float(tracking_loss_adjoint(st, target)[0]))
        tr.set_coefficients(pStar=p0)
        fd = (Ls[0] - Ls[1]) / (2 * hP)

    line = {"metric": "trajectory (forward + adjoint) / forward time", "value": (t_f2 + t_adj) / t_fwd,
            "unit": "x", "higher_is_better": False, "dtype": args.adjoint_precision, "data": "synthetic",
            "config": {"workload": name, "nx": c["nx"], "ny": c["ny"], "steps": n_steps,
                       "subcycles": int(sett.nEVPsteps), "dt_s": c["dt"],
                       "snapshots": tr.snaps, "evp_checkpoint_every": tr.K, "evp_tape": tr.tapes is not None,
                       "evpAlpha": float(sett.evpAlpha), "evpBeta": float(sett.evpBeta),
                       "target": "P* x 1.2 and seed+1 winds", "loss": "interior sum (u-u*)^2+(v-v*)^2+(A-A*)^2"},
            "forward_ms": t_fwd, "forward_with_snapshots_ms": t_f2, "adjoint_ms": t_adj,
            "stats": stats, "loss": L0,
            "dL_dpStar": {"adjoint": dLdP, "centred_difference": fd,
                          "rel_diff": None if fd is None else abs(dLdP - fd) / max(abs(fd), 1e-300)},
            "peak_hbm_gb": peak, "cost_model_steps": tr.cost[tr.n][tr.snaps],
            "gpu_launches_per_forward_step": tr.eng.launches_per_step}
    print(json.dumps(line))
    return 0


def run_ensemble(args):
    """512 independent domains (nx, ny drawn from {64..512} x {64..384} in
    steps of 32, winds scaled by U(0.5, 1.5)), 100 float32 subcycles per step,
    20 steps, one captured graph per step; against the same members run one
    after another through the single-domain float32 solver."""
    import torch
    torch.cuda.set_device(0)
    from __graft_entry__ import build
    build()
    from veris_gb300 import autotune
    from veris_gb300.ensemble import Ensemble, sequential_baseline
    from veris_gb300.state import VerisState
    from veris_gb300.synthetic import CONFIGS, config_settings, ensemble_members, make_state

    c = CONFIGS["c4_ensemble"]
    n_sub = args.subcycles or c["n_evp"]
    n_steps = c["steps"]
    sett = config_settings("c4_ensemble")
    sett.nEVPsteps = n_sub
    specs = ensemble_members(args.members, seed=args.seed)
    t0 = time.perf_counter()
    members = []
    for sp in specs:
        arrays = make_state(sp["nx"], sp["ny"], seed=sp["seed"], wind_scale=sp["wind_scale"])
        members.append(VerisState.from_numpy(arrays, sett))
    t_gen = time.perf_counter() - t0
    cells = sum(sp["nx"] * sp["ny"] for sp in specs)
    ens = Ensemble(members, n_sub)
    ens.step()                               # first step: eager, configures the kernels
    if args.ens_shape is not None:           # a fixed launch (profiling): no tuning
        ens.set_launch(args.ens_shape, args.ens_blocks_per_sm)
        tuned = {"shape": args.ens_shape, "blocks_per_sm": args.ens_blocks_per_sm, "trials": [], "fixed": True}
    else:
        tuned = autotune.tune(ens, use_cache=False)
    ens.capture()
    for _ in range(max(0, args.warmup - 1)):
        ens.step()
    torch.cuda.synchronize()
    clocks = ClockSampler(0)
    clocks.start()
    time.sleep(0.3)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(n_steps):
        ens.step()
    b.record()
    b.synchronize()
    clk = clocks.stop()
    ms = a.elapsed_time(b)
    value = cells * n_sub * n_steps / (ms / 1e3) / 1e9

    # sequential single-domain calls, one step of every member, eager
    outs = [[torch.empty(m.shape, dtype=torch.float32, device="cuda") for _ in range(5)] for m in members]
    import ctypes
    wss = [torch.empty(ens.lib.veris_evp_fast_workspace_bytes(ctypes.byref(ens.grids[k]), 4),
                       dtype=torch.uint8, device="cuda") for k in range(len(members))]
    sequential_baseline(members, n_sub, outs, wss)
    torch.cuda.synchronize()
    seq = []
    for _ in range(2):
        a2, b2 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a2.record()
        sequential_baseline(members, n_sub, outs, wss)
        b2.record()
        b2.synchronize()
        seq.append(a2.elapsed_time(b2))
    seq_ms = min(seq)
    seq_value = cells * n_sub / (seq_ms / 1e3) / 1e9
    line = {"metric": "ensemble EVP Gcell-subcycles/s", "value": value, "unit": "Gcell-subcycles/s",
            "higher_is_better": True, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "c4_ensemble", "members": len(specs), "cells": cells, "subcycles": n_sub,
                       "steps": n_steps, "min_member": [min(sp["nx"] for sp in specs), min(sp["ny"] for sp in specs)],
                       "max_member": [max(sp["nx"] for sp in specs), max(sp["ny"] for sp in specs)],
                       "graph": "one CUDA graph per ensemble step", "tiles_per_subcycle": ens.total_tiles},
            "ms_per_step": ms / n_steps, "tuned": {k: tuned.get(k) for k in ("shape", "blocks_per_sm", "ms_per_subcycle", "fixed")},
            "tuning_trials": tuned.get("trials"),
            "sequential": {"value": seq_value, "ms_per_step": seq_ms,
                           "what": "one veris_evp_fast_solver_f32 call per member, eager, one after another"},
            "speedup_vs_sequential": value / seq_value, "clocks": clk, "generate_s": t_gen,
            "gpu_launches_per_step": n_sub + 2}
    print(json.dumps(line))
    return 0


def main():
    args = parse()
    if args.ensemble:
        return run_ensemble(args)
    if args.adjoint:
        return run_adjoint(args)
    if args.routines_only and args.impl != "reference":
        return run_routines(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())

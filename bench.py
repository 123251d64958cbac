#!/usr/bin/env python
"""Benchmark of the sea-ice step: EVP Gcell-subcycles/s on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (default): the 0.25-degree single domain, 1440 x 720 interior cells,
500 mEVP subcycles per step, dt = 1800 s, seeded synthetic fields.  One
bench step is one full sea-ice time step (dynamics preparation, 500 EVP
subcycles, ocean stress, advection, clean-up, growth, halo fills).

The headline ``value`` is the float64 step (the drop-in arithmetic, the
same precision as the reference's NumPy path) replayed as one CUDA graph,
with inputs resident in HBM; L2 is flushed (a 512 MiB write) before every
timed step and the flush is outside the timed events.  The metric counts
interior cells x subcycles over the whole step time.  ``e2e`` is the same
step through the host coupling (pinned host arrays uploaded, the step's
outputs downloaded, every step).  ``roofline`` is the float64 subcycle
kernel's: bound by GB300's float64 pipe (2 lanes per SM and cycle), with
its HBM fraction beside it.

Also reported, each in its own block: ``fp32`` (the mixed-precision step:
float32 EVP and advection, float64 thermodynamics and budgets; its rate,
end-to-end rate, walk-kernel HBM roofline, error against the float64 step
after one and N steps, and the branch flips behind the error), ``c5``
(the 3600 x 1800 grid: float64 and float32 step rates, walk roofline,
float32 errors, and the error float64 arithmetic makes from inputs rounded
to float32), ``routines`` (free drift, bulk formula, residuals),
``conservation`` (float64 budgets of the timed steps) and ``cpu_baseline``
(the NumPy oracle on one core, bounded sample).

``--impl reference`` times the reference's CPU algorithm (the NumPy oracle,
a restatement of the reference that is bit-identical to it on the golden
fixtures) on all host cores, each step a bounded sample of 20 subcycles
extrapolated to a full step.

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
# EVP subcycles each CPU sample times (the rest of the step is timed once)
CPU_SAMPLE_SUBCYCLES = 20
# float64 lanes GB300's float64 pipe retires per SM and cycle
FP64_LANES_PER_SM_CYCLE = 2


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=("ours", "reference"))
    ap.add_argument("--config", default="c2_quarterdeg")
    ap.add_argument("--precision", default="f64", choices=("f32", "f64"),
                    help="precision of the headline step (f64: the drop-in arithmetic)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp32", action="store_true", help="skip the float32 block")
    ap.add_argument("--no-fp64", action="store_true", help="(--precision f32) skip the float64 comparison")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-c5", action="store_true", help="skip the 3600 x 1800 block")
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
    ap.add_argument("--walk-persistent", type=int, default=-1, choices=(-1, 0, 1),
                    help="float32 walk subcycles per launch: 0 one, 1 all but the last (-1: tuned)")
    ap.add_argument("--f64-tile-rows", type=int, default=-1, choices=(-1, 0, 16, 24, 32),
                    help="rows per tile of the float64 subcycle kernel (0: the library's default; "
                         "-1: tuned on the workload)")
    ap.add_argument("--adjoint", action="store_true",
                    help="time a trajectory's forward + adjoint against its forward (float64)")
    ap.add_argument("--adjoint-config", default="c3_1deg")
    ap.add_argument("--adjoint-steps", type=int, default=None)
    ap.add_argument("--adjoint-precision", default="f64", choices=("f64", "f32"))
    ap.add_argument("--snapshots", type=int, default=None, help="step snapshots (default: all)")
    ap.add_argument("--evp-checkpoint-every", type=int, default=None,
                    help="EVP subcycle checkpoint interval inside a step's adjoint "
                         "(0: keep all; default: keep all when it fits in device memory)")
    ap.add_argument("--tape", default="auto", choices=("auto", "on", "off", "step"),
                    help="keep every EVP subcycle state during the forward (step: float32, one step's "
                         "tape written during the reverse)")
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


def workload_config(name, c, sett, n_sub):
    """The workload's defining keys, printed alike by both arms."""
    return {"workload": name, "nx": c["nx"], "ny": c["ny"], "subcycles": int(n_sub),
            "evpAlpha": float(sett.evpAlpha), "evpBeta": float(sett.evpBeta),
            "adaptive_evp": bool(sett.useAdaptiveEVP), "dt_s": float(c["dt"]), "cells": c["nx"] * c["ny"]}


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

def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def hbm_peak():
    hbm = measured_peaks().get("hbm_gbs")
    return (float(hbm), "measured") if hbm else (6800.0, "fallback")


def fp64_peak(sm_count):
    """GB300's float64 pipe: 2 lanes per SM and cycle at the measured maximum
    SM clock, in G float64 operations per second."""
    mhz = measured_peaks().get("sm_max_mhz") or 2070.0
    return FP64_LANES_PER_SM_CYCLE * sm_count * float(mhz) * 1e6 / 1e9, float(mhz)


def recorded(kernel, workload, what="traffic", form=None):
    """A per-launch figure of ``kernel`` on ``workload`` from an ncu capture
    (profiles/roofline_traffic.json): DRAM bytes ("traffic") or float64-pipe
    lane operations ("fp64_lane_ops"), of the kernel's ``form`` (e.g. the
    float64 subcycle's unit height "rows16") where one is recorded; None
    when not recorded."""
    path = os.path.join(ROOT, "profiles", "roofline_traffic.json")
    try:
        with open(path) as f:
            rec = json.load(f)
    except (OSError, ValueError):
        return None
    key = f"{kernel}/{workload}" + ("" if what == "traffic" else f":{what}")
    if form is not None and f"{key}@{form}" in rec:
        return rec[f"{key}@{form}"]
    return rec.get(key)


def f64_rows(tuning, args):
    """The float64 subcycle's unit height in use: the tuner's choice, the
    one asked for, or the library default (24)."""
    if isinstance(tuning, dict) and "rows" in tuning:
        return int(tuning["rows"])
    return args.f64_tile_rows if args.f64_tile_rows > 0 else 24


# ----------------------------------------------------------------- CPU legs

def cpu_fixed(arrays, sett):
    """The oracle (the reference's NumPy algorithm, one core) on the parts of
    a step outside the EVP subcycles: dynamics preparation, ocean stress,
    advection, clean-up, growth.  Returns (seconds, the prepared state)."""
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
    prepared = SimpleNamespace(variables=SimpleNamespace(**vars(v)), settings=st.settings)
    v.OceanStressU, v.OceanStressV = O.OceanStressUV(st)
    v.hIceMean, v.hSnowMean, v.Area = O.Advection(st)
    out = O.clean_up_advection(st)
    v.hIceMean, v.hSnowMean, v.Area, v.TSurf, v.os_hIceMean, v.os_hSnowMean = out
    v.Area = O.ridging(st)
    O.Growth(st)
    t2 = time.perf_counter()
    return (t1 - t0) + (t2 - t1), prepared


def cpu_subcycles(prepared, n):
    """Seconds per EVP subcycle of the oracle over n subcycles (one core)."""
    from oracle import veris_oracle as O
    c = O.evp_carry(prepared)
    t0 = time.perf_counter()
    for _ in range(n):
        O.evp_subcycle(prepared, c)
    return (time.perf_counter() - t0) / n


def cpu_step_estimate(arrays, sett, n_sample, n_full):
    """One-core seconds per full step: the fixed parts timed once, plus
    ``n_sample`` subcycles timed and scaled to ``n_full``."""
    fixed, prepared = cpu_fixed(arrays, sett)
    per_sub = cpu_subcycles(prepared, n_sample)
    return fixed + per_sub * n_full, fixed, per_sub


def _reference_worker(job):
    """One replica of the oracle in a worker process (one core): the fixed
    parts timed once, then one sample of subcycles per bench step."""
    import os as _os
    _os.environ.setdefault("OMP_NUM_THREADS", "1")
    config, seed, n_sample, steps, warmup = job
    from veris_gb300.synthetic import CONFIGS, make_state, config_settings
    c = CONFIGS[config]
    arrays = make_state(c["nx"], c["ny"], seed=seed)
    sett = config_settings(config)
    cpu_fixed(arrays, sett)                              # warm-up
    fixed, prepared = cpu_fixed(arrays, sett)
    for _ in range(warmup):
        cpu_subcycles(prepared, 2)
    per_sub = [cpu_subcycles(prepared, n_sample) for _ in range(steps)]
    return fixed, per_sub


def jax_probe():
    """Whether the reference's JAX backend could be timed on this host."""
    try:
        import jax  # noqa: F401
        return "importable (not timed: the reference's JAX path needs Veros)"
    except Exception as e:   # noqa: BLE001
        return f"unavailable: {type(e).__name__}: {e}"


def run_reference(args):
    """The reference's CPU algorithm (the NumPy oracle) on all host cores:
    one independent replica of the workload per core (NumPy elementwise code
    uses one core each).  Every replica times the step's parts outside the
    EVP once and, per bench step, a sample of 20 subcycles; a step's time is
    the fixed parts plus the sample scaled to the step's subcycles, and the
    value is all replicas' cells x subcycles over the slowest replica's time."""
    ws, rank = int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    import multiprocessing as mp
    from veris_gb300.synthetic import CONFIGS, config_settings
    c = CONFIGS[args.config]
    sett = config_settings(args.config)
    n_full = args.subcycles or c["n_evp"]
    sett.nEVPsteps = n_full
    cells = c["nx"] * c["ny"]
    n_sample = min(CPU_SAMPLE_SUBCYCLES, n_full)
    cores = max(1, os.cpu_count() or 1)
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(cores) as pool:
        res = pool.map(_reference_worker, [(args.config, args.seed + r, n_sample, args.steps, args.warmup)
                                           for r in range(cores)])
    wall = time.perf_counter() - t0
    # step k takes, on replica r, fixed_r + per_sub_r[k] * n_full; the job's
    # step time is the slowest replica's
    step_s = [max(fx + ps[k] * n_full for fx, ps in res) for k in range(args.steps)]
    sec = float(np.sum(step_s))
    value = cores * cells * n_full * args.steps / sec / 1e9
    fixed_med = float(np.median([fx for fx, _ in res]))
    sub_med = float(np.median([np.median(ps) for _, ps in res]))
    sample = (f"{cores} processes, NumPy oracle on one core each: per bench step {n_sample} EVP subcycles "
              f"timed and scaled x{n_full / n_sample:g} to {n_full}, plus the step's other routines "
              f"(preparation, ocean stress, advection, clean-up, growth) timed once "
              f"(median {fixed_med:.2f} s; {sub_med:.3f} s per subcycle)")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Gcell-subcycles/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": sec / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(args.config, c, sett, n_full),
        "run": {"parallelism": f"{cores} CPU replicas", "l2": "n/a (CPU)",
                "extrapolation": {"subcycles_timed_per_step": n_sample, "subcycles_per_step": n_full,
                                  "factor": n_full / n_sample},
                "wall_s": wall, "jax_cpu": jax_probe()},
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


def make_engine(arrays, sett, dev, precision, args, walk_variant=None, budgets=False, tune=False):
    """A captured SeaIceStep on a fresh device copy of ``arrays`` (the
    capture runs one eager step first); the float32 walk is tuned on the
    workload unless a variant is given."""
    from veris_gb300.engine import SeaIceStep
    from veris_gb300.state import VerisState
    state = VerisState.from_numpy(arrays, sett, device=dev)
    wv = max(0, args.walk_variant) if walk_variant is None else walk_variant
    eng = SeaIceStep(state, precision=precision, evp=args.evp, f32_kernel=args.f32_kernel,
                     walk_rows=args.walk_rows, walk_variant=wv, budgets=budgets)
    tuning = None
    persist = (0, 1) if args.walk_persistent < 0 else (args.walk_persistent,)
    if precision == "f32" and eng.f32_kernel == "walk" and eng.evp_form == "fast":
        if walk_variant is None and args.walk_variant < 0:
            from veris_gb300.autotune import tune_walk
            tuning = tune_walk(eng, persistent=persist)
        elif args.walk_persistent >= 0:
            eng.lib.veris_evp_walk_persistent(args.walk_persistent)
    if precision == "f64" and eng.evp_form == "fast" and args.f64_tile_rows < 0 and tune:
        from veris_gb300.autotune import tune_f64_tile
        tuning = tune_f64_tile(eng)
    eng.capture()
    return eng, tuning


def time_steps(eng, steps, warmup, flush, ws, dev, clocks=None):
    """CUDA-event milliseconds of ``steps`` graph replays (L2 flushed before
    each, outside the events), max over ranks; and the host wall seconds."""
    import torch
    for _ in range(warmup):
        eng.step()
    torch.cuda.synchronize(dev)
    if clocks is not None:
        clocks.start()
        time.sleep(0.3)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    barrier(ws)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for k in range(steps):
        flush.zero_()
        starts[k].record()
        eng.step()
        ends[k].record()
    torch.cuda.synchronize(dev)
    barrier(ws)
    wall = time.perf_counter() - t0
    clk = clocks.stop() if clocks is not None else None
    ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends))
    return max_over_ranks(ms, ws), wall, clk


def evp_kernel_name(eng):
    if eng.evp_form != "fast":
        return f"evp_subcycle_kernel<{'double' if eng.precision == 'f64' else 'float'}>"
    if eng.precision == "f64":
        return "evp_f64_kernel"
    return "evp_walk_kernel" if eng.f32_kernel == "walk" else "evp_tma_kernel"


def evp_launch_us(eng, n_sub, flush):
    """Average microseconds per EVP subcycle launch: CUDA events on the
    launching stream around an eager step's EVP phase (the once-per-step
    fold of the constants included), median of three, L2 flushed first."""
    ms = []
    for _ in range(3):
        flush.zero_()
        ms.append(eng.timed_step())
    return float(np.median(ms)) * 1e3 / n_sub


def roofline_hbm(kernel, workload, cells, us, precision, form=None):
    peak, kind = hbm_peak()
    algo = BYTES_PER_CELL_SUBCYCLE[precision] * cells
    achieved = algo / (us * 1e-6) / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": recorded(kernel, workload, form=form), "kernel": kernel, "algorithmic_bytes_per_launch": algo,
            "avg_launch_us": us, "peak_source": f"{kind} HBM copy bandwidth"}


def roofline_fp64(kernel, workload, cells, us, sm_count, rows=None):
    """The float64 subcycle's roofline: GB300's float64 pipe (its bound),
    with the HBM fraction of the algorithmic bytes beside it.  ``achieved``
    = the kernel's float64-pipe lane operations per launch (ncu, recorded in
    profiles/roofline_traffic.json) over the live launch duration."""
    peak, mhz = fp64_peak(sm_count)
    form = f"rows{rows}" if rows else None
    ops = recorded(kernel, workload, "fp64_lane_ops", form)
    achieved = ops / (us * 1e-6) / 1e9 if ops else None
    return {"bound": "fp64_pipe", "achieved": achieved, "peak": peak, "unit": "Gop/s",
            "frac": achieved / peak if achieved else None, "traffic": recorded(kernel, workload, form=form),
            "kernel": kernel, "unit_rows": rows, "avg_launch_us": us, "fp64_lane_ops_per_launch": ops,
            "fp64_lane_ops_per_cell": ops / cells if ops else None,
            "peak_source": f"{FP64_LANES_PER_SM_CYCLE} float64 lanes per SM and cycle x {sm_count} SMs x "
                           f"{mhz:g} MHz (the measured maximum SM clock)",
            "hbm": roofline_hbm(kernel, workload, cells, us, "f64", form)}


def e2e_of(eng, args, ws, cells, n_sub):
    """The step through the host coupling: pinned host inputs uploaded and
    outputs downloaded every step (HostCoupledStep, one graph per step)."""
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
    e2e_s = max_over_ranks(time.perf_counter() - t0, ws)
    return {"value": ws * cells * n_sub * ke / e2e_s / 1e9, "unit": "Gcell-subcycles/s",
            "h2d_bytes_per_step": host.h2d_bytes, "d2h_bytes_per_step": host.d2h_bytes, "steps": ke,
            "ms_per_step": e2e_s / ke * 1e3,
            "api": "veris_gb300.host.HostCoupledStep.step (pinned host arrays)"}


def branch_states(v, s):
    """Which side of the step's switches each interior cell (or face) is on
    at the state ``v`` (torch tensors on the device): the ocean-drag floor
    (veris/dynamics_routines.py:21-52), the thin-ice cut-off and the area
    clips (veris/clean_up.py:5-47), the surface-temperature clamp at melting
    (veris/solve4temp.py:146-157), the upwind direction and the superbee
    branch of the zonal flux of hIceMean (veris/advection.py:94-175)."""
    import torch
    I = (slice(2, -2), slice(2, -2))
    du = (v.uIce - v.uOcean) * v.maskInU
    dv = (v.vIce - v.vOcean) * v.maskInV
    a = du + torch.roll(du, -1, 0)
    b = dv + torch.roll(dv, -1, 1)
    t = 0.25 * (a * a + b * b)
    dc = torch.where(v.fCori < 0, s.waterIceDrag_south, s.waterIceDrag) * s.rhoSea
    out = {"ocean_drag_floor": ((dc * dc * t <= s.cDragMin ** 2) & (v.iceMask != 0))[I],
           "no_ice": (v.hIceMean <= 0)[I],
           "area_at_1": (v.Area >= 1.0)[I],
           "area_at_min": ((v.Area <= s.Area_min) & (v.hIceMean > 0))[I],
           "tsurf_at_melting": ((v.TSurf >= s.celsius2K) & (v.hIceMean > 0))[I]}
    h = v.hIceMean
    mask = v.iceMaskU * v.maskInU
    uT = v.uIce * v.dyG * v.iceMaskU
    Rjp = (h[3:] - h[2:-1]) * mask[3:]
    Rj = (h[2:-1] - h[1:-2]) * mask[2:-1]
    Rjm = (h[1:-2] - h[:-3]) * mask[1:-2]
    up = uT[2:-1] > 0
    cr = torch.where(up, Rjm, Rjp)
    cr = torch.where(Rj.abs() * s.CrMax > cr.abs(), cr / Rj, torch.sign(cr) * s.CrMax * torch.sign(Rj))
    region = torch.bucketize(cr.nan_to_num(0.0).contiguous(),
                             torch.tensor([0.0, 0.5, 1.0, 2.0], dtype=cr.dtype, device=cr.device))
    out["upwind_direction"] = up[:, 2:-2]
    out["superbee_branch"] = region[:, 2:-2]
    return out


def branch_flips(v_a, v_b, s):
    """Cells (faces) where two states sit on different sides of a switch."""
    sa, sb = branch_states(v_a, s), branch_states(v_b, s)
    flips = {k: int((sa[k] != sb[k]).sum()) for k in sa}
    flips["cells"] = int(sa["no_ice"].numel())
    return flips


def compare_precisions(arrays, sett, dev, args, n_steps, walk_variant):
    """The float32 and float64 steps from the same initial state: field
    errors and branch flips after one and after ``n_steps`` steps."""
    import torch
    names = ("uIce", "vIce", "hIceMean", "hSnowMean", "Area", "TSurf", "Qnet")
    e32, _ = make_engine(arrays, sett, dev, "f32", args, walk_variant=walk_variant)   # capture ran step 1
    e64, _ = make_engine(arrays, sett, dev, "f64", args)
    torch.cuda.synchronize(dev)
    v32, v64 = e32.state.variables, e64.state.variables
    errs1 = {n: rel_errors(getattr(v32, n), getattr(v64, n)) for n in names}
    flips1 = branch_flips(v32, v64, sett)
    for _ in range(n_steps - 1):
        e64.step()
        e32.step()
    torch.cuda.synchronize(dev)
    errs = {n: rel_errors(getattr(v32, n), getattr(v64, n)) for n in names}
    flips = branch_flips(v32, v64, sett)
    return {"after_1_step": errs1, "steps": n_steps, "fields": errs,
            "branch_flips": {"after_1_step": flips1, f"after_{n_steps}_steps": flips},
            "definition": "max_rel = max|a-b| / max|b|, rms_rel = rms(a-b) / max|b|; a branch flip is an "
                          "interior cell (face) on different sides of a switch in the two states"}


def conservation_summary(eng, steps):
    """The float64 budgets of the last ``steps`` recorded steps: the drift
    of the ice and snow volumes and the ice area over them, what advection,
    the clean-up and the thermodynamics changed per step, and the ocean's
    heat, fresh-water and salt fluxes (area-weighted interior sums)."""
    rec = {k: v[-steps:] for k, v in eng.budget_records().items()}

    def drift(start, end):
        a, b = float(rec[start][0]), float(rec[end][-1])
        return {"first": a, "last": b, "rel_change": (b - a) / a if a else None}

    adv = max(abs(float(x - y) / float(y)) if y else 0.0
              for x, y in zip(rec["ice_volume_advected"], rec["ice_volume_start"]))
    return {"steps": len(rec["ice_volume_start"]),
            "ice_volume_m3": drift("ice_volume_start", "ice_volume_end"),
            "snow_volume_m3": drift("snow_volume_start", "snow_volume_end"),
            "ice_area_m2": drift("ice_area_start", "ice_area_end"),
            "advection_ice_volume_rel_change_max": adv,
            "cleanup_ice_volume_change_m3_per_step": float(np.mean(rec["ice_volume_cleaned"]
                                                                   - rec["ice_volume_advected"])),
            "ice_overshoot_m3_per_step": float(np.mean(rec["ice_overshoot"])),
            "thermodynamic_ice_volume_change_m3_per_step": float(np.mean(rec["ice_volume_end"]
                                                                         - rec["ice_volume_cleaned"])),
            "ocean_heat_loss_W": float(np.mean(rec["ocean_heat_loss"])),
            "fresh_water_flux_kg_s": float(np.mean(rec["fresh_water_flux"])),
            "salt_flux_kg_s": float(np.mean(rec["salt_flux"])),
            "how": "float64 area-weighted interior sums inside the step's graph (veris_budget_sums_f64)"}


def fp32_block(arrays, sett, dev, args, flush, ws, workload, cells, n_sub):
    """The mixed-precision step (float32 EVP and advection, float64
    thermodynamics, budgets and master state) on the same workload."""
    eng, tuning = make_engine(arrays, sett, dev, "f32", args)
    ms, wall, _ = time_steps(eng, args.steps, args.warmup, flush, ws, dev)
    value = replica_value(cells, n_sub, args.steps, ms, ws)
    us = evp_launch_us(eng, n_sub, flush)
    out = {"value": value, "unit": "Gcell-subcycles/s", "ms_per_step": ms / args.steps, "dtype": "f32",
           "gpu_launches": eng.launches_per_step * args.steps,
           "roofline": roofline_hbm(evp_kernel_name(eng), workload, cells, us, "f32"),
           "evp_form": eng.evp_form, "f32_kernel": eng.f32_kernel,
           "walk": {"rows": eng.walk_rows or "auto", "variant": eng.walk_variant,
                    "persistent": bool(tuning["persistent"]) if tuning else args.walk_persistent == 1,
                    "tuning": tuning}}
    if not args.no_e2e:
        out["e2e"] = e2e_of(eng, args, ws, cells, n_sub)
    wv = eng.walk_variant
    del eng
    out["error_vs_fp64"] = compare_precisions(arrays, sett, dev, args, max(2, args.warmup + args.steps), wv)
    return out


def c5_block(args, dev, flush):
    """The 3600 x 1800 workload (500 subcycles, dt 600 s): float64 and
    float32 step rates, the walk's HBM roofline, float32 errors after one
    step, and the error float64 arithmetic makes from every input rounded to
    float32 (the conditioning of the step at this resolution)."""
    import torch
    from veris_gb300.engine import SeaIceStep
    from veris_gb300.state import VerisState
    from veris_gb300.synthetic import CONFIGS, make_state, config_settings
    name = "c5_tenthdeg"
    c = CONFIGS[name]
    arrays = make_state(c["nx"], c["ny"], seed=args.seed)
    sett = config_settings(name)
    n_sub = int(sett.nEVPsteps)
    cells = c["nx"] * c["ny"]
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    out = {"config": workload_config(name, c, sett, n_sub)}
    e64, tuning64 = make_engine(arrays, sett, dev, "f64", args, tune=True)
    ms64, _, _ = time_steps(e64, 2, 1, flush, 1, dev)
    us64 = evp_launch_us(e64, n_sub, flush)
    out["fp64"] = {"value": cells * n_sub * 2 / (ms64 / 1e3) / 1e9, "ms_per_step": ms64 / 2, "steps": 2,
                   "roofline": roofline_fp64(evp_kernel_name(e64), name, cells, us64, sms, f64_rows(tuning64, args)),
                   "f64_tile": tuning64}
    del e64
    e32, tuning = make_engine(arrays, sett, dev, "f32", args)
    ms32, _, _ = time_steps(e32, 5, 2, flush, 1, dev)
    us32 = evp_launch_us(e32, n_sub, flush)
    wv = e32.walk_variant
    out["fp32"] = {"value": cells * n_sub * 5 / (ms32 / 1e3) / 1e9, "ms_per_step": ms32 / 5, "steps": 5,
                   "roofline": roofline_hbm(evp_kernel_name(e32), name, cells, us32, "f32"),
                   "walk": {"variant": wv, "tuning": tuning}}
    out["fp32_over_fp64_speedup"] = out["fp32"]["value"] / out["fp64"]["value"]
    del e32
    torch.cuda.empty_cache()
    # one step from the same state: float64, float32, float64 on float32-rounded inputs
    names = ("uIce", "vIce", "hIceMean", "hSnowMean", "Area")
    runs = {}
    for key, arr, prec in (("f64", arrays, "f64"), ("f32", arrays, "f32"),
                           ("f64_rounded_inputs", {k: a.astype(np.float32).astype(np.float64)
                                                   for k, a in arrays.items()}, "f64")):
        st = VerisState.from_numpy(arr, sett, device=dev)
        eng = SeaIceStep(st, precision=prec, walk_variant=wv)
        eng.step()
        torch.cuda.synchronize(dev)
        runs[key] = st.variables
        del eng
    ref = runs["f64"]
    out["error_after_1_step"] = {
        k: {n: rel_errors(getattr(runs[k], n), getattr(ref, n)) for n in names} for k in ("f32", "f64_rounded_inputs")}
    out["branch_flips_after_1_step"] = {k: branch_flips(runs[k], ref, sett) for k in ("f32", "f64_rounded_inputs")}
    out["note"] = ("f64_rounded_inputs: float64 arithmetic throughout, every input rounded to float32 first; "
                   "its error is the part of the float32 error no float32 arithmetic can remove")
    del runs, ref
    torch.cuda.empty_cache()
    return out


def run_ours(args):
    import torch
    ws, rank, local = dist_init(args)
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from __graft_entry__ import build
    if rank == 0 or ws == 1:
        build()
    barrier(ws)
    from veris_gb300 import _abi
    _abi.check("evp_f64_tile_rows", _abi.load().veris_evp_f64_tile_rows(max(0, args.f64_tile_rows)))
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
    n_sub = int(sett.nEVPsteps)
    cells = c["nx"] * c["ny"]
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    # the headline step, graph-replayed, inputs resident
    eng, tuning = make_engine(arrays, sett, dev, args.precision, args, budgets=True, tune=True)
    ms, wall, clk = time_steps(eng, args.steps, args.warmup, flush, ws, dev, clocks=ClockSampler(local))
    conservation = conservation_summary(eng, args.steps)
    value = replica_value(cells, n_sub, args.steps, ms, ws)
    us = evp_launch_us(eng, n_sub, flush)
    phases = eng.phase_times()
    kernel = evp_kernel_name(eng)
    roof = (roofline_fp64(kernel, args.config, cells, us, sms, f64_rows(tuning, args)) if args.precision == "f64"
            else roofline_hbm(kernel, args.config, cells, us, "f32"))
    line = {"metric": METRIC, "value": value, "unit": "Gcell-subcycles/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": args.precision, "data": "synthetic (seeded generators of the workload's fields)",
            "config": workload_config(args.config, c, sett, n_sub),
            "run": {"parallelism": "replicas" if ws > 1 else "single-gpu",
                    "l2": "flushed before every timed step (512 MiB write)", "graph": "one CUDA graph per step",
                    "evp_form": eng.evp_form, "evp_kernel": kernel,
                    "walk": ({"rows": eng.walk_rows or "auto", "variant": eng.walk_variant, "tuning": tuning}
                             if args.precision == "f32" and eng.f32_kernel == "walk" else None),
                    "f64_tile": tuning if args.precision == "f64" else None},
            "roofline": roof, "gpu_launches": eng.launches_per_step * args.steps, "clocks": clk,
            "conservation": conservation,
            "wall_s_timed_region": wall, "evp_ms_per_step": us * n_sub / 1e3,
            "phase_ms": {k: round(v, 4) for k, v in phases.items()}}
    if not args.no_e2e:
        line["e2e"] = e2e_of(eng, args, ws, cells, n_sub)
    del eng
    torch.cuda.empty_cache()

    if args.precision == "f64" and not args.no_fp32:
        line["fp32"] = fp32_block(arrays, sett, dev, args, flush, ws, args.config, cells, n_sub)
        line["fp32"]["speedup_vs_fp64"] = line["fp32"]["value"] / value
    elif args.precision == "f32" and not args.no_fp64:
        e64, _ = make_engine(arrays, sett, dev, "f64", args)
        ms64, _, _ = time_steps(e64, max(1, args.steps // 2), 1, flush, ws, dev)
        line["fp64"] = {"value": replica_value(cells, n_sub, max(1, args.steps // 2), ms64, ws),
                        "ms_per_step": ms64 / max(1, args.steps // 2)}
        del e64
    torch.cuda.empty_cache()

    if ws == 1 and not args.no_routines:
        line["routines"] = measure_routines(arrays, sett, dev, flush)
    if ws == 1 and not args.no_c5 and args.config != "c5_tenthdeg":
        line["c5"] = c5_block(args, dev, flush)

    if rank == 0 and not args.no_cpu_baseline:
        n_sample = min(CPU_SAMPLE_SUBCYCLES, n_sub)
        sec, fixed, per_sub = cpu_step_estimate(arrays, sett, n_sample, n_sub)
        line["cpu_baseline"] = {
            "value": cells * n_sub / sec / 1e9, "unit": "Gcell-subcycles/s", "cores": 1, "kind": "port",
            "sample": (f"NumPy oracle, 1 thread: {n_sample} EVP subcycles timed ({per_sub * n_sample:.1f} s) and "
                       f"scaled x{n_sub / n_sample:g} to {n_sub}, plus preparation, ocean stress, advection, "
                       f"clean-up and growth timed once ({fixed:.1f} s)"),
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
    tape = {"auto": "auto", "on": True, "off": False, "step": "step"}[args.tape]
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
                       "snapshots": tr.snaps, "evp_checkpoint_every": tr.K, "evp_tape": tr.tape_mode,
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
    20 steps.  Headline: whole sea-ice steps of every member (per-member
    preparation, the batched EVP, per-member ocean stress, advection,
    clean-up, Growth and fills on parallel branches), one captured graph per
    ensemble step, against the same members' whole steps one after another
    (each member's own captured float32 step).  Also: the batched EVP alone
    (the dynamics-only form) against the single-domain solver per member."""
    import torch
    torch.cuda.set_device(0)
    from __graft_entry__ import build
    build()
    from veris_gb300 import autotune
    from veris_gb300.engine import SeaIceStep
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

    def timed(step, n):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record()
        for _ in range(n):
            step()
        b.record()
        b.synchronize()
        return a.elapsed_time(b)

    # the batched EVP alone: tuned launch shape
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
    ms_evp = timed(ens.step, n_steps)
    evp_value = cells * n_sub * n_steps / (ms_evp / 1e3) / 1e9
    outs = [[torch.empty(m.shape, dtype=torch.float32, device="cuda") for _ in range(5)] for m in members]
    import ctypes
    wss = [torch.empty(ens.lib.veris_evp_fast_workspace_bytes(ctypes.byref(ens.grids[k]), 4),
                       dtype=torch.uint8, device="cuda") for k in range(len(members))]
    sequential_baseline(members, n_sub, outs, wss)
    seq_evp_ms = min(timed(lambda: sequential_baseline(members, n_sub, outs, wss), 1) for _ in range(2))
    del ens, outs, wss
    torch.cuda.empty_cache()

    # whole steps, batched
    full = Ensemble(members, n_sub, shape=tuned["shape"], blocks_per_sm=tuned["blocks_per_sm"], full_step=True)
    full.step()
    full.capture()
    for _ in range(max(0, args.warmup - 1)):
        full.step()
    clocks = ClockSampler(0)
    clocks.start()
    time.sleep(0.3)
    ms = timed(full.step, n_steps)
    clk = clocks.stop()
    value = cells * n_sub * n_steps / (ms / 1e3) / 1e9
    del full
    torch.cuda.empty_cache()

    # whole steps, one member after another (each its own captured step)
    engines = []
    for st in members:
        e = SeaIceStep(st, precision="f32", check_finite=False)
        e.capture()
        engines.append(e)

    def sequential_step():
        for e in engines:
            e.step()

    sequential_step()
    seq_ms = min(timed(sequential_step, 1) for _ in range(2))
    seq_value = cells * n_sub / (seq_ms / 1e3) / 1e9
    line = {"metric": "ensemble EVP Gcell-subcycles/s (whole sea-ice steps)", "value": value,
            "unit": "Gcell-subcycles/s", "higher_is_better": True, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "c4_ensemble", "members": len(specs), "cells": cells, "subcycles": n_sub,
                       "steps": n_steps, "min_member": [min(sp["nx"] for sp in specs), min(sp["ny"] for sp in specs)],
                       "max_member": [max(sp["nx"] for sp in specs), max(sp["ny"] for sp in specs)],
                       "graph": "one CUDA graph per ensemble step (per-member work on 16 parallel branches)",
                       "tiles_per_subcycle": int(ens_tiles(members, n_sub, tuned))},
            "ms_per_step": ms / n_steps, "clocks": clk, "generate_s": t_gen,
            "tuned": {k: tuned.get(k) for k in ("shape", "blocks_per_sm", "ms_per_subcycle", "fixed")},
            "tuning_trials": tuned.get("trials"),
            "sequential": {"value": seq_value, "ms_per_step": seq_ms,
                           "what": "each member's own captured float32 SeaIceStep, one after another"},
            "speedup_vs_sequential": value / seq_value,
            "dynamics_only": {"value": evp_value, "ms_per_step": ms_evp / n_steps,
                              "sequential_value": cells * n_sub / (seq_evp_ms / 1e3) / 1e9,
                              "sequential_ms_per_step": seq_evp_ms,
                              "speedup_vs_sequential": evp_value / (cells * n_sub / (seq_evp_ms / 1e3) / 1e9),
                              "what": "the batched EVP alone against one veris_evp_fast_solver_f32 call per "
                                      "member, eager, one after another"}}
    print(json.dumps(line))
    return 0


def ens_tiles(members, n_sub, tuned):
    import ctypes
    from veris_gb300 import _abi
    from veris_gb300.ensemble import _grid_of
    lib = _abi.load()
    grids = (_abi.VerisGrid * len(members))(*[_grid_of(m) for m in members])
    return lib.veris_batch_tiles(len(members), grids, int(tuned["shape"]))


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

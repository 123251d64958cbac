"""Autotuners: the launch shape of the batched ensemble, the compiled
register budget of the single-domain walking EVP kernel, and the tile
height of the float64 EVP kernel.

For an ``Ensemble`` it times every candidate (tile shape x CTAs per SM) on a
few subcycles with CUDA events, keeps the fastest and caches the choice per
workload signature (member shapes, subcycles, GPU name) in a JSON file
(``$VERIS_TUNE_CACHE``, default ``~/.cache/veris_gb300/tune.json``).  The
ensemble's state is saved before the trials and restored after them, so
tuning does not advance the members.
"""
import hashlib
import json
import os

import torch

from .ensemble import SHAPES

DEFAULT_CANDIDATES = tuple((s, b) for s in SHAPES for b in ((1, 2, 3, 4) if s < 4 else (2, 3, 4)))


def _cache_path():
    return os.environ.get("VERIS_TUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "veris_gb300", "tune.json"))


def signature(ens):
    dev = torch.cuda.get_device_name(ens.device)
    key = json.dumps({"shapes": ens.shapes, "n_sub": ens.n_sub, "device": dev})
    return hashlib.sha1(key.encode()).hexdigest()


def _load():
    try:
        with open(_cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(cache):
    path = _cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "w") as f:
            json.dump(cache, f, indent=1)
    except OSError:
        pass


def tune(ens, candidates=DEFAULT_CANDIDATES, subcycles=10, repeats=3, use_cache=True):
    """Pick (shape, blocks_per_sm) for ``ens``; sets it and returns
    {"shape", "blocks_per_sm", "ms_per_subcycle", "trials": [...], "cached"}."""
    sig = signature(ens)
    cache = _load() if use_cache else {}
    if sig in cache:
        best = cache[sig]
        ens.set_launch(best["shape"], best["blocks_per_sm"])
        return dict(best, cached=True)
    snap = ens.ws.clone()
    buf0 = ens.buf
    trials = []
    for shape, bps in candidates:
        ens.set_launch(shape, bps)
        ens._enqueue(False, ens.buf, n_sub=2)    # configures the kernel, warms up
        times = []
        for _ in range(repeats):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record()
            ens._enqueue(False, ens.buf, n_sub=subcycles)
            b.record()
            b.synchronize()
            times.append(a.elapsed_time(b) / subcycles)
        trials.append({"shape": shape, "tile": SHAPES[shape], "blocks_per_sm": bps,
                       "ms_per_subcycle": sorted(times)[len(times) // 2]})
    ens.ws.copy_(snap)
    ens.buf = buf0
    del snap
    best = min(trials, key=lambda t: t["ms_per_subcycle"])
    ens.set_launch(best["shape"], best["blocks_per_sm"])
    choice = {"shape": best["shape"], "blocks_per_sm": best["blocks_per_sm"],
              "ms_per_subcycle": best["ms_per_subcycle"]}
    if use_cache:
        cache[sig] = choice
        _store(cache)
    return dict(choice, trials=trials, cached=False)


def tune_walk(eng, variants=(0, 1, 2, 3), persistent=(0, 1), subcycles=10, repeats=3):
    """Pick the walking kernel's compiled register budget (variant) and its
    subcycles per launch (one, or all but the last in one persistent launch)
    for a float32 ``SeaIceStep`` by timing each pair on ``subcycles``
    subcycles of the engine's state (outputs go to scratch: the state is not
    advanced).  More resident warps hide more latency but force shorter
    walks (all walks stay in one wave), so the best budget depends on the
    grid.  Sets the subcycles per launch process-wide
    (veris_evp_walk_persistent) and drops the engine's captured graph."""
    from ._abi import check
    outs = [torch.empty(eng.shape, dtype=torch.float32, device=eng.device) for _ in range(5)]
    ptrs = [t.data_ptr() for t in outs]
    ws = (eng.ws_evp.data_ptr(), eng.ws_evp.numel(), eng.stream)
    r64 = eng._refs(eng.f64)
    trials = []
    try:
        for p in persistent:
            check("evp_walk_persistent", eng.lib.veris_evp_walk_persistent(p))
            for v in variants:
                run = lambda n: check("evp_walk_f32", eng.lib.veris_evp_walk_solver_f32(*r64, n, eng.walk_rows, v,
                                                                                       *ptrs, *ws))
                run(3)
                times = []
                for _ in range(repeats):
                    a = torch.cuda.Event(enable_timing=True)
                    b = torch.cuda.Event(enable_timing=True)
                    a.record()
                    run(subcycles)
                    b.record()
                    b.synchronize()
                    times.append(a.elapsed_time(b) / subcycles)
                trials.append({"variant": v, "persistent": bool(p), "ms_per_subcycle": sorted(times)[len(times) // 2]})
    finally:
        check("evp_walk_persistent", eng.lib.veris_evp_walk_persistent(0))
    best = min(trials, key=lambda t: t["ms_per_subcycle"])
    eng.walk_variant = best["variant"]
    check("evp_walk_persistent", eng.lib.veris_evp_walk_persistent(int(best["persistent"])))
    eng.graph = None
    return {"variant": best["variant"], "persistent": best["persistent"], "trials": trials}


F64_TILE_ROWS = (16, 24, 32)


def tune_f64_tile(eng, rows=F64_TILE_ROWS, subcycles=10, repeats=3):
    """Pick the float64 EVP kernel's tile height (16, 24 or 32 rows of 32
    columns: 4, 3 or 2 CTAs per SM; smaller tiles keep more warps resident
    to cover the float64 pipe's latency, larger ones do less ring work) for
    a float64 ``SeaIceStep`` by timing ``subcycles`` subcycles of the
    engine's state for each (outputs to scratch: the state is not advanced).
    Sets the choice process-wide (veris_evp_f64_tile_rows) and drops the
    engine's captured graph."""
    from ._abi import check
    if eng.precision != "f64" or eng.evp_form != "fast":
        raise ValueError("tune_f64_tile: a float64 engine with the fast EVP form")
    outs = [torch.empty(eng.shape, dtype=torch.float64, device=eng.device) for _ in range(5)]
    ptrs = [t.data_ptr() for t in outs]
    ws = (eng.ws_evp.data_ptr(), eng.ws_evp.numel(), eng.stream)
    r64 = eng._refs(eng.f64)
    trials = []
    for r in rows:
        check("evp_f64_tile_rows", eng.lib.veris_evp_f64_tile_rows(r))
        run = lambda n: check("evp_fast_f64", eng.lib.veris_evp_fast_solver_f64(*r64, n, *ptrs, *ws))
        run(2)
        times = []
        for _ in range(repeats):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record()
            run(subcycles)
            b.record()
            b.synchronize()
            times.append(a.elapsed_time(b) / subcycles)
        trials.append({"rows": r, "ms_per_subcycle": sorted(times)[len(times) // 2]})
    best = min(trials, key=lambda t: t["ms_per_subcycle"])
    check("evp_f64_tile_rows", eng.lib.veris_evp_f64_tile_rows(best["rows"]))
    eng.graph = None
    return {"rows": best["rows"], "trials": trials}

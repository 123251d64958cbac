"""Loading of the golden fixtures (made by tests/golden/make_golden.py)."""
import json
import os
from types import SimpleNamespace

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ("c1", "moving", "small_a", "small_b", "noice")


def load(case):
    d = np.load(os.path.join(GOLDEN, f"{case}.npz"), allow_pickle=False)
    return {k: d[k] for k in d.files}


def initial_state(g):
    variables = {k[3:]: v.copy() for k, v in g.items() if k.startswith("in.")}
    settings = json.loads(str(g["settings"]))
    return SimpleNamespace(variables=SimpleNamespace(**variables),
                           settings=SimpleNamespace(**settings))


def sequence(g):
    """[(index, routine, {output: array})] in call order."""
    calls = {}
    for k, v in g.items():
        if k.startswith("seq."):
            _, idx, routine, out = k.split(".")
            calls.setdefault((int(idx), routine), {})[out] = v
    return [(i, r, calls[(i, r)]) for (i, r) in sorted(calls)]


def sub(g, routine):
    p = f"sub.{routine}."
    return {k[len(p):]: v for k, v in g.items() if k.startswith(p)}


def state_before(g, index):
    """The state just before call ``index`` of the recorded sequence."""
    st = initial_state(g)
    for i, _r, outs in sequence(g):
        if i >= index:
            break
        for n, a in outs.items():
            setattr(st.variables, n, a.copy())
    return st


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = np.max(np.abs(b))
    if scale == 0:
        return float(np.max(np.abs(a)))
    return float(np.max(np.abs(a - b)) / scale)


def load_forcing():
    """forcing.npz: free drift (``fd.<case>.*``) and the bulk formula (``bulk.*``)."""
    return load("forcing")


def freedrift_case(g, case):
    """(state, {uIce, vIce}) of one free-drift record of forcing.npz."""
    p = f"fd.{case}.in."
    variables = {k[len(p):]: v.copy() for k, v in g.items() if k.startswith(p)}
    settings = json.loads(str(g[f"fd.{case}.settings"]))
    st = SimpleNamespace(variables=SimpleNamespace(**variables),
                         settings=SimpleNamespace(**settings))
    return st, {n: g[f"fd.{case}.{n}"] for n in ("uIce", "vIce")}


BULK_IN = ("uw", "vw", "ta", "qa", "tsf", "ocn_mask")
BULK_OUT = ("flwupa", "flha", "fsha", "df0dT", "ust", "vst", "evp", "ssq", "dEvdT")
FREEDRIFT_CASES = ("moving", "small_b")


def bulk_case(g):
    """(settings, inputs in BULK_IN order, {output: array})."""
    settings = SimpleNamespace(**json.loads(str(g["bulk.settings"])))
    return settings, [g[f"bulk.in.{n}"] for n in BULK_IN], {n: g[f"bulk.{n}"] for n in BULK_OUT}

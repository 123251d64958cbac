"""The routines of the step as maps for the dot-product tests: inputs,
outputs and how the oracle computes them, with forward-mode derivatives
(tests/tangent.py) through the oracle.

Each case names the input fields a routine's hand-written adjoint returns
adjoints for, the output fields whose adjoints it takes, and a function that
runs the oracle's restatement of the routine on a state.  ``tangent(case,
state, dx)`` gives J dx exactly, J the routine's Jacobian at ``state``.
"""
import copy
from types import SimpleNamespace

import numpy as np

from oracle import veris_oracle as O
from tests import golden_io as G
from tests.tangent import Tangent, derivative

EVP_STATE = ("uIce", "vIce", "sigma1", "sigma2", "sigma12")
EVP_FIELDS = ("SeaIceStrength", "SeaIceMassC", "SeaIceMassU", "SeaIceMassV", "WindForcingX", "WindForcingY",
              "AreaW", "AreaS", "uOcean", "vOcean", "hIceMean", "Area")
ICE = ("hIceMean", "hSnowMean", "Area", "TSurf")
PREP_OUT = ("SeaIceStrength", "SeaIceMassC", "SeaIceMassU", "SeaIceMassV", "AreaW", "AreaS",
            "WindForcingX", "WindForcingY")


def _prep(st):
    """The dynamics preparation in the step's order, each result stored
    before the next routine reads it (seaice_global_4deg.py:879-888)."""
    v = st.variables
    v.SeaIceMassC, v.SeaIceMassU, v.SeaIceMassV = O.SeaIceMass(st)
    v.AreaW, v.AreaS = O.AreaWS(st)
    v.WindForcingX, v.WindForcingY = O.WindForcingXY(st)
    v.SeaIceStrength = O.SeaIceStrength(st)
    return {k: getattr(v, k) for k in PREP_OUT}


def _advection(st):
    return dict(zip(ICE[:3], O.Advection(st)))


def _cleanup(st):
    v = st.variables
    h, hs, A, T, _os_h, _os_hs = O.clean_up_advection(st)
    v.hIceMean, v.hSnowMean, v.Area, v.TSurf = h, hs, A, T
    return dict(hIceMean=h, hSnowMean=hs, Area=O.ridging(st), TSurf=T)


def _growth(st):
    return dict(zip(ICE, O.Growth(st)[:4]))


def _evp(n):
    def run(st):
        c = O.evp_carry(st)
        for _ in range(n):
            O.evp_subcycle(st, c)
        return {"uIce": c["u"], "vIce": c["v"], "sigma1": c["sigma1"], "sigma2": c["sigma2"],
                "sigma12": c["sigma12"]}
    return run


# case -> (routine the golden state precedes, input fields, output fields, oracle map)
CASES = {
    "prep": ("SeaIceMass", ("hIceMean", "hSnowMean", "Area", "uIce", "vIce"), PREP_OUT, _prep),
    "advection": ("Advection", ("hIceMean", "hSnowMean", "Area", "uIce", "vIce"), ICE[:3], _advection),
    "cleanup": ("clean_up_advection", ICE, ICE, _cleanup),
    "growth": ("Growth", ICE, ICE, _growth),
    "evp": ("IceVelocities", EVP_STATE + EVP_FIELDS, EVP_STATE, _evp(3)),
}


class _NumPyMaking(SimpleNamespace):
    """numpy with zeros/full making Tangent arrays (the oracle builds some
    outputs by slice assignment into fresh arrays)."""

    def __getattr__(self, name):
        return getattr(np, name)


_TANGENT_NP = _NumPyMaking(zeros=lambda *a, **k: Tangent(np.zeros(*a, **k)),
                           full=lambda *a, **k: Tangent(np.full(*a, **k)))


def golden_state(case_name, golden="moving"):
    """The reference's recorded state just before the routine of a case."""
    routine = CASES[case_name][0]
    g = G.load(golden)
    idx = [i for i, r, _o in G.sequence(g) if r == routine][0]
    return G.state_before(g, idx)


def jitter(st, rng, eps=1e-3):
    """Break exact ties (flat fields give zero limiter denominators; zero
    thicknesses sit on the clips' kinks), as the finite-difference tests do."""
    v = st.variables
    for n in ("hIceMean", "hSnowMean", "Area"):
        x = getattr(v, n)
        setattr(v, n, x + eps * rng.random(x.shape) * (x > 0))
    return st


# fields a direction may move everywhere; the others only where they are
# non-zero (a thickness, concentration, mass or strength moved off zero
# switches the step's branches: thin-ice cut-off, mass != 0 switches, clips)
SMOOTH = ("uIce", "vIce", "sigma1", "sigma2", "sigma12", "WindForcingX", "WindForcingY", "uOcean", "vOcean")


def directions(st, names, rng):
    """Random directions over the named inputs, scaled by each field's size.
    The surface temperature moves only under ice and away from the melting
    point, where the albedo switches (veris/solve4temp.py:53-79) and where
    the previous step's clamp left it exactly."""
    out = {}
    v = st.variables
    for k in names:
        x = getattr(v, k)
        scale = float(np.abs(x).max()) or 1.0
        d = rng.standard_normal(x.shape) * scale
        if k == "TSurf":
            d = d * 1e-3 * (v.hIceMean > 0) * (np.abs(x - st.settings.celsius2K) > 1e-3)
        elif k not in SMOOTH:
            d = d * (x != 0)
        out[k] = d
    return out


def evaluate(case_name, st):
    """The outputs of a case's oracle map at ``st`` (a copy is modified)."""
    st = SimpleNamespace(variables=SimpleNamespace(**dict(vars(st.variables))), settings=copy.copy(st.settings))
    return CASES[case_name][3](st)


def tangent(case_name, st, dx):
    """{output: J dx} of a case at ``st``; ``dx``: {input field: direction}."""
    v = {k: (Tangent(a, dx[k]) if k in dx else a) for k, a in vars(st.variables).items()}
    tst = SimpleNamespace(variables=SimpleNamespace(**v), settings=copy.copy(st.settings))
    saved = O.np
    O.np = _TANGENT_NP
    try:
        out = CASES[case_name][3](tst)
    finally:
        O.np = saved
    return {k: np.array(derivative(x), dtype=np.float64) if isinstance(x, Tangent) else np.zeros(np.shape(x))
            for k, x in out.items()}

"""Adjoints of the sea-ice step on the GPU (hand-written kernels).

``evp_adjoint`` is the reverse-mode derivative of the EVP subcycle loop
(veris/evp_solver.py:257-319) in float64: the adjoints of its five outputs
in, the adjoints of its five inputs, of the step-constant fields it reads and
of the water drag coefficients out.  The other routines of the step have one
function each (``fill_overlap_adjoint``, ``advection_adjoint``,
``cleanup_adjoint``, ``growth_adjoint``, ``prep_adjoint``); each takes the
state its forward read and the adjoints of its outputs.  ``trajectory``
chains them over many steps.
"""
import ctypes

import torch

from ._abi import VerisFields, check
from .state import Call

EVP_STATE = ("uIce", "vIce", "sigma1", "sigma2", "sigma12")
EVP_FIELDS = ("SeaIceStrength", "SeaIceMassC", "SeaIceMassU", "SeaIceMassV", "WindForcingX", "WindForcingY",
              "AreaW", "AreaS", "uOcean", "vOcean", "hIceMean", "Area")


def evp_adjoint(state, lam_out, n_subcycles=None, checkpoint_every=0, precision="f64", tape=False):
    """Reverse-mode derivative of ``n_subcycles`` EVP subcycles.

    ``lam_out``: {name: float64 CUDA tensor} adjoints of uIce, vIce, sigma1,
    sigma2, sigma12 after the loop (missing names count as zero).  Returns
    (adjoints of the initial state {name: tensor}, adjoints of the constant
    fields {name: tensor}, {"waterIceDrag": float tensor, "waterIceDrag_south": ...}).
    ``precision`` "f32": the float32 loop (its forward recomputed in float32,
    the state adjoints float32, returned as float64 tensors).  ``tape``: run
    the fast forward with its tape first (the float32 one is the register
    walk: cell areas varying along j only) and the adjoint on that tape.
    """
    s = state.settings
    n = int(s.nEVPsteps if n_subcycles is None else n_subcycles)
    c = Call(state)
    f32 = precision == "f32"
    dt = torch.float32 if f32 else torch.float64
    zeros = lambda d=torch.float64: torch.zeros(c.shape, dtype=d, device=c.device)
    lam = [lam_out[k].to(dt).contiguous() if k in lam_out else zeros(dt) for k in EVP_STATE]
    lo = [t.data_ptr() if f32 else c.arg(t, "lam_" + k) for k, t in zip(EVP_STATE, lam)]
    li = [zeros(dt) for _ in EVP_STATE]
    lf = {k: zeros() for k in EVP_FIELDS}
    table = VerisFields(**{k: t.data_ptr() for k, t in lf.items()})
    scal = torch.zeros(2, dtype=torch.float64, device=c.device)
    esize = 4 if f32 else 8
    if tape:
        g = c.refs()[0]
        tb = int(c.lib.veris_evp_tape_bytes(g, esize, n))
        tp = torch.empty(tb // esize, dtype=dt, device=c.device)
        outs = [torch.empty(c.shape, dtype=dt, device=c.device) for _ in EVP_STATE]
        fws, fwsb = c.workspace(c.lib.veris_evp_fast_workspace_bytes(g, esize))
        fwd = c.lib.veris_evp_fast_tape_f32 if f32 else c.lib.veris_evp_fast_tape_f64
        check("evp_tape", fwd(*c.refs(), n, *[t.data_ptr() for t in outs], tp.data_ptr(), tb, fws, fwsb, c.stream))
        ws, wsb = c.workspace(c.lib.veris_evp_adjoint_taped_workspace_bytes_f32(g, n) if f32 else
                              c.lib.veris_evp_adjoint_taped_workspace_bytes(g, n))
        fn = c.lib.veris_evp_adjoint_taped_f32 if f32 else c.lib.veris_evp_adjoint_taped_f64
        check("evp_adjoint_taped", fn(*c.refs(), n, tp.data_ptr(), tb, *lo, *[t.data_ptr() for t in li],
                                      ctypes.byref(table), scal.data_ptr(), ws, wsb, c.stream))
    else:
        wsb = c.lib.veris_evp_adjoint_workspace_bytes(c.refs()[0], esize, n, int(checkpoint_every))
        ws, wsb = c.workspace(wsb)
        fn = c.lib.veris_evp_adjoint_f32 if f32 else c.lib.veris_evp_adjoint_f64
        check("evp_adjoint", fn(*c.refs(), n, int(checkpoint_every), *lo, *[t.data_ptr() for t in li],
                                ctypes.byref(table), scal.data_ptr(), ws, wsb, c.stream))
    return (dict(zip(EVP_STATE, [t.double() for t in li])), lf,
            {"waterIceDrag": scal[0], "waterIceDrag_south": scal[1]})


ICE = ("hIceMean", "hSnowMean", "Area", "TSurf")
PREP_OUT = ("SeaIceStrength", "SeaIceMassC", "SeaIceMassU", "SeaIceMassV", "AreaW", "AreaS",
            "WindForcingX", "WindForcingY")


def fill_overlap_adjoint(state, lam):
    """Transpose of veris/fill_overlap.py:6-18 applied to ``lam``."""
    c = Call(state)
    out = c.empty()
    check("fill_overlap_adjoint", c.lib.veris_fill_overlap_adjoint_f64(
        c.refs()[0], c.refs()[1], c.arg(lam, "lam"), out.data_ptr(), c.stream))
    return out


def advection_adjoint(state, lam_out):
    """Adjoint of veris/advection.py:15-91 at ``state``.  ``lam_out``: adjoints
    of the advected (hIceMean, hSnowMean, Area).  Returns ({hIceMean,
    hSnowMean, Area: adjoint of the input}, {uIce, vIce: adjoint})."""
    c = Call(state)
    lo = [c.arg(lam_out[k], "lam_" + k) for k in ICE[:3]]
    z = lambda: torch.zeros(c.shape, dtype=torch.float64, device=c.device)
    li, lu, lv = [z() for _ in range(3)], z(), z()
    ws, wsb = c.workspace(c.lib.veris_advection_adjoint_workspace_bytes(c.refs()[0]))
    check("advection_adjoint", c.lib.veris_advection_adjoint_f64(
        *c.refs(), *lo, *[t.data_ptr() for t in li], lu.data_ptr(), lv.data_ptr(), ws, wsb, c.stream))
    return dict(zip(ICE[:3], li)), {"uIce": lu, "vIce": lv}


def _pointwise4(name, fn, state, lam_out):
    c = Call(state)
    lo = [c.arg(lam_out[k], "lam_" + k) for k in ICE]
    out = c.empty(4)
    check(name, fn(*c.refs(), *lo, *[t.data_ptr() for t in out], c.stream))
    return dict(zip(ICE, out))


def cleanup_adjoint(state, lam_out):
    """Adjoint of clean_up_advection followed by ridging (veris/clean_up.py:5-47)
    for (hIceMean, hSnowMean, Area, TSurf) at ``state``."""
    return _pointwise4("cleanup_adjoint", Call(state).lib.veris_cleanup_adjoint_f64, state, lam_out)


def growth_adjoint(state, lam_out):
    """Adjoint of Growth (veris/growth.py:8-397) for (hIceMean, hSnowMean, Area,
    TSurf) at ``state``, whose forcing fields must be the ones Growth read."""
    return _pointwise4("growth_adjoint", Call(state).lib.veris_growth_adjoint_f64, state, lam_out)


def prep_adjoint(state, lam_prep):
    """Adjoint of SeaIceMass, AreaWS, WindForcingXY and SeaIceStrength at
    ``state``.  ``lam_prep``: {name in PREP_OUT: adjoint}.  Returns
    ({hIceMean, hSnowMean, Area, uIce, vIce: adjoint},
    {pStar, airIceDrag, airIceDrag_south: 0-d tensor})."""
    c = Call(state)
    z = lambda: torch.zeros(c.shape, dtype=torch.float64, device=c.device)
    lp = {k: (lam_prep[k] if k in lam_prep else z()) for k in PREP_OUT}
    table = VerisFields(**{k: c.arg(t, "lam_" + k) for k, t in lp.items()})
    names = ("hIceMean", "hSnowMean", "Area", "uIce", "vIce")
    out = {k: z() for k in names}
    scal = torch.zeros(3, dtype=torch.float64, device=c.device)
    ws, wsb = c.workspace(c.lib.veris_prep_adjoint_workspace_bytes(c.refs()[0]))
    check("prep_adjoint", c.lib.veris_prep_adjoint_f64(
        *c.refs(), ctypes.byref(table), *[out[k].data_ptr() for k in names], scal.data_ptr(), ws, wsb,
        c.stream))
    return out, {"pStar": scal[0], "airIceDrag": scal[1], "airIceDrag_south": scal[2]}

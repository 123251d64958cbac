"""Adjoints of the sea-ice step on the GPU (hand-written kernels).

``evp_adjoint`` is the reverse-mode derivative of the EVP subcycle loop
(veris/evp_solver.py:257-319) in float64: the adjoints of its five outputs
in, the adjoints of its five inputs, of the step-constant fields it reads and
of the water drag coefficients out.
"""
import ctypes

import torch

from ._abi import VerisFields, check
from .state import Call

EVP_STATE = ("uIce", "vIce", "sigma1", "sigma2", "sigma12")
EVP_FIELDS = ("SeaIceStrength", "SeaIceMassC", "SeaIceMassU", "SeaIceMassV", "WindForcingX", "WindForcingY",
              "AreaW", "AreaS", "uOcean", "vOcean", "hIceMean", "Area")


def evp_adjoint(state, lam_out, n_subcycles=None, checkpoint_every=0):
    """Reverse-mode derivative of ``n_subcycles`` EVP subcycles.

    ``lam_out``: {name: float64 CUDA tensor} adjoints of uIce, vIce, sigma1,
    sigma2, sigma12 after the loop (missing names count as zero).  Returns
    (adjoints of the initial state {name: tensor}, adjoints of the constant
    fields {name: tensor}, {"waterIceDrag": float tensor, "waterIceDrag_south": ...}).
    """
    s = state.settings
    n = int(s.nEVPsteps if n_subcycles is None else n_subcycles)
    c = Call(state)
    zeros = lambda: torch.zeros(c.shape, dtype=torch.float64, device=c.device)
    lo = [c.arg(lam_out[k], "lam_" + k) if k in lam_out else c.arg(zeros()) for k in EVP_STATE]
    li = c.empty(5)
    lf = {k: zeros() for k in EVP_FIELDS}
    table = VerisFields(**{k: t.data_ptr() for k, t in lf.items()})
    scal = torch.zeros(2, dtype=torch.float64, device=c.device)
    wsb = c.lib.veris_evp_adjoint_workspace_bytes(c.refs()[0], 8, n, int(checkpoint_every))
    ws, wsb = c.workspace(wsb)
    check("evp_adjoint", c.lib.veris_evp_adjoint_f64(
        *c.refs(), n, int(checkpoint_every), *lo, *[t.data_ptr() for t in li], ctypes.byref(table),
        scal.data_ptr(), ws, wsb, c.stream))
    return (dict(zip(EVP_STATE, li)), lf,
            {"waterIceDrag": scal[0], "waterIceDrag_south": scal[1]})

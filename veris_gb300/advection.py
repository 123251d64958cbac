"""Drop-ins for veris/advection.py: flux-limited advection on the GPU."""
import torch

from ._abi import check
from .hostarrays import accepts_host_state
from .state import Call


@accepts_host_state
def Advection(state):
    """veris/advection.py:15-25 -> (hIceMean, hSnowMean, Area)."""
    c = Call(state)
    h, hs, A = c.empty(3)
    ws, wsb = c.workspace(c.lib.veris_advection_workspace_bytes(c.refs()[0], 8))
    check("Advection", c.lib.veris_advection_f64(*c.refs(), h.data_ptr(), hs.data_ptr(), A.data_ptr(),
                                                  ws, wsb, c.stream))
    return h, hs, A


@accepts_host_state
def calc_Advection(state, field):
    """veris/advection.py:28-91 (extensive fields) -> the advected field."""
    c = Call(state)
    out = c.empty()
    ws, wsb = c.workspace(c.lib.veris_advection_workspace_bytes(c.refs()[0], 8))
    check("calc_Advection", c.lib.veris_calc_advection_f64(*c.refs(), c.arg(field, "field"),
                                                            out.data_ptr(), ws, wsb, c.stream))
    return out


@accepts_host_state
def calc_ZonalFlux(state, field, uTrans):
    """veris/advection.py:94-129 -> the zonal flux, halo-filled."""
    c = Call(state)
    F = c.empty()
    check("calc_ZonalFlux", c.lib.veris_calc_zonal_flux_f64(
        *c.refs(), c.arg(field, "field"), c.arg(uTrans, "uTrans"), F.data_ptr(), c.stream))
    return F


@accepts_host_state
def calc_MeridionalFlux(state, field, vTrans):
    """veris/advection.py:132-167 -> the meridional flux, halo-filled."""
    c = Call(state)
    G = c.empty()
    check("calc_MeridionalFlux", c.lib.veris_calc_meridional_flux_f64(
        *c.refs(), c.arg(field, "field"), c.arg(vTrans, "vTrans"), G.data_ptr(), c.stream))
    return G


def limiter(Cr):
    """veris/advection.py:170-175: the superbee limiter, elementwise (a
    NumPy array in, a NumPy array out)."""
    from ._abi import load
    from .hostarrays import is_host_array, to_device, to_host
    if is_host_array(Cr):
        return to_host(limiter(to_device(Cr)))
    if not (isinstance(Cr, torch.Tensor) and Cr.is_cuda and Cr.dtype == torch.float64):
        raise TypeError("Cr must be a float64 CUDA tensor")
    Cr = Cr.contiguous()
    phi = torch.empty_like(Cr)
    check("limiter", load().veris_limiter_f64(Cr.data_ptr(), phi.data_ptr(), Cr.numel(),
                                              torch.cuda.current_stream(Cr.device).cuda_stream))
    return phi

"""Drop-ins for veris/dynsolver.py: air-ice stress, wind forcing, solver dispatch."""
from ._abi import check
from .state import Call
from .evp_solver import evp_solver


def tauXY(state):
    """veris/dynsolver.py:7-47 -> (tauX, tauY) at U and V points."""
    c = Call(state)
    tX, tY = c.empty(2)
    check("tauXY", c.lib.veris_tau_xy_f64(*c.refs(), tX.data_ptr(), tY.data_ptr(), c.stream))
    return tX, tY


def WindForcingXY(state):
    """veris/dynsolver.py:50-84 -> (WindForcingX, WindForcingY)."""
    c = Call(state)
    fx, fy = c.empty(2)
    check("WindForcingXY", c.lib.veris_wind_forcing_xy_f64(*c.refs(), fx.data_ptr(), fy.data_ptr(),
                                                             c.stream))
    return fx, fy


def IceVelocities(state):
    """veris/dynsolver.py:87-102 -> (uIce, vIce, sigma1, sigma2, sigma12).

    The free-drift branch of the reference is not selectable: it reads an
    undefined name (veris/dynsolver.py:95) and is not part of the step.
    """
    if state.settings.useFreedrift and not state.settings.useEVP:
        raise NotImplementedError("free drift is not part of the GPU step")
    return evp_solver(state)

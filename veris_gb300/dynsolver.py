"""Drop-ins for veris/dynsolver.py: air-ice stress, wind forcing, solver dispatch."""
from ._abi import check
from .hostarrays import accepts_host_state
from .state import Call
from .evp_solver import evp_solver
from .freedrift_solver import freedrift_solver


@accepts_host_state
def tauXY(state):
    """veris/dynsolver.py:7-47 -> (tauX, tauY) at U and V points."""
    c = Call(state)
    tX, tY = c.empty(2)
    check("tauXY", c.lib.veris_tau_xy_f64(*c.refs(), tX.data_ptr(), tY.data_ptr(), c.stream))
    return tX, tY


@accepts_host_state
def WindForcingXY(state):
    """veris/dynsolver.py:50-84 -> (WindForcingX, WindForcingY)."""
    c = Call(state)
    fx, fy = c.empty(2)
    check("WindForcingXY", c.lib.veris_wind_forcing_xy_f64(*c.refs(), fx.data_ptr(), fy.data_ptr(),
                                                             c.stream))
    return fx, fy


@accepts_host_state
def IceVelocities(state):
    """veris/dynsolver.py:87-102 -> (uIce, vIce, sigma1, sigma2, sigma12).

    ``useFreedrift``: the free-drift velocities with the stresses as they
    are (the reference's branch means this but reads an unbound name,
    veris/dynsolver.py:95-97); ``useEVP`` (checked second, so it wins when
    both are set, as in the reference): the EVP loop.
    """
    s = state.settings
    if s.useEVP:
        return evp_solver(state)
    if s.useFreedrift:
        u, v = freedrift_solver(state)
        vs = state.variables
        return u, v, vs.sigma1.clone(), vs.sigma2.clone(), vs.sigma12.clone()
    raise ValueError("IceVelocities: neither useEVP nor useFreedrift is set")

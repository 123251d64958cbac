"""Drop-in for veris/growth.py: thermodynamic growth and ocean budgets in float64."""
from ._abi import check
from .hostarrays import accepts_host_state
from .state import Call


@accepts_host_state
def Growth(state):
    """veris/growth.py:8-397 -> (hIceMean, hSnowMean, Area, TSurf, EmPmR,
    forc_salt_surface, Qsw, Qnet, SeaIceLoad, IcePenetSW, recip_hIceMean)."""
    c = Call(state)
    out = c.empty(11)
    check("Growth", c.lib.veris_growth_f64(*c.refs(), *[t.data_ptr() for t in out], c.stream))
    return tuple(out)

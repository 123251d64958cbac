"""Drop-ins for veris/clean_up.py."""
from ._abi import check
from .hostarrays import accepts_host_state
from .state import Call


@accepts_host_state
def clean_up_advection(state):
    """veris/clean_up.py:5-39 -> (hIceMean, hSnowMean, Area, TSurf, os_hIceMean, os_hSnowMean)."""
    c = Call(state)
    out = c.empty(6)
    check("clean_up_advection", c.lib.veris_clean_up_advection_f64(
        *c.refs(), *[t.data_ptr() for t in out], c.stream))
    return tuple(out)


@accepts_host_state
def ridging(state):
    """veris/clean_up.py:42-47 -> Area capped at 1."""
    c = Call(state)
    A = c.empty()
    check("ridging", c.lib.veris_ridging_f64(*c.refs(), A.data_ptr(), c.stream))
    return A

"""Drop-in for veris/solve4temp.py: the float64 surface-temperature Newton solve."""
from ._abi import check
from .hostarrays import accepts_host_state
from .state import Call


@accepts_host_state
def solve4temp(state, hIceActual, hSnowActual, TSurfIn, TempFrz):
    """veris/solve4temp.py:5-174 -> (TSurfOut, F_io_net, F_ia_net, IcePenetSW, FWsublim)."""
    c = Call(state)
    out = c.empty(5)
    check("solve4temp", c.lib.veris_solve4temp_f64(
        *c.refs(), c.arg(hIceActual, "hIceActual"), c.arg(hSnowActual, "hSnowActual"),
        c.arg(TSurfIn, "TSurfIn"), c.arg(TempFrz, "TempFrz"), *[t.data_ptr() for t in out],
        c.stream))
    return tuple(out)

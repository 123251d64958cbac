"""Drop-in for veris/averaging.py."""
from ._abi import check
from .hostarrays import accepts_host_state
from .state import Call


@accepts_host_state
def c_point_to_z_point(state, Cfield, noSlip=True):
    """veris/averaging.py:4-19 -> the field averaged to Z points."""
    c = Call(state)
    Z = c.empty()
    check("c_point_to_z_point", c.lib.veris_c_point_to_z_point_f64(
        *c.refs(), c.arg(Cfield, "Cfield"), int(bool(noSlip)), Z.data_ptr(), c.stream))
    return Z

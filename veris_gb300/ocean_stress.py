"""Drop-in for veris/ocean_stress.py."""
from ._abi import check
from .hostarrays import accepts_host_state
from .state import Call


@accepts_host_state
def OceanStressUV(state):
    """veris/ocean_stress.py:8-40 -> (OceanStressU, OceanStressV), halo-filled."""
    c = Call(state)
    su, sv = c.empty(2)
    check("OceanStressUV", c.lib.veris_ocean_stress_uv_f64(*c.refs(), su.data_ptr(), sv.data_ptr(),
                                                             c.stream))
    return su, sv

"""Drop-ins for veris/area_mass.py: ice mass and concentration at U/V points."""
from ._abi import check
from .hostarrays import accepts_host_state
from .state import Call


@accepts_host_state
def AreaWS(state):
    """veris/area_mass.py:5-14 -> (AreaW, AreaS)."""
    c = Call(state)
    AW, AS = c.empty(2)
    check("AreaWS", c.lib.veris_area_ws_f64(*c.refs(), AW.data_ptr(), AS.data_ptr(), c.stream))
    return AW, AS


@accepts_host_state
def SeaIceMass(state):
    """veris/area_mass.py:17-28 -> (SeaIceMassC, SeaIceMassU, SeaIceMassV)."""
    c = Call(state)
    mC, mU, mV = c.empty(3)
    check("SeaIceMass", c.lib.veris_sea_ice_mass_f64(*c.refs(), mC.data_ptr(), mU.data_ptr(),
                                                       mV.data_ptr(), c.stream))
    return mC, mU, mV

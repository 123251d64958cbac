"""Drop-ins for veris/dynamics_routines.py: ice strength, drag coefficients,
strain rates, viscosities and stress divergence."""
from ._abi import check
from .hostarrays import accepts_host_state
from .state import Call


@accepts_host_state
def SeaIceStrength(state):
    """veris/dynamics_routines.py:5-18 -> SeaIceStrength."""
    c = Call(state)
    P = c.empty()
    check("SeaIceStrength", c.lib.veris_sea_ice_strength_f64(*c.refs(), P.data_ptr(), c.stream))
    return P


@accepts_host_state
def ocean_drag_coeffs(state, uIce, vIce):
    """veris/dynamics_routines.py:21-52 -> cDrag at C points."""
    c = Call(state)
    cd = c.empty()
    check("ocean_drag_coeffs", c.lib.veris_ocean_drag_coeffs_f64(
        *c.refs(), c.arg(uIce, "uIce"), c.arg(vIce, "vIce"), cd.data_ptr(), c.stream))
    return cd


@accepts_host_state
def basal_drag_coeffs(state, uIce, vIce):
    """veris/dynamics_routines.py:55-96 -> cBot at C points."""
    c = Call(state)
    cb = c.empty()
    check("basal_drag_coeffs", c.lib.veris_basal_drag_coeffs_f64(
        *c.refs(), c.arg(uIce, "uIce"), c.arg(vIce, "vIce"), cb.data_ptr(), c.stream))
    return cb


@accepts_host_state
def side_drag(state, uIce, vIce):
    """veris/dynamics_routines.py:99-140 -> (SideDragU, SideDragV)."""
    c = Call(state)
    sU, sV = c.empty(2)
    check("side_drag", c.lib.veris_side_drag_f64(
        *c.refs(), c.arg(uIce, "uIce"), c.arg(vIce, "vIce"), sU.data_ptr(), sV.data_ptr(), c.stream))
    return sU, sV


@accepts_host_state
def strainrates(state, uIce, vIce):
    """veris/dynamics_routines.py:143-217 -> (e11, e22, e12)."""
    c = Call(state)
    e11, e22, e12 = c.empty(3)
    check("strainrates", c.lib.veris_strainrates_f64(
        *c.refs(), c.arg(uIce, "uIce"), c.arg(vIce, "vIce"), e11.data_ptr(), e22.data_ptr(),
        e12.data_ptr(), c.stream))
    return e11, e22, e12


@accepts_host_state
def viscosities(state, e11, e22, e12):
    """veris/dynamics_routines.py:220-268 -> (zeta, eta, press)."""
    c = Call(state)
    zeta, eta, press = c.empty(3)
    check("viscosities", c.lib.veris_viscosities_f64(
        *c.refs(), c.arg(e11, "e11"), c.arg(e22, "e22"), c.arg(e12, "e12"), zeta.data_ptr(),
        eta.data_ptr(), press.data_ptr(), c.stream))
    return zeta, eta, press


@accepts_host_state
def stressdiv(state, sig11, sig22, sig12):
    """veris/dynamics_routines.py:284-303 -> (stressDivX, stressDivY)."""
    c = Call(state)
    dX, dY = c.empty(2)
    check("stressdiv", c.lib.veris_stressdiv_f64(
        *c.refs(), c.arg(sig11, "sig11"), c.arg(sig22, "sig22"), c.arg(sig12, "sig12"),
        dX.data_ptr(), dY.data_ptr(), c.stream))
    return dX, dY

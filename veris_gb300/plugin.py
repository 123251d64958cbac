"""The host model's plugin interface (veris/__init__.py:17-23).

Veros loads a plugin by importing it and reading its ``__VEROS_INTERFACE__``:
a name, a setup entry point run once after the host model's grid exists, a
run entry point called every step, and the plugin's settings and variables
tables.  ``veris_gb300`` exports the same dictionary, so a setup that lists
the plugin gets this package's settings and variables (same names and
defaults, veris/settings.py:4-176, veris/variables.py:4-106), its
``set_inits`` and its no-op ``model``; the setup's step then calls the
routines of ``veris_gb300.<module>`` where it called ``veris.<module>``
(veris/setup/seaice_global_4deg/seaice_global_4deg.py:9-16, 878-932).

When Veros is importable the tables hold its own ``Setting`` and
``Variable`` objects; otherwise stand-ins with the same fields.
"""
import numpy as np

from .model import model
from .settings import SETTINGS as _SETTING_TABLE
from .variables import ALL, DERIVED, FORCING, GRID, MASKS, PROGNOSTIC

try:   # the host model's own descriptor classes when it is installed
    from veros.settings import Setting
    from veros.variables import Variable
except Exception:   # noqa: BLE001
    class Setting:
        """A plugin setting: default value, type and description."""

        def __init__(self, default, type, description=""):
            self.default = default
            self.type = type
            self.description = description

    class Variable:
        """A plugin variable: description, grid dimensions and units."""

        def __init__(self, name, dims, units="", long_description="", **kwargs):
            self.name = name
            self.dims = dims
            self.units = units
            self.long_description = long_description


SETTINGS = {name: Setting(default, typ, meaning) for name, (default, typ, meaning) in _SETTING_TABLE.items()}

_GRID_DIMS = ("xt", "yt")
_UNITS = dict(hIceMean="m", hSnowMean="m", Area=" ", TSurf="K", uIce="m/s", vIce="m/s",
              sigma1="N/m2", sigma2="N/m2", sigma12="N/m2", SeaIceMassC="kg", SeaIceMassU="kg",
              SeaIceMassV="kg", SeaIceStrength="N/m", AreaW=" ", AreaS=" ", WindForcingX="N",
              WindForcingY="N", os_hIceMean="m", os_hSnowMean="m", recip_hIceMean="1/m",
              SeaIceLoad="kg/m2", IcePenetSW="W/m2", OceanStressU="N/m2", OceanStressV="N/m2",
              forc_salt_surface_ice="g/(m2 s)", uOcean="m/s", vOcean="m/s", theta="K", ocSalt="g/kg",
              Qnet="W/m2", Qsw="W/m2", ssh_an="m", R_low="m", uWind="m/s", vWind="m/s", wSpeed="m/s",
              surfPress="Pa", SWdown="W/m2", LWdown="W/m2", ATemp="K", aqh="kg/kg", precip="m/s",
              snowfall="m/s", evap="m/s", runoff="m/s", EmPmR="kg/(m2 s)", saltflux="g/(m2 s)",
              fCori="1/s", rA="m2", rAu="m2", rAv="m2", rAz="m2", recip_rA="1/m2", recip_rAu="1/m2",
              recip_rAv="1/m2", recip_rAz="1/m2")
for _n in ("dxC", "dyC", "dxG", "dyG", "dxU", "dyU", "dxV", "dyV"):
    _UNITS[_n] = "m"
    _UNITS["recip_" + _n] = "1/m"


def _describe(name):
    for group, what in ((PROGNOSTIC, "prognostic sea-ice state"), (DERIVED, "derived each step"),
                        (FORCING, "ocean or atmosphere forcing"), (MASKS, "land-sea mask"),
                        (GRID, "grid metric")):
        if name in group:
            return f"{name} ({what})"
    return name


VARIABLES = {name: Variable(_describe(name), _GRID_DIMS, _UNITS.get(name, " ")) for name in ALL}


def set_inits(state):
    """veris/set_inits.py:6-59: the masks and grid metrics of the sea-ice
    variables from the host model's grid (maskT/U/V at the surface level,
    ht, coriolis_t, dxt, dyt, dxu, dyu, area_t/u/v), and TSurf = 273 K.

    Computed once, on the GPU; the results take the array type of the
    state's grid variables (NumPy arrays for a NumPy host model)."""
    import torch
    from .hostarrays import _device, is_host_array
    vs = state.variables
    host = is_host_array(vs.maskT)
    dev = _device()

    def dv(a):
        return (torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64)).to(dev) if is_host_array(a)
                else a.to(device=dev, dtype=torch.float64))

    surface = lambda m: dv(m)[:, :, -1]
    out = {}
    out["iceMask"], out["iceMaskU"], out["iceMaskV"] = surface(vs.maskT), surface(vs.maskU), surface(vs.maskV)
    out["maskInC"], out["maskInU"], out["maskInV"] = out["iceMask"], out["iceMaskU"], out["iceMaskV"]
    out["R_low"] = dv(vs.ht)
    out["fCori"] = dv(vs.coriolis_t)
    ones = torch.ones_like(out["maskInC"])
    out["dxC"] = ones * dv(vs.dxt)[:, None]
    out["dyC"] = ones * dv(vs.dyt)
    out["dxU"] = ones * dv(vs.dxu)[:, None]
    out["dyU"] = ones * dv(vs.dyu)
    out["dxG"] = 0.5 * (out["dxU"] + torch.roll(out["dxU"], 1, 1))
    out["dyG"] = 0.5 * (out["dyU"] + torch.roll(out["dyU"], 1, 0))
    out["dxV"] = 0.5 * (out["dxC"] + torch.roll(out["dxC"], 1, 1))
    out["dyV"] = 0.5 * (out["dyC"] + torch.roll(out["dyC"], 1, 0))
    out["rA"], out["rAu"], out["rAv"] = dv(vs.area_t), dv(vs.area_u), dv(vs.area_v)
    out["rAz"] = 0.25 * torch.roll(out["rA"] + torch.roll(out["rA"], 1, 0), 1, 1)
    for n in ("dxC", "dyC", "dxG", "dyG", "dxU", "dyU", "dxV", "dyV", "rA", "rAu", "rAv", "rAz"):
        out["recip_" + n] = 1 / out[n]
    out["TSurf"] = ones * 273
    for name, t in out.items():
        setattr(vs, name, t.cpu().numpy() if host else t.contiguous())
    return state


__VEROS_INTERFACE__ = dict(
    name="veris",
    setup_entrypoint=set_inits,
    run_entrypoint=model,
    settings=SETTINGS,
    variables=VARIABLES,
)

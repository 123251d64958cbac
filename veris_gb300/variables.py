"""Names of the 2-D state variables of the sea-ice step.

Every variable is a 2-D ``(nx + 2*olx, ny + 2*oly)`` array, C order, axis 0 =
x, so y is the contiguous axis.  The names are the plugin's variable table
(veris/variables.py:4-106); the grouping below is this package's own and
drives which fields the C ABI's ``VerisFields`` struct carries.
"""

# prognostic ice state
PROGNOSTIC = (
    "hIceMean", "hSnowMean", "Area", "TSurf",
    "uIce", "vIce", "sigma1", "sigma2", "sigma12",
)

# derived each step by the dynamics preparation
DERIVED = (
    "SeaIceMassC", "SeaIceMassU", "SeaIceMassV", "SeaIceStrength",
    "AreaW", "AreaS", "WindForcingX", "WindForcingY",
    "os_hIceMean", "os_hSnowMean", "recip_hIceMean", "SeaIceLoad", "IcePenetSW",
    "OceanStressU", "OceanStressV", "forc_salt_surface_ice",
)

# ocean and atmosphere forcing
FORCING = (
    "uOcean", "vOcean", "theta", "ocSalt", "Qnet", "Qsw", "ssh_an", "R_low",
    "uWind", "vWind", "wSpeed", "surfPress", "SWdown", "LWdown", "ATemp", "aqh",
    "precip", "snowfall", "evap", "runoff", "EmPmR", "saltflux",
)

MASKS = ("maskInC", "maskInU", "maskInV", "iceMask", "iceMaskU", "iceMaskV")

GRID = (
    "k1AtC", "k2AtC", "k1AtZ", "k2AtZ", "Fu", "Fv", "fCori",
    "dxC", "dyC", "dxG", "dyG", "dxU", "dyU", "dxV", "dyV",
    "recip_dxC", "recip_dyC", "recip_dxG", "recip_dyG",
    "recip_dxU", "recip_dyU", "recip_dxV", "recip_dyV",
    "rA", "rAu", "rAv", "rAz", "recip_rA", "recip_rAu", "recip_rAv", "recip_rAz",
)

ALL = PROGNOSTIC + DERIVED + FORCING + MASKS + GRID

# The order of the pointer members of the C struct ``VerisFields``
# (include/veris_gb300.h).  Changing it changes the ABI.
ABI_ORDER = ALL

"""Scalar settings of the sea-ice step.

The names and default values are the plugin's settings table
(veris/settings.py:4-176); the kernels read them through the flat
``VerisParams`` struct that ``veris_gb300._abi.params_from_settings`` packs.
Only the settings the sea-ice step reads are listed; the bulk-forcing
constants of the reference (veris/settings.py:144-175) belong to the
atmosphere/ocean flux formulas that run before the step and are not part of
this package.
"""
from types import SimpleNamespace

# name -> (default, python type, meaning)
SETTINGS = dict(
    deltatTherm=(86400.0, float, "time step of the thermodynamics and advection [s]"),
    recip_deltatTherm=(1 / 86400, float, "1 / deltatTherm [1/s]"),
    deltatDyn=(86400.0, float, "time step of the dynamics [s]"),
    recip_deltatDyn=(1 / 86400, float, "1 / deltatDyn [1/s]"),
    olx=(2, int, "halo width in x"),
    oly=(2, int, "halo width in y"),
    gridcellWidth=(444709.893408, float, "grid cell width [m]"),
    nITC=(5, int, "number of ice thickness categories"),
    recip_nITC=(1 / 5, float, "1 / nITC"),
    noSlip=(True, bool, "no-slip lateral boundary condition"),
    useRelativeWind=(True, bool, "wind stress from the wind-ice velocity difference"),
    secondOrderBC=(False, bool, "second-order no-slip boundary terms"),
    extensiveFld=(True, bool, "advected fields are extensive"),
    useRealFreshWaterFlux=(False, bool, "sea-ice load enters the surface tilt"),
    useFreedrift=(False, bool, "use the free-drift solver"),
    useEVP=(True, bool, "use the EVP solver"),
    evpAlpha=(500.0, float, "mEVP stress relaxation parameter"),
    evpBeta=(500.0, float, "mEVP momentum relaxation parameter"),
    useAdaptiveEVP=(False, bool, "adaptive relaxation parameters (aEVP)"),
    aEVPalphaMin=(5.0, float, "lower limit of the adaptive alpha"),
    aEvpCoeff=(0.5, float, "largest stabilised frequency of the aEVP"),
    explicitDrag=(True, bool, "explicit or implicit drag (unused by the step)"),
    nEVPsteps=(400, int, "number of EVP subcycles per step"),
    computeEvpResidual=(False, bool, "EVP residual diagnostics"),
    veros_fill=(True, bool, "halo fill through the host model's cyclic-x copy"),
    use_coastline=(False, bool, "coastline form factor for the side drag"),
    enable_cyclic_x=(True, bool, "domain is periodic in x (host model setting)"),
    rhoIce=(900.0, float, "ice density [kg/m3]"),
    rhoFresh=(1000.0, float, "fresh water density [kg/m3]"),
    rhoSea=(1026.0, float, "sea water density [kg/m3]"),
    rhoAir=(1.3, float, "air density [kg/m3]"),
    rhoSnow=(330.0, float, "snow density [kg/m3]"),
    recip_rhoFresh=(1 / 1000, float, "1 / rhoFresh"),
    recip_rhoSea=(1 / 1026, float, "1 / rhoSea"),
    rhoIce2rhoSnow=(900 / 330, float, "rhoIce / rhoSnow"),
    rhoIce2rhoFresh=(900 / 1000, float, "rhoIce / rhoFresh"),
    rhoFresh2rhoSnow=(1000 / 330, float, "rhoFresh / rhoSnow"),
    dryIceAlb=(0.75, float, "dry ice albedo"),
    dryIceAlb_south=(0.75, float, "dry ice albedo, southern hemisphere"),
    wetIceAlb=(0.66, float, "wet ice albedo"),
    wetIceAlb_south=(0.66, float, "wet ice albedo, southern hemisphere"),
    drySnowAlb=(0.84, float, "dry snow albedo"),
    drySnowAlb_south=(0.84, float, "dry snow albedo, southern hemisphere"),
    wetSnowAlb=(0.7, float, "wet snow albedo"),
    wetSnowAlb_south=(0.7, float, "wet snow albedo, southern hemisphere"),
    wetAlbTemp=(0.0, float, "temperature above which wet albedos apply [degC]"),
    lhFusion=(3.34e5, float, "latent heat of fusion [J/kg]"),
    lhEvap=(2.5e6, float, "latent heat of evaporation [J/kg]"),
    lhSublim=(3.34e5 + 2.5e6, float, "latent heat of sublimation [J/kg]"),
    cpAir=(1005.0, float, "heat capacity of air [J/kg K]"),
    cpWater=(3986.0, float, "heat capacity of water [J/kg K]"),
    stefBoltz=(5.67e-8, float, "Stefan-Boltzmann constant"),
    iceEmiss=(0.95, float, "ice long-wave emissivity"),
    snowEmiss=(0.95, float, "snow long-wave emissivity"),
    iceConduct=(2.1656, float, "ice conductivity"),
    snowConduct=(0.31, float, "snow conductivity"),
    hCut=(0.15, float, "snow thickness above which snow is opaque [m]"),
    shortwave=(0.3, float, "short-wave ice penetration factor"),
    tempFrz=(-1.96, float, "freezing temperature [degC]"),
    dtempFrz_dS=(0.0, float, "d(freezing temperature)/d(salinity)"),
    saltIce_ref=(0.0, float, "reference ice salinity [g/kg]"),
    saltOcn_ref=(34.7, float, "reference ocean salinity [g/kg]"),
    minLWdown=(60.0, float, "minimum downward long-wave radiation"),
    maxTIce=(30.0, float, "maximum ice temperature"),
    minTIce=(-50.0, float, "minimum ice temperature [degC]"),
    minTAir=(-50.0, float, "minimum air temperature [degC]"),
    dalton=(0.00175, float, "Dalton number"),
    Area_reg=(0.15 ** 2, float, "regularisation of the ice concentration"),
    hIce_reg=(0.10 ** 2, float, "regularisation of the ice thickness"),
    celsius2K=(273.15, float, "0 degC in K"),
    stantonNr=(0.0056, float, "Stanton number"),
    uStarBase=(0.0125, float, "friction velocity beneath the ice [m/s]"),
    McPheeTaperFac=(12.5, float, "tapering factor at the ice bottom"),
    h0=(0.5, float, "lead closing parameter"),
    recip_h0=(1 / 0.5, float, "1 / h0"),
    h0_south=(0.5, float, "lead closing parameter, southern hemisphere"),
    recip_h0_south=(1 / 0.5, float, "1 / h0_south"),
    airTurnAngle=(0.0, float, "air-ice stress turning angle [deg]"),
    waterTurnAngle=(0.0, float, "water-ice stress turning angle [deg]"),
    sinWat=(0.0, float, "sin(waterTurnAngle)"),
    cosWat=(1.0, float, "cos(waterTurnAngle)"),
    wSpeedMin=(1e-10, float, "minimum wind speed [m/s]"),
    hIce_min=(1e-5, float, "minimum ice thickness [m]"),
    Area_min=(1e-5, float, "minimum ice concentration"),
    airIceDrag=(0.0012, float, "air-ice drag coefficient"),
    airIceDrag_south=(0.0012, float, "air-ice drag coefficient, southern hemisphere"),
    waterIceDrag=(0.0055, float, "water-ice drag coefficient"),
    waterIceDrag_south=(0.0055, float, "water-ice drag coefficient, southern hemisphere"),
    cDragMin=(0.25, float, "minimum linear ice-ocean drag coefficient"),
    seaIceLoadFac=(1.0, float, "sea-ice load scale factor"),
    gravity=(9.81, float, "gravitational acceleration"),
    PlasDefCoeff=(2.0, float, "axis ratio e of the elliptical yield curve"),
    deltaMin=(2e-9, float, "minimum of Delta"),
    pressReplFac=(1, int, "replacement pressure switch"),
    pStar=(27.5e3, float, "ice strength parameter P* [N/m2]"),
    cStar=(20.0, float, "ice strength parameter C*"),
    basalDragU0=(5e-5, float, "basal drag velocity parameter"),
    basalDragK1=(8.0, float, "basal drag parameter K1"),
    basalDragK2=(0.0, float, "basal drag parameter K2"),
    cBasalStar=(20.0, float, "basal drag parameter C_b"),
    tensileStrFac=(0.0, float, "tensile strength factor"),
    CrMax=(1e6, float, "slope-ratio bound of the flux limiter"),
    sideDragCoeff=(0.001, float, "side drag coefficient"),
    sideDragU0=(0.01, float, "side drag velocity [m/s]"),
    # bulk formulae over open ocean (veris/settings.py:156-173, veris/heat_flux_MITgcm.py)
    zvir=(0.608, float, "dry-air / water-vapour molecular mass ratio term"),
    cpdair=(1.00464e3, float, "specific heat of dry air [J/K/kg]"),
    karman=(0.4, float, "von Karman constant"),
    latvap=(2.501e6, float, "latent heat of evaporation [J/kg]"),
    ocean_emissivity=(0.985, float, "ocean surface emissivity"),
    gamma_blk=(0.010, float, "adiabatic lapse rate [K/m]"),
    grav=(9.81, float, "gravitational acceleration of the host model (bulk formulae)"),
    # the rest of the plugin's forcing table (veris/settings.py:144-175): read
    # by the host model's setup and by the bulk formulae that run before the
    # step (the CESM ones are not part of this package); listed so that a
    # setup finds every setting it knows
    umin_o=(0.5, float, "minimum wind speed over the ocean [m/s]"),
    umin_i=(1.0, float, "minimum wind speed over ice [m/s]"),
    zref=(10.0, float, "reference height of the wind [m]"),
    ztref=(2.0, float, "reference height of the air temperature [m]"),
    bolzc=(1.38065e-23, float, "Boltzmann constant [J/K/molecule]"),
    avogad=(6.02214e26, float, "Avogadro number [molecules/kmole]"),
    rgas=(8314.47, float, "ideal gas constant [J/K/kmole]"),
    mwdair=(28.966, float, "molecular weight of dry air [kg/kmole]"),
    mwwv=(18.016, float, "molecular weight of water vapour [kg/kmole]"),
    rdair=(287.042, float, "gas constant of dry air [J/K/kg]"),
    rwv=(461.505, float, "gas constant of water vapour [J/K/kg]"),
    cpwv=(1.810e3, float, "specific heat of water vapour [J/K/kg]"),
    cpvir=(0.802, float, "specific-heat ratio term"),
    p0=(1e5, float, "reference pressure of the potential temperature [Pa]"),
    cappa=(0.286, float, "R / cp"),
    zzsice=(0.0005, float, "ice surface roughness [m]"),
    ch=(1e-3, float, "bulk transfer coefficient of sensible heat"),
    ce=(1.15e-3, float, "bulk transfer coefficient of latent heat"),
    eps2=(1e-20, float, "threshold"),
    emissivity=(1.0, float, "surface emissivity"),
    snow_emissivity=(0.98, float, "snow surface emissivity"),
    ice_emissivity=(0.98, float, "ice surface emissivity"),
    tf0kel=(273.15, float, "freezing temperature of fresh water [K]"),
    ocean_albedo=(0.1, float, "ocean albedo"),
    ice_albedo=(0.7, float, "ice albedo"),
)


def default_settings(**overrides):
    """A settings namespace with the defaults above and ``overrides`` applied.

    Unknown names raise ``KeyError`` so that a typo never silently keeps a
    default.  Reciprocal pairs (``recip_deltatDyn`` and friends) are NOT
    derived automatically, as in the host model: set both.
    """
    values = {k: v[0] for k, v in SETTINGS.items()}
    for k, v in overrides.items():
        if k not in SETTINGS:
            raise KeyError(f"unknown sea-ice setting {k!r}")
        values[k] = v
    return SimpleNamespace(**values)


def with_timesteps(sett, dt_dyn, dt_therm=None, n_evp=None):
    """Set the dynamic/thermodynamic time steps and their reciprocals."""
    dt_therm = dt_dyn if dt_therm is None else dt_therm
    sett.deltatDyn = float(dt_dyn)
    sett.recip_deltatDyn = 1.0 / float(dt_dyn)
    sett.deltatTherm = float(dt_therm)
    sett.recip_deltatTherm = 1.0 / float(dt_therm)
    if n_evp is not None:
        sett.nEVPsteps = int(n_evp)
    return sett

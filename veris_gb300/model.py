"""The sea-ice step, drop-in form.

``model(state)`` is the plugin's run entry point, a no-op as in the reference
(veris/model.py:1-9): the host model's setup drives the step.  ``step(state)``
is that setup's sea-ice section (veris/setup/seaice_global_4deg/
seaice_global_4deg.py:878-932) over the GPU drop-ins, in the same order, with
two deliberate differences from the published setup:

* all five results of ``IceVelocities`` are stored (the setup unpacks two of
  five at :891, which raises in the reference);
* the stresses sigma1, sigma2, sigma12 are stored back into the state, so the
  next step's EVP starts from them.
"""
from . import area_mass, dynsolver, dynamics_routines, ocean_stress, advection, clean_up, growth
from .fill_overlap import fill_overlap


def model(state):
    """veris/model.py:1-9: the plugin's run entry point does nothing."""
    return None


STEP = (
    ("SeaIceMass", area_mass.SeaIceMass, ("SeaIceMassC", "SeaIceMassU", "SeaIceMassV")),
    ("AreaWS", area_mass.AreaWS, ("AreaW", "AreaS")),
    ("WindForcingXY", dynsolver.WindForcingXY, ("WindForcingX", "WindForcingY")),
    ("SeaIceStrength", dynamics_routines.SeaIceStrength, ("SeaIceStrength",)),
    ("IceVelocities", dynsolver.IceVelocities, ("uIce", "vIce", "sigma1", "sigma2", "sigma12")),
    ("OceanStressUV", ocean_stress.OceanStressUV, ("OceanStressU", "OceanStressV")),
    ("Advection", advection.Advection, ("hIceMean", "hSnowMean", "Area")),
    ("clean_up_advection", clean_up.clean_up_advection,
     ("hIceMean", "hSnowMean", "Area", "TSurf", "os_hIceMean", "os_hSnowMean")),
    ("ridging", clean_up.ridging, ("Area",)),
    ("Growth", growth.Growth, ("hIceMean", "hSnowMean", "Area", "TSurf", "EmPmR",
                               "forc_salt_surface_ice", "Qsw", "Qnet", "SeaIceLoad", "IcePenetSW",
                               "recip_hIceMean")),
)
FILLED_AFTER_GROWTH = ("hIceMean", "hSnowMean", "Area", "forc_salt_surface_ice", "Qnet")


def step(state, record=None):
    """One sea-ice step on the GPU, float64 throughout (the drop-in path).

    ``record(name, {output: tensor})`` is called after every routine.
    """
    v = state.variables
    for name, fn, outs in STEP:
        vals = fn(state)
        if not isinstance(vals, tuple):
            vals = (vals,)
        if record is not None:
            record(name, dict(zip(outs, vals)))
        for n, x in zip(outs, vals):
            setattr(v, n, x)
    for n in FILLED_AFTER_GROWTH:
        x = fill_overlap(state, getattr(v, n).clone())
        if record is not None:
            record("fill_overlap", {n: x})
        setattr(v, n, x)
    return state

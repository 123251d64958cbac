"""Seeded synthetic sea-ice states for the benchmark and test workloads.

The host model's setup reads ERA5/ECMWF forcing files; these generators stand
in for them with fields of the same kind, shapes and value ranges:

* lat-lon grid over latitudes -80..80, periodic in x, 2-cell halos;
* land mask: smoothed seeded Gaussian noise thresholded to 25 % land;
* hIceMean lognormal with mean 1.5 m and log-sigma 0.5 where |lat| > 55 deg,
  else 0; Area = min(1, hIceMean/0.5) * U(0.8, 1); hSnowMean = 0.2 hIceMean;
* winds N(0, 8 m/s) smoothed with a 3-cell Gaussian (rescaled back to a
  standard deviation of 8 m/s), ocean currents N(0, 0.1 m/s) smoothed;
* SST -1.8 degC under ice, else U(0, 10) degC; air temperature U(-25, 0) degC;
  short-wave U(0, 300) W/m2; long-wave 250 W/m2;
* P* = 27500 N/m2, C* = 20, e = 2.

Fields the workload description leaves open (humidity, precipitation,
evaporation, salinity, sea-surface height, surface pressure, ocean heat loss,
depth) get plausible seeded values documented inline.

All arrays are float64 numpy arrays of shape (nx + 4, ny + 4).
"""
import numpy as np

from .grid import host_grid, velocity_masks, derive_grid_variables, fill_cyclic_x
from .settings import default_settings, with_timesteps

# The five workloads: (nx, ny, subcycles, steps, dt [s])
CONFIGS = {
    "c1_4deg": dict(nx=90, ny=40, n_evp=120, steps=1, dt=3600.0),
    "c2_quarterdeg": dict(nx=1440, ny=720, n_evp=500, steps=10, dt=1800.0),
    "c3_1deg": dict(nx=360, ny=180, n_evp=300, steps=48, dt=3600.0),
    "c4_ensemble": dict(members=512, n_evp=100, steps=20, dt=3600.0),
    "c5_tenthdeg": dict(nx=3600, ny=1800, n_evp=500, steps=24, dt=600.0),
}


def _smooth_periodic(field, sigma):
    """Gaussian smoothing with standard deviation ``sigma`` cells (FFT, periodic)."""
    if sigma <= 0:
        return field
    nxp, nyp = field.shape
    kx = np.fft.fftfreq(nxp)[:, None]
    ky = np.fft.rfftfreq(nyp)[None, :]
    kernel = np.exp(-2.0 * (np.pi * sigma) ** 2 * (kx ** 2 + ky ** 2))
    return np.fft.irfft2(np.fft.rfft2(field) * kernel, s=field.shape)


def _smoothed_normal(rng, shape, std, sigma):
    f = _smooth_periodic(rng.standard_normal(shape), sigma)
    s = f.std()
    return f * (std / s if s > 0 else 0.0)


def make_state(nx, ny, seed=0, wind_scale=1.0, land_fraction=0.25,
               ice_lat=55.0, init_velocity=0.0, init_stress=0.0, olx=2, oly=2,
               land_sigma=None, wet_y_halo=False, land_rows=()):
    """A full sea-ice state (dict name -> array) on an ``nx`` x ``ny`` grid.

    ``init_velocity``/``init_stress`` > 0 start the ice with random smooth
    velocities (m/s) and stresses (N/m2) instead of rest, which exercises more
    of the stencil in parity tests.  ``wet_y_halo`` makes the y-halo rows
    partly wet (the stencils then wrap over the padded array in y, as the
    reference's ``roll`` does) and ``land_rows`` lists interior rows (0-based
    interior y index) forced to land.
    """
    rng = np.random.default_rng(seed)
    g = host_grid(nx, ny, olx=olx, oly=oly)
    NX, NY = nx + 2 * olx, ny + 2 * oly
    lat = np.broadcast_to(g["yt"][None, :], (NX, NY))

    # land mask on the interior, periodic in x, land in the y halo
    if land_sigma is None:
        land_sigma = max(1.0, nx / 45.0)
    noise = _smooth_periodic(rng.standard_normal((nx, ny)), land_sigma)
    maskT = np.zeros((NX, NY))
    if land_fraction > 0:
        thr = np.quantile(noise, land_fraction)
        maskT[olx:-olx, oly:-oly] = (noise > thr).astype(np.float64)
    else:
        maskT[olx:-olx, oly:-oly] = 1.0
    for r in land_rows:
        maskT[:, oly + r] = 0.0
    if wet_y_halo:
        maskT[:, :oly] = (rng.random((NX, oly)) > 0.3)
        maskT[:, -oly:] = (rng.random((NX, oly)) > 0.3)
    fill_cyclic_x(maskT, olx)
    maskU, maskV = velocity_masks(maskT, olx)

    # depth of the ocean (positive, as the host model's ``ht``)
    ht = (50.0 + 4950.0 * rng.random((NX, NY))) * maskT

    v = derive_grid_variables(g, maskT, maskU, maskV, ht)

    # ice fields
    polar = np.abs(lat) > ice_lat
    mu = np.log(1.5) - 0.5 * 0.5 ** 2
    h = np.exp(mu + 0.5 * rng.standard_normal((NX, NY))) * polar * maskT
    area = np.minimum(1.0, h / 0.5) * rng.uniform(0.8, 1.0, (NX, NY)) * (h > 0)
    for a in (h, area):
        fill_cyclic_x(a, olx)
    v["hIceMean"] = h
    v["Area"] = area
    v["hSnowMean"] = 0.2 * h

    # winds and currents
    v["uWind"] = fill_cyclic_x(_smoothed_normal(rng, (NX, NY), 8.0 * wind_scale, 3.0), olx)
    v["vWind"] = fill_cyclic_x(_smoothed_normal(rng, (NX, NY), 8.0 * wind_scale, 3.0), olx)
    v["wSpeed"] = np.sqrt(v["uWind"] ** 2 + v["vWind"] ** 2)
    v["uOcean"] = fill_cyclic_x(_smoothed_normal(rng, (NX, NY), 0.1, 3.0) * maskU, olx)
    v["vOcean"] = fill_cyclic_x(_smoothed_normal(rng, (NX, NY), 0.1, 3.0) * maskV, olx)

    # thermodynamic forcing
    sst = np.where(h > 0, -1.8, rng.uniform(0.0, 10.0, (NX, NY)))
    v["theta"] = sst + 273.15
    v["ATemp"] = rng.uniform(-25.0, 0.0, (NX, NY)) + 273.15
    v["SWdown"] = rng.uniform(0.0, 300.0, (NX, NY))
    v["LWdown"] = np.full((NX, NY), 250.0)
    v["aqh"] = rng.uniform(0.3e-3, 2.5e-3, (NX, NY))          # kg/kg
    v["precip"] = rng.uniform(0.0, 3e-8, (NX, NY))            # m/s, <= 2.6 mm/day
    v["snowfall"] = v["precip"] * rng.uniform(0.0, 1.0, (NX, NY))
    v["evap"] = -rng.uniform(0.0, 3e-8, (NX, NY))             # <0 increases salinity
    v["runoff"] = np.zeros((NX, NY))
    v["ocSalt"] = 34.0 + rng.uniform(-1.0, 1.0, (NX, NY))
    v["Qnet"] = rng.uniform(-50.0, 150.0, (NX, NY))            # ocean heat loss W/m2
    v["Qsw"] = -v["SWdown"]
    v["ssh_an"] = fill_cyclic_x(_smoothed_normal(rng, (NX, NY), 0.1, 3.0), olx)
    v["surfPress"] = fill_cyclic_x(101325.0 + _smoothed_normal(rng, (NX, NY), 500.0, 3.0), olx)

    # dynamic state
    zeros = np.zeros((NX, NY))
    if init_velocity > 0:
        v["uIce"] = fill_cyclic_x(_smoothed_normal(rng, (NX, NY), init_velocity, 2.0) * maskU, olx)
        v["vIce"] = fill_cyclic_x(_smoothed_normal(rng, (NX, NY), init_velocity, 2.0) * maskV, olx)
    else:
        v["uIce"] = zeros.copy()
        v["vIce"] = zeros.copy()
    if init_stress > 0:
        v["sigma1"] = _smoothed_normal(rng, (NX, NY), init_stress, 2.0) * maskT
        v["sigma2"] = _smoothed_normal(rng, (NX, NY), init_stress, 2.0) * maskT
        v["sigma12"] = _smoothed_normal(rng, (NX, NY), init_stress, 2.0)
    else:
        for n in ("sigma1", "sigma2", "sigma12"):
            v[n] = zeros.copy()
    for n in ("SeaIceMassC", "SeaIceMassU", "SeaIceMassV", "SeaIceStrength",
              "AreaW", "AreaS", "WindForcingX", "WindForcingY",
              "os_hIceMean", "os_hSnowMean", "SeaIceLoad", "IcePenetSW",
              "OceanStressU", "OceanStressV", "EmPmR", "saltflux",
              "forc_salt_surface_ice"):
        v[n] = zeros.copy()
    v["recip_hIceMean"] = 1.0 / np.sqrt(h ** 2 + 0.1 ** 2)
    return v


def config_settings(name, **overrides):
    """Settings of one named workload (time steps, subcycles, P*, C*, e)."""
    c = CONFIGS[name]
    s = default_settings(pStar=27500.0, cStar=20.0, PlasDefCoeff=2.0)
    with_timesteps(s, c["dt"], c["dt"], c["n_evp"])
    for k, val in overrides.items():
        if not hasattr(s, k):
            raise KeyError(k)
        setattr(s, k, val)
    return s


def config_state(name, seed=0, **kw):
    c = CONFIGS[name]
    return make_state(c["nx"], c["ny"], seed=seed, **kw)


def ensemble_members(n=512, seed=0):
    """Member shapes and wind scales of the batched-ensemble workload.

    nx is drawn uniformly from {64, 96, ..., 512}, ny from {64, 96, ..., 384},
    and each member's winds are scaled by U(0.5, 1.5).
    """
    rng = np.random.default_rng(seed)
    nxs = rng.choice(np.arange(64, 513, 32), size=n)
    nys = rng.choice(np.arange(64, 385, 32), size=n)
    scales = rng.uniform(0.5, 1.5, size=n)
    return [dict(nx=int(a), ny=int(b), wind_scale=float(s), seed=seed * 100003 + i)
            for i, (a, b, s) in enumerate(zip(nxs, nys, scales))]

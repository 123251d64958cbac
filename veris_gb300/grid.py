"""Lat-lon grid and the sea-ice grid variables derived from it.

``host_grid`` builds the few host-model (Veros) grid arrays the plugin starts
from: x/y spacings per column/row, cell areas, Coriolis parameter and the
tracer/velocity land masks.  ``derive_grid_variables`` then follows the
plugin's initialisation (veris/set_inits.py:5-52) to build the C-grid metric
fields the step reads.  Two properties of that initialisation are kept as
they are because the step depends on them bit for bit:

* the spacings ignore cos(latitude) (veris/set_inits.py:22-25) while the
  areas include it;
* ``rAz = 0.25 * roll(rA + roll(rA, 1, 0), 1, 1)`` is a quarter of a shifted
  two-point sum (veris/set_inits.py:33-34), i.e. half of the four-point mean.

Velocity points follow the MITgcm C grid used by the plugin: U(i, j) sits on
the west face of cell (i, j), V(i, j) on its south face, Z(i, j) on its
south-west corner.
"""
import numpy as np

EARTH_RADIUS = 6370e3
OMEGA = np.pi / 43082.0
DEGTOM = EARTH_RADIUS * np.pi / 180.0


def fill_cyclic_x(a, olx=2):
    """Periodic copy of the x halo in place, in the host model's order.

    The last ``olx`` columns receive interior columns ``olx..2*olx-1`` first,
    then the first ``olx`` columns receive columns ``-2*olx..-olx-1``.
    """
    a[-olx:, ...] = a[olx:2 * olx, ...]
    a[:olx, ...] = a[-2 * olx:-olx, ...]
    return a


def host_grid(nx, ny, lat0=-80.0, lat1=80.0, olx=2, oly=2):
    """Spacings, areas and Coriolis of a regular lat-lon grid with halos."""
    NX, NY = nx + 2 * olx, ny + 2 * oly
    dlon = 360.0 / nx
    dlat = (lat1 - lat0) / ny
    yt = lat0 + (np.arange(NY) - oly + 0.5) * dlat
    yu = yt + 0.5 * dlat
    dxt = np.full(NX, dlon * DEGTOM)
    dxu = dxt.copy()
    dyt = np.full(NY, dlat * DEGTOM)
    dyu = dyt.copy()
    # halo rows of coarse grids can reach past a pole: keep their areas positive
    cost = np.cos(np.deg2rad(np.clip(yt, -89.5, 89.5)))
    cosu = np.cos(np.deg2rad(np.clip(yu, -89.5, 89.5)))
    return dict(
        nx=nx, ny=ny, olx=olx, oly=oly, yt=yt, yu=yu,
        dxt=dxt, dxu=dxu, dyt=dyt, dyu=dyu,
        area_t=dxt[:, None] * cost[None, :] * dyt[None, :],
        area_u=dxu[:, None] * cost[None, :] * dyt[None, :],
        area_v=dxt[:, None] * cosu[None, :] * dyu[None, :],
        coriolis_t=np.broadcast_to(2 * OMEGA * np.sin(np.deg2rad(yt))[None, :], (NX, NY)).copy(),
    )


def velocity_masks(maskT, olx=2):
    """U and V masks of the C grid: open only between two wet cells."""
    maskU = maskT * np.roll(maskT, 1, 0)
    maskV = maskT * np.roll(maskT, 1, 1)
    fill_cyclic_x(maskU, olx)
    fill_cyclic_x(maskV, olx)
    return maskU, maskV


def derive_grid_variables(g, maskT, maskU, maskV, ht):
    """The plugin's grid and mask variables (veris/set_inits.py:10-50)."""
    ones2d = np.ones_like(maskT)
    v = {}
    v["iceMask"] = maskT.copy()
    v["iceMaskU"] = maskU.copy()
    v["iceMaskV"] = maskV.copy()
    v["maskInC"] = maskT.copy()
    v["maskInU"] = maskU.copy()
    v["maskInV"] = maskV.copy()
    v["R_low"] = ht.copy()
    v["fCori"] = g["coriolis_t"].copy()
    v["dxC"] = ones2d * g["dxt"][:, None]
    v["dyC"] = ones2d * g["dyt"]
    v["dxU"] = ones2d * g["dxu"][:, None]
    v["dyU"] = ones2d * g["dyu"]
    v["dxG"] = 0.5 * (v["dxU"] + np.roll(v["dxU"], 1, 1))
    v["dyG"] = 0.5 * (v["dyU"] + np.roll(v["dyU"], 1, 0))
    v["dxV"] = 0.5 * (v["dxC"] + np.roll(v["dxC"], 1, 1))
    v["dyV"] = 0.5 * (v["dyC"] + np.roll(v["dyC"], 1, 0))
    v["rA"] = g["area_t"].copy()
    v["rAu"] = g["area_u"].copy()
    v["rAv"] = g["area_v"].copy()
    rAz = v["rA"] + np.roll(v["rA"], 1, 0)
    v["rAz"] = 0.25 * np.roll(rAz, 1, 1)
    for name in ("dxC", "dyC", "dxG", "dyG", "dxU", "dyU", "dxV", "dyV"):
        v["recip_" + name] = 1 / v[name]
    for name in ("rA", "rAu", "rAv", "rAz"):
        v["recip_" + name] = 1 / v[name]
    for name in ("k1AtC", "k2AtC", "k1AtZ", "k2AtZ", "Fu", "Fv"):
        v[name] = np.zeros_like(maskT)
    v["TSurf"] = ones2d * 273
    return v

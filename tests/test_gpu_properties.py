"""Properties of the reference's arithmetic, checked on the GPU kernels.

* Advection (veris/advection.py:15-91) conserves the area integral
  sum(rA * field) of hIceMean, hSnowMean and Area on an all-ocean domain
  that is periodic in x: the zonal fluxes are halo-filled, so their
  divergence telescopes, and the meridional fluxes vanish at the land rows
  of the y halo.  Bars: 1e-12 relative in float64, 1e-6 in float32 (the
  oracle conserves it to round-off on the same state, see
  ``tests/test_oracle_golden.py``).
* A step leaves land at exactly zero in every output the reference masks:
  uIce/vIce and the ocean stress at U/V points without ice mask, sigma1,
  sigma2, hIceMean, hSnowMean and Area at C points without ice mask, EmPmR
  and the salt flux at dry C points; the float64 drop-ins and the float32
  engine alike.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

INTERIOR = (slice(2, -2), slice(2, -2))
ADVECTED = ("hIceMean", "hSnowMean", "Area")
LAND_ZERO = (("uIce", "iceMaskU"), ("vIce", "iceMaskV"), ("sigma1", "iceMask"), ("sigma2", "iceMask"),
             ("hIceMean", "iceMask"), ("hSnowMean", "iceMask"), ("Area", "iceMask"),
             ("EmPmR", "maskInC"), ("forc_salt_surface_ice", "maskInC"),
             ("OceanStressU", "iceMaskU"), ("OceanStressV", "iceMaskV"))


@pytest.fixture(scope="module", autouse=True)
def _lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from veris_gb300 import _abi
    return _abi.load()


def _ocean_state(nx, ny, seed):
    """All-ocean, ice everywhere, moving ice; halos of the advected fields
    and velocities filled as the step leaves them."""
    from veris_gb300.fill_overlap import fill_overlap, fill_overlap_uv
    from veris_gb300.state import VerisState
    from veris_gb300.synthetic import config_settings, make_state
    arrays = make_state(nx, ny, seed=seed, land_fraction=0.0, ice_lat=0.0, init_velocity=0.3)
    st = VerisState.from_numpy(arrays, config_settings("c1_4deg"))
    v = st.variables
    v.uIce, v.vIce = fill_overlap_uv(st, v.uIce, v.vIce)
    for k in ADVECTED:
        setattr(v, k, fill_overlap(st, getattr(v, k)))
    return st


def _area_integral(rA, x):
    return float((rA[INTERIOR].astype(np.float64) * x[INTERIOR].astype(np.float64)).sum())


@pytest.mark.parametrize("nx,ny", [(36, 20), (90, 40), (181, 67)])
def test_advection_conserves_the_area_integral_f64(nx, ny):
    from veris_gb300.advection import Advection
    st = _ocean_state(nx, ny, seed=nx)
    v = st.variables
    rA = v.rA.cpu().numpy()
    out = Advection(st)
    torch.cuda.synchronize()
    for k, new in zip(ADVECTED, out):
        old = getattr(v, k).cpu().numpy()
        new = new.cpu().numpy()
        assert np.abs(new - old).max() > 1e-4 * np.abs(old).max(), k   # the fields did move
        s0, s1 = _area_integral(rA, old), _area_integral(rA, new)
        assert abs(s1 - s0) <= 1e-12 * abs(s0), (k, s0, s1)


@pytest.mark.parametrize("nx,ny", [(36, 20), (181, 67)])
def test_advection_conserves_the_area_integral_f32(nx, ny):
    from veris_gb300 import _abi
    from veris_gb300.state import Call, Variables
    st = _ocean_state(nx, ny, seed=nx + 1)
    v32 = Variables(**{k: t.float() for k, t in vars(st.variables).items() if isinstance(t, torch.Tensor)})
    c = Call(st, dtype=torch.float32, variables=v32)
    h, hs, A = c.empty(3)
    ws, wsb = c.workspace(c.lib.veris_advection_workspace_bytes(c.refs()[0], 4))
    _abi.check("Advection_f32", c.lib.veris_advection_f32(*c.refs(), h.data_ptr(), hs.data_ptr(), A.data_ptr(),
                                                          ws, wsb, c.stream))
    torch.cuda.synchronize()
    rA = v32.rA.cpu().numpy()
    for k, new in zip(ADVECTED, (h, hs, A)):
        old = getattr(v32, k).cpu().numpy()
        s0, s1 = _area_integral(rA, old), _area_integral(rA, new.cpu().numpy())
        assert abs(s1 - s0) <= 1e-6 * abs(s0), (k, s0, s1)


def _land_state():
    from veris_gb300.state import VerisState
    from veris_gb300.synthetic import config_settings, make_state
    arrays = make_state(36, 20, seed=6, land_fraction=0.3, ice_lat=0.0, init_velocity=0.2, init_stress=1000.0)
    return VerisState.from_numpy(arrays, config_settings("c1_4deg", nEVPsteps=10))


def _assert_land_zero(v, what):
    for k, m in LAND_ZERO:
        x = getattr(v, k)[INTERIOR].double().cpu().numpy()
        land = getattr(v, m)[INTERIOR].cpu().numpy() == 0
        assert land.any(), (what, m)
        assert np.all(x[land] == 0.0), (what, k, float(np.abs(x[land]).max()))


def test_float64_step_zeroes_land():
    from veris_gb300 import model
    st = _land_state()
    model.step(st)
    torch.cuda.synchronize()
    _assert_land_zero(st.variables, "float64 drop-ins")


def test_float32_engine_step_zeroes_land():
    from veris_gb300.engine import SeaIceStep
    st = _land_state()
    SeaIceStep(st, precision="f32").step()
    torch.cuda.synchronize()
    _assert_land_zero(st.variables, "float32 engine")

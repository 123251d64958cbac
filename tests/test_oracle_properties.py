"""Randomised properties of the oracle (hypothesis; CPU only).

The fixtures pin the oracle on fixed cases; these check properties the
reference's arithmetic has for any input:

* the superbee limiter (veris/advection.py:170-175) stays in [0, 2], is 0
  for non-positive ratios and is non-decreasing;
* the halo fill (veris/fill_overlap.py:6-18) is idempotent and leaves the
  interior alone, with either fill;
* advection (veris/advection.py:15-91) conserves sum(rA * field) on an
  all-ocean domain periodic in x, for any seeded velocity field.
"""
from types import SimpleNamespace

import numpy as np
import pytest

hypothesis = pytest.importorskip("hypothesis")
from hypothesis import given, settings, strategies as st  # noqa: E402

from oracle import veris_oracle as O  # noqa: E402

finite = st.floats(min_value=-1e6, max_value=1e6, allow_nan=False, allow_infinity=False)


@given(st.lists(finite, min_size=1, max_size=64))
def test_limiter_range_sign_and_monotonicity(xs):
    cr = np.sort(np.asarray(xs, dtype=np.float64))
    phi = O.limiter(cr)
    assert np.all((phi >= 0) & (phi <= 2))
    assert np.all(phi[cr <= 0] == 0)
    assert np.all(np.diff(phi) >= 0)


@settings(max_examples=40, deadline=None)
@given(nx=st.integers(4, 24), ny=st.integers(4, 24), seed=st.integers(0, 2**31 - 1),
       veros_fill=st.booleans(), cyclic=st.booleans())
def test_fill_idempotent_and_interior_untouched(nx, ny, seed, veros_fill, cyclic):
    s = SimpleNamespace(veros_fill=veros_fill, enable_cyclic_x=cyclic, olx=2, oly=2)
    state = SimpleNamespace(settings=s)
    a = np.random.default_rng(seed).standard_normal((nx + 4, ny + 4))
    once = O.fill_overlap(state, a.copy())
    twice = O.fill_overlap(state, once.copy())
    np.testing.assert_array_equal(once, twice)
    np.testing.assert_array_equal(once[2:-2, 2:-2], a[2:-2, 2:-2])


@settings(max_examples=12, deadline=None)
@given(seed=st.integers(0, 10_000), speed=st.floats(0.01, 0.6))
def test_advection_conserves_on_a_periodic_ocean(seed, speed):
    from veris_gb300.synthetic import config_settings, make_state
    a = make_state(24, 14, seed=seed, land_fraction=0.0, ice_lat=0.0, init_velocity=speed)
    state = SimpleNamespace(variables=SimpleNamespace(**a), settings=config_settings("c1_4deg"))
    v = state.variables
    v.uIce, v.vIce = O.fill_overlap_uv(state, v.uIce.copy(), v.vIce.copy())
    for k in ("hIceMean", "hSnowMean", "Area"):
        setattr(v, k, O.fill_overlap(state, getattr(v, k).copy()))
    interior = (slice(2, -2), slice(2, -2))
    with np.errstate(all="ignore"):
        out = O.Advection(state)
    for k, new in zip(("hIceMean", "hSnowMean", "Area"), out):
        old = getattr(v, k)
        s0, s1 = (v.rA[interior] * old[interior]).sum(), (v.rA[interior] * new[interior]).sum()
        assert abs(s1 - s0) <= 1e-12 * abs(s0), (k, s0, s1)

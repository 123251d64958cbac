"""The CPU oracle against the golden fixtures made by running the reference.

The oracle restates the reference's arithmetic in its order of operations, so
the bar here is bit-exact equality (NaN == NaN never occurs: the fixtures are
finite).
"""
import os

import numpy as np
import pytest

from oracle import veris_oracle as O
from tests import golden_io as G


@pytest.mark.parametrize("case", G.CASES)
def test_step_sequence_bit_exact(case):
    g = G.load(case)
    st = G.initial_state(g)
    seq = G.sequence(g)
    got = []
    n_steps = sum(1 for _i, r, _o in seq if r == "SeaIceMass")
    for _ in range(n_steps):
        O.step(st, record=lambda name, outs: got.append((name, outs)))
    assert [r for _i, r, _o in seq] == [name for name, _o in got]
    for (i, r, ref), (_n, outs) in zip(seq, got):
        for k, a in ref.items():
            np.testing.assert_array_equal(outs[k], a, err_msg=f"{case} call {i} {r}.{k}")


@pytest.mark.parametrize("case", G.CASES)
def test_inner_routines_bit_exact(case):
    g = G.load(case)
    first_evp = [i for i, r, _o in G.sequence(g) if r == "IceVelocities"][0]
    st = G.state_before(g, first_evp)
    v = st.variables
    u, vv = v.uIce, v.vIce
    e11, e22, e12 = O.strainrates(st, u, vv)
    ref = G.sub(g, "strainrates")
    for k, a in zip(("e11", "e22", "e12"), (e11, e22, e12)):
        np.testing.assert_array_equal(a, ref[k], err_msg=k)
    zeta, eta, press = O.viscosities(st, ref["e11"], ref["e22"], ref["e12"])
    ref = G.sub(g, "viscosities")
    for k, a in zip(("zeta", "eta", "press"), (zeta, eta, press)):
        np.testing.assert_array_equal(a, ref[k], err_msg=k)
    np.testing.assert_array_equal(O.c_point_to_z_point(st, ref["zeta"]),
                                  G.sub(g, "c_point_to_z_point")["zetaZ"])
    np.testing.assert_array_equal(O.ocean_drag_coeffs(st, u, vv), G.sub(g, "ocean_drag_coeffs")["cDrag"])
    np.testing.assert_array_equal(O.basal_drag_coeffs(st, u, vv), G.sub(g, "basal_drag_coeffs")["cBot"])
    sU, sV = O.side_drag(st, u, vv)
    ref = G.sub(g, "side_drag")
    np.testing.assert_array_equal(sU, ref["SideDragU"])
    np.testing.assert_array_equal(sV, ref["SideDragV"])
    dX, dY = O.stressdiv(st, v.sigma1, v.sigma2, v.sigma12)
    ref = G.sub(g, "stressdiv")
    np.testing.assert_array_equal(dX, ref["stressDivX"])
    np.testing.assert_array_equal(dY, ref["stressDivY"])
    tX, tY = O.tauXY(st)
    ref = G.sub(g, "tauXY")
    np.testing.assert_array_equal(tX, ref["tauX"])
    np.testing.assert_array_equal(tY, ref["tauY"])
    out = O.evp_solver(st, n=1)
    ref = G.sub(g, "evp_1")
    for k, a in zip(("uIce", "vIce", "sigma1", "sigma2", "sigma12"), out):
        np.testing.assert_array_equal(a, ref[k], err_msg=k)


@pytest.mark.parametrize("case", G.CASES)
def test_advection_and_thermo_routines_bit_exact(case):
    g = G.load(case)
    seq = G.sequence(g)
    adv = [i for i, r, _o in seq if r == "Advection"][0]
    st = G.state_before(g, adv)
    v = st.variables
    uT = v.uIce * v.dyG * v.iceMaskU
    vT = v.vIce * v.dxG * v.iceMaskV
    np.testing.assert_array_equal(O.calc_ZonalFlux(st, v.hIceMean.copy(), uT),
                                  G.sub(g, "calc_ZonalFlux")["ZonalFlux"])
    np.testing.assert_array_equal(O.calc_MeridionalFlux(st, v.hIceMean.copy(), vT),
                                  G.sub(g, "calc_MeridionalFlux")["MeridionalFlux"])
    np.testing.assert_array_equal(O.calc_Advection(st, v.Area.copy()),
                                  G.sub(g, "calc_Advection")["field"])
    lim = G.sub(g, "limiter")
    np.testing.assert_array_equal(O.limiter(lim["Cr"]), lim["phi"])

    gr = [i for i, r, _o in seq if r == "Growth"][0]
    st = G.state_before(g, gr)
    v, s = st.variables, st.settings
    ref = G.sub(g, "solve4temp")
    TempFrz = s.tempFrz + s.dtempFrz_dS * v.ocSalt + s.celsius2K
    out = O.solve4temp(st, ref["in_hIceActual"], ref["in_hSnowActual"], v.TSurf, TempFrz)
    for k, a in zip(("TSurfOut", "F_io_net", "F_ia_net", "IcePenetSW", "FWsublim"), out):
        np.testing.assert_array_equal(a, ref[k], err_msg=k)


def test_limiter_range():
    cr = np.linspace(-50, 50, 10001)
    phi = O.limiter(cr)
    assert phi.min() >= 0 and phi.max() <= 2


def test_advection_conserves_the_area_integral():
    """On an all-ocean domain periodic in x the zonal flux divergence
    telescopes and the meridional fluxes vanish at the y-halo land rows."""
    from types import SimpleNamespace
    from veris_gb300.synthetic import config_settings, make_state
    a = make_state(36, 20, seed=5, land_fraction=0.0, ice_lat=0.0, init_velocity=0.3)
    st = SimpleNamespace(variables=SimpleNamespace(**a), settings=config_settings("c1_4deg"))
    v = st.variables
    v.uIce, v.vIce = O.fill_overlap_uv(st, v.uIce.copy(), v.vIce.copy())
    for k in ("hIceMean", "hSnowMean", "Area"):
        setattr(v, k, O.fill_overlap(st, getattr(v, k).copy()))
    I = (slice(2, -2), slice(2, -2))
    for k, new in zip(("hIceMean", "hSnowMean", "Area"), O.Advection(st)):
        old = getattr(v, k)
        assert np.abs(new - old).max() > 1e-4 * np.abs(old).max(), k
        s0, s1 = (v.rA[I] * old[I]).sum(), (v.rA[I] * new[I]).sum()
        assert abs(s1 - s0) <= 1e-13 * abs(s0), (k, s0, s1)


def test_step_zeroes_land():
    """The outputs the reference masks are exactly zero on land after a step."""
    from types import SimpleNamespace
    from veris_gb300.synthetic import config_settings, make_state
    a = make_state(36, 20, seed=6, land_fraction=0.3, ice_lat=0.0, init_velocity=0.2, init_stress=1000.0)
    st = SimpleNamespace(variables=SimpleNamespace(**a), settings=config_settings("c1_4deg", nEVPsteps=10))
    O.step(st)
    v = st.variables
    I = (slice(2, -2), slice(2, -2))
    for k, m in (("uIce", "iceMaskU"), ("vIce", "iceMaskV"), ("sigma1", "iceMask"), ("sigma2", "iceMask"),
                 ("hIceMean", "iceMask"), ("hSnowMean", "iceMask"), ("Area", "iceMask"),
                 ("EmPmR", "maskInC"), ("forc_salt_surface_ice", "maskInC"),
                 ("OceanStressU", "iceMaskU"), ("OceanStressV", "iceMaskV")):
        land = getattr(v, m)[I] == 0
        assert land.any(), m
        assert np.all(getattr(v, k)[I][land] == 0.0), k


def test_fill_overlap_idempotent():
    g = G.load("c1")
    st = G.initial_state(g)
    a = np.random.default_rng(0).random(st.variables.iceMask.shape)
    once = O.fill_overlap(st, a.copy())
    twice = O.fill_overlap(st, once.copy())
    np.testing.assert_array_equal(once, twice)


@pytest.mark.parametrize("case", G.FREEDRIFT_CASES)
def test_freedrift_bit_exact(case):
    st, ref = G.freedrift_case(G.load_forcing(), case)
    u, v = O.freedrift_solver(st)
    np.testing.assert_array_equal(u, ref["uIce"])
    np.testing.assert_array_equal(v, ref["vIce"])


def test_freedrift_fixture_reaches_the_zero_branches():
    st, ref = G.freedrift_case(G.load_forcing(), "small_b")
    v = st.variables
    calm = (v.WindForcingX == 0) & (v.WindForcingY == 0) & (v.uOcean == 0) & (v.vOcean == 0)
    assert calm.sum() > 50 and np.abs(ref["uIce"]).max() > 0


def test_bulk_formula_bit_exact():
    from types import SimpleNamespace
    sett, args, ref = G.bulk_case(G.load_forcing())
    got = O.bulkf_formula_lanl(SimpleNamespace(settings=sett), *args)
    for n, a in zip(G.BULK_OUT, got):
        np.testing.assert_array_equal(a, ref[n], err_msg=n)


def test_bulk_fixture_spans_stable_and_unstable_layers():
    _sett, (uw, vw, ta, qa, tsf, _m), _ref = G.bulk_case(G.load_forcing())
    dT = ta - tsf
    assert (dT > 1).any() and (dT < -1).any()
    assert (np.hypot(uw, vw) < 1).any() and (np.hypot(uw, vw) == 0).any()


def test_evp_residuals_match_the_plain_loop():
    """The residual loop leaves the EVP result unchanged and its sums are
    non-negative; with the state at rest and no forcing they are zero."""
    g = G.load("moving")
    first_evp = [i for i, r, _o in G.sequence(g) if r == "IceVelocities"][0]
    st = G.state_before(g, first_evp)
    u, v, s1, s2, s12, resU, resSig = O.evp_residuals(st, n=6)
    ref = O.evp_solver(G.state_before(g, first_evp), n=6)
    for a, b in zip((u, v, s1, s2, s12), ref):
        np.testing.assert_array_equal(a, b)
    assert resU.shape == (6,) and (resU > 0).all() and (resSig > 0).all()


@pytest.mark.parametrize("case", ("moving", "small_a", "small_b"))
def test_evp_residuals_against_the_reference(case):
    """The residuals of the reference's own branch (veris/evp_solver.py:
    51-56, 191-230, its two unbound names patched to the stress components
    they stand for; tests/golden/make_golden.py --residuals) equal the
    oracle's restatement, and the solve is unchanged."""
    z = np.load(os.path.join(G.GOLDEN, "residuals.npz"))
    g = G.load(case)
    first_evp = [i for i, r, _o in G.sequence(g) if r == "IceVelocities"][0]
    st = G.state_before(g, first_evp)
    n = len(z[f"res.{case}.resU"])
    out = O.evp_residuals(st, n=n)
    for k, name in enumerate(("uIce", "vIce", "sigma1", "sigma2", "sigma12")):
        np.testing.assert_array_equal(out[k], z[f"res.{case}.{name}"])
    np.testing.assert_allclose(out[5], z[f"res.{case}.resU"], rtol=1e-14, atol=0)
    np.testing.assert_allclose(out[6], z[f"res.{case}.resSig"], rtol=1e-14, atol=0)

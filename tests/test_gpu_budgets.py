"""Float64 conservation diagnostics of the step engine against NumPy sums.

The engine records, every step, area-weighted interior sums of the ice and
snow volumes and the ice area at four points of the step, the advection
overshoots, and the ocean's heat, fresh-water and salt fluxes from Growth
(veris/growth.py:296-383).  They are checked against float64 NumPy sums of
the oracle's own step (veris/setup/seaice_global_4deg/seaice_global_4deg.py:
878-932 order), and against NumPy sums of the engine's own fields."""
import copy
from types import SimpleNamespace

import numpy as np
import pytest

from oracle import veris_oracle as O

pytestmark = pytest.mark.gpu

I = (slice(2, -2), slice(2, -2))


def _sum(rA, x):
    return float(np.sum(rA[I] * x[I]))


def _mag(rA, x):
    return float(np.sum(np.abs(rA[I] * x[I])))


def _oracle_budgets(arrays, sett, steps):
    """The BUDGET_SLOTS of every step, from the oracle's step records."""
    st = SimpleNamespace(variables=SimpleNamespace(**{k: v.copy() for k, v in arrays.items()}),
                         settings=copy.copy(sett))
    v = st.variables
    rA = v.rA
    rows = []
    for _ in range(steps):
        row = {"ice_volume_start": _sum(rA, v.hIceMean), "snow_volume_start": _sum(rA, v.hSnowMean),
               "ice_area_start": _sum(rA, v.Area)}

        def record(name, outs):
            if name == "Advection":
                row.update(ice_volume_advected=_sum(rA, outs["hIceMean"]),
                           snow_volume_advected=_sum(rA, outs["hSnowMean"]),
                           ice_area_advected=_sum(rA, outs["Area"]))
            elif name == "clean_up_advection":
                row.update(ice_volume_cleaned=_sum(rA, outs["hIceMean"]),
                           snow_volume_cleaned=_sum(rA, outs["hSnowMean"]),
                           ice_overshoot=_sum(rA, outs["os_hIceMean"]),
                           snow_overshoot=_sum(rA, outs["os_hSnowMean"]))

        O.step(st, record=record)
        row.update(ice_volume_end=_sum(rA, v.hIceMean), snow_volume_end=_sum(rA, v.hSnowMean),
                   ice_area_end=_sum(rA, v.Area), ocean_heat_loss=_sum(rA, v.Qnet),
                   fresh_water_flux=_sum(rA, v.EmPmR), salt_flux=_sum(rA, v.forc_salt_surface_ice))
        # magnitudes of the fluxes' terms (their sums cancel)
        row.update(mag_ocean_heat_loss=_mag(rA, v.Qnet), mag_fresh_water_flux=_mag(rA, v.EmPmR),
                   mag_salt_flux=_mag(rA, v.forc_salt_surface_ice))
        rows.append(row)
    return rows


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_budgets_against_numpy_sums(precision):
    import torch
    from veris_gb300.engine import BUDGET_SLOTS, SeaIceStep
    from veris_gb300.state import VerisState
    from veris_gb300.synthetic import config_settings, make_state

    arrays = make_state(40, 24, seed=5, init_velocity=0.1, ice_lat=25.0)
    sett = config_settings("c1_4deg", nEVPsteps=40)
    steps = 3
    st = VerisState.from_numpy(arrays, sett, device="cuda:0")
    eng = SeaIceStep(st, precision=precision, budgets=True)
    own = []
    for k in range(steps):
        eng.step()
        v = st.variables
        rA = v.rA.cpu().numpy()
        own.append({"ice_volume_end": _sum(rA, v.hIceMean.cpu().numpy()),
                    "ocean_heat_loss": _sum(rA, v.Qnet.cpu().numpy()),
                    "fresh_water_flux": _sum(rA, v.EmPmR.cpu().numpy())})
    torch.cuda.synchronize()
    rec = eng.budget_records()
    assert set(rec) == set(BUDGET_SLOTS) and all(len(x) == steps for x in rec.values())
    # the device sums equal NumPy's sums of the engine's own fields
    for k in range(steps):
        for name, val in own[k].items():
            assert abs(rec[name][k] - val) <= 1e-13 * max(abs(val), 1e-300), (name, k, rec[name][k], val)
    # and the oracle's step to the parity tolerance of the path
    ref = _oracle_budgets(arrays, sett, steps)
    tol = 1e-12 if precision == "f64" else 1e-4
    for k in range(steps):
        for name in BUDGET_SLOTS:
            a, b = rec[name][k], ref[k][name]
            if "volume" in name or "overshoot" in name:
                scale = abs(ref[k]["ice_volume_start"]) if name.startswith("ice") or name == "ice_overshoot" \
                    else abs(ref[k]["snow_volume_start"])
            else:
                scale = ref[k].get("mag_" + name, abs(b))
            assert abs(a - b) <= tol * max(scale, abs(b), 1e-300), (precision, name, k, a, b)


def test_budgets_are_reproducible_and_graph_safe():
    """Two engines from the same state record bit-identical budgets, one
    eager and one replaying a captured graph (the slot advances in the
    graph)."""
    import torch
    from veris_gb300.engine import SeaIceStep
    from veris_gb300.state import VerisState
    from veris_gb300.synthetic import config_settings, make_state

    arrays = make_state(64, 40, seed=6, init_velocity=0.05, ice_lat=30.0)
    sett = config_settings("c1_4deg", nEVPsteps=30)
    a = SeaIceStep(VerisState.from_numpy(arrays, sett, device="cuda:0"), precision="f64", budgets=True)
    b = SeaIceStep(VerisState.from_numpy(arrays, sett, device="cuda:0"), precision="f64", budgets=True)
    for _ in range(4):
        a.step()
    b.capture()            # one eager step, then the captured step
    for _ in range(3):
        b.step()
    torch.cuda.synchronize()
    ra, rb = a.budget_records(), b.budget_records()
    for name in ra:
        assert len(ra[name]) == 4 and len(rb[name]) == 4
        assert np.array_equal(ra[name], rb[name]), name

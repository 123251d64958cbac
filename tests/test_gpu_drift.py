"""Drift of the float64 GPU step from the reference algorithm over many
steps (the CPU oracle, bit-identical to the reference on the fixtures):
one step must agree to 1e-10; the difference after ten steps is printed and
bounded (rounding differences of the regrouped fast-form arithmetic grow
through the nonlinear rheology)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

FIELDS = ("uIce", "vIce", "hIceMean", "Area")


def _rel(a, b):
    scale = max(float(np.max(np.abs(b))), 1e-300)
    return float(np.max(np.abs(a - b))) / scale


@pytest.mark.parametrize("evp", ("plain", "fast"))
def test_float64_drift_over_ten_steps(evp):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from types import SimpleNamespace
    from oracle import veris_oracle as O
    from veris_gb300.engine import SeaIceStep
    from veris_gb300.state import VerisState
    from veris_gb300.synthetic import config_settings, make_state
    arrays = make_state(90, 40, seed=11, init_velocity=0.05)
    sett = config_settings("c1_4deg")
    ref = SimpleNamespace(variables=SimpleNamespace(**{k: v.copy() for k, v in arrays.items()}), settings=sett)
    st = VerisState.from_numpy(arrays, sett)
    eng = SeaIceStep(st, precision="f64", evp=evp)
    drift = []
    for step in range(10):
        O.step(ref)
        eng.step()
        torch.cuda.synchronize()
        drift.append({n: _rel(getattr(st.variables, n).cpu().numpy(), getattr(ref.variables, n)) for n in FIELDS})
    print(f"\nfloat64 drift ({evp} EVP form), max-norm relative to the field maximum, per step:")
    for k, d in enumerate(drift):
        print(f"  step {k + 1:2d}: " + ", ".join(f"{n} {e:.1e}" for n, e in d.items()))
    assert max(drift[0].values()) <= 1e-10
    assert max(drift[-1].values()) <= 1e-6

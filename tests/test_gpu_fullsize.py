"""The path at the workloads' full sizes.

* 360 x 180 (the one-degree workload, 300 subcycles, dt 3600 s): one whole
  float64 step of the drop-ins and of the step engine against the oracle,
  bar 1e-10.
* 1440 x 720 (the quarter-degree workload): one whole step against the
  oracle (two subcycles keep the NumPy side to seconds), bar 1e-10.
* 3600 x 1800 (the tenth-degree workload): one whole float64 step with two
  subcycles (advection and growth in full) against the oracle, bar 1e-10.
* Members of the ensemble workload (sizes and wind scales drawn by its
  generator, 100 subcycles): one float64 step each against the oracle.
* 3600 x 1800 (the tenth-degree workload), properties that do not depend on
  an oracle: the float64 fast EVP form equals the plain float64 kernel to
  1e-10, the float32 walk equals the shared-memory float32 form to 1e-5, a
  float32 engine step is bit-reproducible, the halo fill is idempotent and
  the deterministic global sum repeats bit for bit.
"""
import numpy as np
import pytest

from tests import golden_io as G

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from veris_gb300 import _abi
    return _abi.load()


def _prepared(st):
    from veris_gb300 import model
    for name in ("SeaIceMass", "AreaWS", "WindForcingXY", "SeaIceStrength"):
        fn, outs = [(f, o) for n, f, o in model.STEP if n == name][0]
        vals = fn(st)
        vals = vals if isinstance(vals, tuple) else (vals,)
        for o, x in zip(outs, vals):
            setattr(st.variables, o, x)
    return st


def test_quarter_degree_step_against_the_oracle():
    from types import SimpleNamespace
    from oracle import veris_oracle as O
    from veris_gb300 import model
    from veris_gb300.state import VerisState
    from veris_gb300.synthetic import config_settings, config_state
    arrays = config_state("c2_quarterdeg", seed=3, init_velocity=0.05, init_stress=1000.0)
    sett = config_settings("c2_quarterdeg", nEVPsteps=2)
    ref = SimpleNamespace(variables=SimpleNamespace(**{k: v.copy() for k, v in arrays.items()}), settings=sett)
    O.step(ref)
    st = VerisState.from_numpy(arrays, sett)
    model.step(st)
    torch.cuda.synchronize()
    for k in ("uIce", "vIce", "sigma1", "sigma2", "sigma12", "hIceMean", "hSnowMean", "Area", "TSurf",
              "Qnet", "EmPmR", "forc_salt_surface_ice"):
        e = G.rel_err(getattr(st.variables, k).cpu().numpy(), getattr(ref.variables, k))
        assert e <= 1e-10, (k, e)


STEP_FIELDS = ("uIce", "vIce", "sigma1", "sigma2", "sigma12", "hIceMean", "hSnowMean", "Area", "TSurf",
               "Qnet", "EmPmR", "forc_salt_surface_ice", "OceanStressU", "OceanStressV")


def _step_against_oracle(arrays, sett, engine=False, tol=1e-10):
    """One float64 step of the drop-ins (and of the float64 step engine, fast
    EVP form) from ``arrays``, against the oracle's step."""
    from types import SimpleNamespace
    from oracle import veris_oracle as O
    from veris_gb300 import model
    from veris_gb300.engine import SeaIceStep
    from veris_gb300.state import VerisState
    ref = SimpleNamespace(variables=SimpleNamespace(**{k: v.copy() for k, v in arrays.items()}), settings=sett)
    O.step(ref)
    runs = {"drop-ins": VerisState.from_numpy(arrays, sett)}
    model.step(runs["drop-ins"])
    if engine:
        runs["engine"] = VerisState.from_numpy(arrays, sett)
        eng = SeaIceStep(runs["engine"], precision="f64")
        assert eng.evp_form == "fast"
        eng.step()
    torch.cuda.synchronize()
    for name, st in runs.items():
        for k in STEP_FIELDS:
            e = G.rel_err(getattr(st.variables, k).cpu().numpy(), getattr(ref.variables, k))
            assert e <= tol, (name, k, e)


def test_one_degree_step_against_the_oracle():
    from veris_gb300.synthetic import config_settings, config_state
    arrays = config_state("c3_1deg", seed=2, init_velocity=0.05, init_stress=500.0)
    _step_against_oracle(arrays, config_settings("c3_1deg"), engine=True)


def test_tenth_degree_step_against_the_oracle(tenth):
    from veris_gb300.synthetic import config_settings
    arrays, _sett = tenth
    _step_against_oracle(arrays, config_settings("c5_tenthdeg", nEVPsteps=2), engine=True)


@pytest.mark.parametrize("member", (0, 1, 2, 3))
def test_ensemble_members_against_the_oracle(member):
    from veris_gb300.synthetic import config_settings, ensemble_members, make_state
    sp = ensemble_members(512, seed=0)[member]
    arrays = make_state(sp["nx"], sp["ny"], seed=sp["seed"], wind_scale=sp["wind_scale"])
    _step_against_oracle(arrays, config_settings("c4_ensemble"))


@pytest.fixture(scope="module")
def tenth():
    from veris_gb300.state import VerisState
    from veris_gb300.synthetic import config_settings, config_state
    arrays = config_state("c5_tenthdeg", seed=1, init_velocity=0.05)
    return arrays, config_settings("c5_tenthdeg")


def test_tenth_degree_fast_forms_agree(tenth):
    from veris_gb300.evp_solver import evp_solver, evp_solver_fast
    from veris_gb300.state import VerisState
    arrays, sett = tenth
    st = _prepared(VerisState.from_numpy(arrays, sett))
    plain = evp_solver(st, 3)
    fast = evp_solver_fast(st, "f64", "smem", n_subcycles=3)
    for k in range(5):
        e = G.rel_err(fast[k].cpu().numpy(), plain[k].cpu().numpy())
        assert e <= 1e-10, (k, e)
    walk = evp_solver_fast(st, "f32", "walk", n_subcycles=10, rows=0, variant=2)
    smem = evp_solver_fast(st, "f32", "smem", n_subcycles=10)
    for k in range(5):
        e = G.rel_err(walk[k].double().cpu().numpy(), smem[k].double().cpu().numpy())
        assert e <= 1e-5, (k, e)


def test_tenth_degree_step_is_reproducible_and_fill_idempotent(tenth):
    from veris_gb300.engine import SeaIceStep
    from veris_gb300.fill_overlap import fill_overlap
    from veris_gb300.global_sum import interior_sum
    from veris_gb300.state import VerisState
    arrays, sett = tenth
    sett = type(sett)(**vars(sett))
    sett.nEVPsteps = 50
    outs = []
    for _ in range(2):
        st = VerisState.from_numpy(arrays, sett)
        SeaIceStep(st, precision="f32").step()
        torch.cuda.synchronize()
        outs.append({k: getattr(st.variables, k).clone() for k in ("uIce", "vIce", "hIceMean", "Area", "Qnet")})
    for k in outs[0]:
        assert torch.equal(outs[0][k], outs[1][k]), k
    h = outs[0]["hIceMean"]
    once = fill_overlap(st, h.clone())
    twice = fill_overlap(st, once.clone())
    assert torch.equal(once, twice)
    rA = st.variables.rA
    s1 = interior_sum(h, rA)
    s2 = interior_sum(h, rA)
    assert torch.equal(s1, s2)
    ref = float((h[2:-2, 2:-2] * rA[2:-2, 2:-2]).sum())
    assert abs(float(s1) - ref) <= 1e-12 * abs(ref)

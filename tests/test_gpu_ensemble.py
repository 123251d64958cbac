"""Batched ensemble: members of uneven sizes advanced by one persistent,
work-queue kernel per subcycle equal the single-domain shared-memory form
bit for bit, under every tile shape, eagerly and as a captured graph."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

SIZES = ((64, 64), (96, 64), (64, 128), (160, 96), (128, 160))
N_SUB = 7


@pytest.fixture(scope="module", autouse=True)
def _lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from veris_gb300 import _abi
    return _abi.load()


def _members(seed=0):
    from veris_gb300.state import VerisState
    from veris_gb300.synthetic import config_settings, make_state
    sett = config_settings("c4_ensemble")
    out = []
    for k, (nx, ny) in enumerate(SIZES):
        arrays = make_state(nx, ny, seed=seed + k, wind_scale=0.5 + 0.25 * k, init_velocity=0.05)
        out.append(VerisState.from_numpy(arrays, sett))
    return out


def _single(member, n):
    from veris_gb300.evp_solver import evp_solver_fast
    return evp_solver_fast(member, "f32", form="smem", n_subcycles=n)


@pytest.mark.parametrize("shape", (0, 1, 2, 3))
def test_batch_equals_single_domain(shape):
    """Shared-memory tiles: bit for bit the single-domain shared-memory form."""
    from veris_gb300.ensemble import EVP_STATE, Ensemble
    members = _members()
    ens = Ensemble(members, N_SUB, shape=shape, blocks_per_sm=2)
    ens.step()
    torch.cuda.synchronize()
    for m, st in enumerate(members):
        ref = _single(st, N_SUB)
        got = ens.state(m)
        for k, r in zip(EVP_STATE, ref):
            assert torch.equal(got[k], r), (shape, m, k, float((got[k] - r).abs().max()))


@pytest.mark.parametrize("shape", (4, 5, 6))
def test_batch_walks_equal_single_domain_walks(shape):
    """Register walks: bit for bit the single-domain walking form with the
    same walk length."""
    from veris_gb300.ensemble import EVP_STATE, SHAPES, Ensemble
    from veris_gb300.evp_solver import evp_solver_fast
    members = _members()
    ens = Ensemble(members, N_SUB, shape=shape, blocks_per_sm=3)
    ens.step()
    torch.cuda.synchronize()
    for m, st in enumerate(members):
        ref = evp_solver_fast(st, "f32", "walk", n_subcycles=N_SUB, rows=SHAPES[shape][0], variant=2)
        got = ens.state(m)
        for k, r in zip(EVP_STATE, ref):
            assert torch.equal(got[k], r), (shape, m, k, float((got[k] - r).abs().max()))


def test_graph_steps_equal_eager_steps():
    from veris_gb300.ensemble import EVP_STATE, Ensemble
    a = Ensemble(_members(1), N_SUB, shape=1)
    b = Ensemble(_members(1), N_SUB, shape=1)
    for _ in range(3):
        a.step()
    b.step()            # first step eagerly (no refold), then the captured one
    b.capture()
    b.step()
    b.step()
    torch.cuda.synchronize()
    assert a.buf == b.buf
    for m in range(len(SIZES)):
        sa, sb = a.state(m), b.state(m)
        for k in EVP_STATE:
            assert torch.equal(sa[k], sb[k]), (m, k)


def test_refold_matches_a_fresh_single_domain_step():
    """After one ensemble step the refold re-forms the momentum constant from
    the new velocities, as a new single-domain call's preparation does (up to
    the float32 rounding of that fold)."""
    from veris_gb300.ensemble import EVP_STATE, Ensemble
    members = _members(2)
    ens = Ensemble(members, N_SUB, shape=0)
    ens.step()
    # the single-domain path: write the first step's result back, solve again
    for m, st in enumerate(members):
        s1 = ens.state(m, dtype=torch.float64)
        for k in EVP_STATE:
            getattr(st.variables, k).copy_(s1[k])
    ens.step()
    for m, st in enumerate(members):
        ref = _single(st, N_SUB)
        got = ens.state(m)
        for k, r in zip(EVP_STATE, ref):
            scale = float(r.abs().max()) or 1.0
            assert float((got[k] - r).abs().max()) <= 1e-5 * scale, (m, k)


def test_autotune_picks_a_candidate_and_restores_the_state(tmp_path, monkeypatch):
    from veris_gb300 import autotune
    from veris_gb300.ensemble import EVP_STATE, Ensemble
    monkeypatch.setenv("VERIS_TUNE_CACHE", str(tmp_path / "tune.json"))
    ens = Ensemble(_members(3), N_SUB)
    ens.step()
    before = [ens.state(m) for m in range(len(SIZES))]
    res = autotune.tune(ens, candidates=((0, 2), (1, 3), (3, 4)), subcycles=3, repeats=2)
    assert (res["shape"], res["blocks_per_sm"]) in ((0, 2), (1, 3), (3, 4))
    assert not res["cached"] and len(res["trials"]) == 3
    for m in range(len(SIZES)):
        after = ens.state(m)
        for k in EVP_STATE:
            assert torch.equal(before[m][k], after[k])
    again = autotune.tune(ens, candidates=((0, 2), (1, 3), (3, 4)))
    assert again["cached"] and again["shape"] == res["shape"]


FIELDS = ("uIce", "vIce", "hIceMean", "hSnowMean", "Area", "TSurf", "Qnet")


def _member_arrays(seed=0):
    from veris_gb300.synthetic import make_state
    return [make_state(nx, ny, seed=seed + k, wind_scale=0.5 + 0.25 * k, init_velocity=0.05)
            for k, (nx, ny) in enumerate(SIZES)]


def test_full_steps_advance_every_member_like_a_single_domain_step():
    """Whole steps (per-member preparation, the batched EVP, per-member ocean
    stress, advection, clean-up, Growth and fills on parallel branches): each
    member equals a single-domain float32 engine step whose EVP is the same
    shared-memory tile (fed through the engine's external-EVP input) bit for
    bit, and the float64 oracle's step to float32 tolerance."""
    import copy
    from types import SimpleNamespace
    from oracle import veris_oracle as O
    from veris_gb300.engine import SeaIceStep
    from veris_gb300.ensemble import Ensemble
    from veris_gb300.evp_solver import evp_solver_fast
    from veris_gb300.state import VerisState
    from veris_gb300.synthetic import config_settings
    sett = config_settings("c4_ensemble", nEVPsteps=N_SUB)
    arrays = _member_arrays()
    members = [VerisState.from_numpy(a, sett) for a in arrays]
    ens = Ensemble(members, N_SUB, shape=0, blocks_per_sm=2, full_step=True, branches=3)
    ens.step()
    torch.cuda.synchronize()
    for m, a in enumerate(arrays):
        st = VerisState.from_numpy(a, sett)
        eng = SeaIceStep(st, precision="f32", evp="external", check_finite=False)
        eng._enqueue_prep()
        for t, r in zip(eng.evp_out32, evp_solver_fast(st, "f32", form="smem", n_subcycles=N_SUB)):
            t.copy_(r)
        eng._enqueue_evp()
        eng._enqueue_post()
        ref = SimpleNamespace(variables=SimpleNamespace(**{k: v.copy() for k, v in a.items()}),
                              settings=copy.copy(sett))
        O.step(ref)
        torch.cuda.synchronize()
        for k in FIELDS:
            got = getattr(members[m].variables, k)
            assert torch.equal(got, getattr(st.variables, k)), (m, k)
            b = getattr(ref.variables, k)
            e = float(np.abs(got.cpu().numpy() - b).max() / max(np.abs(b).max(), 1e-300))
            assert e <= 1e-4, (m, k, e)


def test_full_steps_graph_equals_eager():
    from veris_gb300.ensemble import Ensemble
    from veris_gb300.state import VerisState
    from veris_gb300.synthetic import config_settings
    sett = config_settings("c4_ensemble", nEVPsteps=N_SUB)
    arrays = _member_arrays(5)
    a = Ensemble([VerisState.from_numpy(x, sett) for x in arrays], N_SUB, shape=6, full_step=True, branches=4)
    b = Ensemble([VerisState.from_numpy(x, sett) for x in arrays], N_SUB, shape=6, full_step=True, branches=4)
    for _ in range(3):
        a.step()
    b.step()
    b.capture()
    b.step()
    b.step()
    torch.cuda.synchronize()
    for m in range(len(arrays)):
        for k in FIELDS:
            assert torch.equal(getattr(a.members[m].variables, k), getattr(b.members[m].variables, k)), (m, k)

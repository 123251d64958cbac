"""Dot-product tests of the hand-written adjoint kernels.

For each routine y = f(x) of the step and random x-directions dx and
y-weights w: <J dx, w> = <dx, J^T w>, with J dx the exact tangent of the
oracle's restatement of the routine (forward-mode derivatives through NumPy,
tests/tangent.py, itself checked against centred differences on the CPU) and
J^T w from the GPU adjoint kernel.  No finite differences, no step size: the
two sides agree to rounding (bar 1e-10 of the magnitude of the terms).
Routines: the dynamics preparation (SeaIceMass, AreaWS, WindForcingXY,
SeaIceStrength), the EVP loop (3 subcycles: every input state field and
step-constant field), advection, clean-up with ridging, and Growth with
solve4temp.  States: the reference's own recorded states (golden fixtures),
jittered off exact ties, directions off the branch switches as in
tests/transpose_cases.py.
"""
import numpy as np
import pytest

from tests.transpose_cases import CASES, directions, golden_state, jitter, tangent

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-10


@pytest.fixture(scope="module", autouse=True)
def _lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from veris_gb300 import _abi
    return _abi.load()


def _adjoint(case, gst, lam):
    from veris_gb300 import adjoint as A
    if case == "prep":
        out, _scal = A.prep_adjoint(gst, lam)
        return out
    if case == "advection":
        fields, vel = A.advection_adjoint(gst, lam)
        return dict(fields, **vel)
    if case == "cleanup":
        return A.cleanup_adjoint(gst, lam)
    if case == "growth":
        return A.growth_adjoint(gst, lam)
    if case == "evp":
        state, fields, _drag = A.evp_adjoint(gst, lam, n_subcycles=3)
        return dict(state, **fields)
    raise KeyError(case)


@pytest.mark.parametrize("golden", ["moving", "c1", "small_b"])
@pytest.mark.parametrize("case", list(CASES))
def test_adjoint_is_the_transpose_of_the_tangent(case, golden):
    from veris_gb300.state import VerisState
    if case == "evp" and golden == "small_b":
        pytest.skip("second-order boundary terms: the EVP adjoint covers the fast form's settings")
    rng = np.random.default_rng(5)
    st = jitter(golden_state(case, golden), rng)
    _routine, ins, outs, _f = CASES[case]
    dx = directions(st, ins, rng)
    jd = tangent(case, st, dx)
    w = {k: rng.standard_normal(jd[k].shape) for k in outs}
    lhs_terms = [w[k] * jd[k] for k in outs]
    lhs = sum(float(t.sum()) for t in lhs_terms)

    gst = VerisState.from_numpy(vars(st.variables), st.settings)
    lam = {k: torch.as_tensor(w[k], device="cuda") for k in outs}
    adj = _adjoint(case, gst, lam)
    torch.cuda.synchronize()
    rhs_terms = [dx[k] * adj[k].cpu().numpy() for k in ins]
    rhs = sum(float(t.sum()) for t in rhs_terms)
    mag = sum(float(np.abs(t).sum()) for t in lhs_terms + rhs_terms)
    assert mag > 0
    assert abs(lhs - rhs) <= TOL * mag, f"{case}/{golden}: <J dx, w> {lhs:.12e} <dx, J^T w> {rhs:.12e}"


@pytest.mark.parametrize("golden", ["moving", "c1"])
@pytest.mark.parametrize("form,tape", [(1, False), (2, False), (2, True)])
def test_float32_evp_adjoint_is_the_transpose_to_float32_rounding(golden, form, tape):
    """The float32 EVP adjoint (form 1: the tile kernel; 2: the gather passes,
    which recompute Delta, zeta and cDrag in float32, or with ``tape`` read
    the register walk's own from its tape) against the float64 oracle's exact
    tangent: <J dx, w> = <dx, J^T w> to float32 rounding of the state, the
    linearisation and the adjoint sweep (bar 1e-4 of the magnitude of the
    terms)."""
    from veris_gb300 import _abi
    from veris_gb300 import adjoint as A
    from veris_gb300.state import VerisState
    lib = _abi.load()
    rng = np.random.default_rng(5)
    st = jitter(golden_state("evp", golden), rng)
    _routine, ins, outs, _f = CASES["evp"]
    dx = directions(st, ins, rng)
    jd = tangent("evp", st, dx)
    w = {k: rng.standard_normal(jd[k].shape) for k in outs}
    lhs_terms = [w[k] * jd[k] for k in outs]
    lhs = sum(float(t.sum()) for t in lhs_terms)
    gst = VerisState.from_numpy(vars(st.variables), st.settings)
    lam = {k: torch.as_tensor(w[k], device="cuda") for k in outs}
    try:
        assert lib.veris_evp_adjoint_f32_form(form) == 0
        state, fields, _drag = A.evp_adjoint(gst, lam, n_subcycles=3, precision="f32", tape=tape)
    finally:
        lib.veris_evp_adjoint_f32_form(0)
    adj = dict(state, **fields)
    torch.cuda.synchronize()
    rhs_terms = [dx[k] * adj[k].cpu().numpy() for k in ins]
    rhs = sum(float(t.sum()) for t in rhs_terms)
    mag = sum(float(np.abs(t).sum()) for t in lhs_terms + rhs_terms)
    assert mag > 0
    assert abs(lhs - rhs) <= 1e-4 * mag, \
        f"evp f32 form {form} tape {tape}/{golden}: {lhs:.9e} vs {rhs:.9e} ({abs(lhs - rhs) / mag:.2e})"
    assert lib.veris_evp_adjoint_f32_form(4) != 0


@pytest.mark.parametrize("golden,veros_fill", [("c1", True), ("c1", False), ("moving", True)])
@pytest.mark.parametrize("tape", [False, True])
def test_float32_linked_passes_equal_the_separate_ones(golden, veros_fill, tape):
    """The float32 gather passes with P4 of each subcycle fused with P1 of
    the one before it (form 2) against every pass in its own launch (form
    3), with the x halo or both halos filled (the fused pass evaluates P4 at
    a point's images itself): the same state and field adjoints bit for bit,
    the drag scalars up to the order of their per-warp atomics."""
    from veris_gb300 import _abi
    from veris_gb300 import adjoint as A
    from veris_gb300.state import VerisState
    lib = _abi.load()
    rng = np.random.default_rng(9)
    st = jitter(golden_state("evp", golden), rng)
    st.settings.veros_fill = veros_fill
    _routine, _ins, outs, _f = CASES["evp"]
    gst = VerisState.from_numpy(vars(st.variables), st.settings)
    lam = {k: torch.as_tensor(rng.standard_normal(getattr(st.variables, k).shape), device="cuda") for k in outs}
    res = {}
    try:
        for form in (2, 3):
            assert lib.veris_evp_adjoint_f32_form(form) == 0
            res[form] = A.evp_adjoint(gst, lam, n_subcycles=4, precision="f32", tape=tape)
    finally:
        lib.veris_evp_adjoint_f32_form(0)
    torch.cuda.synchronize()
    (s2, f2, d2), (s3, f3, d3) = res[2], res[3]
    for k in s2:
        assert torch.equal(s2[k], s3[k]), k
    for k in f2:
        assert torch.equal(f2[k], f3[k]), k
    for k in d2:
        a, b = float(d2[k]), float(d3[k])
        assert abs(a - b) <= 1e-12 * max(abs(b), 1e-30), (k, a, b)


def test_evp_adjoint_is_the_transpose_with_both_halos_refreshed():
    """The float64 EVP adjoint with veros_fill off (the x and the y halo
    refreshed after every subcycle): the adjoints of both halos' images go
    back to their sources; against the oracle's exact tangent to 1e-10."""
    from veris_gb300.state import VerisState
    rng = np.random.default_rng(7)
    st = jitter(golden_state("evp", "c1"), rng)
    st.settings.veros_fill = False
    _routine, ins, outs, _f = CASES["evp"]
    dx = directions(st, ins, rng)
    jd = tangent("evp", st, dx)
    w = {k: rng.standard_normal(jd[k].shape) for k in outs}
    lhs_terms = [w[k] * jd[k] for k in outs]
    lhs = sum(float(t.sum()) for t in lhs_terms)
    gst = VerisState.from_numpy(vars(st.variables), st.settings)
    lam = {k: torch.as_tensor(w[k], device="cuda") for k in outs}
    adj = _adjoint("evp", gst, lam)
    torch.cuda.synchronize()
    rhs_terms = [dx[k] * adj[k].cpu().numpy() for k in ins]
    rhs = sum(float(t.sum()) for t in rhs_terms)
    mag = sum(float(np.abs(t).sum()) for t in lhs_terms + rhs_terms)
    assert abs(lhs - rhs) <= TOL * mag, f"{lhs:.12e} vs {rhs:.12e}"

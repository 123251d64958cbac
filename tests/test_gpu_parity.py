"""GPU float64 drop-ins against the golden fixtures (made by running the
reference) and against the CPU oracle.

Bar: 1e-10 relative max-norm (max |gpu - ref| / max |ref|) for every output
of every routine, and for one or two full steps.
"""
import numpy as np
import pytest

from tests import golden_io as G

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-10


@pytest.fixture(scope="module", autouse=True)
def _lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from veris_gb300 import _abi
    return _abi.load()


def to_gpu(st):
    from veris_gb300.state import VerisState
    return VerisState.from_numpy(vars(st.variables), st.settings)


def cpu(t):
    return t.detach().cpu().numpy()


def assert_close(got, ref, what, tol=TOL):
    got = cpu(got) if hasattr(got, "detach") else np.asarray(got)
    assert np.all(np.isfinite(got)), f"{what}: non-finite values"
    e = G.rel_err(got, ref)
    assert e <= tol, f"{what}: relative max-norm error {e:.3e} > {tol:.0e}"


@pytest.mark.parametrize("case", G.CASES)
def test_step_sequence(case):
    from veris_gb300 import model
    g = G.load(case)
    st = to_gpu(G.initial_state(g))
    seq = G.sequence(g)
    got = []
    n_steps = sum(1 for _i, r, _o in seq if r == "SeaIceMass")
    for _ in range(n_steps):
        model.step(st, record=lambda name, outs: got.append((name, {k: cpu(v) for k, v in outs.items()})))
    assert [r for _i, r, _o in seq] == [n for n, _o in got]
    for (i, r, ref), (_n, outs) in zip(seq, got):
        for k, a in ref.items():
            assert_close(outs[k], a, f"{case} call {i} {r}.{k}")


@pytest.mark.parametrize("case", G.CASES)
def test_each_routine_from_recorded_state(case):
    """Every routine of the step, each from the reference's own input state."""
    from veris_gb300 import model
    g = G.load(case)
    fns = {name: fn for name, fn, _o in model.STEP}
    for i, r, ref in G.sequence(g):
        if r == "fill_overlap":
            continue
        st = to_gpu(G.state_before(g, i))
        vals = fns[r](st)
        if not isinstance(vals, tuple):
            vals = (vals,)
        for (k, a), v in zip(ref.items(), vals):
            assert_close(v, a, f"{case} call {i} {r}.{k}")


@pytest.mark.parametrize("case", G.CASES)
def test_inner_routines(case):
    from veris_gb300 import dynamics_routines as D, averaging, dynsolver, evp_solver
    g = G.load(case)
    first_evp = [i for i, r, _o in G.sequence(g) if r == "IceVelocities"][0]
    st = to_gpu(G.state_before(g, first_evp))
    v = st.variables
    ref = G.sub(g, "strainrates")
    for k, a in zip(("e11", "e22", "e12"), D.strainrates(st, v.uIce, v.vIce)):
        assert_close(a, ref[k], f"{case} strainrates.{k}")
    e = [torch.as_tensor(ref[k]).cuda() for k in ("e11", "e22", "e12")]
    ref = G.sub(g, "viscosities")
    for k, a in zip(("zeta", "eta", "press"), D.viscosities(st, *e)):
        assert_close(a, ref[k], f"{case} viscosities.{k}")
    zeta = torch.as_tensor(ref["zeta"]).cuda()
    assert_close(averaging.c_point_to_z_point(st, zeta), G.sub(g, "c_point_to_z_point")["zetaZ"],
                 f"{case} c_point_to_z_point")
    assert_close(D.ocean_drag_coeffs(st, v.uIce, v.vIce), G.sub(g, "ocean_drag_coeffs")["cDrag"],
                 f"{case} ocean_drag_coeffs")
    assert_close(D.basal_drag_coeffs(st, v.uIce, v.vIce), G.sub(g, "basal_drag_coeffs")["cBot"],
                 f"{case} basal_drag_coeffs")
    ref = G.sub(g, "side_drag")
    sU, sV = D.side_drag(st, v.uIce, v.vIce)
    assert_close(sU, ref["SideDragU"], f"{case} side_drag.U")
    assert_close(sV, ref["SideDragV"], f"{case} side_drag.V")
    ref = G.sub(g, "stressdiv")
    dX, dY = D.stressdiv(st, v.sigma1, v.sigma2, v.sigma12)
    assert_close(dX, ref["stressDivX"], f"{case} stressdiv.X")
    assert_close(dY, ref["stressDivY"], f"{case} stressdiv.Y")
    ref = G.sub(g, "tauXY")
    tX, tY = dynsolver.tauXY(st)
    assert_close(tX, ref["tauX"], f"{case} tauXY.X")
    assert_close(tY, ref["tauY"], f"{case} tauXY.Y")
    ref = G.sub(g, "evp_1")
    out = evp_solver.evp_solver(st, n_subcycles=1)
    for k, a in zip(("uIce", "vIce", "sigma1", "sigma2", "sigma12"), out):
        assert_close(a, ref[k], f"{case} evp_1.{k}")


@pytest.mark.parametrize("case", G.CASES)
def test_advection_and_thermo_routines(case):
    from veris_gb300 import advection as A, solve4temp as S
    g = G.load(case)
    seq = G.sequence(g)
    adv = [i for i, r, _o in seq if r == "Advection"][0]
    st = to_gpu(G.state_before(g, adv))
    v = st.variables
    uT = v.uIce * v.dyG * v.iceMaskU
    vT = v.vIce * v.dxG * v.iceMaskV
    assert_close(A.calc_ZonalFlux(st, v.hIceMean, uT), G.sub(g, "calc_ZonalFlux")["ZonalFlux"],
                 f"{case} calc_ZonalFlux")
    assert_close(A.calc_MeridionalFlux(st, v.hIceMean, vT),
                 G.sub(g, "calc_MeridionalFlux")["MeridionalFlux"], f"{case} calc_MeridionalFlux")
    assert_close(A.calc_Advection(st, v.Area), G.sub(g, "calc_Advection")["field"],
                 f"{case} calc_Advection")
    lim = G.sub(g, "limiter")
    assert_close(A.limiter(torch.as_tensor(lim["Cr"]).cuda()), lim["phi"], f"{case} limiter", tol=0)

    gr = [i for i, r, _o in seq if r == "Growth"][0]
    st = to_gpu(G.state_before(g, gr))
    v, s = st.variables, st.settings
    ref = G.sub(g, "solve4temp")
    TF = s.tempFrz + s.dtempFrz_dS * v.ocSalt + s.celsius2K
    out = S.solve4temp(st, torch.as_tensor(ref["in_hIceActual"]).cuda(),
                       torch.as_tensor(ref["in_hSnowActual"]).cuda(), v.TSurf, TF)
    for k, a in zip(("TSurfOut", "F_io_net", "F_ia_net", "IcePenetSW", "FWsublim"), out):
        assert_close(a, ref[k], f"{case} solve4temp.{k}")


def test_global_sum_deterministic():
    from veris_gb300.global_sum import interior_sum
    x = torch.rand(1444, 724, dtype=torch.float64, device="cuda")
    s1 = interior_sum(x).item()
    s2 = interior_sum(x).item()
    assert s1 == s2
    ref = x[2:-2, 2:-2].double().sum().item()
    assert abs(s1 - ref) <= 1e-12 * abs(ref)

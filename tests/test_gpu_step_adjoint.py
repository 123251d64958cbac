"""Hand-written adjoints of the step's routines and of whole trajectories
against centred finite differences of the same float64 forward.

For a routine y = f(x) and random weights W, L = <W, y>; along a direction d
the adjoint's <dL/dx, d> must match (L(x + h d) - L(x - h d)) / 2h.  The
directions avoid the points where a routine has a kink at the state itself
(max(x, 0) at x = 0, a limiter ratio with a zero denominator): a centred
difference there measures the mean of two one-sided slopes, not a derivative.
"""
import numpy as np
import pytest

from tests import golden_io as G

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

H = 1e-6
TOL = 2e-6


@pytest.fixture(scope="module", autouse=True)
def _lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from veris_gb300 import _abi
    return _abi.load()


def _state(case, routine, call=0):
    """The reference's state just before its ``call``-th call of ``routine``."""
    from veris_gb300.state import VerisState
    g = G.load(case)
    idx = [i for i, r, _o in G.sequence(g) if r == routine][call]
    st = G.state_before(g, idx)
    return VerisState.from_numpy(vars(st.variables), st.settings)


def _jitter(st, rng, names=("hIceMean", "hSnowMean", "Area"), eps=1e-3):
    """Break exact ties (flat fields give zero limiter denominators)."""
    v = st.variables
    for n in names:
        x = getattr(v, n)
        setattr(v, n, x + eps * torch.as_tensor(rng.random(tuple(x.shape)), device=x.device) * (x > 0))


def _check(fd, ad, what, floor=1e-12):
    """``floor``: the rounding noise of the difference quotient itself."""
    assert abs(fd - ad) <= TOL * max(abs(fd), abs(ad)) + floor, f"{what}: fd {fd:.9e} ad {ad:.9e}"


def _noise(W, outs, scale, h=H):
    """Rounding noise of (L+ - L-) / 2h for L = <W, y>: eps * sum|W y| / (h scale), x100."""
    s = sum(float((w * o).abs().sum()) for w, o in zip(W, outs))
    return 100 * 2.2e-16 * s / (h * scale)


def _fd(loss, st, name, d, scale, h=H):
    v = st.variables
    x0 = getattr(v, name).clone()
    setattr(v, name, x0 + h * scale * d)
    lp = loss(st)
    setattr(v, name, x0 - h * scale * d)
    lm = loss(st)
    setattr(v, name, x0)
    return (lp - lm) / (2 * h * scale)


def _rand(rng, like):
    return torch.as_tensor(rng.standard_normal(tuple(like.shape)), device=like.device)


def test_fill_adjoint_is_the_transpose():
    from veris_gb300.adjoint import fill_overlap_adjoint
    from veris_gb300.fill_overlap import fill_overlap
    rng = np.random.default_rng(1)
    for case in ("c1", "small_b"):
        st = _state(case, "SeaIceMass")
        x = _rand(rng, st.variables.iceMask)
        y = _rand(rng, st.variables.iceMask)
        lhs = float((fill_overlap(st, x.clone()) * y).sum())
        rhs = float((x * fill_overlap_adjoint(st, y)).sum())
        assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), 1.0), (case, lhs, rhs)


@pytest.mark.parametrize("case,call", (("moving", 0), ("moving", 1), ("c1", 1)))
def test_advection_adjoint(case, call):
    from veris_gb300.adjoint import advection_adjoint
    from veris_gb300.advection import Advection
    rng = np.random.default_rng(2)
    st = _state(case, "Advection", call)
    _jitter(st, rng)
    v = st.variables
    W = [_rand(rng, v.iceMask) for _ in range(3)]
    loss = lambda s: sum(float((w * o).sum()) for w, o in zip(W, Advection(s)))
    outs = Advection(st)
    lin, luv = advection_adjoint(st, dict(zip(("hIceMean", "hSnowMean", "Area"), W)))
    grads = dict(lin, **luv)
    for name in ("hIceMean", "hSnowMean", "Area", "uIce", "vIce"):
        x = getattr(v, name)
        tracer = name in ("hIceMean", "hSnowMean", "Area")
        # a face between two zero cells has a zero limiter denominator: keep
        # the tracer perturbations on the nonzero cells; the limiter ratios
        # of small tracer differences move fast, so the tracer step is
        # smaller (at 1e-6 x max a few faces cross a superbee breakpoint)
        d = _rand(rng, x) * ((x != 0) if tracer else 1)
        scale = float(x.abs().max()) or 1.0
        h = H / 10 if tracer else H
        _check(_fd(loss, st, name, d, scale, h), float((grads[name] * d).sum()), f"{case} {name}",
               floor=_noise(W, outs, scale, h))


def _safe_ice(v):
    """Points away from the clean-up's and Growth's clipping thresholds."""
    return ((v.hIceMean > 0.05) & (v.hSnowMean > 1e-3) & (v.Area > 0.05) & (v.Area < 0.95)
            & (v.iceMask > 0)).to(torch.float64)


@pytest.mark.parametrize("case", ("moving", "c1", "small_a"))
def test_cleanup_adjoint(case):
    from veris_gb300.adjoint import cleanup_adjoint
    from veris_gb300.clean_up import clean_up_advection, ridging
    rng = np.random.default_rng(3)
    st = _state(case, "clean_up_advection")
    v = st.variables
    W = [_rand(rng, v.iceMask) for _ in range(4)]

    def loss(s):
        h, hs, A, T, _a, _b = clean_up_advection(s)
        keep = (s.variables.hIceMean, s.variables.hSnowMean, s.variables.Area, s.variables.TSurf)
        s.variables.hIceMean, s.variables.hSnowMean, s.variables.Area, s.variables.TSurf = h, hs, A, T
        A2 = ridging(s)
        s.variables.hIceMean, s.variables.hSnowMean, s.variables.Area, s.variables.TSurf = keep
        return sum(float((w * o).sum()) for w, o in zip(W, (h, hs, A2, T)))

    g = cleanup_adjoint(st, dict(zip(("hIceMean", "hSnowMean", "Area", "TSurf"), W)))
    m = _safe_ice(v)
    for name in ("hIceMean", "hSnowMean", "Area", "TSurf"):
        x = getattr(v, name)
        d = _rand(rng, x) * m
        scale = float(x.abs().max()) or 1.0
        _check(_fd(loss, st, name, d, scale), float((g[name] * d).sum()), f"{case} {name}")


@pytest.mark.parametrize("case", ("moving", "c1", "small_a", "small_b"))
def test_growth_adjoint(case):
    from veris_gb300.adjoint import growth_adjoint
    from veris_gb300.growth import Growth
    rng = np.random.default_rng(4)
    st = _state(case, "Growth")
    v = st.variables
    W = [_rand(rng, v.iceMask) for _ in range(4)]
    loss = lambda s: sum(float((w * o).sum()) for w, o in zip(W, Growth(s)[:4]))
    outs = Growth(st)[:4]
    g = growth_adjoint(st, dict(zip(("hIceMean", "hSnowMean", "Area", "TSurf"), W)))
    m = _safe_ice(v)
    for name in ("hIceMean", "hSnowMean", "Area", "TSurf"):
        x = getattr(v, name)
        d = _rand(rng, x) * m
        scale = float(x.abs().max()) or 1.0
        _check(_fd(loss, st, name, d, scale), float((g[name] * d).sum()), f"{case} {name}",
               floor=_noise(W, outs, scale))


@pytest.mark.parametrize("case,call", (("moving", 0), ("moving", 1), ("c1", 1)))
def test_prep_adjoint(case, call):
    from veris_gb300 import area_mass, dynamics_routines, dynsolver
    from veris_gb300.adjoint import PREP_OUT, prep_adjoint
    rng = np.random.default_rng(5)
    st = _state(case, "SeaIceMass", call)
    v = st.variables
    W = {k: _rand(rng, v.iceMask) for k in PREP_OUT}

    def outputs(s):
        o = {}
        o["SeaIceMassC"], o["SeaIceMassU"], o["SeaIceMassV"] = area_mass.SeaIceMass(s)
        o["AreaW"], o["AreaS"] = area_mass.AreaWS(s)
        keep = {k: getattr(s.variables, k) for k in ("SeaIceMassU", "SeaIceMassV", "AreaW", "AreaS")}
        for k in keep:
            setattr(s.variables, k, o[k])
        o["WindForcingX"], o["WindForcingY"] = dynsolver.WindForcingXY(s)
        for k, t in keep.items():
            setattr(s.variables, k, t)
        o["SeaIceStrength"] = dynamics_routines.SeaIceStrength(s)
        return o

    loss = lambda s: sum(float((W[k] * t).sum()) for k, t in outputs(s).items())
    g, scal = prep_adjoint(st, W)
    for name in ("hIceMean", "hSnowMean", "Area"):
        x = getattr(v, name)
        d = _rand(rng, x)
        scale = float(x.abs().max()) or 1.0
        _check(_fd(loss, st, name, d, scale), float((g[name] * d).sum()), f"{case} {name}")
    # the velocities enter the wind forcing only; the other outputs are
    # large and would bury their difference quotient in rounding noise
    Wuv = {k: W[k] for k in ("WindForcingX", "WindForcingY")}
    loss_uv = lambda s: sum(float((Wuv[k] * outputs(s)[k]).sum()) for k in Wuv)
    o = outputs(st)
    guv, _ = prep_adjoint(st, Wuv)
    for name in ("uIce", "vIce"):
        x = getattr(v, name)
        d = _rand(rng, x)
        scale = float(x.abs().max()) or 1.0
        _check(_fd(loss_uv, st, name, d, scale), float((guv[name] * d).sum()), f"{case} {name}",
               floor=_noise(list(Wuv.values()), [o[k] for k in Wuv], scale))
    # each coefficient against the outputs it enters (smaller rounding noise)
    s = st.settings
    for name, pair, outs in (("pStar", ("pStar",), ("SeaIceStrength",)),
                             ("airIceDrag", ("airIceDrag", "airIceDrag_south"), ("WindForcingX", "WindForcingY"))):
        Wc = {k: W[k] for k in outs}
        _g, sc = prep_adjoint(st, Wc)
        lossc = lambda st_: sum(float((Wc[k] * outputs(st_)[k]).sum()) for k in Wc)
        base = {k: getattr(s, k) for k in pair}
        hs = H * base[pair[0]]
        for k in pair:
            setattr(s, k, base[k] + hs)
        lp = lossc(st)
        for k in pair:
            setattr(s, k, base[k] - hs)
        lm = lossc(st)
        for k in pair:
            setattr(s, k, base[k])
        ad = sum(float(sc[k]) for k in pair)
        floor = _noise(list(Wc.values()), [o[k] for k in outs], base[pair[0]])
        _check((lp - lm) / (2 * hs), ad, f"{case} {name}", floor=floor)


# ------------------------------------------------------------- trajectories

N_STEPS = 3
N_SUB = 12


def _trajectory_state(case="moving"):
    from veris_gb300.state import VerisState
    g = G.load(case)
    st = G.initial_state(g)
    return VerisState.from_numpy(vars(st.variables), st.settings)


def test_trajectory_gradients_match_finite_differences():
    from veris_gb300.trajectory import COEFFS, Trajectory, tracking_loss_adjoint
    rng = np.random.default_rng(7)
    st = _trajectory_state()
    v = st.variables
    tr = Trajectory(st, N_STEPS, n_subcycles=N_SUB)
    x0 = {k: getattr(v, k).clone() for k in ("uIce", "vIce", "sigma1", "sigma2", "sigma12",
                                             "hIceMean", "hSnowMean", "Area", "TSurf")}
    target = {k: getattr(v, k) + 0.01 * _rand(rng, v.iceMask) * v.iceMask for k in ("uIce", "vIce", "Area")}
    target = {k: t.clone() for k, t in target.items()}

    def run():
        for k, t in x0.items():
            getattr(v, k).copy_(t)
        tr.forward()
        L, lam = tracking_loss_adjoint(st, target)
        return float(L), lam

    L0, lam = run()
    grads, coeffs, _ = tr.backward(lam)
    m = _safe_ice(v)
    for name in ("hIceMean", "Area", "uIce", "hSnowMean"):
        d = _rand(rng, v.iceMask) * m
        scale = float(x0[name].abs().max()) or 1.0
        base = x0[name].clone()
        x0[name] = base + H * scale * d
        lp, _ = run()
        x0[name] = base - H * scale * d
        lm, _ = run()
        x0[name] = base
        _check((lp - lm) / (2 * H * scale), float((grads[name] * d).sum()), f"trajectory d/d {name}")
    s = st.settings
    for name in COEFFS:
        c0 = getattr(s, name)
        hs = H * c0
        tr.set_coefficients(**{name: c0 + hs})
        lp, _ = run()
        tr.set_coefficients(**{name: c0 - hs})
        lm, _ = run()
        tr.set_coefficients(**{name: c0})
        _check((lp - lm) / (2 * hs), float(coeffs[name]), f"trajectory d/d {name}")


def test_trajectory_checkpointing_is_exact():
    """Fewer snapshots recompute steps, and the EVP tape skips the subcycle
    recomputation, but all give the same gradients."""
    from veris_gb300.trajectory import CARRIED, Trajectory
    rng = np.random.default_rng(8)
    st = _trajectory_state()
    v = st.variables
    x0 = {k: getattr(v, k).clone() for k in CARRIED}
    lam = {k: _rand(rng, v.iceMask) for k in ("uIce", "vIce", "Area", "hIceMean")}
    out = []
    for snaps, tape in ((None, False), (1, False), (0, False), (None, True)):
        for k, t in x0.items():
            getattr(v, k).copy_(t)
        tr = Trajectory(st, 5, n_subcycles=N_SUB, snapshots=snaps, evp_checkpoint_every=0 if snaps else 4,
                        tape=tape)
        assert (tr.tapes is not None) == tape
        tr.forward()
        g, c, _ = tr.backward(lam)
        out.append((g, c, dict(tr.stats)))
    assert out[0][2]["recomputed_steps"] == 0 and out[3][2]["recomputed_steps"] == 0
    assert out[1][2]["recomputed_steps"] > 0 and out[2][2]["recomputed_steps"] > out[1][2]["recomputed_steps"]
    for g, c, _ in out[1:]:
        for k in CARRIED:
            e = G.rel_err(g[k].cpu().numpy(), out[0][0][k].cpu().numpy())
            assert e <= 1e-12, (k, e)
        for k in c:
            assert abs(float(c[k]) - float(out[0][1][k])) <= 1e-12 * max(abs(float(out[0][1][k])), 1e-30), k


def test_trajectory_autograd_function():
    from veris_gb300.trajectory import COEFFS, Trajectory, sea_ice_trajectory
    rng = np.random.default_rng(9)
    st = _trajectory_state()
    v = st.variables
    s = st.settings
    tr = Trajectory(st, 2, n_subcycles=N_SUB)
    x0 = {k: getattr(v, k).clone() for k in ("uIce", "vIce", "sigma1", "sigma2", "sigma12", "hSnowMean", "TSurf")}
    h0 = v.hIceMean.clone().requires_grad_(True)
    A0 = v.Area.clone().requires_grad_(True)
    c = torch.tensor([float(getattr(s, k)) for k in COEFFS], dtype=torch.float64, device="cuda",
                     requires_grad=True)
    u, vv, A = sea_ice_trajectory(tr, h0, A0, c)
    W = [_rand(rng, v.iceMask) for _ in range(3)]
    L = sum((w * o).sum() for w, o in zip(W, (u, vv, A)))
    L.backward()
    assert h0.grad is not None and A0.grad is not None and c.grad is not None
    assert torch.isfinite(h0.grad).all() and torch.isfinite(c.grad).all()
    # the same numbers through Trajectory.backward
    for k, t in x0.items():
        getattr(v, k).copy_(t)
    v.hIceMean.copy_(h0.detach())
    v.Area.copy_(A0.detach())
    tr.forward()
    g, cg, _ = tr.backward({"uIce": W[0], "vIce": W[1], "Area": W[2]})
    assert G.rel_err(h0.grad.cpu().numpy(), g["hIceMean"].cpu().numpy()) <= 1e-12
    assert G.rel_err(A0.grad.cpu().numpy(), g["Area"].cpu().numpy()) <= 1e-12


@pytest.mark.parametrize("rows,variant", ((0, 0), (16, 1), (32, 2), (8, 3)))
def test_float32_tape_is_the_walks_trajectory(rows, variant):
    """The float32 tape (veris_evp_fast_tape_f32, automatic walk length,
    variant 0) holds the states the engine's tuned walk computes: its final
    state equals the walk solver's bit for bit for any walk length and
    register variant, so a tape written during the reverse sweep linearises
    the forward's own trajectory."""
    import ctypes
    from veris_gb300.evp_solver import evp_solver_fast
    from veris_gb300.state import Call
    from veris_gb300._abi import check
    st = _trajectory_state()
    want = evp_solver_fast(st, "f32", form="walk", n_subcycles=N_SUB, rows=rows, variant=variant)
    c = Call(st)
    g = c.refs()[0]
    tape = torch.empty(int(c.lib.veris_evp_tape_bytes(g, 4, N_SUB)) // 4, dtype=torch.float32, device=c.device)
    out = [torch.empty(c.shape, dtype=torch.float32, device=c.device) for _ in range(5)]
    ws, wsb = c.workspace(c.lib.veris_evp_fast_workspace_bytes(g, 4))
    check("evp_tape_f32", c.lib.veris_evp_fast_tape_f32(*c.refs(), N_SUB, *[t.data_ptr() for t in out],
                                                         tape.data_ptr(), tape.numel() * 4, ws, wsb, c.stream))
    torch.cuda.synchronize()
    for a, b in zip(out, want):
        assert torch.equal(a, b)


def test_float32_step_tape_gives_the_all_steps_gradients():
    """tape="step" (one step's tape written by the walk during the reverse)
    against the tapes of all steps written during the forward: the same
    state gradients bit for bit and the same coefficient gradients up to the
    order of the per-warp drag sums' atomics, with the gather passes (the
    tile kernel this small grid would take sums with shared-memory atomics,
    so no two of its runs agree bit for bit); the shared-memory recompute
    (tape off) within float32 rounding of them."""
    from veris_gb300 import _abi
    from veris_gb300.trajectory import Trajectory, tracking_loss_adjoint
    lib = _abi.load()
    assert lib.veris_evp_adjoint_f32_form(2) == 0
    try:
        _step_tape_case()
    finally:
        lib.veris_evp_adjoint_f32_form(0)


def _step_tape_case():
    from veris_gb300.trajectory import Trajectory, tracking_loss_adjoint
    rng = np.random.default_rng(11)
    st = _trajectory_state()
    v = st.variables
    names = ("uIce", "vIce", "sigma1", "sigma2", "sigma12", "hIceMean", "hSnowMean", "Area", "TSurf")
    x0 = {k: getattr(v, k).clone() for k in names}
    target = {k: (getattr(v, k) + 0.01 * _rand(rng, v.iceMask) * v.iceMask).clone() for k in ("uIce", "vIce", "Area")}
    res = {}
    for tape in (True, "step", False):
        for k, t in x0.items():
            getattr(v, k).copy_(t)
        tr = Trajectory(st, N_STEPS, n_subcycles=N_SUB, precision="f32", tape=tape)
        assert tr.tape_mode == {True: "all", "step": "step", False: "off"}[tape]
        tr.forward()
        L, lam = tracking_loss_adjoint(st, target)
        res[tape] = tr.backward(lam)
    (ga, ca, _), (gs, cs, _), (go, co, _) = res[True], res["step"], res[False]
    for k in ga:
        assert torch.equal(ga[k], gs[k]), k
    for k in ca:
        assert abs(float(cs[k]) - float(ca[k])) <= 1e-12 * max(abs(float(ca[k])), 1e-30), (k, cs[k], ca[k])
        assert abs(float(co[k]) - float(ca[k])) <= 5e-3 * max(abs(float(ca[k])), 1e-30), (k, co[k], ca[k])


@pytest.mark.parametrize("tape", (True, False))
def test_float32_trajectory_gradients(tape):
    """The float32 trajectory (float32 EVP and advection forward, float32 EVP
    adjoint): its gradients against the float64 ones (1e-2), and dL/dP*
    against a centred difference of its own forward with a step large enough
    for float32 rounding."""
    from veris_gb300.trajectory import Trajectory, tracking_loss_adjoint
    rng = np.random.default_rng(10)
    st = _trajectory_state()
    v = st.variables
    names = ("uIce", "vIce", "sigma1", "sigma2", "sigma12", "hIceMean", "hSnowMean", "Area", "TSurf")
    x0 = {k: getattr(v, k).clone() for k in names}
    target = {k: (getattr(v, k) + 0.01 * _rand(rng, v.iceMask) * v.iceMask).clone() for k in ("uIce", "vIce", "Area")}
    grads = {}
    for prec in ("f64", "f32"):
        for k, t in x0.items():
            getattr(v, k).copy_(t)
        tr = Trajectory(st, N_STEPS, n_subcycles=N_SUB, precision=prec, tape=tape)
        tr.forward()
        L, lam = tracking_loss_adjoint(st, target)
        grads[prec] = tr.backward(lam)
    g64, c64, _ = grads["f64"]
    g32, c32, _ = grads["f32"]
    for name in ("pStar", "airIceDrag", "waterIceDrag"):
        a, b = float(c32[name]), float(c64[name])
        assert abs(a - b) <= 1e-2 * max(abs(b), 1e-30), (name, a, b)
    m = _safe_ice(v)
    d = _rand(rng, v.iceMask) * m
    a, b = float((g32["hIceMean"] * d).sum()), float((g64["hIceMean"] * d).sum())
    assert abs(a - b) <= 1e-2 * max(abs(b), 1e-30), ("hIceMean", a, b)
    # centred difference of the float32 forward in P*: this small trajectory's
    # loss moves by ~1e-6 of itself per 1e-3 of P*, where float32 rounding
    # of the state is ~1e-7, so the step is 1e-2 of P*
    s = st.settings
    p0 = s.pStar
    hP = 1e-2 * p0
    Ls = []
    for pv in (p0 + hP, p0 - hP):
        for k, t in x0.items():
            getattr(v, k).copy_(t)
        tr.set_coefficients(pStar=pv)
        tr.forward()
        Ls.append(float(tracking_loss_adjoint(st, target)[0]))
    tr.set_coefficients(pStar=p0)
    fd = (Ls[0] - Ls[1]) / (2 * hP)
    assert abs(fd - float(c32["pStar"])) <= 5e-2 * max(abs(fd), 1e-30), (fd, float(c32["pStar"]))

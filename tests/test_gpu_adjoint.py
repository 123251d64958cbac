"""Hand-written adjoint of the EVP loop against centred finite differences.

Loss L = sum_k <W_k, out_k> over the five outputs of n subcycles with random
weights W_k.  For a direction d in one input X, the adjoint's <dL/dX, d> must
match (L(X + h d) - L(X - h d)) / 2h computed with the same float64 forward.
"""
import numpy as np
import pytest

from tests import golden_io as G

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

N_SUB = 12
H = 1e-6
TOL = 2e-6


@pytest.fixture(scope="module", autouse=True)
def _lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from veris_gb300 import _abi
    return _abi.load()


def _state(case, call=0, **overrides):
    """The reference's input state of its ``call``-th EVP call."""
    from veris_gb300.state import VerisState
    g = G.load(case)
    evp_calls = [i for i, r, _o in G.sequence(g) if r == "IceVelocities"]
    st0 = G.state_before(g, evp_calls[call])
    for k, v in overrides.items():
        setattr(st0.settings, k, v)
    return VerisState.from_numpy(vars(st0.variables), st0.settings)


def _loss(st, W):
    from veris_gb300.evp_solver import evp_solver_fast
    out = evp_solver_fast(st, "f64", n_subcycles=N_SUB)
    return sum(float((w * o).sum()) for w, o in zip(W, out))


def _direction(st, name, rng):
    v = st.variables
    x = getattr(v, name)
    d = torch.as_tensor(rng.standard_normal(tuple(x.shape)), device=x.device)
    if name in ("SeaIceMassU", "SeaIceMassV", "SeaIceMassC", "SeaIceStrength", "AreaW", "AreaS"):
        d = d * (x != 0)    # keep the mass != 0 switches and masks where they are
    scale = float(x.abs().max()) or 1.0
    return d, scale


# c1 starts from rest, where Delta = 0 and zeta = P/deltaMin: a finite
# difference of any affordable size then measures a secant of zeta(Delta),
# not its derivative, so c1 is checked from the start of its second step.
@pytest.mark.parametrize("case,call,fill", (("c1", 1, True), ("moving", 0, True), ("moving", 1, True),
                                            ("c1", 1, False)))
def test_evp_adjoint_matches_finite_differences(case, call, fill):
    """fill False: both halos refreshed after every subcycle (veros_fill off),
    so the adjoint also moves the y-halo images' adjoints to their sources."""
    from veris_gb300.adjoint import evp_adjoint
    rng = np.random.default_rng(5)
    st = _state(case, call, veros_fill=fill)
    shape = tuple(st.variables.iceMask.shape)
    W = [torch.as_tensor(rng.standard_normal(shape), device="cuda") for _ in range(5)]
    lam_in, lam_f, scal = evp_adjoint(st, dict(zip(("uIce", "vIce", "sigma1", "sigma2", "sigma12"), W)),
                                      n_subcycles=N_SUB)
    checks = [("uIce", lam_in["uIce"]), ("vIce", lam_in["vIce"]), ("sigma1", lam_in["sigma1"]),
              ("sigma12", lam_in["sigma12"]), ("SeaIceStrength", lam_f["SeaIceStrength"]),
              ("WindForcingX", lam_f["WindForcingX"]), ("AreaS", lam_f["AreaS"]),
              ("uOcean", lam_f["uOcean"]), ("SeaIceMassU", lam_f["SeaIceMassU"]),
              ("SeaIceMassC", lam_f["SeaIceMassC"])]
    if st.settings.basalDragK2:
        checks.append(("hIceMean", lam_f["hIceMean"]))
    v = st.variables
    for name, lam in checks:
        d, scale = _direction(st, name, rng)
        x0 = getattr(v, name).clone()
        setattr(v, name, x0 + H * scale * d)
        lp = _loss(st, W)
        setattr(v, name, x0 - H * scale * d)
        lm = _loss(st, W)
        setattr(v, name, x0)
        fd = (lp - lm) / (2 * H * scale)
        ad = float((lam * d).sum())
        assert abs(fd - ad) <= TOL * max(abs(fd), abs(ad), 1e-12), f"{case} {name}: fd {fd:.9e} ad {ad:.9e}"

    # the water drag coefficient (northern and southern values moved together)
    s = st.settings
    w0, w0s = s.waterIceDrag, s.waterIceDrag_south
    hs = H * w0
    s.waterIceDrag, s.waterIceDrag_south = w0 + hs, w0s + hs
    lp = _loss(st, W)
    s.waterIceDrag, s.waterIceDrag_south = w0 - hs, w0s - hs
    lm = _loss(st, W)
    s.waterIceDrag, s.waterIceDrag_south = w0, w0s
    fd = (lp - lm) / (2 * hs)
    ad = float(scal["waterIceDrag"] + scal["waterIceDrag_south"])
    assert abs(fd - ad) <= TOL * max(abs(fd), abs(ad), 1e-12), f"{case} waterIceDrag: fd {fd:.9e} ad {ad:.9e}"


def test_evp_adjoint_checkpointing_is_exact():
    """Recomputing segments from checkpoints gives the same adjoint as storing
    every state."""
    from veris_gb300.adjoint import evp_adjoint
    rng = np.random.default_rng(6)
    st = _state("moving")
    shape = tuple(st.variables.iceMask.shape)
    W = {k: torch.as_tensor(rng.standard_normal(shape), device="cuda")
         for k in ("uIce", "vIce", "sigma1", "sigma2", "sigma12")}
    a = evp_adjoint(st, W, n_subcycles=N_SUB, checkpoint_every=0)
    b = evp_adjoint(st, W, n_subcycles=N_SUB, checkpoint_every=5)
    for k in a[0]:
        e = G.rel_err(b[0][k].cpu().numpy(), a[0][k].cpu().numpy())
        assert e <= 1e-12, (k, e)
    for k in ("SeaIceStrength", "WindForcingX", "uOcean"):
        e = G.rel_err(b[1][k].cpu().numpy(), a[1][k].cpu().numpy())
        assert e <= 1e-12, (k, e)

"""The routines beside the step on the GPU: free drift, the bulk formula and
the EVP residual diagnostics, against the golden fixtures (made by running
the reference) and the CPU oracle.

Bars: float64 1e-10 relative max-norm (max |gpu - ref| / max |ref|); float32
1e-5 (free drift) and 1e-4 (bulk formula, five iterations of logs and
divisions).  The residuals are sums of squared differences of consecutive
subcycle states, so they carry the states' rounding divided by the size of
the change: float64 bar 1e-8 relative per subcycle.
"""
import numpy as np
import pytest

from oracle import veris_oracle as O
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


def cpu(t):
    return t.detach().cpu().numpy()


def assert_close(got, ref, what, tol=TOL):
    got = cpu(got) if hasattr(got, "detach") else np.asarray(got)
    assert np.all(np.isfinite(got)), f"{what}: non-finite values"
    e = G.rel_err(got, ref)
    assert e <= tol, f"{what}: relative max-norm error {e:.3e} > {tol:.0e}"


def _fd_state(case, dtype=torch.float64):
    """A full GPU state of the fixture's grid carrying the fixture's inputs."""
    from tests.golden.make_golden import CASES
    from veris_gb300.state import VerisState
    from veris_gb300.synthetic import make_state
    st, ref = G.freedrift_case(G.load_forcing(), case)
    arrays = make_state(**CASES[case]["grid"])
    arrays.update(vars(st.variables))
    return VerisState.from_numpy(arrays, st.settings, dtype=dtype), st, ref


@pytest.mark.parametrize("case", G.FREEDRIFT_CASES)
def test_freedrift_matches_reference(case):
    from veris_gb300.freedrift_solver import freedrift_solver
    gst, _st, ref = _fd_state(case)
    u, v = freedrift_solver(gst)
    assert_close(u, ref["uIce"], f"{case} uIce")
    assert_close(v, ref["vIce"], f"{case} vIce")


@pytest.mark.parametrize("case", G.FREEDRIFT_CASES)
def test_freedrift_f32(case):
    from veris_gb300.freedrift_solver import freedrift_solver_f32
    gst, _st, ref = _fd_state(case, dtype=torch.float32)
    u, v = freedrift_solver_f32(gst)
    assert u.dtype == torch.float32
    assert_close(u, ref["uIce"], f"{case} uIce f32", 1e-5)
    assert_close(v, ref["vIce"], f"{case} vIce f32", 1e-5)


@pytest.mark.parametrize("nx,ny", ((1440, 720), (37, 11), (4, 4), (4, 61)))
def test_freedrift_sizes_against_oracle(nx, ny):
    """Sizes that leave partial strips and bands, and the smallest grid."""
    from veris_gb300.freedrift_solver import freedrift_solver
    from veris_gb300.state import VerisState
    from veris_gb300.synthetic import config_settings, make_state
    from types import SimpleNamespace
    arrays = make_state(nx, ny, seed=nx + ny, wind_scale=2.0, init_velocity=0.1)
    sett = config_settings("c2_quarterdeg")
    rng = np.random.default_rng(5)
    arrays["WindForcingX"] = rng.normal(0, 0.2, arrays["hIceMean"].shape)
    arrays["WindForcingY"] = rng.normal(0, 0.2, arrays["hIceMean"].shape)
    gst = VerisState.from_numpy(arrays, sett)
    u, v = freedrift_solver(gst)
    ou, ov = O.freedrift_solver(SimpleNamespace(variables=SimpleNamespace(**arrays), settings=sett))
    assert_close(u, ou, f"{nx}x{ny} uIce")
    assert_close(v, ov, f"{nx}x{ny} vIce")


def test_ice_velocities_dispatch():
    """useFreedrift: free drift with the stresses as they are; useEVP wins."""
    import copy
    from veris_gb300.dynsolver import IceVelocities
    from veris_gb300.evp_solver import evp_solver
    from veris_gb300.freedrift_solver import freedrift_solver
    gst, _st, _ref = _fd_state("moving")
    s = copy.copy(gst.settings)
    s.useFreedrift, s.useEVP = True, False
    gst.settings = s
    out = IceVelocities(gst)
    u, v = freedrift_solver(gst)
    assert torch.equal(out[0], u) and torch.equal(out[1], v)
    for k, t in zip(("sigma1", "sigma2", "sigma12"), out[2:]):
        assert torch.equal(t, getattr(gst.variables, k))
    s.useEVP = True
    s.nEVPsteps = 3
    both = IceVelocities(gst)
    ref = evp_solver(gst)
    for a, b in zip(both, ref):
        assert torch.equal(a, b)


def _bulk_gpu(dtype, outputs=None):
    from veris_gb300.heat_flux_MITgcm import BULK_OUTPUTS, bulkf_formula_lanl
    from types import SimpleNamespace
    sett, args, ref = G.bulk_case(G.load_forcing())
    t = [torch.as_tensor(a, dtype=dtype, device="cuda") for a in args]
    out = bulkf_formula_lanl(SimpleNamespace(settings=sett), *t, outputs=outputs or BULK_OUTPUTS)
    return out, ref


def test_bulk_formula_matches_reference():
    out, ref = _bulk_gpu(torch.float64)
    for n, a in zip(G.BULK_OUT, out):
        assert_close(a, ref[n], f"bulk {n}")


def test_bulk_formula_f32():
    out, ref = _bulk_gpu(torch.float32)
    for n, a in zip(G.BULK_OUT, out):
        assert a.dtype == torch.float32
        assert_close(a, ref[n], f"bulk {n} f32", 1e-4)


def test_bulk_formula_skips_outputs_and_agrees():
    full, _ref = _bulk_gpu(torch.float64)
    part, _ref = _bulk_gpu(torch.float64, outputs=("flwupa", "flha", "fsha", "df0dT", "ust", "vst"))
    assert part[6] is None and part[7] is None and part[8] is None
    for a, b in zip(full[:6], part[:6]):
        assert torch.equal(a, b)


def test_bulk_formula_large_against_oracle():
    """A full quarter-degree field of air/sea states against the oracle."""
    from veris_gb300.heat_flux_MITgcm import bulkf_formula_lanl
    from veris_gb300.synthetic import config_settings
    from types import SimpleNamespace
    rng = np.random.default_rng(11)
    shape = (1444, 724)
    uw, vw = rng.normal(0, 7, shape), rng.normal(0, 7, shape)
    tsf = 271 + 30 * rng.random(shape)
    ta = tsf + rng.normal(0, 5, shape)
    qa = 0.02 * rng.random(shape)
    mask = np.ones(shape)
    st = SimpleNamespace(settings=config_settings("c2_quarterdeg"))
    ref = O.bulkf_formula_lanl(st, uw, vw, ta, qa, tsf, mask)
    t = [torch.as_tensor(a, device="cuda") for a in (uw, vw, ta, qa, tsf, mask)]
    out = bulkf_formula_lanl(st, *t)
    for n, a, r in zip(G.BULK_OUT, out, ref):
        assert_close(a, r, f"bulk {n}")


def _residual_state(case, n):
    g = G.load(case)
    first_evp = [i for i, r, _o in G.sequence(g) if r == "IceVelocities"][0]
    st = G.state_before(g, first_evp)
    from veris_gb300.state import VerisState
    return VerisState.from_numpy(vars(st.variables), st.settings), st


@pytest.mark.parametrize("case", ("moving", "small_a", "small_b"))
def test_evp_residuals_against_oracle(case):
    """small_a runs the adaptive EVP (alpha and beta fields of each subcycle)."""
    from veris_gb300.evp_solver import evp_solver, evp_solver_residuals
    n = 8
    gst, st = _residual_state(case, n)
    out = evp_solver_residuals(gst, n)
    ref = O.evp_residuals(st, n)
    plain = evp_solver(gst, n)
    for a, b in zip(out[:5], plain):
        assert torch.equal(a, b), "the residual loop changed the solve"
    for k, (a, r) in enumerate(zip(out[:5], ref[:5])):
        assert_close(a, r, f"{case} field {k}")
    for name, a, r in (("resU", out[5], ref[5]), ("resSig", out[6], ref[6])):
        got = cpu(a)
        assert got.shape == (n,)
        rel = np.abs(got - r) / np.maximum(np.abs(r), 1e-300)
        assert rel.max() <= 1e-8, f"{case} {name}: {rel.max():.3e}"


@pytest.mark.parametrize("case", ("moving", "small_a", "small_b"))
def test_evp_residuals_against_the_reference(case):
    """The residuals of the reference's own branch (its two unbound names
    patched to the stress components they stand for; residuals.npz, made by
    tests/golden/make_golden.py --residuals), to the same 1e-8 as against
    the oracle."""
    import os
    from veris_gb300.evp_solver import evp_solver_residuals
    z = np.load(os.path.join(G.GOLDEN, "residuals.npz"))
    n = len(z[f"res.{case}.resU"])
    gst, _st = _residual_state(case, n)
    out = evp_solver_residuals(gst, n)
    for k, name in enumerate(("uIce", "vIce", "sigma1", "sigma2", "sigma12")):
        assert_close(out[k], z[f"res.{case}.{name}"], f"{case} {name}")
    for name, a in (("resU", out[5]), ("resSig", out[6])):
        r = z[f"res.{case}.{name}"]
        rel = np.abs(cpu(a) - r) / np.maximum(np.abs(r), 1e-300)
        assert rel.max() <= 1e-8, f"{case} {name}: {rel.max():.3e}"


def test_evp_residuals_deterministic_and_f32():
    from veris_gb300.evp_solver import evp_solver_residuals
    from veris_gb300.state import VerisState
    from veris_gb300.synthetic import config_settings, make_state
    arrays = make_state(360, 180, seed=3, init_velocity=0.1, init_stress=2000.0)
    sett = config_settings("c3_1deg")
    gst = VerisState.from_numpy(arrays, sett)
    a = evp_solver_residuals(gst, 20)
    b = evp_solver_residuals(gst, 20)
    assert torch.equal(a[5], b[5]) and torch.equal(a[6], b[6])
    s32 = VerisState.from_numpy(arrays, sett, dtype=torch.float32)
    c = evp_solver_residuals(s32, 20, precision="f32")
    assert c[0].dtype == torch.float32 and c[5].dtype == torch.float64
    ru, rs = cpu(a[5]), cpu(a[6])
    assert (ru > 0).all() and (rs > 0).all()
    # float32 states: the early, large changes agree to float32 rounding
    np.testing.assert_allclose(cpu(c[5])[:5], ru[:5], rtol=1e-3)
    np.testing.assert_allclose(cpu(c[6])[:5], rs[:5], rtol=1e-3)


def test_evp_solver_prints_residuals(capsys):
    import copy
    from veris_gb300 import evp_solver as E
    gst, _st = _residual_state("moving", 4)
    s = copy.copy(gst.settings)
    s.computeEvpResidual = True
    gst.settings = s
    E.printEvpResidual = True
    try:
        out = E.evp_solver(gst, 4)
    finally:
        E.printEvpResidual = False
    lines = capsys.readouterr().out.strip().splitlines()
    assert len(out) == 5 and len(lines) == 4
    assert lines[0].startswith("evp resU, resSigma: 0 ")
    assert E.last_residuals[0].shape == (4,)


def test_abi_argument_checks():
    """Status codes of the new entry points for bad arguments (nothing is
    launched for them)."""
    import ctypes
    from veris_gb300 import _abi
    from veris_gb300.state import Call
    lib = _abi.load()
    gst, _st, _ref = _fd_state("moving")
    c = Call(gst)
    u = c.empty()
    assert lib.veris_freedrift_solver_f64(*c.refs(), u.data_ptr(), None, c.stream) == 6   # invalid argument
    p = _abi.params_from_settings(gst.settings)
    assert lib.veris_bulkf_formula_lanl_f64(ctypes.byref(p), 0, *([None] * 15), c.stream) == 0   # n = 0: nothing to do
    assert lib.veris_bulkf_formula_lanl_f64(ctypes.byref(p), -1, *([None] * 15), c.stream) == 6
    assert lib.veris_bulkf_formula_lanl_f64(ctypes.byref(p), 16, *([None] * 15), c.stream) == 6   # inputs missing
    need = lib.veris_evp_residual_workspace_bytes(c.refs()[0], 8, 4)
    assert need > 0
    res = torch.zeros(8, dtype=torch.float64, device="cuda")
    ws = torch.empty(need - 8, dtype=torch.uint8, device="cuda")
    outs = c.empty(5)
    st = lib.veris_evp_residual_solver_f64(*c.refs(), 4, *[t.data_ptr() for t in outs], res.data_ptr(),
                                           res[4:].data_ptr(), ws.data_ptr(), ws.numel(), c.stream)
    assert st == 8   # workspace too small

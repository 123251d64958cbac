"""The persistent-buffer engine: float64 mode reproduces the golden step
sequence (1e-10), graph replay equals eager stepping bit for bit, the mixed
float32 mode stays within the stated error of float64, and the host-coupled
step returns what the device holds."""
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


def gpu_state(case):
    from veris_gb300.state import VerisState
    g = G.load(case)
    st = G.initial_state(g)
    return g, VerisState.from_numpy(vars(st.variables), st.settings)


def final_reference(g):
    """The last recorded value of every variable after the recorded steps."""
    out = {}
    for _i, _r, outs in G.sequence(g):
        out.update(outs)
    return out


@pytest.mark.parametrize("case", G.CASES)
def test_engine_f64_matches_golden(case):
    from veris_gb300.engine import SeaIceStep
    g, st = gpu_state(case)
    n_steps = sum(1 for _i, r, _o in G.sequence(g) if r == "SeaIceMass")
    eng = SeaIceStep(st, precision="f64")
    for _ in range(n_steps):
        eng.step()
    torch.cuda.synchronize()
    for k, ref in final_reference(g).items():
        got = getattr(st.variables, k).cpu().numpy()
        e = G.rel_err(got, ref)
        assert e <= 1e-10, f"{case}.{k}: {e:.3e}"


def test_graph_replay_equals_eager():
    from veris_gb300.engine import SeaIceStep
    _g, a = gpu_state("moving")
    _g, b = gpu_state("moving")
    ea = SeaIceStep(a, precision="f64")
    eb = SeaIceStep(b, precision="f64")
    eb.capture()          # one eager step, then the captured graph
    ea.step()
    for _ in range(2):
        ea.step()
        eb.step()
    torch.cuda.synchronize()
    for k in ("uIce", "vIce", "sigma12", "hIceMean", "Area", "Qnet"):
        assert torch.equal(getattr(a.variables, k), getattr(b.variables, k)), k


@pytest.mark.parametrize("case", ("c1", "moving"))
def test_engine_f32_close_to_f64(case):
    from veris_gb300.engine import SeaIceStep
    _g, a = gpu_state(case)
    _g, b = gpu_state(case)
    e64 = SeaIceStep(a, precision="f64")
    e32 = SeaIceStep(b, precision="f32")
    for _ in range(2):
        e64.step()
        e32.step()
    torch.cuda.synchronize()
    tol = {"uIce": 1e-4, "vIce": 1e-4, "hIceMean": 1e-6, "hSnowMean": 1e-6, "Area": 1e-5}
    for k, t in tol.items():
        x = getattr(b.variables, k).cpu().numpy()
        y = getattr(a.variables, k).cpu().numpy()
        e = G.rel_err(x, y)
        assert e <= t, f"{case}.{k}: float32 vs float64 {e:.3e} > {t:.0e}"


def test_host_coupled_step_roundtrip():
    from veris_gb300.engine import SeaIceStep
    from veris_gb300.host import HostCoupledStep
    _g, st = gpu_state("moving")
    eng = SeaIceStep(st, precision="f64")
    host = HostCoupledStep(eng)
    h_in, h_out = host.host_buffers()
    host.step(h_in, h_out)
    for n in host.outputs:
        assert torch.equal(h_out[n], getattr(st.variables, n).cpu()), n
    assert host.h2d_bytes == len(host.inputs) * st.variables.iceMask.numel() * 8


@pytest.mark.parametrize("precision,veros_fill", [("f64", True), ("f32", True), ("f64", False)])
def test_host_coupled_graph_equals_plain_steps(precision, veros_fill):
    """The captured host exchange (side-stream uploads of the Growth forcing,
    early downloads of the dynamics outputs and the clean-up overshoots,
    Growth's outputs by row blocks while Growth runs, the rows the halo fill
    rewrites after it; with both halos filled the filled fields wait for the
    fill) gives the host exactly what an engine step followed by plain copies
    gives, step after step, with new host inputs every step."""
    from veris_gb300.engine import SeaIceStep
    from veris_gb300.host import HostCoupledStep
    from veris_gb300.state import VerisState
    from veris_gb300.synthetic import config_settings, make_state
    arrays = make_state(120, 80, seed=2, init_velocity=0.05)
    sett = config_settings("c3_1deg", nEVPsteps=40, veros_fill=veros_fill)
    a = VerisState.from_numpy(arrays, sett)
    b = VerisState.from_numpy(arrays, sett)
    host = HostCoupledStep(SeaIceStep(a, precision=precision))
    eng_b = SeaIceStep(b, precision=precision)
    h_in, h_out = host.host_buffers()
    rng = np.random.default_rng(0)
    for k in range(4):
        # the host model changes its forcing between steps
        for n in ("Qnet", "ATemp", "uWind", "theta"):
            h_in[n].mul_(float(1.0 + 0.01 * rng.standard_normal()))
        host.step(h_in, h_out)
        for n in host.inputs:
            getattr(b.variables, n).copy_(h_in[n].cuda())
        eng_b.step()
        torch.cuda.synchronize()
        for n in host.outputs:
            assert torch.equal(h_out[n], getattr(b.variables, n).cpu()), (k, n)
        # the host keeps stepping from what the step returned
        for n in host.outputs:
            if n in h_in:
                h_in[n].copy_(h_out[n])
    assert len(host.graphs) == 1


@pytest.mark.parametrize("case", G.CASES)
def test_fast_form_support_and_parity(case):
    """The fast EVP form covers the default rheology; in float64 it matches
    the reference's EVP results to 1e-10 wherever it applies."""
    from veris_gb300.engine import SeaIceStep
    g, st = gpu_state(case)
    eng = SeaIceStep(st, precision="f64", evp="auto")
    expected_fast = case in ("c1", "moving", "noice")
    assert (eng.evp_form == "fast") == expected_fast, (case, hex(eng.fast_violations))
    if not expected_fast:
        return
    n_steps = sum(1 for _i, r, _o in G.sequence(g) if r == "SeaIceMass")
    evp_refs = [o for _i, r, o in G.sequence(g) if r == "IceVelocities"]
    for k in range(n_steps):
        eng.step()
        torch.cuda.synchronize()
        for name, ref in evp_refs[k].items():
            # the state holds later values of u, v: compare the EVP outputs kept by the engine
            got = eng.evp_out[("uIce", "vIce", "sigma1", "sigma2", "sigma12").index(name)].cpu().numpy()
            e = G.rel_err(got, ref)
            assert e <= 1e-10, f"{case} step {k} {name}: {e:.3e}"


@pytest.mark.parametrize("case", ("c1", "moving", "noice"))
def test_tma_form_matches_smem_form_and_f64(case):
    """The TMA-staged float32 kernel against the shared-memory float32 kernel
    (same arithmetic) and the float64 fast form, from the reference's own
    input state of the first EVP call; the device status word stays clean."""
    from veris_gb300.evp_solver import evp_solver_fast
    g = G.load(case)
    first_evp = [i for i, r, _o in G.sequence(g) if r == "IceVelocities"][0]
    from veris_gb300.state import VerisState
    st0 = G.state_before(g, first_evp)
    st = VerisState.from_numpy(vars(st0.variables), st0.settings)
    tma, status = evp_solver_fast(st, "f32", "tma", return_status=True)
    assert status == 0
    smem = evp_solver_fast(st, "f32", "smem")
    f64 = evp_solver_fast(st, "f64")
    ref = [o for _i, r, o in G.sequence(g) if r == "IceVelocities"][0]
    for k, name in enumerate(("uIce", "vIce", "sigma1", "sigma2", "sigma12")):
        a, b = tma[k].double().cpu().numpy(), smem[k].double().cpu().numpy()
        assert G.rel_err(a, b) <= 1e-5, f"{case}.{name}: tma vs smem {G.rel_err(a, b):.2e}"
        assert G.rel_err(f64[k].cpu().numpy(), ref[name]) <= 1e-10
        if name in ("uIce", "vIce"):
            e = G.rel_err(a, ref[name])
            assert e <= 1e-3, f"{case}.{name}: float32 vs reference {e:.2e}"


@pytest.mark.parametrize("case", ("c1", "moving", "noice"))
@pytest.mark.parametrize("rows,variant", ((4, 0), (7, 1), (16, 2), (64, 3), (16, 1)))
def test_walk_form_matches_tma_and_smem_forms(case, rows, variant):
    """The register-walking float32 kernel (any walk length, with ragged last
    walks) against the TMA-staged and the shared-memory float32 kernels from
    the reference's input state of the first EVP call."""
    from veris_gb300.evp_solver import evp_solver_fast
    from veris_gb300.state import VerisState
    g = G.load(case)
    first_evp = [i for i, r, _o in G.sequence(g) if r == "IceVelocities"][0]
    st0 = G.state_before(g, first_evp)
    st = VerisState.from_numpy(vars(st0.variables), st0.settings)
    try:
        smem = evp_solver_fast(st, "f32", "smem")
    except Exception as e:   # settings the fast forms do not cover
        pytest.skip(str(e))
    walk = evp_solver_fast(st, "f32", "walk", rows=rows, variant=variant)
    tma = evp_solver_fast(st, "f32", "tma")
    for k, name in enumerate(("uIce", "vIce", "sigma1", "sigma2", "sigma12")):
        a = walk[k].double().cpu().numpy()
        assert G.rel_err(a, smem[k].double().cpu().numpy()) <= 1e-5, f"{case}.{name} rows {rows}: walk vs smem"
        assert G.rel_err(a, tma[k].double().cpu().numpy()) <= 1e-5, f"{case}.{name} rows {rows}: walk vs tma"


def test_walk_form_on_a_larger_synthetic_grid():
    """Many strips and walks, the cyclic x-halo images and the array edges."""
    from veris_gb300.evp_solver import evp_solver_fast
    from veris_gb300.state import VerisState
    from veris_gb300.synthetic import config_settings, make_state
    st = VerisState.from_numpy(make_state(300, 150, seed=4, init_velocity=0.05), config_settings("c3_1deg"))
    from veris_gb300 import model
    for name in ("SeaIceMass", "AreaWS", "WindForcingXY", "SeaIceStrength"):
        fn, outs = [(f, o) for n, f, o in model.STEP if n == name][0]
        vals = fn(st)
        vals = vals if isinstance(vals, tuple) else (vals,)
        for o, x in zip(outs, vals):
            setattr(st.variables, o, x)
    smem = evp_solver_fast(st, "f32", "smem", n_subcycles=20)
    for rows, variant in ((16, 0), (33, 1), (8, 3), (0, 2)):
        walk = evp_solver_fast(st, "f32", "walk", n_subcycles=20, rows=rows, variant=variant)
        for k in range(5):
            e = G.rel_err(walk[k].double().cpu().numpy(), smem[k].double().cpu().numpy())
            assert e <= 1e-5, (rows, k, e)


@pytest.mark.parametrize("nx,ny", ((297, 151), (61, 9), (5, 57)))
def test_walk_on_odd_and_narrow_widths(nx, ny):
    """Odd padded widths, and grids narrower than one strip (the strip
    covers the periodic width several times over)."""
    from veris_gb300.evp_solver import evp_solver_fast
    from veris_gb300.state import VerisState
    from veris_gb300.synthetic import config_settings, make_state
    st = VerisState.from_numpy(make_state(nx, ny, seed=nx, init_velocity=0.05, ice_lat=0.0),
                               config_settings("c3_1deg"))
    from veris_gb300 import model
    for name in ("SeaIceMass", "AreaWS", "WindForcingXY", "SeaIceStrength"):
        fn, outs = [(f, o) for n, f, o in model.STEP if n == name][0]
        vals = fn(st)
        vals = vals if isinstance(vals, tuple) else (vals,)
        for o, x in zip(outs, vals):
            setattr(st.variables, o, x)
    smem = evp_solver_fast(st, "f32", "smem", n_subcycles=12)
    for rows, variant in ((16, 2), (5, 1), (0, 3), (8, 0)):
        walk = evp_solver_fast(st, "f32", "walk", n_subcycles=12, rows=rows, variant=variant)
        for k in range(5):
            e = G.rel_err(walk[k].double().cpu().numpy(), smem[k].double().cpu().numpy())
            assert e <= 1e-5, (nx, ny, rows, variant, k, e)


def _prepared(nx, ny, seed, **overrides):
    from veris_gb300 import model
    from veris_gb300.state import VerisState
    from veris_gb300.synthetic import config_settings, make_state
    sett = config_settings("c3_1deg", **overrides)
    st = VerisState.from_numpy(make_state(nx, ny, seed=seed, init_velocity=0.05, init_stress=2000.0, ice_lat=30.0),
                               sett)
    for name in ("SeaIceMass", "AreaWS", "WindForcingXY", "SeaIceStrength"):
        fn, outs = [(f, o) for n, f, o in model.STEP if n == name][0]
        vals = fn(st)
        vals = vals if isinstance(vals, tuple) else (vals,)
        for o, x in zip(outs, vals):
            setattr(st.variables, o, x)
    return st


@pytest.mark.parametrize("nx,ny,rows,variant", ((120, 90, 0, 2), (61, 33, 7, 0), (200, 150, 16, 3)))
def test_walk_adaptive_evp(nx, ny, rows, variant):
    """Adaptive EVP in the register-walking kernel against the plain float64
    and float32 loops (alphaC from zeta per subcycle, alphaZ and the betas
    averaged from it)."""
    from veris_gb300.evp_solver import evp_solver, evp_solver_f32, evp_solver_fast
    from veris_gb300.state import VerisState
    st = _prepared(nx, ny, nx, useAdaptiveEVP=True)
    n = 20
    walk = evp_solver_fast(st, "f32", "walk", n_subcycles=n, rows=rows, variant=variant)
    ref = evp_solver(st, n)
    st32 = VerisState({k: getattr(st.variables, k).float() for k in st.variables.names()}, st.settings)
    plain32 = evp_solver_f32(st32, n)
    for k in range(5):
        w = walk[k].double().cpu().numpy()
        e64 = G.rel_err(w, ref[k].cpu().numpy())
        e32 = G.rel_err(w, plain32[k].double().cpu().numpy())
        assert e64 <= 1e-3, (k, e64)
        assert e32 <= 1e-3, (k, e32)
    # and it is not the constant-alpha solve
    st_c = _prepared(nx, ny, nx)
    const = evp_solver_fast(st_c, "f32", "walk", n_subcycles=n, rows=rows, variant=variant)
    assert G.rel_err(walk[0].double().cpu().numpy(), const[0].double().cpu().numpy()) > 1e-3


def test_engine_f32_runs_adaptive_evp_in_the_walk():
    from veris_gb300.engine import SeaIceStep
    from veris_gb300.state import VerisState
    from veris_gb300.synthetic import config_settings, make_state
    sett = config_settings("c3_1deg", useAdaptiveEVP=True, nEVPsteps=30)
    arrays = make_state(96, 64, seed=9, init_velocity=0.05)
    s32 = VerisState.from_numpy(arrays, sett)
    s64 = VerisState.from_numpy(arrays, sett)
    e32 = SeaIceStep(s32, precision="f32")
    e64 = SeaIceStep(s64, precision="f64", evp="plain")
    assert e32.evp_form == "fast"
    e32.step()
    e64.step()
    torch.cuda.synchronize()
    for k in ("uIce", "vIce", "hIceMean", "Area"):
        e = G.rel_err(getattr(s32.variables, k).cpu().numpy(), getattr(s64.variables, k).cpu().numpy())
        assert e <= 1e-3, (k, e)


def test_engine_free_drift_step():
    """useFreedrift without useEVP: the engine's step runs free drift, like the
    drop-in sequence (IceVelocities), and keeps the stresses."""
    from veris_gb300 import model
    from veris_gb300.engine import SeaIceStep
    from veris_gb300.state import VerisState
    from veris_gb300.synthetic import config_settings, make_state
    sett = config_settings("c3_1deg", useFreedrift=True, useEVP=False)
    arrays = make_state(96, 64, seed=5, init_velocity=0.05, init_stress=500.0)
    ref = VerisState.from_numpy(arrays, sett)
    model.step(ref)
    for precision, tol in (("f64", 1e-10), ("f32", 1e-4)):
        st = VerisState.from_numpy(arrays, sett)
        SeaIceStep(st, precision=precision).step()
        torch.cuda.synchronize()
        for k in ("uIce", "vIce", "hIceMean", "Area", "TSurf"):
            e = G.rel_err(getattr(st.variables, k).cpu().numpy(), getattr(ref.variables, k).cpu().numpy())
            assert e <= tol, (precision, k, e)
        assert torch.equal(st.variables.sigma1, torch.as_tensor(arrays["sigma1"], device="cuda"))


@pytest.mark.parametrize("nx,ny", ((120, 90), (61, 33)))
def test_walk_with_both_halos_refreshed(nx, ny):
    """veros_fill = False refreshes both halos from periodic images: the walk's
    own state layout keeps a halo point's own stresses and its velocity
    images apart."""
    from veris_gb300.evp_solver import evp_solver_fast
    st = _prepared(nx, ny, nx + 1, veros_fill=False)
    smem = evp_solver_fast(st, "f32", "smem", n_subcycles=12)
    for rows, variant in ((0, 2), (7, 0), (16, 3)):
        walk = evp_solver_fast(st, "f32", "walk", n_subcycles=12, rows=rows, variant=variant)
        for k in range(5):
            e = G.rel_err(walk[k].double().cpu().numpy(), smem[k].double().cpu().numpy())
            assert e <= 1e-5, (nx, ny, rows, variant, k, e)


def test_areas_along_both_axes_take_the_tile_form():
    """Cell areas that vary along i as well: the engine runs the TMA-staged
    form instead of the register walk (which holds the areas per column),
    and the walk drop-in refuses the state."""
    from veris_gb300.engine import SeaIceStep
    from veris_gb300.evp_solver import evp_solver_fast
    st = _prepared(96, 64, 5)
    v = st.variables
    scale = torch.linspace(0.9, 1.1, v.rA.shape[0], dtype=torch.float64, device="cuda")[:, None]
    for n in ("rA", "rAu", "rAv", "rAz"):
        getattr(v, n).mul_(scale)
    for n, src in (("recip_rA", "rA"), ("recip_rAu", "rAu"), ("recip_rAv", "rAv")):
        getattr(v, n).copy_(1.0 / getattr(v, src))
    eng = SeaIceStep(st, precision="f32")
    assert eng.area2d and eng.evp_form == "fast" and eng.f32_kernel == "tma"
    with pytest.raises(ValueError):
        evp_solver_fast(st, "f32", "walk", n_subcycles=3)
    smem = evp_solver_fast(st, "f32", "smem", n_subcycles=10)
    tma = evp_solver_fast(st, "f32", "tma", n_subcycles=10)
    for k in range(5):
        assert G.rel_err(tma[k].double().cpu().numpy(), smem[k].double().cpu().numpy()) <= 1e-5


def test_growth_by_row_blocks_equals_one_launch():
    """veris_growth_rows_f64 over uneven row blocks that tile the padded
    array gives Growth's eleven outputs bit for bit; ranges outside the
    array are refused before any launch."""
    from veris_gb300.growth import Growth
    from veris_gb300.state import Call
    _g, st = gpu_state("moving")
    whole = Growth(st)
    c = Call(st)
    out = c.empty(11)
    NX = st.variables.iceMask.shape[0]
    cuts = [0, 3, 7, NX // 2, NX - 1, NX]
    for a, b in zip(cuts[:-1], cuts[1:]):
        assert c.lib.veris_growth_rows_f64(*c.refs(), *[t.data_ptr() for t in out], a, b, c.stream) == 0
    torch.cuda.synchronize()
    for q, (x, y) in enumerate(zip(out, whole)):
        assert torch.equal(x, y), q
    ptrs = [t.data_ptr() for t in out]
    for a, b in ((-1, 4), (4, 4), (5, 3), (0, NX + 1)):
        assert c.lib.veris_growth_rows_f64(*c.refs(), *ptrs, a, b, c.stream) == 6, (a, b)


def test_float64_tile_heights_give_the_same_values_and_the_tuner_picks_one():
    """The float64 subcycle's tile height (16, 24, 32 rows) changes only the
    launch: every height gives the same values bit for bit; the tuner keeps
    one of them and leaves the state alone."""
    import ctypes
    from veris_gb300 import _abi
    from veris_gb300.autotune import tune_f64_tile
    from veris_gb300.engine import SeaIceStep
    from veris_gb300.state import Call, VerisState
    from veris_gb300.synthetic import config_settings, make_state
    arrays = make_state(150, 70, seed=4, init_velocity=0.1, init_stress=800.0, ice_lat=30.0)
    sett = config_settings("c1_4deg", nEVPsteps=9)
    st = VerisState.from_numpy(arrays, sett)
    lib = _abi.load()
    c = Call(st)
    ws, wsb = c.workspace(lib.veris_evp_fast_workspace_bytes(c.refs()[0], 8))
    res = []
    try:
        for rows in (16, 24, 32):
            assert lib.veris_evp_f64_tile_rows(rows) == 0
            out = c.empty(5)
            assert lib.veris_evp_fast_solver_f64(*c.refs(), 9, *[t.data_ptr() for t in out], ws, wsb, c.stream) == 0
            res.append(out)
        assert lib.veris_evp_f64_tile_rows(20) == 6
        for out in res[1:]:
            for a, b in zip(out, res[0]):
                assert torch.equal(a, b)
        eng = SeaIceStep(VerisState.from_numpy(arrays, sett), precision="f64")
        before = eng.state.variables.uIce.clone()
        t = tune_f64_tile(eng, subcycles=3, repeats=1)
        assert t["rows"] in (16, 24, 32) and len(t["trials"]) == 3
        assert torch.equal(before, eng.state.variables.uIce)
    finally:
        lib.veris_evp_f64_tile_rows(0)


@pytest.mark.parametrize("nx,ny", ((1203, 611), (4001, 97)))
def test_f64_units_on_large_odd_grids(nx, ny):
    """Grids where every unit height leaves a last round of small pieces at
    the bottom of each strip (more full pieces than resident CTA slots):
    16-, 24- and 32-row units give the same values bit for bit, and those
    match the plain float64 loop to 1e-10."""
    from veris_gb300 import _abi
    from veris_gb300.evp_solver import evp_solver
    from veris_gb300.state import Call
    st = _prepared(nx, ny, nx + ny)
    lib = _abi.load()
    c = Call(st)
    ws, wsb = c.workspace(lib.veris_evp_fast_workspace_bytes(c.refs()[0], 8))
    n = 6
    res = []
    try:
        for rows in (16, 24, 32):
            assert lib.veris_evp_f64_tile_rows(rows) == 0
            out = c.empty(5)
            assert lib.veris_evp_fast_solver_f64(*c.refs(), n, *[t.data_ptr() for t in out], ws, wsb, c.stream) == 0
            res.append(out)
    finally:
        lib.veris_evp_f64_tile_rows(0)
    for out in res[1:]:
        for a, b in zip(out, res[0]):
            assert torch.equal(a, b)
    ref = evp_solver(st, n)
    for k in range(5):
        e = G.rel_err(res[0][k].cpu().numpy(), ref[k].cpu().numpy())
        assert e <= 1e-10, (k, e)


_TURN = dict(waterTurnAngle=15.0, sinWat=float(np.sin(np.radians(15.0))), cosWat=float(np.cos(np.radians(15.0))))


@pytest.mark.parametrize("nx,ny,fill,n,extra", ((300, 150, True, 25, {}), (61, 33, True, 9, {}),
                                                (120, 90, False, 14, {}), (1440, 720, True, 40, {}),
                                                (200, 120, True, 12, {"useAdaptiveEVP": True}),
                                                (200, 120, False, 12, dict(_TURN, basalDragK2=15.0))))
def test_persistent_walk_gives_the_same_values(nx, ny, fill, n, extra):
    """Several float32 subcycles per persistent launch (each walk waiting on
    its neighbours' progress counters) against one launch per subcycle: bit
    for bit, for several walk lengths and compiled forms, with the cyclic
    x-halo images (veros_fill) and with both halos refreshed, and with the
    adaptive EVP, basal drag and turning angles."""
    from veris_gb300 import _abi
    from veris_gb300.evp_solver import evp_solver_fast
    lib = _abi.load()
    st = _prepared(nx, ny, nx + 7, veros_fill=fill, **extra)
    try:
        for rows, variant in ((0, 2), (16, 0), (0, 3)):
            assert lib.veris_evp_walk_persistent(0) == 0
            one = evp_solver_fast(st, "f32", "walk", n_subcycles=n, rows=rows, variant=variant)
            assert lib.veris_evp_walk_persistent(1) == 0
            many, status = evp_solver_fast(st, "f32", "walk", n_subcycles=n, rows=rows, variant=variant,
                                           return_status=True)
            assert status == 0, status
            for k in range(5):
                assert torch.equal(one[k], many[k]), (rows, variant, k)
    finally:
        lib.veris_evp_walk_persistent(0)
    assert lib.veris_evp_walk_persistent(2) != 0

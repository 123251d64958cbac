"""Failure detection without a GPU fault.

* The bounded mbarrier wait of the TMA-staged kernel gives up on a barrier
  nothing arrives on, reports the timeout bit through its status word, and
  the context stays usable.
* The non-finite check flags a NaN or an infinity anywhere in its arrays;
  the engine runs it once per step and the host exchange raises
  VerisError(VERIS_ERR_NAN) after a step that met a NaN in its forcing.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from veris_gb300 import _abi
    return _abi.load()


def test_bounded_wait_gives_up_and_reports(lib):
    status = torch.full((2,), -1, dtype=torch.int32, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    assert lib.veris_mbarrier_wait_probe(1, 4096, status[0:1].data_ptr(), s) == 0   # arrives: completes
    assert lib.veris_mbarrier_wait_probe(0, 4096, status[1:2].data_ptr(), s) == 0   # nothing arrives
    torch.cuda.synchronize()
    assert status.tolist() == [0, 1]
    # limits outside (0, 2^20] are refused before any launch
    assert lib.veris_mbarrier_wait_probe(0, 0, status[1:2].data_ptr(), s) == 6
    assert lib.veris_mbarrier_wait_probe(0, (1 << 20) + 1, status[1:2].data_ptr(), s) == 6


def test_context_usable_after_a_timed_out_wait(lib):
    from veris_gb300.evp_solver import evp_solver_fast
    from veris_gb300.state import VerisState
    from veris_gb300.synthetic import config_settings, make_state
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert lib.veris_mbarrier_wait_probe(0, 4096, status.data_ptr(), torch.cuda.current_stream().cuda_stream) == 0
    torch.cuda.synchronize()
    assert int(status) == 1
    st = VerisState.from_numpy(make_state(64, 48, seed=1, init_velocity=0.05), config_settings("c3_1deg"))
    out = evp_solver_fast(st, "f32", "tma", n_subcycles=5)
    torch.cuda.synchronize()
    assert all(bool(torch.isfinite(t).all()) for t in out)


# Non-finite detection: bad input made on the host (a NaN or an infinity in
# a forcing array).  Every loop of the step's kernels has a fixed trip count
# and no address depends on a field value, so non-finite data only flows
# through the arithmetic.

@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_check_finite_flags_nan_and_inf(lib, dtype):
    import ctypes
    from veris_gb300 import _abi
    nx, ny = 40, 30
    g = _abi.VerisGrid(nx, ny, 2, 2, ny + 4)
    fn = lib.veris_check_finite_f64 if dtype == torch.float64 else lib.veris_check_finite_f32
    s = torch.cuda.current_stream().cuda_stream
    arrays = [torch.rand(nx + 4, ny + 4, dtype=dtype, device="cuda") for _ in range(3)]
    status = torch.zeros(1, dtype=torch.int32, device="cuda")

    def run(flag=2):
        ptrs = (ctypes.c_void_p * 3)(*[a.data_ptr() for a in arrays])
        assert fn(ctypes.byref(g), ptrs, 3, flag, status.data_ptr(), s) == 0
        torch.cuda.synchronize()
        return int(status)

    assert run() == 0
    arrays[2][0, ny + 3] = float("nan")    # a halo corner of the last array
    assert run() == 2
    status.zero_()
    arrays[2][0, ny + 3] = 0.5
    arrays[1][nx // 2, ny // 2] = float("-inf")
    assert run(flag=4) == 4
    # argument checks refuse before any launch
    ptrs = (ctypes.c_void_p * 3)(*[a.data_ptr() for a in arrays])
    assert fn(ctypes.byref(g), ptrs, 0, 2, status.data_ptr(), s) == 6
    assert fn(ctypes.byref(g), ptrs, 9, 2, status.data_ptr(), s) == 6
    assert fn(ctypes.byref(g), ptrs, 3, 0, status.data_ptr(), s) == 6


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_engine_reports_a_nan_in_the_forcing(lib, precision):
    from veris_gb300._abi import VerisError
    from veris_gb300.engine import SeaIceStep
    from veris_gb300.host import HostCoupledStep
    from veris_gb300.state import VerisState
    from veris_gb300.synthetic import config_settings, make_state
    arrays = make_state(48, 32, seed=2, init_velocity=0.05)
    eng = SeaIceStep(VerisState.from_numpy(arrays, config_settings("c1_4deg", nEVPsteps=10)), precision=precision)
    eng.step()
    eng.check()                       # a clean step: no flag
    assert eng.status() == 0
    host = HostCoupledStep(eng)
    h_in, h_out = host.host_buffers()
    host.step(h_in, h_out)            # clean, through the host exchange
    # an interior ice point with wet U and V faces: the wind stress there
    # feeds the momentum equation (a NaN in a halo point would stay in the
    # halo, which the fill overwrites from the interior)
    I = (slice(2, -2), slice(2, -2))
    ok = ((arrays["hIceMean"][I] > 0) & (arrays["iceMaskU"][I] == 1) & (arrays["iceMaskV"][I] == 1)
          & (arrays["iceMaskU"][3:-1, 2:-2] == 1))
    ice = np.argwhere(ok)[0] + 2
    h_in["uWind"][tuple(ice)] = float("nan")
    with pytest.raises(VerisError) as e:
        host.step(h_in, h_out)
    assert e.value.status == 3
    assert eng.status() & 2
    with pytest.raises(VerisError):
        eng.check()
    # every prognostic field comes from h_in each step: with the forcing
    # finite again the next step is clean
    eng.clear_status()
    h_in["uWind"][tuple(ice)] = 0.0
    host.step(h_in, h_out)
    assert eng.status() == 0
    assert all(bool(torch.isfinite(h_out[n]).all()) for n in ("uIce", "vIce", "hIceMean", "TSurf"))

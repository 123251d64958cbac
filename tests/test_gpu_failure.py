"""Failure detection without a GPU fault: the bounded mbarrier wait of the
TMA-staged kernel gives up on a barrier nothing arrives on, reports the
timeout bit through its status word, and the context stays usable."""
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

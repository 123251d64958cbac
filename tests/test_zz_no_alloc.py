"""The allocation-free EVP entry point, through the C ABI.

veris_evp_solver_f64_noalloc exists for callers that cannot allocate device
memory (a host model's time loop calling the C ABI without a device allocator
of its own, or a caller held to a device-memory budget fixed at start-up): it
keeps its scratch in a fixed array inside the library instead of a
caller-provided workspace.  It runs the same kernels as the workspace-taking
veris_evp_solver_f64 on the same stream, so this test checks that two calls
in a row give that entry point's results bit for bit, for the workload's
subcycle count and for 0 and 1 subcycles (which never touch the scratch).

The file is named so that pytest collects it last: a run that stops at the
first failure has then already run every other test.
"""
import ctypes

import numpy as np
import pytest

from tests import golden_io as G

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from veris_gb300 import _abi
    return _abi.load()


def _call_args(case):
    from veris_gb300.state import VerisState, Call
    g = G.load(case)
    first_evp = [i for i, r, _o in G.sequence(g) if r == "IceVelocities"][0]
    st0 = G.state_before(g, first_evp)
    st = VerisState.from_numpy(vars(st0.variables), st0.settings)
    return Call(st), int(st.settings.nEVPsteps)


@pytest.mark.parametrize("case,subcycles", [("c1", None), ("moving", None), ("small_a", None),
                                             ("c1", 0), ("c1", 1), ("moving", 1)])
def test_noalloc_matches_workspace_entry_point_twice(lib, case, subcycles):
    c, n = _call_args(case)
    n = n if subcycles is None else subcycles
    ref = c.empty(5)
    for t in ref:
        t.fill_(np.nan)
    ws, wsb = c.workspace(lib.veris_evp_workspace_bytes(c.refs()[0], 8))
    assert lib.veris_evp_solver_f64(*c.refs(), n, *[t.data_ptr() for t in ref], ws, wsb, c.stream) == 0
    for call in range(2):
        out = c.empty(5)
        for t in out:
            t.fill_(np.nan)
        st = lib.veris_evp_solver_f64_noalloc(*c.refs(), n, *[t.data_ptr() for t in out], c.stream)
        assert st == 0, lib.veris_status_string(st)
        torch.cuda.synchronize()
        for name, a, b in zip(("uIce", "vIce", "sigma1", "sigma2", "sigma12"), out, ref):
            assert torch.isfinite(b).all(), f"{case} n={n} {name}: the workspace entry point left gaps"
            assert torch.equal(a, b), f"{case} n={n} call {call} {name} differs from veris_evp_solver_f64"


def test_noalloc_rejects_grids_beyond_its_scratch(lib):
    from veris_gb300 import _abi
    c, n = _call_args("c1")
    big = _abi.VerisGrid(1024, 512, 2, 2, 516)     # 1028 * 516 padded cells > 262144
    out = c.empty(5)
    st = lib.veris_evp_solver_f64_noalloc(ctypes.byref(big), *c.refs()[1:], n, *[t.data_ptr() for t in out],
                                          c.stream)
    assert st == 9
    assert b"fixed scratch" in lib.veris_status_string(st)

"""Host-side logic that needs no GPU: the binomial checkpoint schedule of the
multi-step adjoint, the choice of the EVP checkpoint spacing and of the EVP
tape policy from free device memory, and the host exchange's plan of which
rows of Growth's outputs can go to the host before the halo fill."""
import functools
from types import SimpleNamespace

import pytest

torch = pytest.importorskip("torch")


def test_binomial_schedule_closed_forms_and_monotonicity():
    from veris_gb300.trajectory import binomial_schedule
    n, s = 40, 6
    cost, split = binomial_schedule(n, s)
    for k in range(2, n + 1):
        assert cost[k][0] == k * (k - 1) // 2
        for t in range(1, s + 1):
            assert cost[k][t] <= cost[k][t - 1]           # a free slot never costs more
            assert cost[k][t] >= k - 1                     # every step but the last is advanced once
            if t >= k - 1:
                assert cost[k][t] == k - 1
            assert 1 <= split[k][t] <= k - 1


def test_binomial_schedule_is_optimal_on_small_cases():
    """Against an independent exhaustive recursion over every first split."""
    from veris_gb300.trajectory import binomial_schedule

    @functools.lru_cache(maxsize=None)
    def best(k, t):
        if k <= 1:
            return 0
        if t == 0:
            return k * (k - 1) // 2
        return min(m + best(k - m, t - 1) + best(m, t) for m in range(1, k))

    cost, split = binomial_schedule(24, 4)
    for k in range(1, 25):
        for t in range(0, 5):
            assert cost[k][t] == best(k, t), (k, t)
            if k >= 2 and t >= 1 and t < k - 1:
                m = split[k][t]
                assert m + cost[k - m][t - 1] + cost[m][t] == cost[k][t]


class _FakeLib:
    """veris_evp_adjoint_workspace_bytes of the real layout's shape: fixed
    part, checkpoints every K subcycles, a segment of K + 1 states."""

    def __init__(self, state_bytes, fixed):
        self.state_bytes, self.fixed = state_bytes, fixed

    def veris_evp_adjoint_workspace_bytes(self, g, esize, n, K):
        if K <= 0 or K > n:
            K = n
        ncp = (n + K - 1) // K
        return self.fixed + (ncp + K + 1 + 2) * self.state_bytes


def _traj(n_sub, lib):
    from veris_gb300.trajectory import Trajectory
    tr = Trajectory.__new__(Trajectory)
    tr.eng = SimpleNamespace(n_sub=n_sub, device="cpu")
    tr.lib = lib
    return tr


def test_checkpoint_spacing_one_segment_when_it_fits(monkeypatch):
    lib = _FakeLib(state_bytes=100, fixed=1000)
    tr = _traj(500, lib)
    need = lib.veris_evp_adjoint_workspace_bytes(None, 8, 500, 0)
    monkeypatch.setattr(torch.cuda, "mem_get_info", lambda dev=None: (int(need / 0.6) + 10, 0))
    assert tr._fitting_checkpoint_spacing(None, 8, 0.6) == 0


def test_checkpoint_spacing_smallest_workspace_otherwise(monkeypatch):
    lib = _FakeLib(state_bytes=100, fixed=1000)
    tr = _traj(500, lib)
    monkeypatch.setattr(torch.cuda, "mem_get_info", lambda dev=None: (10_000, 0))
    K = tr._fitting_checkpoint_spacing(None, 8, 0.6)
    ws = lambda k: lib.veris_evp_adjoint_workspace_bytes(None, 8, 500, k)
    assert 1 <= K < 500
    assert ws(K) == min(ws(k) for k in range(1, 500))
    assert 15 <= K <= 30                                   # about sqrt(500)


@pytest.mark.parametrize("veros_fill", [True, False])
def test_growth_row_plan(veros_fill):
    from veris_gb300.host import EARLY_OUTPUTS, HOST_OUTPUTS, MID_OUTPUTS, growth_row_plan
    from veris_gb300.engine import FILLED_AFTER_GROWTH, GROWTH_OUT
    NX, olx = 100, 2
    early = tuple(n for n in HOST_OUTPUTS if n in EARLY_OUTPUTS)
    mid = tuple(n for n in HOST_OUTPUTS if n in MID_OUTPUTS)
    plan = growth_row_plan(HOST_OUTPUTS, early, mid, NX, olx, veros_fill)
    for n in HOST_OUTPUTS:
        if n not in GROWTH_OUT or n in early or n in mid:
            assert n not in plan, n
        elif n not in FILLED_AFTER_GROWTH:
            assert plan[n] == (0, NX), n                   # the fill never touches it
        elif veros_fill:
            assert plan[n] == (olx, NX - olx), n           # the fill rewrites the x-halo rows
        else:
            assert n not in plan, n                        # columns of every row: after the fill
    assert "TSurf" in plan and "hIceMean" in plan if veros_fill else "hIceMean" not in plan


def test_tape_policy():
    """All steps' tapes when they fit beside every snapshot; else, in float32,
    one step's tape written during the reverse; else the recompute."""
    from veris_gb300.trajectory import tape_mode
    G = 1 << 30
    tb, ws = 65 * G, 1 * G   # one 0.1-degree float32 step's tape, the taped adjoint's workspace
    # 24 steps do not fit in 60 % of 250 GB; one step does
    assert tape_mode("auto", True, True, 24, tb, ws, 250 * G, 0.6) == "step"
    assert tape_mode("auto", False, True, 24, tb, ws, 250 * G, 0.6) is False   # float64: recompute
    # two steps fit: every step taped during the forward
    assert tape_mode("auto", True, True, 1, tb, ws, 250 * G, 0.6) is True
    assert tape_mode("auto", False, True, 1, tb, ws, 250 * G, 0.6) is True
    # without a snapshot of every step the forward cannot keep per-step tapes
    assert tape_mode("auto", True, False, 1, tb, ws, 250 * G, 0.6) == "step"
    # not even one step fits
    assert tape_mode("auto", True, True, 24, tb, ws, 100 * G, 0.6) is False
    # explicit choices
    assert tape_mode("step", True, True, 24, tb, ws, 0, 0.6) == "step"
    assert tape_mode(False, True, True, 24, tb, ws, 0, 0.6) is False
    assert tape_mode(True, True, True, 24, tb, ws, 0, 0.6) is True
    with pytest.raises(ValueError):
        tape_mode("step", False, True, 24, tb, ws, 0, 0.6)
    with pytest.raises(ValueError):
        tape_mode(True, True, False, 24, tb, ws, 0, 0.6)

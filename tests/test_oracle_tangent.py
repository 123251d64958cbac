"""The forward-mode derivatives of the oracle (tests/tangent.py) against
centred differences of the oracle, for every routine the dot-product tests
use: the tangent-linear map J dx the GPU adjoints are checked against is
itself checked here, on the CPU."""
import numpy as np
import pytest

from tests.transpose_cases import CASES, directions, evaluate, golden_state, jitter, tangent


def _directions(st, names, rng):
    return directions(st, names, rng)


@pytest.mark.parametrize("case", list(CASES))
def test_tangent_matches_centred_differences(case):
    rng = np.random.default_rng(11)
    st = jitter(golden_state(case), rng)
    _routine, ins, outs, _f = CASES[case]
    dx = _directions(st, ins, rng)
    base = evaluate(case, st)
    w = {k: rng.standard_normal(np.shape(base[k])) for k in outs}
    jd = tangent(case, st, dx)
    ad = sum(float(np.sum(w[k] * jd[k])) for k in outs)

    h = 1e-7

    def loss(sign):
        v = dict(vars(st.variables))
        for k in ins:
            v[k] = v[k] + sign * h * dx[k]
        from types import SimpleNamespace
        s2 = SimpleNamespace(variables=SimpleNamespace(**v), settings=st.settings)
        out = evaluate(case, s2)
        return sum(float(np.sum(w[k] * out[k])) for k in outs)

    fd = (loss(+1) - loss(-1)) / (2 * h)
    mag = sum(float(np.sum(np.abs(w[k] * base[k]))) for k in outs)
    noise = 100 * 2.2e-16 * mag / h
    assert abs(fd - ad) <= 1e-5 * max(abs(fd), abs(ad)) + noise, (case, fd, ad, noise)

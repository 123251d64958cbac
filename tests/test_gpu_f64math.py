"""The float64 division, reciprocal and square roots of the float64 kernels.

The float64 EVP subcycle, its adjoint, the free drift and the bulk formula
take a/b, 1/b, sqrt(b) and 1/sqrt(b) from the hardware's approximate
reciprocal (square root) refined by the series of the exact correction
(veris_gb300/csrc/f64math.cuh), not from IEEE division and square root.
``veris_f64_math_check`` evaluates every form elementwise; here they are
measured against correctly rounded results (NumPy's IEEE division and square
root; the reciprocal square root through extended precision where NumPy has
it) over operands spanning the float64 range, and against IEEE special
values: zeros, subnormals, negatives, infinities and NaN.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

FORMS = ("div64", "div_lane", "rcp64", "rcp_lane", "sqrt64", "sqrt_lane", "rsqrt64", "rsqrt_lane")
ULP_BOUND = 1   # the series forms against the correctly rounded value


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from veris_gb300 import _abi
    return _abi.load()


def _run(lib, a, b):
    n = a.size
    da = torch.from_numpy(a).cuda()
    db = torch.from_numpy(b).cuda()
    out = torch.empty(8 * n, dtype=torch.float64, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    assert lib.veris_f64_math_check(da.data_ptr(), db.data_ptr(), n, out.data_ptr(), s) == 0
    torch.cuda.synchronize()
    return out.cpu().numpy().reshape(8, n)


def _references(a, b):
    """Correctly rounded a/b, 1/b, sqrt(b) and 1/sqrt(b) (the last within
    half an ulp more where NumPy has no extended precision)."""
    with np.errstate(all="ignore"):
        div = a / b
        rcp = 1.0 / b
        root = np.sqrt(b)
        if np.finfo(np.longdouble).nmant >= 63:
            rroot = (1.0 / np.sqrt(b.astype(np.longdouble))).astype(np.float64)
            extra = 0
        else:
            rroot = 1.0 / np.sqrt(b)
            extra = 1
    return (div, div, rcp, rcp, root, root, rroot, rroot), extra


def _ordered(x):
    """float64 bits as integers ordered like the values (+0 and -0 both 0)."""
    i = x.view(np.int64)
    return np.where(i >= 0, i, -(i & np.int64(0x7FFFFFFFFFFFFFFF)))


def _ulps(x, ref):
    both_nan = np.isnan(x) & np.isnan(ref)
    ox, oy = _ordered(x), _ordered(ref)
    same = (ox >= 0) == (oy >= 0)   # the integer difference cannot overflow there
    d = np.where(same, np.abs(np.where(same, ox - oy, 0)).astype(np.float64),
                 np.abs(ox).astype(np.float64) + np.abs(oy).astype(np.float64))
    d[both_nan] = 0.0
    d[np.isnan(x) != np.isnan(ref)] = np.inf
    return d


def _check(out, a, b):
    refs, extra = _references(a, b)
    worst = {}
    for k, name in enumerate(FORMS):
        bound = ULP_BOUND + (extra if name.startswith("rsqrt") else 0)
        d = _ulps(out[k], refs[k])
        worst[name] = float(d.max())
        bad = np.flatnonzero(d > bound)
        assert bad.size == 0, (name, a[bad[:4]], b[bad[:4]], out[k][bad[:4]], refs[k][bad[:4]])
    return worst


def _in_seed_range(b):
    """positive, normal and at least 2^64 inside both ends of the exponent range"""
    hi = (b.view(np.int64) >> 32).astype(np.int64)
    return (hi >= (64 << 20)) & (hi < (1984 << 20))


def test_series_forms_within_one_ulp(lib):
    """Operands inside the seed range (every warp takes the series)."""
    rng = np.random.default_rng(20261204)
    n = 1 << 20
    a = np.ldexp(rng.uniform(0.5, 1.0, n), rng.integers(-500, 500, n)) * rng.choice((-1.0, 1.0), n)
    b = np.ldexp(rng.uniform(0.5, 1.0, n), rng.integers(-900, 900, n))
    worst = _check(_run(lib, a, b), a, b)
    print("worst ulps:", worst)


def test_special_operands_give_ieee_results(lib):
    """Edge operands mixed into the warps: the warp forms fall back to IEEE
    for the whole warp, the lane forms for the lane."""
    rng = np.random.default_rng(7)
    n = 1 << 16
    a = np.ldexp(rng.uniform(0.5, 1.0, n), rng.integers(-1070, 1020, n)) * rng.choice((-1.0, 1.0), n)
    b = np.ldexp(rng.uniform(0.5, 1.0, n), rng.integers(-1070, 1020, n))
    special = np.array([0.0, -0.0, 5e-324, 1e-310, 2.2250738585072014e-308, 1e-300, 1e300,
                        np.finfo(np.float64).max, np.inf, -np.inf, np.nan, -1.0, -3e-200, 1.0, 4.0])
    idx = rng.choice(n, 4096, replace=False)
    b[idx] = special[rng.integers(0, special.size, idx.size)]
    idx = rng.choice(n, 1024, replace=False)
    a[idx] = special[rng.integers(0, special.size, idx.size)]
    out = _run(lib, a, b)
    _check(out, a, b)
    # IEEE results exactly: per lane where the operand leaves the seed range,
    # and on every lane of a warp (32 consecutive elements) that holds one
    out_lane = ~_in_seed_range(b)
    warp = lambda lane: np.repeat(lane.reshape(-1, 32).any(axis=1), 32)
    out_warp = warp(out_lane)
    out_warp_root = warp(out_lane & (b != 0.0))   # sqrt64 takes zeros in the series path
    with np.errstate(all="ignore"):
        ieee = (a / b, 1.0 / b, np.sqrt(b), 1.0 / np.sqrt(b))
        for k, name in enumerate(FORMS):
            sel = (out_warp_root if name == "sqrt64" else out_warp) if name.endswith("64") else out_lane
            got, want = out[k][sel], ieee[k // 2][sel]
            if name == "sqrt64":   # -0 gives +0 in a warp that takes the series, -0 in one that does not
                want = np.where(want == 0.0, 0.0, want)
                got = np.where(got == 0.0, 0.0, got)
            assert np.array_equal(got.view(np.int64)[~np.isnan(want)], want.view(np.int64)[~np.isnan(want)]), name
            assert np.all(np.isnan(got[np.isnan(want)])), name
        assert 0 < out_lane.sum() < out_warp.sum() < b.size


def test_empty_and_bad_arguments(lib):
    s = torch.cuda.current_stream().cuda_stream
    assert lib.veris_f64_math_check(None, None, 0, None, s) == 0
    assert lib.veris_f64_math_check(None, None, 4, None, s) != 0
    assert lib.veris_f64_math_check(None, None, -1, None, s) != 0

"""Forward-mode derivatives of NumPy code: the tangent-linear map of the oracle.

Test infrastructure.  ``Tangent`` is an array that carries a value and one
directional derivative through the NumPy operations the oracle uses
(arithmetic, powers, square root, exp/log, trigonometry, min/max, abs, sign,
``where``, ``roll``, ``clip``, slicing and slice assignment).  Running an
oracle routine on Tangent inputs whose derivative parts hold a direction dx
gives J dx exactly (to rounding), with J the Jacobian of that routine at the
inputs' values; the dot-product tests compare <J dx, w> with <dx, J^T w>
from the GPU's hand-written adjoint kernels.

Branches follow the values, as in the forward code.  At a tie of max/min
the first argument's derivative is taken; sqrt(0) has derivative 0 (the
subgradient the adjoint kernels use); sign and comparisons have none.
"""
import numpy as np

_HANDLED = {}


def _val(x):
    return x.v if isinstance(x, Tangent) else x


def _der(x):
    return x.d if isinstance(x, Tangent) else 0.0


def _implements(fn):
    def deco(f):
        _HANDLED[fn] = f
        return f
    return deco


class Tangent(np.lib.mixins.NDArrayOperatorsMixin):
    __array_priority__ = 1000

    def __init__(self, v, d=None):
        self.v = np.array(v, dtype=np.float64)
        self.d = np.zeros_like(self.v) if d is None else np.broadcast_to(np.asarray(d, np.float64),
                                                                          self.v.shape).copy()

    # ---- array-like surface
    shape = property(lambda self: self.v.shape)
    ndim = property(lambda self: self.v.ndim)
    dtype = property(lambda self: self.v.dtype)
    size = property(lambda self: self.v.size)

    def __len__(self):
        return len(self.v)

    def __getitem__(self, idx):
        return Tangent(self.v[idx], self.d[idx])

    def __setitem__(self, idx, x):
        self.v[idx] = _val(x)
        self.d[idx] = _der(x)

    def copy(self):
        return Tangent(self.v.copy(), self.d.copy())

    def sum(self, *a, **kw):
        return Tangent(self.v.sum(*a, **kw), self.d.sum(*a, **kw))

    def astype(self, dtype):
        return self.copy()

    def __repr__(self):
        return f"Tangent(v={self.v!r}, d={self.d!r})"

    # ---- ufuncs
    def __array_ufunc__(self, ufunc, method, *inputs, **kw):
        if method != "__call__" or kw.get("out") is not None:
            return NotImplemented
        vals = [_val(x) for x in inputs]
        ders = [_der(x) for x in inputs]
        rule = _RULES.get(ufunc)
        if rule is None:
            if ufunc in _NO_DERIVATIVE:
                return ufunc(*vals)
            raise TypeError(f"Tangent: no rule for {ufunc.__name__}")
        v, d = rule(vals, ders)
        return Tangent(v, d)

    def __array_function__(self, func, types, args, kwargs):
        f = _HANDLED.get(func)
        if f is None:
            raise TypeError(f"Tangent: no rule for {func.__name__}")
        return f(*args, **kwargs)


def _pow(vals, ders):
    a, b = vals
    da, db = ders
    v = a ** b
    d = 0.0
    if not (np.isscalar(da) and da == 0.0):
        with np.errstate(all="ignore"):
            d = d + np.where(a != 0, b * a ** (b - 1.0), np.where(b == 1.0, 1.0, 0.0)) * da
    if not (np.isscalar(db) and db == 0.0):
        with np.errstate(all="ignore"):
            d = d + v * np.log(np.where(a > 0, a, 1.0)) * db
    return v, d


def _sqrt(vals, ders):
    v = np.sqrt(vals[0])
    with np.errstate(all="ignore"):
        g = np.where(v > 0, 0.5 / np.where(v > 0, v, 1.0), 0.0)
    return v, g * ders[0]


def _div(vals, ders):
    a, b = vals
    v = a / b
    return v, (ders[0] - v * ders[1]) / b


def _maximum(vals, ders):
    a, b = vals
    first = a >= b
    return np.maximum(a, b), np.where(first, ders[0], ders[1])


def _minimum(vals, ders):
    a, b = vals
    first = a <= b
    return np.minimum(a, b), np.where(first, ders[0], ders[1])


_RULES = {
    np.add: lambda v, d: (v[0] + v[1], d[0] + d[1]),
    np.subtract: lambda v, d: (v[0] - v[1], d[0] - d[1]),
    np.multiply: lambda v, d: (v[0] * v[1], d[0] * v[1] + v[0] * d[1]),
    np.true_divide: _div,
    np.negative: lambda v, d: (-v[0], -d[0]),
    np.positive: lambda v, d: (v[0], d[0]),
    np.power: _pow,
    np.float_power: _pow,
    np.square: lambda v, d: (v[0] * v[0], 2.0 * v[0] * d[0]),
    np.sqrt: _sqrt,
    np.exp: lambda v, d: (np.exp(v[0]), np.exp(v[0]) * d[0]),
    np.log: lambda v, d: (np.log(v[0]), d[0] / v[0]),
    np.log10: lambda v, d: (np.log10(v[0]), d[0] / (v[0] * np.log(10.0))),
    np.sin: lambda v, d: (np.sin(v[0]), np.cos(v[0]) * d[0]),
    np.cos: lambda v, d: (np.cos(v[0]), -np.sin(v[0]) * d[0]),
    np.arctan: lambda v, d: (np.arctan(v[0]), d[0] / (1.0 + v[0] * v[0])),
    np.arctan2: lambda v, d: (np.arctan2(v[0], v[1]),
                              (v[1] * d[0] - v[0] * d[1]) / np.where(v[0] * v[0] + v[1] * v[1] > 0,
                                                                     v[0] * v[0] + v[1] * v[1], 1.0)),
    np.absolute: lambda v, d: (np.abs(v[0]), np.sign(v[0]) * d[0]),
    np.fabs: lambda v, d: (np.abs(v[0]), np.sign(v[0]) * d[0]),
    np.maximum: _maximum,
    np.minimum: _minimum,
    np.fmax: _maximum,
    np.fmin: _minimum,
    np.sign: lambda v, d: (np.sign(v[0]), np.zeros_like(np.asarray(v[0], dtype=np.float64))),
}
_NO_DERIVATIVE = {np.greater, np.less, np.greater_equal, np.less_equal, np.equal, np.not_equal,
                  np.logical_and, np.logical_or, np.logical_not, np.isfinite, np.isnan}


@_implements(np.where)
def _where(cond, a, b):
    cond = _val(cond)
    return Tangent(np.where(cond, _val(a), _val(b)), np.where(cond, _der(a), _der(b)))


@_implements(np.roll)
def _roll(a, shift, axis=None):
    return Tangent(np.roll(_val(a), shift, axis), np.roll(np.broadcast_to(_der(a), np.shape(_val(a))), shift,
                                                           axis))


@_implements(np.clip)
def _clip(a, lo, hi, **kw):
    return np.minimum(np.maximum(a, lo), hi)


@_implements(np.zeros_like)
def _zeros_like(a, *args, **kw):
    return Tangent(np.zeros_like(_val(a), dtype=np.float64))


@_implements(np.ones_like)
def _ones_like(a, *args, **kw):
    return Tangent(np.ones_like(_val(a), dtype=np.float64))


@_implements(np.full_like)
def _full_like(a, fill, *args, **kw):
    return Tangent(np.full_like(_val(a), _val(fill), dtype=np.float64))


@_implements(np.copy)
def _copy(a, *args, **kw):
    return a.copy()


@_implements(np.array)
def _array(a, *args, **kw):
    return a.copy()


@_implements(np.asarray)
def _asarray(a, *args, **kw):
    return a


@_implements(np.shape)
def _shape(a):
    return np.shape(_val(a))


@_implements(np.sum)
def _sum(a, *args, **kw):
    return a.sum(*args, **kw)


def seed(value, direction):
    """A Tangent at ``value`` with derivative part ``direction``."""
    return Tangent(value, direction)


def values(x):
    return _val(x)


def derivative(x):
    d = _der(x)
    return np.broadcast_to(d, np.shape(_val(x))) if np.isscalar(d) else d

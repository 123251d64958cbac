"""Host-model states: the drop-ins on a state whose variables are NumPy arrays.

A host model such as Veros with its NumPy backend keeps ``state.variables``
as NumPy arrays on the host and calls the plugin's routines with that state
(veris/setup/seaice_global_4deg/seaice_global_4deg.py:878-932).  Every
drop-in routine of this package accepts such a state: the decorator below
mirrors the variables the kernels read onto the GPU, runs the routine there
(the CUDA kernels; nothing is computed on the host), and returns NumPy arrays
as the reference's functional kernels do.

Grid and mask variables (the ones ``set_inits`` derives once,
veris/set_inits.py:6-59, and the host model never changes afterwards) are
uploaded once per array object and kept on the device while the array lives;
all other variables are uploaded on every call, since the host model may
update them in place between calls.  ``forget_device_copies()`` drops the kept
copies (call it after changing a grid or mask array in place).
"""
import functools
import weakref

import numpy as np
import torch

from .state import VerisState
from .variables import ABI_ORDER, GRID, MASKS

STATIC = frozenset(GRID + MASKS)
_kept = {}   # id(array) -> (weakref to it, data pointer, shape, strides, device tensor)


def is_host_array(x):
    return isinstance(x, np.ndarray)


def is_host_state(state):
    """True when the state's variables are host (NumPy) arrays."""
    v = getattr(state, "variables", None)
    ref = getattr(v, "iceMask", None) if v is not None else None
    return is_host_array(ref)


def _device():
    if not torch.cuda.is_available():
        raise RuntimeError("veris_gb300 runs its routines on a CUDA device; none is available "
                           "(there is no CPU implementation)")
    return torch.device("cuda", torch.cuda.current_device())


def to_device(a, dev=None):
    """A float64 device copy of a host array (any strides)."""
    dev = dev or _device()
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64)).to(dev)


def _kept_copy(a, dev):
    key = id(a)
    ent = _kept.get(key)
    ptr = a.__array_interface__["data"][0]
    if ent is not None:
        ref, p, shape, strides, t = ent
        if ref() is a and p == ptr and shape == a.shape and strides == a.strides and t.device == dev:
            return t
    t = to_device(a, dev)
    _kept[key] = (weakref.ref(a), ptr, a.shape, a.strides, t)
    return t


def forget_device_copies():
    """Drop the device copies kept for grid and mask arrays."""
    _kept.clear()


def device_state(state):
    """A VerisState of CUDA tensors mirroring a host state's variables."""
    dev = _device()
    v = state.variables
    out = {}
    for name in ABI_ORDER:
        a = getattr(v, name, None)
        if a is None:
            continue
        if not is_host_array(a):
            a = np.asarray(a)
        out[name] = _kept_copy(a, dev) if name in STATIC else to_device(a, dev)
    return VerisState(out, state.settings)


def to_host(x):
    """Device results -> NumPy arrays (tuples element by element)."""
    if isinstance(x, tuple):
        return tuple(to_host(y) for y in x)
    if isinstance(x, list):
        return [to_host(y) for y in x]
    if isinstance(x, torch.Tensor):
        return x.detach().cpu().numpy()
    return x


def accepts_host_state(fn):
    """Lets a drop-in ``fn(state, *arrays, **kw)`` take a host state: the
    state and any NumPy array arguments are mirrored onto the GPU, ``fn``
    runs there, and its tensors come back as NumPy arrays.  States of CUDA
    tensors pass straight through."""
    @functools.wraps(fn)
    def wrapper(state, *args, **kw):
        if not (is_host_state(state) or any(is_host_array(a) for a in args)):
            return fn(state, *args, **kw)
        dstate = device_state(state) if is_host_state(state) else state
        dev = _device()
        dargs = [to_device(a, dev) if is_host_array(a) else a for a in args]
        return to_host(fn(dstate, *dargs, **kw))
    wrapper.__wrapped_device__ = fn
    return wrapper


def accepts_host_arrays(fn):
    """The same for a routine that reads only the settings of its state
    (the pointwise bulk formula): NumPy array arguments are mirrored, the
    state is not."""
    @functools.wraps(fn)
    def wrapper(state, *args, **kw):
        if not any(is_host_array(a) for a in args):
            return fn(state, *args, **kw)
        dev = _device()
        dargs = [to_device(a, dev) if is_host_array(a) else a for a in args]
        return to_host(fn(state, *dargs, **kw))
    wrapper.__wrapped_device__ = fn
    return wrapper

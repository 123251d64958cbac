"""The sea-ice state on the GPU: ``state.variables`` and ``state.settings``.

Mirrors the host model's state interface that the plugin's kernels read
(``state.variables.<name>`` arrays, ``state.settings.<name>`` scalars), with
the variables held as CUDA tensors (PyTorch owns the memory).  Every
variable is a 2-D ``(nx + 4, ny + 4)`` tensor, y contiguous.
"""
from types import SimpleNamespace

import numpy as np
import torch

from . import _abi
from .variables import ABI_ORDER


class Variables(SimpleNamespace):
    """Attribute container of the state's 2-D tensors."""

    def names(self):
        return [k for k, v in vars(self).items() if isinstance(v, torch.Tensor)]


class VerisState:
    def __init__(self, variables, settings):
        self.variables = variables if isinstance(variables, Variables) else Variables(**variables)
        self.settings = settings

    @classmethod
    def from_numpy(cls, arrays, settings, device="cuda", dtype=torch.float64):
        v = {k: torch.as_tensor(np.ascontiguousarray(a), dtype=dtype).to(device) for k, a in arrays.items()}
        return cls(v, settings)

    def to_numpy(self, names=None):
        names = names or self.variables.names()
        return {n: getattr(self.variables, n).detach().cpu().numpy() for n in names}

    @property
    def shape(self):
        return tuple(self.variables.iceMask.shape)


def require_device(t, name, dtype, shape):
    if not isinstance(t, torch.Tensor):
        raise TypeError(f"state variable {name} must be a torch tensor, got {type(t).__name__}")
    if not t.is_cuda:
        raise ValueError(f"state variable {name} must live on a CUDA device (no CPU path exists)")
    if t.dtype != dtype:
        raise TypeError(f"state variable {name} must be {dtype}, got {t.dtype}")
    if tuple(t.shape) != shape:
        raise ValueError(f"state variable {name} has shape {tuple(t.shape)}, expected {shape}")
    return t if t.is_contiguous() else t.contiguous()


class Call:
    """Grid, params and field table of one C-ABI call, with keep-alive refs."""

    def __init__(self, state, dtype=torch.float64, variables=None):
        v = state.variables if variables is None else variables
        sett = state.settings
        ref = v.iceMask
        if ref.dim() != 2:
            raise ValueError("state variables must be 2-D")
        self.shape = tuple(ref.shape)
        self.dtype = dtype
        self.device = ref.device
        NX, NY = self.shape
        olx, oly = int(sett.olx), int(sett.oly)
        self.grid = _abi.VerisGrid(NX - 2 * olx, NY - 2 * oly, olx, oly, NY)
        self.params = _abi.params_from_settings(sett)
        self.fields = _abi.VerisFields()
        self.keep = []
        for n in ABI_ORDER:
            t = getattr(v, n, None)
            if t is None:
                continue
            t = require_device(t, n, dtype, self.shape)
            self.keep.append(t)
            setattr(self.fields, n, t.data_ptr())
        self.stream = torch.cuda.current_stream(self.device).cuda_stream
        self.lib = _abi.load()

    def empty(self, n=1):
        out = [torch.empty(self.shape, dtype=self.dtype, device=self.device) for _ in range(n)]
        return out if n > 1 else out[0]

    def arg(self, t, name="array"):
        t = require_device(t, name, self.dtype, self.shape)
        self.keep.append(t)
        return t.data_ptr()

    def workspace(self, nbytes):
        ws = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=self.device)
        self.keep.append(ws)
        return ws.data_ptr(), ws.numel()

    def refs(self):
        return (ctypes_ref(self.grid), ctypes_ref(self.params), ctypes_ref(self.fields))


def ctypes_ref(x):
    import ctypes
    return ctypes.byref(x)

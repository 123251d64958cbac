"""veris/global_sum.py:1-4 is the identity on one process; ``global_sum`` keeps
that contract.  ``interior_sum`` is the deterministic float64 device
reduction used by the conservation diagnostics."""
import ctypes

import torch

from ._abi import VerisGrid, check, load


def global_sum(A):
    """veris/global_sum.py:1-4 (one process: the identity)."""
    return A


def interior_sum(A, weight=None, olx=2, oly=2):
    """Sum of ``A * weight`` over the interior, float64, run-to-run reproducible.

    Returns a 0-d float64 CUDA tensor (no host synchronisation).
    """
    if not (A.is_cuda and A.dtype == torch.float64 and A.dim() == 2 and A.is_contiguous()):
        raise TypeError("A must be a contiguous 2-D float64 CUDA tensor")
    NX, NY = A.shape
    g = VerisGrid(NX - 2 * olx, NY - 2 * oly, olx, oly, NY)
    lib = load()
    ws = torch.empty(lib.veris_reduce_workspace_bytes(ctypes.byref(g)), dtype=torch.uint8, device=A.device)
    out = torch.empty((), dtype=torch.float64, device=A.device)
    wp = None
    if weight is not None:
        weight = weight.contiguous()
        wp = weight.data_ptr()
    check("interior_sum", lib.veris_global_sum_f64(ctypes.byref(g), A.data_ptr(), wp, out.data_ptr(),
                                                   ws.data_ptr(), ws.numel(),
                                                   torch.cuda.current_stream(A.device).cuda_stream))
    return out

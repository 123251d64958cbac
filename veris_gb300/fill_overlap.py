"""Drop-ins for veris/fill_overlap.py: the halo fill, in place."""
import torch

from ._abi import check, load, params_from_settings, VerisGrid


def fill_overlap(state, A):
    """veris/fill_overlap.py:6-18: fills A's halos in place and returns A
    (a NumPy array is filled on the GPU and updated in place)."""
    import ctypes
    from .hostarrays import is_host_array, to_device
    if is_host_array(A):
        t = fill_overlap(state, to_device(A))
        A[...] = t.cpu().numpy()
        return A
    s = state.settings
    if not (isinstance(A, torch.Tensor) and A.is_cuda and A.dim() == 2 and A.is_contiguous()):
        raise TypeError("A must be a contiguous 2-D CUDA tensor")
    NX, NY = A.shape
    g = VerisGrid(NX - 2 * s.olx, NY - 2 * s.oly, s.olx, s.oly, NY)
    p = params_from_settings(s)
    lib = load()
    stream = torch.cuda.current_stream(A.device).cuda_stream
    if A.dtype == torch.float64:
        st = lib.veris_fill_overlap_f64(ctypes.byref(g), ctypes.byref(p), A.data_ptr(), stream)
    elif A.dtype == torch.float32:
        st = lib.veris_fill_overlap_f32(ctypes.byref(g), ctypes.byref(p), A.data_ptr(), stream)
    else:
        raise TypeError("A must be float64 or float32")
    check("fill_overlap", st)
    return A


def fill_overlap_uv(state, U, V):
    """veris/fill_overlap.py:21-23."""
    return fill_overlap(state, U), fill_overlap(state, V)

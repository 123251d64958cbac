"""Drop-in for veris/heat_flux_MITgcm.py: the bulk-formula fluxes over open
ocean that produce the atmospheric forcing of the sea-ice step."""
import torch

from . import _abi
from ._abi import check
from .hostarrays import accepts_host_arrays

BULK_OUTPUTS = ("flwupa", "flha", "fsha", "df0dT", "ust", "vst", "evp", "ssq", "dEvdT")


@accepts_host_arrays
def bulkf_formula_lanl(state, uw, vw, ta, qa, tsf, ocn_mask, outputs=BULK_OUTPUTS):
    """veris/heat_flux_MITgcm.py:5-123 -> (flwupa, flha, fsha, df0dT, ust,
    vst, evp, ssq, dEvdT).

    The inputs are CUDA tensors of one shape and one dtype (float64, or
    float32 for the float32 kernel); the formula is pointwise, so any shape
    works.  ``ocn_mask`` only fixes the shape, as in the reference.  Outputs
    not named in ``outputs`` are not computed and come back as None (the
    reference's own caller discards evp, ssq and dEvdT,
    veris/setup/seaice_global_4deg/seaice_global_4deg.py:761)."""
    args = [uw, vw, ta, qa, tsf]
    dtype = uw.dtype
    if dtype not in (torch.float64, torch.float32):
        raise TypeError(f"bulkf_formula_lanl: float64 or float32 inputs, got {dtype}")
    shape = tuple(uw.shape)
    for name, t in zip(("uw", "vw", "ta", "qa", "tsf", "ocn_mask"), args + [ocn_mask]):
        if not (torch.is_tensor(t) and t.is_cuda):
            raise TypeError(f"bulkf_formula_lanl: {name} must be a CUDA tensor")
        if tuple(t.shape) != shape:
            raise ValueError(f"bulkf_formula_lanl: {name} has shape {tuple(t.shape)}, expected {shape}")
    args = [t.to(dtype).contiguous() for t in args]
    unknown = set(outputs) - set(BULK_OUTPUTS)
    if unknown:
        raise ValueError(f"bulkf_formula_lanl: unknown outputs {sorted(unknown)}")
    outs = [torch.empty(shape, dtype=dtype, device=uw.device) if n in outputs else None for n in BULK_OUTPUTS]
    lib = _abi.load()
    p = _abi.params_from_settings(state.settings)
    fn = lib.veris_bulkf_formula_lanl_f64 if dtype == torch.float64 else lib.veris_bulkf_formula_lanl_f32
    import ctypes
    stream = torch.cuda.current_stream(uw.device).cuda_stream
    check("bulkf_formula_lanl", fn(ctypes.byref(p), uw.numel(), *[t.data_ptr() for t in args], None,
                                   *[0 if t is None else t.data_ptr() for t in outs], stream))
    return tuple(outs)

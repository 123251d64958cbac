"""ctypes binding of the C ABI declared in ``include/veris_gb300.h``.

This is the Python host's side of the boundary: it loads the in-tree CUDA
library, declares the argument types of every entry point and packs the
settings into the ``VerisParams`` struct.  The library is required: there is
no CPU fallback, and a missing or unloadable library raises ``VerisError``.
"""
import ctypes
import os

import numpy as np

from .variables import ABI_ORDER

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "_lib", "libveris_gb300.so")

STATUS = {
    0: "ok", 1: "bad grid shape, halo width or pitch", 2: "misaligned pointer or pitch",
    3: "non-finite value detected", 4: "device-side wait timed out",
    5: "CUDA launch or API call failed", 6: "invalid argument",
    7: "settings not supported by this entry point", 8: "workspace missing or too small",
    9: "grid larger than a fixed-size entry point's scratch",
}
VERIS_ERR_NAN = 3


class VerisError(RuntimeError):
    def __init__(self, where, status):
        self.status = status
        super().__init__(f"{where}: status {status} ({STATUS.get(status, 'unknown')})")


# Order and names of the VerisParams members (the X-macro lists of the header)
PARAM_DOUBLES = (
    "deltatTherm recip_deltatTherm deltatDyn recip_deltatDyn evpAlpha evpBeta aEVPalphaMin "
    "EVPcFac rhoIce rhoFresh rhoSea rhoAir rhoSnow recip_rhoFresh recip_rhoSea rhoIce2rhoSnow "
    "rhoIce2rhoFresh rhoFresh2rhoSnow dryIceAlb dryIceAlb_south wetIceAlb wetIceAlb_south "
    "drySnowAlb drySnowAlb_south wetSnowAlb wetSnowAlb_south wetAlbTemp lhFusion lhEvap "
    "lhSublim cpAir cpWater stefBoltz iceEmiss snowEmiss iceConduct snowConduct hCut shortwave "
    "tempFrz dtempFrz_dS saltIce_ref minLWdown minTIce minTAir dalton Area_reg hIce_reg "
    "celsius2K stantonNr uStarBase McPheeTaperFac recip_h0 recip_h0_south recip_nITC sinWin "
    "cosWin sinWat cosWat sinWatOcn cosWatOcn wSpeedMin hIce_min Area_min airIceDrag "
    "airIceDrag_south waterIceDrag waterIceDrag_south cDragMin seaIceLoadFac gravity "
    "PlasDefCoeff deltaMin pressReplFac pStar cStar basalDragU0 basalDragK1 basalDragK2 "
    "cBasalStar tensileStrFac CrMax sideDragCoeff sideDragU0 "
    "s4t_cc0 s4t_cc1 s4t_cc2 s4t_d1 s4t_d1i "
    "zvir cpdair karman latvap ocean_emissivity gamma_blk grav"
).split()
PARAM_INTS = (
    "nITC noSlip secondOrderBC useRelativeWind useRealFreshWaterFlux useAdaptiveEVP "
    "veros_fill enable_cyclic_x use_coastline extensiveFld nEVPsteps pad_"
).split()


class VerisGrid(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("olx", ctypes.c_int32),
                ("oly", ctypes.c_int32), ("ld", ctypes.c_int64)]


class VerisParams(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in PARAM_DOUBLES] + [(n, ctypes.c_int32) for n in PARAM_INTS]


class VerisFields(ctypes.Structure):
    """One device pointer per state variable (VerisFieldsF64 / VerisFieldsF32)."""
    _fields_ = [(n, ctypes.c_void_p) for n in ABI_ORDER]


BULK_PARAMS = ("zvir", "cpdair", "karman", "latvap", "ocean_emissivity", "gamma_blk", "grav")
DERIVED_PARAMS = ("EVPcFac", "sinWin", "cosWin", "sinWatOcn", "cosWatOcn",
                  "s4t_cc0", "s4t_cc1", "s4t_cc2", "s4t_d1", "s4t_d1i", "pad_")


def params_from_settings(sett):
    """Pack a settings namespace into ``VerisParams``.

    The derived members are computed here the way the reference computes
    them in Python (veris/dynsolver.py:41-42, veris/ocean_stress.py:22-23,
    veris/evp_solver.py:264-268, veris/solve4temp.py:14-27), so both sides
    start from identically rounded constants.
    """
    from .settings import SETTINGS
    p = VerisParams()
    for n in PARAM_DOUBLES:
        if n in DERIVED_PARAMS:
            continue
        if n in BULK_PARAMS and not hasattr(sett, n):
            # host-model constants of the bulk formulae; settings saved before
            # they were carried here hold the defaults
            setattr(p, n, float(SETTINGS[n][0]))
            continue
        setattr(p, n, float(getattr(sett, n)))
    for n in PARAM_INTS:
        if n in DERIVED_PARAMS:
            continue
        setattr(p, n, int(getattr(sett, n)))
    p.sinWin = float(np.sin(np.deg2rad(sett.airTurnAngle)))
    p.cosWin = float(np.cos(np.deg2rad(sett.airTurnAngle)))
    p.sinWatOcn = float(np.sin(np.deg2rad(sett.waterTurnAngle)))
    p.cosWatOcn = float(np.cos(np.deg2rad(sett.waterTurnAngle)))
    p.EVPcFac = float(sett.deltatDyn * 4 * (np.pi * sett.aEvpCoeff) ** 2) if sett.useAdaptiveEVP else 0.0
    aa1, aa2, bb1, pa = 2663.5, 12.537, 0.622, 100000
    cc0 = 10 ** aa2
    p.s4t_cc0 = float(cc0)
    p.s4t_cc1 = float(cc0 * aa1 * bb1 * pa * np.log(10))
    p.s4t_cc2 = float(cc0 * (1 - bb1))
    p.s4t_d1 = float(sett.dalton * sett.cpAir * sett.rhoAir)
    p.s4t_d1i = float(sett.dalton * sett.lhSublim * sett.rhoAir)
    p.pad_ = 0
    return p


_P = ctypes.c_void_p
_G = ctypes.POINTER(VerisGrid)
_Pa = ctypes.POINTER(VerisParams)
_F = ctypes.POINTER(VerisFields)
_I = ctypes.c_int
_S = ctypes.c_size_t
_L = ctypes.c_int64

SIGNATURES = {
    "veris_params_size": ([], _S),
    "veris_fields_count": ([], _S),
    "veris_field_name": ([_S], ctypes.c_char_p),
    "veris_status_string": ([_I], ctypes.c_char_p),
    "veris_device_ok": ([], _I),
    "veris_fill_overlap_f64": ([_G, _Pa, _P, _P], _I),
    "veris_fill_overlap_f32": ([_G, _Pa, _P, _P], _I),
    "veris_sea_ice_mass_f64": ([_G, _Pa, _F, _P, _P, _P, _P], _I),
    "veris_area_ws_f64": ([_G, _Pa, _F, _P, _P, _P], _I),
    "veris_tau_xy_f64": ([_G, _Pa, _F, _P, _P, _P], _I),
    "veris_wind_forcing_xy_f64": ([_G, _Pa, _F, _P, _P, _P], _I),
    "veris_sea_ice_strength_f64": ([_G, _Pa, _F, _P, _P], _I),
    "veris_strainrates_f64": ([_G, _Pa, _F, _P, _P, _P, _P, _P, _P], _I),
    "veris_viscosities_f64": ([_G, _Pa, _F, _P, _P, _P, _P, _P, _P, _P], _I),
    "veris_c_point_to_z_point_f64": ([_G, _Pa, _F, _P, ctypes.c_int32, _P, _P], _I),
    "veris_ocean_drag_coeffs_f64": ([_G, _Pa, _F, _P, _P, _P, _P], _I),
    "veris_basal_drag_coeffs_f64": ([_G, _Pa, _F, _P, _P, _P, _P], _I),
    "veris_side_drag_f64": ([_G, _Pa, _F, _P, _P, _P, _P, _P], _I),
    "veris_stressdiv_f64": ([_G, _Pa, _F, _P, _P, _P, _P, _P, _P], _I),
    "veris_evp_workspace_bytes": ([_G, ctypes.c_int32], _S),
    "veris_evp_solver_f64": ([_G, _Pa, _F, ctypes.c_int32, _P, _P, _P, _P, _P, _P, _S, _P], _I),
    "veris_evp_residual_workspace_bytes": ([_G, ctypes.c_int32, ctypes.c_int32], _S),
    "veris_evp_residual_solver_f64": ([_G, _Pa, _F, ctypes.c_int32] + [_P] * 8 + [_S, _P], _I),
    "veris_evp_residual_solver_f32": ([_G, _Pa, _F, ctypes.c_int32] + [_P] * 8 + [_S, _P], _I),
    "veris_freedrift_solver_f64": ([_G, _Pa, _F, _P, _P, _P], _I),
    "veris_freedrift_solver_f32": ([_G, _Pa, _F, _P, _P, _P], _I),
    "veris_bulkf_formula_lanl_f64": ([_Pa, _L] + [_P] * 15 + [_P], _I),
    "veris_bulkf_formula_lanl_f32": ([_Pa, _L] + [_P] * 15 + [_P], _I),
    "veris_evp_solver_f32": ([_G, _Pa, _F, ctypes.c_int32, _P, _P, _P, _P, _P, _P, _S, _P], _I),
    "veris_evp_fast_workspace_bytes": ([_G, ctypes.c_int32], _S),
    "veris_evp_fast_settings_check": ([_Pa], _I),
    "veris_evp_walk_settings_check": ([_Pa], _I),
    "veris_evp_fast_check": ([_G, _Pa, _F, _P, _P], _I),
    "veris_evp_fast_solver_f32": ([_G, _Pa, _F, ctypes.c_int32, _P, _P, _P, _P, _P, _P, _S, _P], _I),
    "veris_evp_fast_solver_f64": ([_G, _Pa, _F, ctypes.c_int32, _P, _P, _P, _P, _P, _P, _S, _P], _I),
    "veris_evp_f64_tile_rows": ([ctypes.c_int32], _I),
    "veris_evp_walk_persistent": ([ctypes.c_int32], _I),
    "veris_evp_adjoint_f32_form": ([ctypes.c_int32], _I),
    "veris_evp_walk_solver_f32": ([_G, _Pa, _F, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, _P, _P, _P, _P, _P,
                                   _P, _S, _P], _I),
    "veris_evp_smem_solver_f32": ([_G, _Pa, _F, ctypes.c_int32, _P, _P, _P, _P, _P, _P, _S, _P], _I),
    "veris_evp_fast_status": ([_P, ctypes.POINTER(ctypes.c_int32), _P], _I),
    "veris_evp_solver_f64_noalloc": ([_G, _Pa, _F, ctypes.c_int32, _P, _P, _P, _P, _P, _P], _I),
    "veris_evp_adjoint_workspace_bytes": ([_G, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32], _S),
    "veris_evp_adjoint_f64": ([_G, _Pa, _F, ctypes.c_int32, ctypes.c_int32] + [_P] * 10 + [_F, _P, _P, _S, _P], _I),
    "veris_evp_tape_bytes": ([_G, ctypes.c_int32, ctypes.c_int32], _S),
    "veris_evp_fast_tape_f64": ([_G, _Pa, _F, ctypes.c_int32] + [_P] * 6 + [_S, _P, _S, _P], _I),
    "veris_evp_adjoint_taped_workspace_bytes": ([_G, ctypes.c_int32], _S),
    "veris_evp_adjoint_taped_f64": ([_G, _Pa, _F, ctypes.c_int32, _P, _S] + [_P] * 10 + [_F, _P, _P, _S, _P], _I),
    "veris_evp_fast_tape_f32": ([_G, _Pa, _F, ctypes.c_int32] + [_P] * 6 + [_S, _P, _S, _P], _I),
    "veris_evp_adjoint_f32": ([_G, _Pa, _F, ctypes.c_int32, ctypes.c_int32] + [_P] * 10 + [_F, _P, _P, _S, _P], _I),
    "veris_evp_adjoint_taped_workspace_bytes_f32": ([_G, ctypes.c_int32], _S),
    "veris_evp_adjoint_taped_f32": ([_G, _Pa, _F, ctypes.c_int32, _P, _S] + [_P] * 10 + [_F, _P, _P, _S, _P], _I),
    "veris_fill_overlap_adjoint_f64": ([_G, _Pa, _P, _P, _P], _I),
    "veris_advection_adjoint_workspace_bytes": ([_G], _S),
    "veris_advection_adjoint_f64": ([_G, _Pa, _F] + [_P] * 8 + [_P, _S, _P], _I),
    "veris_cleanup_adjoint_f64": ([_G, _Pa, _F] + [_P] * 8 + [_P], _I),
    "veris_growth_adjoint_f64": ([_G, _Pa, _F] + [_P] * 8 + [_P], _I),
    "veris_prep_adjoint_workspace_bytes": ([_G], _S),
    "veris_prep_adjoint_f64": ([_G, _Pa, _F, _F] + [_P] * 6 + [_P, _S, _P], _I),
    "veris_batch_workspace_bytes": ([ctypes.c_int32, _G], _S),
    "veris_batch_init": ([ctypes.c_int32, _G, _Pa, _P, _S], _I),
    "veris_batch_tiles": ([ctypes.c_int32, _G, ctypes.c_int32], _I),
    "veris_batch_prep_member_f32": ([ctypes.c_int32, _G, _Pa, _P, _S, ctypes.c_int32, _F, _P], _I),
    "veris_batch_evp_f32": ([ctypes.c_int32, _G, _Pa, _P, _S] + [ctypes.c_int32] * 5 + [_P], _I),
    "veris_batch_copy_state_f32": ([ctypes.c_int32, _G, _Pa, _P, _S, ctypes.c_int32, ctypes.c_int32]
                                   + [_P] * 5 + [_P], _I),
    "veris_ocean_stress_uv_f64": ([_G, _Pa, _F, _P, _P, _P], _I),
    "veris_limiter_f64": ([_P, _P, _L, _P], _I),
    "veris_calc_zonal_flux_f64": ([_G, _Pa, _F, _P, _P, _P, _P], _I),
    "veris_calc_meridional_flux_f64": ([_G, _Pa, _F, _P, _P, _P, _P], _I),
    "veris_advection_workspace_bytes": ([_G, ctypes.c_int32], _S),
    "veris_calc_advection_f64": ([_G, _Pa, _F, _P, _P, _P, _S, _P], _I),
    "veris_advection_f64": ([_G, _Pa, _F, _P, _P, _P, _P, _S, _P], _I),
    "veris_advection_f32": ([_G, _Pa, _F, _P, _P, _P, _P, _S, _P], _I),
    "veris_clean_up_advection_f64": ([_G, _Pa, _F, _P, _P, _P, _P, _P, _P, _P], _I),
    "veris_ridging_f64": ([_G, _Pa, _F, _P, _P], _I),
    "veris_solve4temp_f64": ([_G, _Pa, _F, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P], _I),
    "veris_growth_f64": ([_G, _Pa, _F] + [_P] * 11 + [_P], _I),
    "veris_growth_rows_f64": ([_G, _Pa, _F] + [_P] * 11 + [ctypes.c_int32, ctypes.c_int32, _P], _I),
    "veris_reduce_workspace_bytes": ([_G], _S),
    "veris_mbarrier_wait_probe": ([ctypes.c_int32, ctypes.c_uint32, _P, _P], _I),
    "veris_global_sum_f64": ([_G, _P, _P, _P, _P, _S, _P], _I),
    "veris_budget_workspace_bytes": ([], _S),
    "veris_budget_sums_f64": ([_G, _P, _P, ctypes.c_int32, ctypes.c_int32, _P, ctypes.c_int32, _P, ctypes.c_int32,
                               _P, _S, _P], _I),
    "veris_check_finite_f64": ([_G, _P, ctypes.c_int32, ctypes.c_int32, _P, _P], _I),
    "veris_check_finite_f32": ([_G, _P, ctypes.c_int32, ctypes.c_int32, _P, _P], _I),
    "veris_convert_f64_to_f32": ([_P, _P, _L, _P], _I),
    "veris_convert_f32_to_f64": ([_P, _P, _L, _P], _I),
    "veris_f64_math_check": ([_P, _P, _L, _P, _P], _I),
}

_lib = None


def load(path=None):
    """Load the CUDA library (once) and declare its entry points."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    path = path or LIBPATH
    if not os.path.exists(path):
        raise VerisError(f"CUDA library {path} is missing; build it with "
                         f"`python -m veris_gb300.build`", 6)
    lib = ctypes.CDLL(path)
    for name, (args, res) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    if lib.veris_params_size() != ctypes.sizeof(VerisParams):
        raise VerisError("VerisParams layout differs between the library and the binding", 6)
    if lib.veris_fields_count() != len(ABI_ORDER):
        raise VerisError("VerisFields layout differs between the library and the binding", 6)
    for k, n in enumerate(ABI_ORDER):
        if lib.veris_field_name(k).decode() != n:
            raise VerisError(f"VerisFields member {k} is {lib.veris_field_name(k)!r}, expected {n}", 6)
    if path == LIBPATH:
        _lib = lib
    return lib


def check(where, status):
    if status != 0:
        raise VerisError(where, status)

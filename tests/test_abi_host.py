"""CPU-side checks of the C-ABI boundary: the library loads, exports every
symbol the header declares, and its struct layouts match the binding.  No
compute call is made (there is no GPU here)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "veris_gb300.h")


@pytest.fixture(scope="module")
def lib():
    from veris_gb300 import build, _abi
    path = build.build()
    return _abi.load(path)


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(veris_[a-z0-9_]+)\s*\(", text)))


def _macro_names(macro):
    text = open(HEADER).read()
    m = re.search(r"#define " + macro + r"\(X\)(.*?)\n\n", text, flags=re.S)
    return re.findall(r"X\((\w+)\)", m.group(1))


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) > 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_declares_every_symbol():
    from veris_gb300 import _abi
    assert set(declared_functions()) <= set(_abi.SIGNATURES)


def test_field_table_layout(lib):
    from veris_gb300 import _abi
    from veris_gb300.variables import ABI_ORDER
    assert _macro_names("VERIS_FIELDS") == list(ABI_ORDER)
    assert lib.veris_fields_count() == len(ABI_ORDER)
    assert [lib.veris_field_name(k).decode() for k in range(len(ABI_ORDER))] == list(ABI_ORDER)
    assert lib.veris_field_name(len(ABI_ORDER)) is None
    assert ctypes.sizeof(_abi.VerisFields) == 8 * len(ABI_ORDER)


def test_params_layout(lib):
    from veris_gb300 import _abi
    assert _macro_names("VERIS_PARAM_DOUBLES") == _abi.PARAM_DOUBLES
    assert _macro_names("VERIS_PARAM_INTS") == _abi.PARAM_INTS
    assert lib.veris_params_size() == ctypes.sizeof(_abi.VerisParams)


def test_status_strings(lib):
    assert lib.veris_status_string(0) == b"ok"
    assert b"workspace" in lib.veris_status_string(8)


def test_shape_validation_without_device(lib):
    """Workspace queries reject bad grids before touching the device."""
    from veris_gb300 import _abi
    good = _abi.VerisGrid(90, 40, 2, 2, 44)
    assert lib.veris_evp_workspace_bytes(ctypes.byref(good), 8) == 5 * ((94 * 44 * 8 + 255) // 256 * 256)
    for bad in (_abi.VerisGrid(90, 40, 3, 2, 44), _abi.VerisGrid(90, 40, 2, 2, 43),
                _abi.VerisGrid(3, 40, 2, 2, 44)):
        assert lib.veris_evp_workspace_bytes(ctypes.byref(bad), 8) == 0
    assert lib.veris_evp_workspace_bytes(ctypes.byref(good), 2) == 0


def test_params_pack_derived_constants():
    import numpy as np
    from veris_gb300 import _abi
    from veris_gb300.settings import default_settings
    s = default_settings(airTurnAngle=25.0, waterTurnAngle=10.0, useAdaptiveEVP=True)
    p = _abi.params_from_settings(s)
    assert p.sinWin == float(np.sin(np.deg2rad(25.0)))
    assert p.cosWatOcn == float(np.cos(np.deg2rad(10.0)))
    assert p.EVPcFac == s.deltatDyn * 4 * (np.pi * 0.5) ** 2
    assert p.s4t_cc0 == 10 ** 12.537
    assert p.useAdaptiveEVP == 1 and p.noSlip == 1


def test_missing_library_fails_loudly(tmp_path):
    from veris_gb300 import _abi
    with pytest.raises(_abi.VerisError):
        _abi.load(str(tmp_path / "nope.so"))

"""The host model's plugin interface without a GPU.

``tests/golden/setup_callsite.json`` holds the sea-ice step of the
reference setup (veris/setup/seaice_global_4deg/seaice_global_4deg.py:
879-932) as the setup's source writes it: each routine it imports from the
plugin, the module, the arguments and the variables it assigns, plus the
names of the plugin's settings and variables tables (veris/settings.py,
veris/variables.py), all read from the reference by
``tests/golden/make_golden.py --plugin``.
"""
import importlib
import inspect
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _site():
    with open(os.path.join(HERE, "golden", "setup_callsite.json")) as f:
        return json.load(f)


def test_interface_dictionary():
    import veris_gb300
    i = veris_gb300.__VEROS_INTERFACE__
    assert set(i) == {"name", "setup_entrypoint", "run_entrypoint", "settings", "variables"}
    assert i["name"] == "veris"
    assert callable(i["setup_entrypoint"]) and callable(i["run_entrypoint"])
    assert i["run_entrypoint"](object()) is None          # veris/model.py:1-9: a no-op
    for s in i["settings"].values():
        assert hasattr(s, "default") and hasattr(s, "type") and hasattr(s, "description")
    for v in i["variables"].values():
        assert v.dims == ("xt", "yt")


def test_tables_cover_the_plugins():
    import veris_gb300
    i = veris_gb300.__VEROS_INTERFACE__
    site = _site()
    assert set(site["plugin_settings"]) <= set(i["settings"]), \
        sorted(set(site["plugin_settings"]) - set(i["settings"]))
    assert set(site["plugin_variables"]) <= set(i["variables"]), \
        sorted(set(site["plugin_variables"]) - set(i["variables"]))


def test_every_routine_the_setup_calls_exists_with_its_signature():
    site = _site()
    assert site["lines"] == [879, 932] and len(site["calls"]) == 15
    for c in site["calls"]:
        assert c["module"].startswith("veris.")
        mod = importlib.import_module("veris_gb300." + c["module"][len("veris."):])
        fn = getattr(mod, c["func"])
        sig = inspect.signature(fn)
        sig.bind(*c["args"])            # the setup's positional arguments fit
        assert c["args"][0] == "state"


def test_no_host_fallback_without_a_device():
    """A host (NumPy) state is mirrored to the GPU; with no GPU the call
    fails loudly instead of computing on the host."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    from types import SimpleNamespace
    from veris_gb300.area_mass import SeaIceMass
    from veris_gb300.settings import default_settings
    a = np.zeros((8, 6))
    st = SimpleNamespace(variables=SimpleNamespace(iceMask=a, hIceMean=a, hSnowMean=a), settings=default_settings())
    with pytest.raises(RuntimeError, match="CUDA"):
        SeaIceMass(st)


def test_host_state_detection():
    from types import SimpleNamespace
    from veris_gb300.hostarrays import is_host_state, to_host
    assert is_host_state(SimpleNamespace(variables=SimpleNamespace(iceMask=np.zeros(3))))
    assert not is_host_state(SimpleNamespace(variables=SimpleNamespace()))
    assert to_host((1, [2.0])) == (1, [2.0])

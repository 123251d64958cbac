"""GB300-native sea-ice step (EVP/mEVP dynamics, advection, thermodynamics).

Importing the package gives the host model's plugin interface,
``__VEROS_INTERFACE__`` (veris/__init__.py:17-23); the routines live in the
modules named as the reference's (``veris_gb300.area_mass``,
``veris_gb300.dynsolver``, ``veris_gb300.advection``, ...).
"""
__version__ = "0.2.0"

from .plugin import __VEROS_INTERFACE__  # noqa: E402,F401

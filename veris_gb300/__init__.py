"""GB300-native sea-ice step (EVP/mEVP dynamics, advection, thermodynamics)."""
__version__ = "0.1.0"

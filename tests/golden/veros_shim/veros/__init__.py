"""Minimal stand-in for the Veros API surface the plugin imports.

Test infrastructure only: it lets ``tests/golden/make_golden.py`` execute the
reference plugin's own NumPy code in this container, where the Veros package
(pinned by the reference at veros 1.4.x) is not installed.  It restates the
single-process NumPy behaviour of the few Veros entry points used:
decorators are identities, ``update`` assigns in place, ``for_loop`` is a
Python loop and ``enforce_boundaries`` copies the periodic x halo.
"""
import logging

logger = logging.getLogger("veros-shim")


def veros_kernel(function=None, **kwargs):
    if function is None:
        return lambda f: f
    return function


veros_routine = veros_kernel


class KernelOutput(dict):
    pass


class VerosSetup:
    pass

"""GB300-native wave-function propagation engine.

Drop-in for the propagation path of WaveFunctionSimPython: the modules
``sim_state``, ``measurement``, ``operators``, ``core_sim``, ``iter_data`` and
``initialisation`` keep the reference's call surface and TOML schema, and call
the CUDA engine (``_wfs.so``, C ABI in ``include/wfs.h``) through ctypes.
"""
from ._lib import Engine, WfsError, load  # noqa: F401

__all__ = ["Engine", "WfsError", "load"]

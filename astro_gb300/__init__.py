"""astro_gb300 — the osbo/astro Barnes-Hut step on one GB300 (sm_103a).

The compute path is libastro_cuda.so (astro_gb300/csrc, C ABI in
include/astro_cuda.h). This package is its Python host side: ctypes
bindings, the byte layouts, a Renderer-like ``Simulation`` and the
stand-alone ``RadixSort``.
"""
from . import layouts
from ._native import AstroError, LIB_PATH
from .layouts import (COLOR_TYPE, OCTREE_NODE, POSITION_MASS, VELOCITY_RADIUS, Params,
                      PRESET_PHYSICAL, PRESET_REFERENCE, FORM_PLAIN, FORM_PRECISION,
                      FLAG_IEEE_EXACT, FLAG_NO_GRAPH, FLAG_PERSISTENT, FLAG_OPEN_DELTA,
                      FLAG_QUADRUPOLE, FLAG_PER_PARTICLE)
from .simulation import Simulation, default_params, version

__all__ = [
    "AstroError", "LIB_PATH", "Simulation", "default_params", "version", "layouts", "Params",
    "POSITION_MASS", "VELOCITY_RADIUS", "COLOR_TYPE", "OCTREE_NODE", "PRESET_PHYSICAL",
    "PRESET_REFERENCE", "FORM_PLAIN", "FORM_PRECISION", "FLAG_IEEE_EXACT", "FLAG_NO_GRAPH",
    "FLAG_PERSISTENT", "FLAG_OPEN_DELTA", "FLAG_QUADRUPOLE", "FLAG_PER_PARTICLE",
]

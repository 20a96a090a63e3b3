"""rendu_gb300 -- GB300 (sm_103a) BVH raycaster and offline path tracer with the API of
kosua20/Rendu's ``Raycaster`` and ``PathTracer``.

The compute path is ``librendu_gb300.so`` (CUDA, built by ``rendu_gb300.build``); the
Python classes here only marshal arguments to its C-ABI (include/rendu_gb300.h).
"""
from ._lib import RenduError, lib  # noqa: F401
from .raycaster import HIT_DTYPE, RAY_DTYPE, Hit, Raycaster  # noqa: F401
from .pathtracer import BatchRenderer, PathTracer  # noqa: F401

__all__ = ["Raycaster", "PathTracer", "BatchRenderer", "Hit", "HIT_DTYPE", "RAY_DTYPE", "RenduError", "lib"]

"""Name -> algorithm instance, as the reference's callers look algorithms up.

``ALGORITHMS[name].process(dem_gpu, **params)`` mirrors the reference's
``ALGORITHMS`` dict (algorithms/dask_registry.py:27-49); the instances here
take one CUDA device array (the single-device loop replaces the Dask arrays).
Only the hot-path algorithms exist: asking for one of the reference's other
names raises the same ``ValueError`` the reference's loader raises for an
algorithm that is not available (core/tile_processor.py:807-820).
"""
from __future__ import annotations

from ._base import TileAlgorithm
from ._impl_ambient_occlusion import AmbientOcclusionAlgorithm
from ._impl_curvature import CurvatureAlgorithm
from ._impl_hillshade import HillshadeAlgorithm
from ._impl_openness import OpennessAlgorithm
from ._impl_slope import SlopeAlgorithm
from ._impl_topousm_fast import TopoUSMFastAlgorithm

# core/tile_processor.py:64-87, restricted to the algorithms built here
DEFAULT_ALGORITHMS = {
    "topousm_fast": "TopoUSMFastAlgorithm",
    "hillshade": "HillshadeAlgorithm",
    "slope": "SlopeAlgorithm",
    "curvature": "CurvatureAlgorithm",
    "ambient_occlusion": "AmbientOcclusionAlgorithm",
    "openness": "OpennessAlgorithm",
}

ALGORITHMS = {
    "topousm_fast": TopoUSMFastAlgorithm(),
    "hillshade": HillshadeAlgorithm(),
    "slope": SlopeAlgorithm(),
    "curvature": CurvatureAlgorithm(),
    "ambient_occlusion": AmbientOcclusionAlgorithm(),
    "openness": OpennessAlgorithm(),
}


def load_algorithm(name: str) -> TileAlgorithm:
    """A new instance of ``algorithms/tile/<name>.py``'s class
    (core/tile_processor.py:807-820); ``ValueError`` for an unknown name."""
    from importlib import import_module

    if name in DEFAULT_ALGORITHMS:
        module = import_module(f"{__package__}.tile.{name}")
        cls = getattr(module, DEFAULT_ALGORITHMS[name], None)
        if cls is not None:
            return cls()
    raise ValueError(f"Algorithm {name} not found or not available on this platform")


__all__ = ["ALGORITHMS", "DEFAULT_ALGORITHMS", "load_algorithm"]

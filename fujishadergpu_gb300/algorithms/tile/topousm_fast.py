"""Tile algorithm module for topousm_fast (algorithms/tile/topousm_fast.py of the reference):
the class the tile loop finds by name, ``TopoUSMFastAlgorithm().process(dem_gpu, **params)``."""
from .._impl_topousm_fast import TopoUSMFastAlgorithm

__all__ = ["TopoUSMFastAlgorithm"]

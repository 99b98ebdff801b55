"""Tile algorithm module for ambient_occlusion (algorithms/tile/ambient_occlusion.py of the reference):
the class the tile loop finds by name, ``AmbientOcclusionAlgorithm().process(dem_gpu, **params)``."""
from .._impl_ambient_occlusion import AmbientOcclusionAlgorithm

__all__ = ["AmbientOcclusionAlgorithm"]

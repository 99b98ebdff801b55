"""Tile algorithm module for curvature (algorithms/tile/curvature.py of the reference):
the class the tile loop finds by name, ``CurvatureAlgorithm().process(dem_gpu, **params)``."""
from .._impl_curvature import CurvatureAlgorithm

__all__ = ["CurvatureAlgorithm"]

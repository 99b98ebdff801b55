"""Tile algorithm module for slope (algorithms/tile/slope.py of the reference):
the class the tile loop finds by name, ``SlopeAlgorithm().process(dem_gpu, **params)``."""
from .._impl_slope import SlopeAlgorithm

__all__ = ["SlopeAlgorithm"]

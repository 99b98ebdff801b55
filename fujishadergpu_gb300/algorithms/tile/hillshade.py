"""Tile algorithm module for hillshade (algorithms/tile/hillshade.py of the reference):
the class the tile loop finds by name, ``HillshadeAlgorithm().process(dem_gpu, **params)``."""
from .._impl_hillshade import HillshadeAlgorithm

__all__ = ["HillshadeAlgorithm"]

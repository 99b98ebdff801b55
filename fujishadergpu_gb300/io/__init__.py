"""Output encoding and raster metadata rules."""

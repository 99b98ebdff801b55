"""fujishadergpu_gb300: the raster hot path of FujiShaderGPU on GB300 (sm_103a).

Hand-written CUDA kernels in ``libfsg.so`` (C ABI: ``include/fsg.h``) behind
the reference's per-algorithm entry points (``fujishadergpu_gb300.algorithms``)
and its single-device tile loop (``fujishadergpu_gb300.core``).
"""
__version__ = "0.1.0"

"""CPU oracle for the raster hot path (test infrastructure only).

``oracle.restated`` restates the reference's NumPy/CuPy algorithms on the CPU;
``tests/`` pin it to golden vectors produced by the reference itself and use it
as the checker for the CUDA kernels.  The product package never imports it.
"""

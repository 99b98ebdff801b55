"""Prepared launches and CUDA-graph replay of the tile loop.

The reference's tile scheduler (core/tile_processor.py:1629-1683) submits one
thread-pool task per tile and per step.  Here a whole tile list of one
kernel is a *plan* (``fsg_plan`` in include/fsg.h): created once, it owns the
uploaded tile tables, and each launch issues only kernels, memsets and
device-side copies.  A sequence of plan launches (the products of a batch of
uneven tiles) is captured once into a CUDA graph and replayed as a single
graph launch per step.
"""
from __future__ import annotations

import ctypes as C
from typing import Callable, Dict, List, Optional, Sequence

from .. import _arrays
from .. import _native as N


class Plan:
    """One prepared library call; keeps the Python objects its device pointers refer to alive."""

    def __init__(self, handle: C.c_void_p, keep=()):
        self._h = handle
        self._keep = list(keep)

    def launch(self, stream: Optional[int] = None) -> None:
        if not self._h:
            raise RuntimeError("plan already destroyed")
        s = _arrays.current_stream_handle() if stream is None else stream
        N.check(N.lib().fsg_plan_launch(self._h, C.c_void_p(s)))

    def close(self) -> None:
        if self._h:
            N.lib().fsg_plan_destroy(self._h)
            self._h = None
            self._keep = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _tiles_array(tiles: Sequence[N.Tile]):
    return (N.Tile * max(1, len(tiles)))(*tiles)


def stencil_plan(view: _arrays.DevView, tiles: Sequence[N.Tile], params: N.StencilParams,
                 planes: Dict[int, N.Plane], keep=()) -> Plan:
    """fsg_stencil prepared over ``tiles`` (planes indexed by FSG_OUT_*)."""
    arr = (N.Plane * N.FSG_STENCIL_NOUT)()
    for idx, pl in planes.items():
        arr[idx] = pl
    h = C.c_void_p()
    N.check(N.lib().fsg_stencil_plan(C.c_void_p(view.ptr), view.ld, view.h, view.w, _tiles_array(tiles), len(tiles),
                                     C.byref(params), arr, C.byref(h)))
    return Plan(h, [view] + list(keep))


def topousm_plan(view: _arrays.DevView, tiles: Sequence[N.Tile], params, plane: N.Plane, keep=()) -> Plan:
    """fsg_topousm prepared over ``tiles`` (strip-path radius lists)."""
    h = C.c_void_p()
    N.check(N.lib().fsg_topousm_plan(C.c_void_p(view.ptr), view.ld, view.h, view.w, _tiles_array(tiles), len(tiles),
                                     C.byref(params), C.byref(plane), C.byref(h)))
    return Plan(h, [view, params] + list(keep))


def openness_plan(view: _arrays.DevView, tiles: Sequence[N.Tile], params, display_plane: Optional[N.Plane] = None,
                  raw=None, keep=()) -> Plan:
    """fsg_openness prepared over ``tiles``."""
    h = C.c_void_p()
    N.check(N.lib().fsg_openness_plan(C.c_void_p(view.ptr), view.ld, view.h, view.w, _tiles_array(tiles), len(tiles),
                                      C.byref(params), C.byref(display_plane) if display_plane is not None else None,
                                      C.c_void_p(raw.data_ptr() if raw is not None else 0),
                                      int(raw.stride(0)) if raw is not None else 0, C.byref(h)))
    return Plan(h, [view, params] + ([raw] if raw is not None else []) + list(keep))


class GraphStep:
    """A step (a callable issuing plan launches on the current stream) captured once
    into a CUDA graph; ``replay()`` runs the whole step as one graph launch."""

    def __init__(self, step: Callable[[], None], warmup: int = 1):
        torch = _arrays._torch()
        self._torch = torch
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):  # first launches outside capture (lazy library set-up)
            for _ in range(max(0, warmup)):
                step()
        torch.cuda.current_stream().wait_stream(side)
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph, capture_error_mode="thread_local"):
            step()
        torch.cuda.synchronize()

    def replay(self) -> None:
        self.graph.replay()


def launch_all(plans: List[Plan], stream: Optional[int] = None) -> None:
    for p in plans:
        p.launch(stream)


__all__ = ["Plan", "stencil_plan", "topousm_plan", "openness_plan", "GraphStep", "launch_all"]

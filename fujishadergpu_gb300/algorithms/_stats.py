"""Global normalisation statistics on the GPU (FP64 order statistics).

``topousm_fast_stat_func`` and ``robust_unsigned_stretch_stat_func`` keep the
reference names and return values (_normalization.py:21-32,
_global_stats.py:181-203); the percentiles come from ``fsg_percentile``
(exact float32 order statistics, numpy 'linear' interpolation in FP64).
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence, Tuple

from .. import _arrays
from .. import _native as N

NORMAL_PERCENTILE = 99.0  # _normalization.py:17


def _flat(values):
    torch = _arrays._torch()
    if isinstance(values, torch.Tensor):
        t = values
    else:
        t = _arrays.as_device_f32_2d(values if getattr(values, "ndim", 2) == 2 else values.reshape(1, -1)).tensor
    if not t.is_cuda:
        t = t.cuda()
    return t.reshape(-1).to(torch.float32).contiguous()


def percentile(values, q: Sequence[float], *, absolute: bool = False) -> Tuple[Tuple[float, ...], int]:
    """(percentiles of the non-NaN values, valid count); ``absolute`` uses |v|."""
    t = _flat(values)
    qs = (C.c_double * len(q))(*[float(x) for x in q])
    out = (C.c_double * len(q))()
    nv = C.c_int64(0)
    N.check(N.lib().fsg_percentile(C.c_void_p(t.data_ptr()), t.numel(), 1 if absolute else 0, qs, len(q), out,
                                   C.byref(nv), C.c_void_p(_arrays.current_stream_handle())))
    return tuple(float(v) for v in out), int(nv.value)


def std(values) -> float:
    t = _flat(values)
    out = C.c_double(0.0)
    N.check(N.lib().fsg_std(C.c_void_p(t.data_ptr()), t.numel(), C.byref(out),
                            C.c_void_p(_arrays.current_stream_handle())))
    return float(out.value)


def topousm_fast_stat_func(data) -> Tuple[float]:
    """p99(|valid|) scale, falling back to std then 1.0 (_normalization.py:21-32)."""
    (p,), n = percentile(data, [NORMAL_PERCENTILE], absolute=True)
    if n > 0:
        if p > 1e-9:
            return (p,)
        s = std(data)
        return (s if s > 1e-9 else 1.0,)
    return (1.0,)


def robust_unsigned_stretch_stat_func(values) -> Tuple[float, float]:
    """(p1, p99 - p1) of the finite values (_global_stats.py:181-203)."""
    if values is None:
        return (0.0, 0.0)
    torch = _arrays._torch()
    t = _flat(values)
    t = torch.where(torch.isfinite(t), t, torch.full_like(t, float("nan")))
    (lo, hi), n = percentile(t, [1.0, 99.0])
    if n == 0:
        return (0.0, 0.0)
    sc = hi - lo
    if not (sc > 1e-12):
        return (lo, 0.0)
    return (lo, sc)

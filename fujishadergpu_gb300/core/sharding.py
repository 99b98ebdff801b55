"""The tile loop sharded over devices (one process per GPU) and the one
exchange step it needs.

Tiles are independent given their halo, so each rank takes a contiguous band
of tile rows and runs the single-device loop on it; nothing is exchanged on
the data path (weak scaling).  The only cross-tile coupling of the hot path is
the global statistics (topousm_fast's p99(|x|), openness' p1 / p99 stretch;
algorithms/_normalization.py:21-41, _global_stats.py:156-203), computed in the
reference on one device.  Here each rank contributes the histogram of its own
values' order-preserving keys to every pass of the radix select that
``fsg_percentile`` runs on one device (11 + 11 + 10 bits); the histograms are
summed across ranks (one all-reduce per pass) and every rank picks the same
bin, so all ranks obtain the exact order statistics of the union of the
shards -- the same numbers ``fsg_percentile`` returns for the concatenated
values.

A histogram source gives a rank's histograms: the GPU
(``DeviceHistograms``, the ``fsg_key_histogram`` kernel) or NumPy
(``NumpyHistograms``, for host-side arrays).  ``allreduce`` sums an int64
NumPy array over the ranks (``torch_allreduce`` wraps torch.distributed).

``core.tile_loop.process_dem_array`` runs sharded when a ``Shard`` is given or
a torch.distributed process group of more than one rank is initialised: each
rank computes its band of tile rows, its round-robin share of the
statistics windows, and the statistics through this merge (the reference
broadcasts them to its Dask workers, core/dask_processor.py:1011-1016).
"""
from __future__ import annotations

import ctypes as C
import math
from typing import Callable, List, Optional, Sequence, Tuple

import numpy as np

PASSES = ((21, 11), (10, 11), (0, 10))   # (shift, bits) of the three radix passes


# ------------------------------------------------------------------ bands
def band_rows(n_tile_rows: int, world: int, rank: int) -> Tuple[int, int]:
    """Contiguous, balanced range [r0, r1) of tile rows owned by ``rank``."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    base, extra = divmod(int(n_tile_rows), world)
    r0 = rank * base + min(rank, extra)
    return r0, r0 + base + (1 if rank < extra else 0)


def shard_tiles(infos: Sequence, world: int, rank: int) -> List:
    """The tiles (``TileInfo``, with ``ty``) of this rank's band of tile rows."""
    if not infos:
        return []
    n_rows = max(int(t.ty) for t in infos) + 1
    r0, r1 = band_rows(n_rows, world, rank)
    return [t for t in infos if r0 <= int(t.ty) < r1]


# ------------------------------------------------------------ key helpers
def ordered_keys(values: np.ndarray, absolute: bool = False) -> np.ndarray:
    """The order-preserving uint32 image of the valid float32 values (NaN dropped)."""
    v = np.asarray(values, dtype=np.float32).ravel()
    v = v[~np.isnan(v)]
    if absolute:
        v = np.abs(v)
    u = v.view(np.uint32)
    return np.where(u & np.uint32(0x80000000), ~u, u | np.uint32(0x80000000)).astype(np.uint32)


def key_to_float(k: int) -> float:
    k = int(k) & 0xFFFFFFFF
    u = (k & 0x7FFFFFFF) if (k & 0x80000000) else (~k & 0xFFFFFFFF)
    return float(np.array([u], dtype=np.uint32).view(np.float32)[0])


class NumpyHistograms:
    """Histogram source over a host array (the same keys as the GPU kernel)."""

    def __init__(self, values, absolute: bool = False):
        self.keys = ordered_keys(values, absolute)

    def count(self) -> int:
        return int(self.keys.size)

    def histogram(self, prefix: int, mask: int, shift: int, bits: int) -> np.ndarray:
        k = self.keys[(self.keys & np.uint32(mask)) == np.uint32(prefix)]
        b = (k >> np.uint32(shift)) & np.uint32((1 << bits) - 1)
        return np.bincount(b.astype(np.int64), minlength=1 << bits).astype(np.int64)


class DeviceHistograms:
    """Histogram source over a float32 device tensor (``fsg_key_histogram``)."""

    def __init__(self, values, absolute: bool = False):
        from .. import _arrays
        from .. import _native as N
        self._N = N
        t = values if hasattr(values, "data_ptr") else _arrays.as_device_f32_2d(values).tensor
        self.t = t.reshape(-1).contiguous().float()
        self.absolute = 1 if absolute else 0
        self._count = None if self.t.numel() > 0 else 0

    def count(self) -> int:
        if self._count is None:
            h = self.histogram(0, 0, 21, 11)
            self._count = int(h.sum())
        return self._count

    def histogram(self, prefix: int, mask: int, shift: int, bits: int) -> np.ndarray:
        from .. import _arrays
        if self.t.numel() == 0:
            return np.zeros(1 << bits, dtype=np.int64)
        out = (C.c_uint64 * (1 << bits))()
        self._N.check(self._N.lib().fsg_key_histogram(
            C.c_void_p(self.t.data_ptr()), int(self.t.numel()), self.absolute, C.c_uint32(prefix),
            C.c_uint32(mask), int(shift), int(bits), out, C.c_void_p(_arrays.current_stream_handle())))
        return np.frombuffer(out, dtype=np.uint64).astype(np.int64)


def torch_allreduce(group=None) -> Callable[[np.ndarray], np.ndarray]:
    """Sum an int64 array over the ranks of ``group`` (gloo on CPU tensors, NCCL on CUDA)."""
    import torch
    import torch.distributed as dist

    def reduce(a: np.ndarray) -> np.ndarray:
        backend = dist.get_backend(group)
        dev = "cuda" if backend == "nccl" else "cpu"
        t = torch.from_numpy(np.ascontiguousarray(a, dtype=np.int64)).to(dev)
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
        return t.cpu().numpy()
    return reduce


# ------------------------------------------------------------ percentiles
def linear_pick(n: int, q: float) -> Tuple[int, int, float]:
    """numpy.percentile 'linear' index arithmetic (as fsg_percentile's linear_pick)."""
    qq = q / 100.0
    virt = (n - 1) * qq   # numpy's 'linear' virtual index
    prev = math.floor(virt)
    gamma = virt - prev
    lo = int(prev)
    hi = lo + 1
    if virt >= n - 1:
        lo = hi = n - 1
    elif virt < 0:
        lo = hi = 0
    return lo, hi, gamma


def lerp_numpy(a: float, b: float, t: float) -> float:
    diff = float(b) - float(a)
    r = float(a) + diff * t
    if t >= 0.5:
        r = float(b) - diff * (1.0 - t)
    return r


def select_key(src, rank_k: int, allreduce: Callable[[np.ndarray], np.ndarray]) -> int:
    """The key of the rank_k-th smallest value (0-based) of the union of all ranks' values."""
    prefix, mask, k = 0, 0, int(rank_k)
    for shift, bits in PASSES:
        h = allreduce(src.histogram(prefix, mask, shift, bits))
        c = np.cumsum(h)
        b = int(np.searchsorted(c, k, side="right"))
        b = min(b, (1 << bits) - 1)
        k -= int(c[b - 1]) if b > 0 else 0
        prefix |= b << shift
        mask |= ((1 << bits) - 1) << shift
    return prefix


def distributed_percentile(src, q: Sequence[float], allreduce: Callable[[np.ndarray], np.ndarray]
                           ) -> Tuple[List[float], int]:
    """Exact numpy.percentile(union of the ranks' valid values, q, 'linear') on every rank,
    FP64 interpolation; returns (values, total valid count)."""
    for x in q:
        if not 0.0 <= float(x) <= 100.0:
            raise ValueError(f"percentile {x} outside [0, 100]")
    n = int(allreduce(np.array([src.count()], dtype=np.int64))[0])
    if n == 0:
        return [float("nan")] * len(q), 0
    picks = [linear_pick(n, float(x)) for x in q]
    ranks = sorted({r for lo, hi, _ in picks for r in (lo, hi)})
    vals = {r: key_to_float(select_key(src, r, allreduce)) for r in ranks}
    return [lerp_numpy(vals[lo], vals[hi], g) for lo, hi, g in picks], n


def distributed_topousm_scale(src, allreduce) -> Tuple[float]:
    """topousm_fast_stat_func's scale p99(|x|) over all shards (src built with absolute=True)."""
    (p99,), n = distributed_percentile(src, [99.0], allreduce)
    return (p99,)


# ------------------------------------------------------- the shard of a run
class Shard:
    """This process's part of a sharded run: ``world`` ranks, this one ``rank``,
    ``allreduce`` the sum over the ranks of an int64 / float64 NumPy array."""

    def __init__(self, world: int, rank: int, allreduce: Callable[[np.ndarray], np.ndarray]):
        if world < 1 or not 0 <= rank < world:
            raise ValueError(f"rank {rank} outside a world of {world}")
        self.world, self.rank, self.allreduce = int(world), int(rank), allreduce

    def mine(self, items: Sequence) -> List:
        """Round-robin share of a list every rank builds identically."""
        return [x for i, x in enumerate(items) if i % self.world == self.rank]


def torch_allreduce_any(group=None) -> Callable[[np.ndarray], np.ndarray]:
    """As torch_allreduce, for int64 or float64 arrays."""
    import torch
    import torch.distributed as dist

    def reduce(a: np.ndarray) -> np.ndarray:
        a = np.ascontiguousarray(a)
        backend = dist.get_backend(group)
        dev = "cuda" if backend == "nccl" else "cpu"
        t = torch.from_numpy(a.copy()).to(dev)
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
        return t.cpu().numpy()
    return reduce


def shard_from_environment(group=None) -> Optional["Shard"]:
    """A Shard over the initialised torch.distributed process group when it has more
    than one rank; None otherwise (single-device run)."""
    try:
        import torch.distributed as dist
    except ImportError:  # pragma: no cover
        return None
    if not (dist.is_available() and dist.is_initialized()):
        return None
    world = dist.get_world_size(group)
    if world <= 1:
        return None
    return Shard(world, dist.get_rank(group), torch_allreduce_any(group))


def _union_std(values: np.ndarray, allreduce) -> float:
    """Population standard deviation of the union of the ranks' valid values (float64 sums)."""
    v = np.asarray(values, dtype=np.float64)
    v = v[~np.isnan(v)]
    tot = allreduce(np.array([v.size, v.sum()], dtype=np.float64))
    n, s = int(tot[0]), float(tot[1])
    if n == 0:
        return 0.0
    mean = s / n
    ss = float(allreduce(np.array([np.square(v - mean).sum()], dtype=np.float64))[0])
    return math.sqrt(ss / n)


def sharded_topousm_stat(src_abs, values_host_fn, allreduce) -> Tuple[float]:
    """topousm_fast_stat_func over the union of the shards: p99(|x|) from the exact
    histogram merge, falling back to the standard deviation, then 1.0
    (_normalization.py:21-32).  ``values_host_fn()`` gives this rank's values on the
    host (only called for the fallback)."""
    (p,), n = distributed_percentile(src_abs, [99.0], allreduce)
    if n > 0:
        if p > 1e-9:
            return (p,)
        sd = _union_std(values_host_fn(), allreduce)
        return (sd if sd > 1e-9 else 1.0,)
    return (1.0,)


def sharded_stretch_stat(src, allreduce) -> Tuple[float, float]:
    """robust_unsigned_stretch_stat_func over the union: (p1, p99 - p1)
    (_global_stats.py:181-203)."""
    (lo, hi), n = distributed_percentile(src, [1.0, 99.0], allreduce)
    if n == 0:
        return (0.0, 0.0)
    sc = hi - lo
    if not (sc > 1e-12):
        return (lo, 0.0)
    return (lo, sc)

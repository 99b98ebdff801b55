"""Sharding of the tile loop and the exact cross-rank percentile merge
(histogram all-reduce in the radix select), on CPU with gloo ranks."""
import os
import socket

import numpy as np
import pytest

from fujishadergpu_gb300.core import sharding as SH


def test_band_rows_partition_every_tile_row_once():
    for n in (1, 2, 7, 8, 33):
        for world in (1, 2, 3, 4, 8):
            rows = []
            for r in range(world):
                a, b = SH.band_rows(n, world, r)
                assert 0 <= a <= b <= n
                rows.extend(range(a, b))
            assert rows == list(range(n))
    with pytest.raises(ValueError):
        SH.band_rows(4, 2, 2)


def test_shard_tiles_cover_the_grid():
    from fujishadergpu_gb300.core.tile_loop import tile_grid
    infos = tile_grid(1000, 900, 256, 64)
    got = []
    for r in range(3):
        got.extend((t.ty, t.tx) for t in SH.shard_tiles(infos, 3, r))
    assert sorted(got) == sorted((t.ty, t.tx) for t in infos)


def _data(n, seed, nan_frac=0.05):
    rng = np.random.default_rng(seed)
    x = (rng.standard_normal(n) * 40.0 + rng.standard_normal(n) ** 3).astype(np.float32)
    x[rng.random(n) < nan_frac] = np.nan
    return x


QS = [0.0, 0.5, 1.0, 25.0, 50.0, 99.0, 99.9, 100.0]


@pytest.mark.parametrize("absolute", [False, True])
def test_single_rank_equals_numpy_percentile(absolute):
    x = _data(50_001, 3)
    src = SH.NumpyHistograms(x, absolute)
    got, n = SH.distributed_percentile(src, QS, lambda a: a)
    v = x[~np.isnan(x)].astype(np.float64)
    if absolute:
        v = np.abs(v)
    assert n == v.size
    assert got == list(np.percentile(v, QS))


def test_key_order_is_the_float_order():
    x = np.array([-np.inf, -3.5, -0.0, 0.0, 1e-30, 2.0, np.inf], np.float32)
    k = SH.ordered_keys(x)
    assert np.all(np.diff(k.astype(np.int64)) >= 0)
    assert [SH.key_to_float(v) for v in k] == [float(v) for v in x]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, shards, qs, out_path):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        src = SH.NumpyHistograms(shards[rank], absolute=True)
        vals, n = SH.distributed_percentile(src, qs, SH.torch_allreduce())
        np.save(out_path % rank, np.array(vals + [float(n)], dtype=np.float64))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_agree_with_the_union(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    x = _data(80_003, 11)
    shards = [x[:30_000], x[30_000:]]           # uneven shards
    out = str(tmp_path / "rank%d.npy")
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, shards, QS, out), nprocs=2, join=True, start_method="spawn")
    v = np.abs(x[~np.isnan(x)].astype(np.float64))
    ref = list(np.percentile(v, QS)) + [float(v.size)]
    for r in range(2):
        assert list(np.load(out % r)) == ref


def _stat_rank(rank, world, port, shards, out_path):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        shard = SH.shard_from_environment()
        assert shard is not None and shard.world == world and shard.rank == rank
        v = shards[rank]
        top = SH.sharded_topousm_stat(SH.NumpyHistograms(v, absolute=True), lambda: v, shard.allreduce)
        flat = SH.sharded_topousm_stat(SH.NumpyHistograms(np.zeros_like(v), absolute=True),
                                       lambda: np.zeros_like(v), shard.allreduce)
        st = SH.sharded_stretch_stat(SH.NumpyHistograms(v), shard.allreduce)
        np.save(out_path % rank, np.array(list(top) + list(flat) + list(st), dtype=np.float64))
    finally:
        dist.destroy_process_group()


def test_sharded_statistics_equal_the_reference_stat_funcs(tmp_path):
    """topousm_fast_stat_func and robust_unsigned_stretch_stat_func of the union, on every rank
    (including the all-zero fallback to the standard deviation, then 1.0)."""
    from oracle import restated as R
    mp = pytest.importorskip("torch.multiprocessing")
    x = _data(60_001, 21)
    shards = [x[:17_000], x[17_000:]]
    out = str(tmp_path / "stat%d.npy")
    mp.start_processes(_stat_rank, args=(2, _free_port(), shards, out), nprocs=2, join=True, start_method="spawn")
    # exact float32 order statistics with FP64 interpolation = np.percentile of the float64 values
    # (the reference's float32 interpolation is within one float32 ulp of it)
    x64 = x[~np.isnan(x)].astype(np.float64)
    p1, p99 = np.percentile(x64, [1.0, 99.0])
    ref = [float(np.percentile(np.abs(x64), 99.0)), 1.0, float(p1), float(p99 - p1)]
    r32 = list(R.topousm_scale(x)) + [1.0] + list(R.stretch_stats(x))
    for r in range(2):
        got = list(np.load(out % r))
        assert got == ref
        assert got == pytest.approx(r32, rel=2e-7)


def test_shard_round_robin_and_validation():
    sh = [SH.Shard(3, r, lambda a: a) for r in range(3)]
    items = list(range(10))
    assert sorted(sum((s.mine(items) for s in sh), [])) == items
    with pytest.raises(ValueError):
        SH.Shard(2, 2, lambda a: a)
    assert SH.shard_from_environment() is None

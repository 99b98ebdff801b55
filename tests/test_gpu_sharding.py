"""The device histogram pass behind the cross-rank percentile merge."""
import numpy as np
import pytest

from fujishadergpu_gb300.core import sharding as SH

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def test_device_histograms_equal_numpy_histograms(cuda):
    rng = np.random.default_rng(5)
    x = (rng.standard_normal(300_001) * 30).astype(np.float32)
    x[rng.random(x.size) < 0.03] = np.nan
    for absolute in (False, True):
        d = SH.DeviceHistograms(torch.from_numpy(x).cuda(), absolute)
        h = SH.NumpyHistograms(x, absolute)
        assert d.count() == h.count()
        k = SH.select_key(h, h.count() // 3, lambda a: a)
        for prefix, mask, (shift, bits) in ((0, 0, SH.PASSES[0]), (k & 0xFFE00000, 0xFFE00000, SH.PASSES[1]),
                                            (k & 0xFFFFFC00, 0xFFFFFC00, SH.PASSES[2])):
            assert np.array_equal(d.histogram(prefix, mask, shift, bits), h.histogram(prefix, mask, shift, bits))


def test_sharded_device_percentiles_equal_fsg_percentile(cuda):
    """Two shards merged through the histogram exchange give fsg_percentile's numbers."""
    from fujishadergpu_gb300.algorithms._stats import percentile
    rng = np.random.default_rng(6)
    x = (rng.standard_normal(200_000) ** 3).astype(np.float32)
    t = torch.from_numpy(x).cuda()
    shards = [SH.DeviceHistograms(t[:77_777]), SH.DeviceHistograms(t[77_777:])]

    class Union:  # the all-reduce of two ranks, in one process
        def count(self):
            return sum(s.count() for s in shards)

        def histogram(self, *a):
            return sum(s.histogram(*a) for s in shards)

    q = [1.0, 50.0, 99.0]
    got, n = SH.distributed_percentile(Union(), q, lambda a: a)
    ref, nref = percentile(t, q)
    assert n == x.size == nref
    assert got == list(ref)


def _free_port():
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _dem_for_sharding():
    from fujishadergpu_gb300 import synth
    d = synth.fbm_ridged(900, 1100, hurst=0.8, seed_fbm=131, seed_ridged=132, lo=0.0, hi=3500.0)
    d[synth.nodata_disks(900, 1100, count=4, seed=133, rmin=5.0, rmax=25.0)] = np.nan
    return d


CASES = {
    "topousm_fast": dict(tile_size=256, pixel_size=10.0, pixel_scale_x=10.0, pixel_scale_y=-10.0,
                         radii=[2, 8, 32, 128, 512], weights=[16 / 31, 8 / 31, 4 / 31, 2 / 31, 1 / 31]),
    "openness": dict(tile_size=256, pixel_size=5.0, pixel_scale_x=5.0, pixel_scale_y=-5.0, mode="local",
                     max_distance=40),
}


def _shard_rank(rank, world, port, out_path):
    import torch.distributed as dist
    import os as _os
    _os.environ["MASTER_ADDR"] = "127.0.0.1"
    _os.environ["MASTER_PORT"] = str(port)
    torch.cuda.set_device(0)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from fujishadergpu_gb300.core import tile_loop
        d = torch.from_numpy(_dem_for_sharding()).cuda()
        for name, kw in CASES.items():
            res = tile_loop.process_dem_array(d, name, **kw)   # sharded: the process group is initialised
            r0, r1 = res.rows
            np.save(out_path % (name, rank), res.output[r0:r1].cpu().numpy())
            np.save(out_path % (name + "_meta", rank), np.array([r0, r1] + list(res.stats), dtype=np.float64))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_reproduce_the_single_device_tile_loop(cuda, tmp_path):
    """Two ranks (processes sharing this GPU, statistics merged over gloo) each run their band
    of tile rows; the bands and the statistics equal the single-device run bit for bit."""
    mp = pytest.importorskip("torch.multiprocessing")
    from fujishadergpu_gb300.core import tile_loop
    out = str(tmp_path / "%s_rank%d.npy")
    mp.start_processes(_shard_rank, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
    d = torch.from_numpy(_dem_for_sharding()).cuda()
    for name, kw in CASES.items():
        ref = tile_loop.process_dem_array(d, name, shard=None, **kw)
        full = ref.output.cpu().numpy()
        covered = []
        for r in range(2):
            meta = np.load(out % (name + "_meta", r))
            r0, r1 = int(meta[0]), int(meta[1])
            assert tuple(meta[2:]) == tuple(ref.stats), (name, r, meta[2:], ref.stats)
            band = np.load(out % (name, r))
            assert np.array_equal(band, full[r0:r1], equal_nan=True), (name, r)
            covered.append((r0, r1))
        assert covered[0][0] == 0 and covered[0][1] == covered[1][0] and covered[1][1] == full.shape[0], covered

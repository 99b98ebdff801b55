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

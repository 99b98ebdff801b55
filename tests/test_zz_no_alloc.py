"""fsg_percentile_noalloc: the percentile entry point for callers that cannot
allocate device memory during a run (an application whose GPU memory is owned
and budgeted by its own pool, or a latency-critical caller that cannot accept
the implicit synchronisation cudaMalloc / cudaFree may cause).

It keeps its scratch in a fixed device array instead of allocating, so its
results must equal those of fsg_percentile, call after call: the array keeps
the previous call's contents and must not leak them into the next result.
This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _call(fn, x, qs, absolute):
    from fujishadergpu_gb300 import _native as N
    q = (C.c_double * len(qs))(*qs)
    out = (C.c_double * len(qs))()
    nv = C.c_int64(-1)
    st = fn(C.c_void_p(x.data_ptr()), x.numel(), 1 if absolute else 0, q, len(qs), out, C.byref(nv),
            C.c_void_p(torch.cuda.current_stream().cuda_stream))
    N.check(st)
    return [float(v) for v in out], int(nv.value)


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fujishadergpu_gb300 import _native as N
    return N.lib()


def test_noalloc_matches_allocating_entry_point_twice(lib):
    rng = np.random.default_rng(123)
    qs = [0.0, 1.0, 25.0, 50.0, 99.0, 100.0]
    cases = []
    for n in (3, 1000, 250_001):
        x = (rng.standard_normal(n) * 50.0).astype(np.float32)
        x[rng.integers(0, n, max(1, n // 20))] = np.nan
        cases.append(torch.from_numpy(x).cuda())
    for x in cases:
        for absolute in (False, True):
            ref, nref = _call(lib.fsg_percentile, x, qs, absolute)
            # two calls in a row: the shared array keeps the previous call's state
            for _ in range(2):
                got, n = _call(lib.fsg_percentile_noalloc, x, qs, absolute)
                assert n == nref
                assert got == pytest.approx(ref, rel=1e-12, abs=0.0)


def test_noalloc_alternating_inputs_do_not_leak_state(lib):
    a = torch.linspace(-5.0, 5.0, 4097, device="cuda")
    b = torch.full((10,), 7.0, device="cuda")
    ra, _ = _call(lib.fsg_percentile, a, [99.0], False)
    rb, _ = _call(lib.fsg_percentile, b, [99.0], False)
    for _ in range(2):
        assert _call(lib.fsg_percentile_noalloc, a, [99.0], False)[0] == pytest.approx(ra, rel=1e-12)
        assert _call(lib.fsg_percentile_noalloc, b, [99.0], False)[0] == pytest.approx(rb, rel=1e-12)


def test_noalloc_rejects_more_percentiles_than_its_array_holds(lib):
    from fujishadergpu_gb300 import _native as N
    x = torch.zeros(8, device="cuda")
    with pytest.raises(N.FsgError) as e:
        _call(lib.fsg_percentile_noalloc, x, [float(i) for i in range(17)], False)
    assert e.value.code == N.FSG_ERR_WORKSPACE


def test_noalloc_draws_nothing_from_the_stream_ordered_pool(lib):
    """The allocating entry point takes its scratch from the library's stream-ordered
    pool (fsg_scratch_high_water reports that pool's high-water mark); the
    allocation-free one must leave the mark where it was."""
    hw = C.c_uint64()

    def get(reset=0):
        assert lib.fsg_scratch_high_water(C.byref(hw), C.c_int32(reset)) == 0
        return int(hw.value)

    x = torch.randn(100_000, device="cuda")
    torch.cuda.synchronize()
    get(reset=1)
    base = get()
    _call(lib.fsg_percentile, x, [50.0, 99.0], False)
    torch.cuda.synchronize()
    assert get() > base, "control: fsg_percentile should draw its scratch from the pool"
    get(reset=1)
    base = get()
    for _ in range(2):
        _call(lib.fsg_percentile_noalloc, x, [50.0, 99.0], False)
    torch.cuda.synchronize()
    assert get() == base

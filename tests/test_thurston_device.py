"""Extremal domino tilings on the GPU equal the host Thurston algorithm (itself equal to the
reference's MaxTiling / MinTiling on the golden cases), including its errors."""
import time

import numpy as np
import pytest


def domains(rt):
    D = rt.DominoTiler
    out = [D.AztecDiamond(n) for n in (1, 2, 5, 16, 64)]
    out += [D.Rectangle(4, 6), D.Rectangle(10, 10), D.Rectangle(32, 64), D.Rectangle(7, 12)]
    out += [D.AztecRectangle(6, [2]), D.AztecRectangle(9, [1, 7])]
    return out


@pytest.mark.gpu
def test_device_extremal_tilings_equal_the_host_algorithm(rt):
    D = rt.DominoTiler
    for d in domains(rt):
        for top in (True, False):
            try:
                host = D.MaxTiling(d) if top else D.MinTiling(d)
            except rt.RTError as e:
                with pytest.raises(rt.RTError) as dev_err:
                    D.ExtremalTilingDevice(d, top)
                assert dev_err.value.args[0].endswith(f"(status {e.args[0].split('status ')[-1]}")
                continue
            assert np.array_equal(D.ExtremalTilingDevice(d, top), host)


@pytest.mark.gpu
def test_device_extremal_tilings_at_order_1024(rt):
    D = rt.DominoTiler
    d = D.AztecDiamond(1024)
    for top in (True, False):
        t0 = time.perf_counter()
        host = D.MaxTiling(d) if top else D.MinTiling(d)
        t1 = time.perf_counter()
        dev = D.ExtremalTilingDevice(d, top)
        t2 = time.perf_counter()
        assert np.array_equal(dev, host)
        print(f"order 1024 {'max' if top else 'min'}: host {1e3 * (t1 - t0):.0f} ms, device {1e3 * (t2 - t1):.0f} ms")


def test_untileable_and_holed_domains_are_refused_before_the_device(rt):
    D = rt.DominoTiler
    with pytest.raises(rt.RTError):
        D.ExtremalTilingDevice(D.Rectangle(3, 3), True)  # odd area: the boundary walk mismatches
    d = D.Rectangle(8, 8).reshape(int(np.sqrt(D.Rectangle(8, 8).size)), -1).copy()
    d[5:7, 5:7] = 0  # a 2 x 2 hole: the boundary is not one walk
    with pytest.raises(rt.RTError):
        D.ExtremalTilingDevice(d.ravel(), True)


@pytest.mark.gpu
def test_device_height_function_equals_the_host_function(rt):
    D = rt.DominoTiler
    for d in [D.AztecDiamond(5), D.AztecDiamond(64), D.Rectangle(10, 16)]:
        tmax = D.MaxTiling(d)
        n = int(np.sqrt(tmax.size))
        t = tmax.copy()
        D(rule="cftp", rng="fast", fast_stream=2).Walk(t, 400, 3)
        for x in (tmax, D.MinTiling(d), t):
            assert np.array_equal(D.TilingToHeightfuncDevice(x, d), D.TilingToHeightfunc(x, d))


@pytest.mark.gpu
def test_sampler_height_sums_equal_host_sums(rt):
    torch = pytest.importorskip("torch")
    D = rt.DominoTiler
    d = D.AztecDiamond(48)
    tmax = D.MaxTiling(d)
    n = int(np.sqrt(tmax.size))
    s = rt.DominoSampler(n, 1, rt.DominoTiler(rule="cftp", rng="fast", fast_stream=5))
    s.load(0, tmax)
    s.set_domain(d)
    sums = torch.zeros(n * n, dtype=torch.int64, device="cuda")
    heights = torch.zeros(n * n, dtype=torch.int32, device="cuda")
    host = np.zeros(n * n, np.int64)
    for k in range(12):
        s.run_fast(31, 40 * k, 40)
        s.accumulate_heights(0, sums.data_ptr(), heights.data_ptr())
        t = s.store(0)
        h = D.TilingToHeightfunc(t, d)
        s.sync()
        torch.cuda.synchronize()
        assert np.array_equal(heights.cpu().numpy(), h)
        host += np.where(h != np.iinfo(np.int32).max, h, 0)
    torch.cuda.synchronize()
    assert np.array_equal(sums.cpu().numpy(), host)
    s.close()

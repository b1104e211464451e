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

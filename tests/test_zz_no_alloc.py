"""rt_dm_sweep_noalloc: the resident sweep for callers that cannot allocate device memory.

The caller (here: the test, through torch) owns the device chains and generator states;
the entry point itself allocates nothing and keeps its scratch in a static device array.
Its tilings must equal those of the existing entry point (rt_domino_walk) exactly, on two
calls in a row that continue the same chains.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _split(t: np.ndarray, n: int, pitch: int) -> np.ndarray:
    """Host tiling -> [colour (0 white, 1 black)][N][pitch] u8, the reference's split."""
    out = np.zeros((2, n, pitch), np.uint8)
    T = t.reshape(n, n)
    for i in range(n):
        j = np.arange(n)
        black = (i + j) % 2 == 0
        out[1, i, j[black] // 2] = T[i, j[black]]
        out[0, i, j[~black] // 2] = T[i, j[~black]]
    return out


def _merge(a: np.ndarray, n: int) -> np.ndarray:
    T = np.zeros((n, n), np.int32)
    for i in range(n):
        j = np.arange(n)
        black = (i + j) % 2 == 0
        T[i, j[black]] = a[1, i, j[black] // 2]
        T[i, j[~black]] = a[0, i, j[~black] // 2]
    return T.ravel()


def _check_two_calls(rt, orc, order, mode, n_chains, s1, s2, seed=2024):
    """A steps = 0 warm-up call (the set-up a caller that cannot allocate later makes
    first), then two sweeping calls that continue the same chains; after each, every chain
    must equal rt_domino_walk run for the same total number of half-sweeps."""
    import torch

    D = rt.DominoTiler
    d = D.AztecDiamond(order)
    tmax, tmin = D.MaxTiling(d), D.MinTiling(d)
    n = int(np.sqrt(tmax.size))
    pitch = (n // 2 + 15) // 16 * 16
    tiler = rt.DominoTiler(rule="cftp_twoperiodic", rng=mode, a=1.0, b=0.5)
    opts = tiler.opts()

    starts = (tmax, tmin)[:n_chains]
    chains = np.stack([_split(t, n, pitch) for t in starts])
    dev_chains = torch.from_numpy(chains).cuda()
    draws = rt.mt19937_draws(seed, 1 + s1 + s2)
    if mode == "tinymt":
        # rt_domino_walk seeds generator k with (first draw + k); later draws pick colours.
        cells = (n - 2) * (n // 2 - 2)
        gens = torch.from_numpy(orc.tmt_seed_states(int(draws[0]), cells).view(np.int32)).cuda()
        gen_ptr = gens.data_ptr()
        colours = (draws[1:] % 2).astype(np.uint8)
    else:
        gen_ptr = None
        colours = None
    lib = rt.lib()
    st = lib.rt_dm_sweep_noalloc(dev_chains.data_ptr(), gen_ptr, n, n_chains, None, 0, seed, 0, C.byref(opts))
    assert st == 0, lib.rt_last_error().decode()
    assert np.array_equal(dev_chains.cpu().numpy(), chains), "a steps = 0 call must leave the chains alone"
    done = 0
    for steps in (s1, s2):
        cptr = colours[done:done + steps].ctypes.data if colours is not None else None
        st = lib.rt_dm_sweep_noalloc(dev_chains.data_ptr(), gen_ptr, n, n_chains, cptr, steps, seed, done,
                                     C.byref(opts))
        assert st == 0, lib.rt_last_error().decode()
        done += steps
        got = dev_chains.cpu().numpy()
        for c, start in enumerate(starts):
            want = start.copy()
            tiler.Walk(want, done, seed)  # the existing entry point
            assert np.array_equal(_merge(got[c], n), want), (mode, n_chains, done, c)


@pytest.mark.parametrize("n_chains", [1, 2])
@pytest.mark.parametrize("mode", ["tinymt", "fast"])
def test_noalloc_sweep_matches_walk_on_two_calls(rt, orc, mode, n_chains):
    _check_two_calls(rt, orc, 60, mode, n_chains, 300, 457)


def test_noalloc_sweep_at_the_size_limit_matches_walk(rt, orc):
    # Aztec order 509: tiling side 1024, the largest the static scratch holds.
    _check_two_calls(rt, orc, 509, "fast", 2, 150, 211)


def test_noalloc_sweep_rejects_sizes_beyond_its_limits(rt):
    import torch

    lib = rt.lib()
    opts = rt.DominoTiler(rule="plain", rng="fast").opts()
    buf = torch.zeros(16, dtype=torch.uint8, device="cuda")
    st = lib.rt_dm_sweep_noalloc(buf.data_ptr(), None, 1026, 1, None, 1, 0, 0, C.byref(opts))
    assert st == rt.RT_ERR_INVALID_ARGUMENT and "1024" in lib.rt_last_error().decode()
    st = lib.rt_dm_sweep_noalloc(buf.data_ptr(), None, 64, 3, None, 1, 0, 0, C.byref(opts))
    assert st == rt.RT_ERR_INVALID_ARGUMENT
    st = lib.rt_dm_sweep_noalloc(buf.data_ptr(), None, 64, 1, None, 65537, 0, 0, C.byref(opts))
    assert st == rt.RT_ERR_INVALID_ARGUMENT and "65536" in lib.rt_last_error().decode()

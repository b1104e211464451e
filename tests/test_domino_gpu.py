"""GPU parity of the domino sweep through the C ABI.

TinyMT mode must equal the reference's own sweep code (golden vectors made from the
reference-compiled kernels) and the oracle bit for bit; fast mode must equal the oracle's
statement of the fast mode bit for bit.  At the full order-1024 size the walk is compared
with the multi-threaded oracle over a short run, and longer runs are checked through
size-independent properties (valid tiling, height function between the extremal ones)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RULE_NAMES = ["plain", "cftp", "twoperiodic", "cftp_twoperiodic"]


def _tiler(rt, rule, rng="tinymt", a=0.7, b=1.0, engine=0):
    return rt.DominoTiler(rule=RULE_NAMES[rule], rng=rng, a=a, b=b, engine=engine)


def _is_valid_tiling(rt, t, d) -> bool:
    """Edge bits agree across every edge and each domain square is covered exactly once."""
    n = int(np.sqrt(t.size))
    T = t.reshape(n, n)
    if np.any((T[:-1, :] & 2) // 2 != (T[1:, :] & 1)):
        return False
    if np.any((T[:, :-1] & 8) // 8 != (T[:, 1:] & 4) // 4):
        return False
    # Each square (i, j) with corners (i, j) .. (i+1, j+1) is crossed by exactly one dimer
    # edge among its four sides when covered: a domino covers it together with a neighbour.
    D = np.asarray(d).reshape(n - 1, n - 1)
    top = (T[:-1, :-1] & 8) // 8      # edge (i, j)-(i, j+1): separates square (i-1, j) and (i, j)
    left = (T[:-1, :-1] & 2) // 2     # edge (i, j)-(i+1, j): separates square (i, j-1) and (i, j)
    bottom = (T[1:, :-1] & 8) // 8
    right = (T[:-1, 1:] & 2) // 2
    cover = top + left + bottom + right
    return bool(np.all(cover[D == 1] == 1) and np.all(cover[D == 0] == 0))


@pytest.mark.parametrize("engine", [1, 2, 3, 4])
def test_golden_reference_vectors(rt, golden, engine):
    for case in golden["cases"]:
        n = case["N"]
        tiler = _tiler(rt, case["rule"], engine=engine)
        if case["kind"] == "walk":
            if "params" in case:
                tiler.LoadTinyMT(np.array(case["params"], np.uint32))
            t = np.array(case["start"], np.int32)
            tiler.Walk(t, case["steps"], case["seed"])
        elif case["kind"] == "epochs":
            t = np.array(case["start"], np.int32)
            tiler.Walk(t, case["steps"], case["seeds"])
        else:
            t, stats = tiler.cftp(case["tmax"], case["tmin"], case["driver_seed"], case["first_steps"],
                                  case["schedule"], 30)
            assert stats["attempts"] == case["attempts"], case["name"]
        assert np.array_equal(t, np.array(case["expected"], np.int32)), case["name"]


@pytest.mark.parametrize("engine", [1, 2, 3, 4])
def test_tinymt_walk_random_cases_match_oracle(rt, orc, engine):
    rng = np.random.default_rng(11)
    D = rt.DominoTiler
    for trial in range(16):
        order = int(rng.integers(1, 70))
        rule = int(rng.integers(0, 4))
        steps = int(rng.integers(0, 400))
        seed = int(rng.integers(-(2**40), 2**40))
        a, b = float(rng.uniform(0.2, 1.5)), float(rng.uniform(0.2, 1.5))
        d = D.AztecDiamond(order)
        t0 = D.MaxTiling(d) if trial % 2 else D.MinTiling(d)
        n = int(np.sqrt(t0.size))
        g = t0.copy()
        _tiler(rt, rule, a=a, b=b, engine=engine).Walk(g, steps, seed)
        o = t0.copy()
        orc.walk_tinymt(o, n, steps, seed, rule=rule, a=a, b=b, threads=4)
        assert np.array_equal(g, o), (order, rule, steps, seed)


@pytest.mark.parametrize("engine", [1, 2, 3, 4])
def test_tinymt_walk_with_parameter_table_and_rectangles(rt, orc, engine):
    D = rt.DominoTiler
    rng = np.random.default_rng(3)
    for rows, cols in [(4, 6), (13, 8), (30, 31), (200, 90)]:
        d = D.Rectangle(rows, cols) if (rows * cols) % 2 == 0 else D.Rectangle(rows, cols + 1)
        t0 = D.MaxTiling(d)
        n = int(np.sqrt(t0.size))
        params = rng.integers(0, 2**32, size=(n * n // 2, 3), dtype=np.uint64).astype(np.uint32)
        tiler = rt.DominoTiler(rule="plain", engine=engine)
        tiler.LoadTinyMT(params)
        g = t0.copy()
        tiler.Walk(g, 150, 77)
        o = t0.copy()
        orc.walk_tinymt(o, n, 150, 77, rule=0, params=params)
        assert np.array_equal(g, o)


@pytest.mark.parametrize("engine", [1, 2, 3, 4])
def test_tinymt_epochs_match_oracle(rt, orc, engine):
    D = rt.DominoTiler
    d = D.AztecDiamond(33)
    t0 = D.MinTiling(d)
    n = int(np.sqrt(t0.size))
    steps, seeds = [100, 0, 37, 256], [5, 6, 2**32 + 7, -3]
    for rule in range(4):
        g = t0.copy()
        _tiler(rt, rule, engine=engine).Walk(g, steps, seeds)
        o = t0.copy()
        orc.walk_epochs_tinymt(o, n, steps, seeds, rule=rule)
        assert np.array_equal(g, o), rule


@pytest.mark.parametrize("engine", [1, 2, 3])
@pytest.mark.parametrize("rule", [0, 1, 2, 3])
def test_fast_walk_matches_oracle(rt, orc, rule, engine):
    D = rt.DominoTiler
    for order, steps, seed, stream in [(3, 50, 1, 0), (20, 301, 2**40 + 5, 17), (47, 200, 9, 65535)]:
        d = D.AztecDiamond(order)
        t0 = D.MaxTiling(d)
        n = int(np.sqrt(t0.size))
        tiler = rt.DominoTiler(rule=RULE_NAMES[rule], rng="fast", a=1.0, b=0.5, fast_stream=stream, engine=engine)
        g = t0.copy()
        tiler.Walk(g, steps, seed)
        o = t0.copy()
        orc.walk_fast(o, n, 0, steps, seed, stream, rule=rule, a=1.0, b=0.5)
        assert np.array_equal(g, o), (order, steps)


@pytest.mark.parametrize("engine", [1, 2, 3])
@pytest.mark.parametrize("rule,a,b", [(1, 1.0, 1.0), (3, 1.0, 0.5)])
def test_fast_cftp_matches_oracle(rt, orc, rule, a, b, engine):
    D = rt.DominoTiler
    for order, seed in [(4, 3), (10, 12345)]:
        d = D.AztecDiamond(order)
        tmax, tmin = D.MaxTiling(d), D.MinTiling(d)
        n = int(np.sqrt(tmax.size))
        tiler = rt.DominoTiler(rule=RULE_NAMES[rule], rng="fast", a=a, b=b, engine=engine)
        out, stats = tiler.cftp(tmax, tmin, seed, first_steps=8, max_attempts=16)
        ref, attempts, used = orc.cftp_fast(tmax, tmin, n, seed, 0, 8, 16, rule=rule, a=a, b=b)
        assert attempts == stats["attempts"] and 2 * used == stats["final_steps"]
        assert np.array_equal(out, ref)
        assert _is_valid_tiling(rt, out, d)


@pytest.mark.parametrize("engine", [1, 2, 3, 4])
def test_tinymt_cftp_doubling_schedule_matches_oracle(rt, orc, engine):
    D = rt.DominoTiler
    d = D.AztecDiamond(8)
    tmax, tmin = D.MaxTiling(d), D.MinTiling(d)
    n = int(np.sqrt(tmax.size))
    for schedule in (0, 1):
        # schedule 0 (the reference's 128 + 256k look-back) coalesces here after 13 attempts,
        # schedule 1 (doubling) after 4.
        tiler = rt.DominoTiler(rule="cftp_twoperiodic", a=1.0, b=0.5, engine=engine)
        out, stats = tiler.cftp(tmax, tmin, 99, 128, schedule, 25)
        ref, attempts, total = orc.cftp_tinymt(tmax, tmin, n, 99, 128, schedule, 25, rule=3, a=1.0, b=0.5)
        assert attempts == stats["attempts"] and total == stats["total_steps"] and np.array_equal(out, ref)


def test_sampler_api(rt):
    D = rt.DominoTiler
    order = 50
    d = D.AztecDiamond(order)
    tmax, tmin = D.MaxTiling(d), D.MinTiling(d)
    n = int(np.sqrt(tmax.size))
    s = rt.DominoSampler(n, 3, rt.DominoTiler(rule="cftp"))
    s.load(0, tmax)
    s.load(1, tmin)
    assert s.interior_vertices == 2 * order * order - 2 * order + 1
    assert np.array_equal(s.store(0), tmax) and np.array_equal(s.store(1), tmin)
    nd = s.diff(0, 1)
    assert nd == int(np.count_nonzero(tmax != tmin))
    s.copy_chain(2, 0)
    assert s.diff(2, 0) == 0
    s.seed(123)
    s.run(np.array([1, 0, 0, 1, 1], np.uint8))
    assert s.launches > 0
    assert _is_valid_tiling(rt, s.store(0), d) and _is_valid_tiling(rt, s.store(1), d)
    s.close()


@pytest.mark.parametrize("engine", [1, 2, 3, 4])
def test_full_size_order_1024_matches_threaded_oracle(rt, orc, engine):
    """Order-1024 Aztec diamond (N = 2054): 40 TinyMT steps of the two-periodic CFTP rule
    equal the oracle bit for bit."""
    D = rt.DominoTiler
    d = D.AztecDiamond(1024)
    t0 = D.MaxTiling(d)
    n = int(np.sqrt(t0.size))
    g = t0.copy()
    rt.DominoTiler(rule="cftp_twoperiodic", a=1.0, b=0.5, engine=engine).Walk(g, 40, 1)
    o = t0.copy()
    orc.walk_tinymt(o, n, 40, 1, rule=3, a=1.0, b=0.5, threads=8)
    assert np.array_equal(g, o)


def test_inconsistent_tiling_takes_the_per_half_sweep_path(rt, orc):
    """A tiling whose edge bits disagree is swept exactly as the reference does (its
    rebuild overwrites such sites); the resident engine declines it."""
    D = rt.DominoTiler
    t0 = D.MaxTiling(D.AztecDiamond(12))
    n = int(np.sqrt(t0.size))
    t0[5 * n + 5] ^= 8
    g = t0.copy()
    rt.DominoTiler(rule="plain").Walk(g, 31, 4)
    o = t0.copy()
    orc.walk_tinymt(o, n, 31, 4, rule=0)
    assert np.array_equal(g, o)
    with pytest.raises(rt.RTError):
        rt.DominoTiler(rule="plain", engine=2).Walk(t0.copy(), 3, 4)


@pytest.mark.gpu
@pytest.mark.parametrize("rng", ["tinymt", "fast"])
def test_arbitrary_edge_masks_sweep_as_the_reference(rt, orc, rng):
    """Every site holding a random edge mask (no tiling at all): the per-half-sweep kernels
    still rotate and rebuild exactly as the reference's kernels do, edges of the array
    included."""
    rnd = np.random.default_rng(2024)
    for n, steps, seed in ((14, 9, 3), (30, 40, 77), (66, 25, 5)):
        t0 = rnd.integers(0, 16, size=n * n).astype(np.int32)
        g = t0.copy()
        tiler = rt.DominoTiler(rule="cftp", rng=rng, fast_stream=2, engine=1)
        tiler.Walk(g, steps, seed)
        o = t0.copy()
        if rng == "tinymt":
            orc.walk_tinymt(o, n, steps, seed, rule=1)
        else:
            orc.walk_fast(o, n, 0, steps, seed, 2, rule=1)
        assert np.array_equal(g, o), (rng, n)


def test_full_size_order_1024_properties(rt):
    """Longer runs at full size: still a valid tiling of the same domain, height function
    between those of the min and max tilings, and the coupled chains stay ordered."""
    D = rt.DominoTiler
    d = D.AztecDiamond(1024)
    tmax, tmin = D.MaxTiling(d), D.MinTiling(d)
    n = int(np.sqrt(tmax.size))
    s = rt.DominoSampler(n, 2, rt.DominoTiler(rule="cftp_twoperiodic", rng="fast", a=1.0, b=0.5))
    s.load(0, tmax)
    s.load(1, tmin)
    s.run_fast(5, -4000, 4000)
    top, bot = s.store(0), s.store(1)
    s.close()
    assert _is_valid_tiling(rt, top, d) and _is_valid_tiling(rt, bot, d)
    hmax = D.TilingToHeightfunc(tmax, d)
    hmin = D.TilingToHeightfunc(tmin, d)
    ht, hb = D.TilingToHeightfunc(top, d), D.TilingToHeightfunc(bot, d)
    inside = hmax != np.iinfo(np.int32).max
    assert (hb[inside] <= ht[inside]).all()  # monotone coupling keeps the order
    assert (hmin[inside] <= hb[inside]).all() and (ht[inside] <= hmax[inside]).all()


@pytest.mark.gpu
@pytest.mark.parametrize("engine", [2, 3])
def test_resident_engine_wait_gives_up_and_the_sampler_stays_usable(rt, engine):
    """Failure detection without a GPU fault, on both resident kernels: band 1 publishes none
    of its boundary rows and a wait gives up after 4096 polls, so its neighbours' waits run
    out; every CTA leaves its loop, the host reads RT_ERR_TIMEOUT, and the same sampler (same
    CUDA context) then reproduces a fresh sampler's walk bit for bit."""
    D = rt.DominoTiler
    d = D.AztecDiamond(64)
    tmax, tmin = D.MaxTiling(d), D.MinTiling(d)
    n = rt.side_of(tmax)
    tiler = rt.DominoTiler(rule="cftp", rng="fast", fast_stream=3, engine=engine)

    def fresh():
        s = rt.DominoSampler(n, 2, tiler)
        s.load(0, tmin)
        s.load(1, tmax)
        return s

    s = fresh()
    info = s.engine_info()
    assert info["engine"] == engine and info["bands"] >= 3
    assert rt.lib().rt_dm_sampler_test_silent_band(s.h, 1, 4096) == rt.RT_OK
    with pytest.raises(rt.RTError) as err:
        s.run_fast(5, 0, 64)
        s.sync()
    assert err.value.status == rt.RT_ERR_TIMEOUT
    assert rt.lib().rt_dm_sampler_test_silent_band(s.h, -1, 0) == rt.RT_OK
    s.load(0, tmin)
    s.load(1, tmax)
    s.run_fast(5, 0, 64)
    got = [s.store(0), s.store(1)]
    s.close()
    ref = fresh()
    ref.run_fast(5, 0, 64)
    want = [ref.store(0), ref.store(1)]
    ref.close()
    assert all(np.array_equal(a, b) for a, b in zip(got, want))
    assert not np.array_equal(want[0], tmin)


@pytest.mark.gpu
def test_bit_plane_engine_wait_gives_up_and_the_sampler_stays_usable(rt):
    """The same failure detection on the bit-plane kernel (TinyMT mode): band 1 publishes none
    of its boundary words, the neighbours' bounded waits run out, the host reads
    RT_ERR_TIMEOUT, and the sampler then reproduces a fresh sampler's walk bit for bit."""
    D = rt.DominoTiler
    d = D.AztecDiamond(64)
    tmax, tmin = D.MaxTiling(d), D.MinTiling(d)
    n = rt.side_of(tmax)
    tiler = rt.DominoTiler(rule="cftp", engine=4)
    cols = rt.mt19937_colours(77, 64)

    def fresh():
        s = rt.DominoSampler(n, 2, tiler)
        s.load(0, tmin)
        s.load(1, tmax)
        s.seed(5)
        return s

    s = fresh()
    info = s.engine_info()
    assert info["engine"] == 4 and info["bands"] >= 3
    assert rt.lib().rt_dm_sampler_test_silent_band(s.h, 1, 4096) == rt.RT_OK
    with pytest.raises(rt.RTError) as err:
        s.run(cols)
        s.sync()
    assert err.value.status == rt.RT_ERR_TIMEOUT
    assert rt.lib().rt_dm_sampler_test_silent_band(s.h, -1, 0) == rt.RT_OK
    s.load(0, tmin)
    s.load(1, tmax)
    s.seed(5)
    s.run(cols)
    got = [s.store(0), s.store(1)]
    s.close()
    ref = fresh()
    ref.run(cols)
    want = [ref.store(0), ref.store(1)]
    ref.close()
    assert all(np.array_equal(a, b) for a, b in zip(got, want))
    assert not np.array_equal(want[0], tmin)


@pytest.mark.gpu
@pytest.mark.parametrize("order", [1, 2, 5, 33, 130, 700])
def test_bit_plane_engine_matches_the_run_kernel(rt, orc, order):
    """Engine 4 (edge bit planes) against the oracle on Aztec diamonds from the smallest to
    ones whose bands span many rows and words, from both extremal tilings, both chain counts,
    with epochs (the in-kernel generator reseeding)."""
    D = rt.DominoTiler
    d = D.AztecDiamond(order)
    tmax, tmin = D.MaxTiling(d), D.MinTiling(d)
    n = rt.side_of(tmax)
    steps, seeds = [37, 64], [12345 + order, 777]
    for rule in ("cftp_twoperiodic", "plain"):
        for start in (tmax, tmin):
            g = start.copy()
            rt.DominoTiler(rule=rule, a=1.0, b=0.5, engine=4).Walk(g, steps, seeds)
            o = start.copy()
            orc.walk_epochs_tinymt(o, n, steps, seeds, rule=3 if rule == "cftp_twoperiodic" else 0, a=1.0, b=0.5,
                                   threads=8)
            assert np.array_equal(g, o), (order, rule)

"""Lozenge tilings: host utilities and the three-colour sweep.

CPU: the oracle and the library's host utilities against vectors made from the reference's
own src/Lozenge code (tests/golden/lozenge_ref_cases.json).  GPU: TinyMT-mode walks and CFTP
bit-exact with those vectors and with the oracle, fast mode bit-exact with the oracle, and
CFTP samples uniform over every lozenge tiling of small hexagons (MacMahon counts)."""
import json
from pathlib import Path

import numpy as np
import pytest

GOLD = json.loads((Path(__file__).parent / "golden/lozenge_ref_cases.json").read_text())


def test_oracle_matches_reference_lozenge_vectors(orc):
    for hc in GOLD["host_cases"]:
        d = orc.lz_almost_hex(hc["n"], hc["m"])
        assert np.array_equal(d, hc["domain"])
        for which in ("max", "min"):
            rc, t = orc.lz_extremal(d, which)
            assert rc == 0 and np.array_equal(t, hc[which])
        assert np.array_equal(orc.lz_tiling_to_heightfunc(hc["max"], d), hc["hf_max"])
    for case in GOLD["cases"]:
        if case["kind"] == "walk":
            t = np.array(case["start"], np.int32)
            orc.lz_walk_tinymt(t, case["N"], case["steps"], case["seed"], params=case.get("params"))
        else:
            t, att, _ = orc.lz_cftp(case["tmax"], case["tmin"], case["N"], case["driver_seed"], case["first_steps"],
                                    case["schedule"], 40)
            assert att == case["attempts"]
        assert np.array_equal(t, case["expected"]), case["name"]


def test_host_utilities_match_reference_lozenge_vectors(rt):
    L = rt.LozengeTiler
    for hc in GOLD["host_cases"]:
        d = L.AlmostHexDomain(hc["n"], hc["m"])
        assert np.array_equal(d, hc["domain"])
        assert np.array_equal(L.DomainToVertices(d), hc["vertices"])
        tmax, tmin = L.MaxTiling(d), L.MinTiling(d)
        assert np.array_equal(tmax, hc["max"]) and np.array_equal(tmin, hc["min"])
        hf = L.TilingToHeightfunc(tmax, d)
        assert np.array_equal(hf, hc["hf_max"])
        assert np.array_equal(L.HeightfuncToTiling(hf, d), tmax)
        assert np.array_equal(L.TilingToDomain(tmax), d)
    # the regular hexagon has 3n^2 - 3n + 1 interior vertices
    for n in (2, 7, 20):
        v = L.DomainToVertices(L.Hexagon(n))
        assert int((v == 1).sum()) == 3 * n * n - 3 * n + 1


def _lz_flip(T, i, j):
    U = T.copy()
    U[i, j] ^= 63
    for (di, dj, bit) in ((0, 1, 4), (-1, 1, 16), (-1, 0, 32), (0, -1, 8), (1, -1, 2), (1, 0, 1)):
        U[i + di, j + dj] ^= bit
    return U


def enumerate_lozenge(rt, n):
    L = rt.LozengeTiler
    d = L.Hexagon(n)
    t0 = L.MaxTiling(d)
    N = int(np.sqrt(t0.size))
    start = t0.reshape(N, N)
    seen = {start.tobytes(): 0}
    frontier, tilings = [start], [start]
    while frontier:
        nxt = []
        for T in frontier:
            for i, j in zip(*np.nonzero((T == 25) | (T == 38))):
                U = _lz_flip(T, i, j)
                k = U.tobytes()
                if k not in seen:
                    seen[k] = len(tilings)
                    tilings.append(U)
                    nxt.append(U)
        frontier = nxt
    return d, N, tilings, seen


def test_lozenge_enumeration_matches_macmahon(rt):
    # boxed plane partitions in an n x n x n box: 20 for n = 2, 980 for n = 3
    assert len(enumerate_lozenge(rt, 2)[2]) == 20
    assert len(enumerate_lozenge(rt, 3)[2]) == 980


@pytest.mark.gpu
def test_lozenge_walk_matches_reference_vectors(rt):
    for case in GOLD["cases"]:
        if case["kind"] == "walk":
            t = np.array(case["start"], np.int32)
            tiler = rt.LozengeTiler()
            if "params" in case:  # LoadTinyMT's per-generator table (LozengeTiler.cpp:161-164)
                tiler.LoadTinyMT(case["params"])
            tiler.Walk(t, case["steps"], case["seed"])
        else:
            t, stats = rt.LozengeTiler().cftp(case["tmax"], case["tmin"], case["driver_seed"], case["first_steps"],
                                              case["schedule"], 40)
            assert stats["attempts"] == case["attempts"]
        assert np.array_equal(t, case["expected"]), case["name"]


@pytest.mark.gpu
def test_lozenge_walks_match_oracle(rt, orc):
    L = rt.LozengeTiler
    rng = np.random.default_rng(5)
    for trial in range(8):
        n, m = int(rng.integers(2, 40)), 0
        m = int(rng.integers(0, n // 2 + 1))
        d = L.AlmostHexDomain(n, m)
        t0 = L.MaxTiling(d) if trial % 2 else L.MinTiling(d)
        N = int(np.sqrt(t0.size))
        steps, seed = int(rng.integers(0, 400)), int(rng.integers(-(2**40), 2**40))
        g = t0.copy()
        L(rng="tinymt").Walk(g, steps, seed)
        o = t0.copy()
        orc.lz_walk_tinymt(o, N, steps, seed)
        assert np.array_equal(g, o), (n, m, steps, seed)
        g = t0.copy()
        L(rng="fast", fast_stream=trial).Walk(g, steps, seed)
        o = t0.copy()
        orc.lz_walk_fast(o, N, 0, steps, seed, trial)
        assert np.array_equal(g, o), ("fast", n, m, steps, seed)


@pytest.mark.gpu
@pytest.mark.parametrize("fast", [False, True])
def test_lozenge_cftp_matches_oracle(rt, orc, fast):
    L = rt.LozengeTiler
    d = L.Hexagon(6)
    tmax, tmin = L.MaxTiling(d), L.MinTiling(d)
    N = int(np.sqrt(tmax.size))
    tiler = L(rng="fast" if fast else "tinymt")
    for seed in (1, 99):
        out, stats = tiler.cftp(tmax, tmin, seed, first_steps=16, schedule=1, max_attempts=20)
        ref, att, total = orc.lz_cftp(tmax, tmin, N, seed, 16, 1, 20, fast=fast)
        assert att == stats["attempts"] and total == stats["total_steps"] and np.array_equal(out, ref)


@pytest.mark.gpu
@pytest.mark.parametrize("rng,n,samples", [("fast", 2, 2000), ("tinymt", 2, 1500), ("fast", 3, 6000)])
def test_lozenge_cftp_is_uniform_over_enumerated_tilings(rt, rng, n, samples):
    from tests.test_cftp_exactness import chi_square_p

    d, N, tilings, seen = enumerate_lozenge(rt, n)
    L = rt.LozengeTiler
    tmax, tmin = L.MaxTiling(d), L.MinTiling(d)
    counts = np.zeros(len(tilings))
    for k in range(samples):
        tiler = L(rng=rng, fast_stream=k & 0xFFFF)
        out, _ = tiler.cftp(tmax, tmin, 5000 + k, first_steps=8, schedule=1, max_attempts=20)
        counts[seen[out.reshape(N, N).tobytes()]] += 1
    p = chi_square_p(counts, np.full(len(tilings), 1.0 / len(tilings)))
    assert p > 1e-3, p


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["tinymt", "fast"])
def test_arbitrary_edge_masks_sweep_as_the_reference(rt, orc, mode):
    """Every vertex holding a random six-bit edge mask (no tiling at all): the per-step
    kernels (rotation, then the word-parallel rebuild of the two other colours) still do
    exactly what the reference's kernels do, array edges included."""
    rnd = np.random.default_rng(99)
    for n, steps, seed in ((12, 7, 1), (33, 40, 8), (66, 25, 3)):
        t0 = rnd.integers(0, 64, size=n * n).astype(np.int32)
        a = t0.copy()
        rt.LozengeTiler(rng=mode, fast_stream=4).Walk(a, steps, seed)
        b = t0.copy()
        if mode == "tinymt":
            orc.lz_walk_tinymt(b, n, steps, seed)
        else:
            orc.lz_walk_fast(b, n, 0, steps, seed, 4)
        assert np.array_equal(a, b), (mode, n)


@pytest.mark.gpu
@pytest.mark.parametrize("rng,q", [("tinymt", None), ("fast", None), ("tinymt", 0.7), ("fast", 1.3)])
def test_resident_engine_equals_per_step_kernels(rt, rng, q):
    """The resident band kernel (engine 2) against the per-step kernels (engine 1): walks of
    one chain and CFTP of the coupled pair give the same tilings and attempt counts, on
    hexagons from 3 bands (side 5) to one band per SM (side 512, a short walk)."""
    L = rt.LozengeTiler
    for side, steps in ((5, 301), (37, 450), (150, 90), (512, 31)):
        d = L.Hexagon(side)
        t0 = L.MaxTiling(d)
        out = []
        for engine in (1, 2):
            t = t0.copy()
            L(rng=rng, fast_stream=11, q=q, engine=engine).Walk(t, steps, 4242 + side)
            out.append(t)
        assert np.array_equal(out[0], out[1]), (rng, q, side)
        assert not np.array_equal(out[1], t0) or side == 512
    d = L.Hexagon(9)
    tmax, tmin = L.MaxTiling(d), L.MinTiling(d)
    res = [L(rng=rng, fast_stream=3, q=q, engine=e).cftp(tmax, tmin, 77, first_steps=8, schedule=1, max_attempts=20)
           for e in (1, 2)]
    assert np.array_equal(res[0][0], res[1][0]) and res[0][1]["attempts"] == res[1][1]["attempts"]


@pytest.mark.gpu
def test_resident_engine_with_a_tinymt_parameter_table(rt):
    L = rt.LozengeTiler
    d = L.Hexagon(20)
    t0 = L.MaxTiling(d)
    n = int(np.sqrt(t0.size))
    rnd = np.random.default_rng(3)
    table = [(0x8F7011EE ^ int(x), 0xFC78FF1F ^ int(y), 0x3793FDFF ^ int(z))
             for x, y, z in rnd.integers(0, 1 << 20, size=(n * (n // 3), 3))]
    out = []
    for engine in (1, 2):
        tiler = L(engine=engine)
        tiler.LoadTinyMT(table)
        t = t0.copy()
        tiler.Walk(t, 200, 9)
        out.append(t)
    assert np.array_equal(out[0], out[1])


def test_resident_engine_refuses_mtgp(rt):
    L = rt.LozengeTiler
    t = L.MaxTiling(L.Hexagon(4))
    with pytest.raises(rt.RTError) as e:
        L(rng="mtgp", engine=2).Walk(t, 3, 1)
    assert e.value.status == rt.RT_ERR_INVALID_ARGUMENT

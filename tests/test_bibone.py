"""Bibone tilings (dimer coverings of the triangular lattice; reference src/TriangleDimer).

CPU: the oracle and the library's host utilities against vectors made from the reference's
own code (tests/golden/bibone_ref_cases.json: its .cl kernels driven by its Walk loop, its
IceCreamCone, and the committed Examples/ExampleOuts/TriangleDimer fixtures); every move maps
dimer coverings to dimer coverings, and the moves connect all coverings of small domains
(counted independently by brute force).
GPU: TinyMT-mode walks bit-exact with the reference's vectors, fast-mode walks bit-exact with
the oracle, the 512 x 512 rhombus from the brick start stays a covering of the same vertex
set, and the fast chain's samples are uniform over the coverings of a small domain."""
import json
from pathlib import Path

import numpy as np
import pytest

GOLD = json.loads((Path(__file__).parent / "golden/bibone_ref_cases.json").read_text())
NEIGHBOURS = ((0, 1), (0, -1), (-1, 0), (1, 0), (-1, 1), (1, -1))


def cover(rt, t):
    """Dimers at each vertex (M x M)."""
    d = rt.TriangleDimerTiler.Dimers(t)
    M = int(np.sqrt(d.size))
    D = d.reshape(M, M)
    c = np.zeros((M + 2, M + 2), int)
    for a, b in zip(*np.nonzero(D & 1)):
        c[a, b] += 1
        c[a, b + 1] += 1
    for a, b in zip(*np.nonzero(D & 2)):
        c[a, b] += 1
        c[a - 1, b] += 1
    for a, b in zip(*np.nonzero(D & 4)):
        c[a, b] += 1
        c[a - 1, b + 1] += 1
    return c[:M, :M]


def count_coverings(vertices):
    """Perfect matchings of the triangular-lattice graph induced on `vertices` (brute force)."""
    vs = sorted(vertices)
    index = {v: k for k, v in enumerate(vs)}
    adj = [[index[(a + da, b + db)] for da, db in NEIGHBOURS if (a + da, b + db) in index] for a, b in vs]

    def rec(used):
        if used == (1 << len(vs)) - 1:
            return 1
        v = next(k for k in range(len(vs)) if not used >> k & 1)
        return sum(rec(used | 1 << v | 1 << w) for w in adj[v] if not used >> w & 1)

    return rec(0)


def flip_all(rt, t):
    """Every covering reachable from t by single moves (breadth first), each move the toggle
    of a lozenge, triangle or butterfly cycle one half of which is covered, written out here
    independently of the oracle and the library as (row, column, edge bit) offsets."""
    T = rt.TriangleDimerTiler
    N = int(np.sqrt(t.size))
    M = N // 2
    cycles = [
        ([(-1, 0, 4), (0, 0, 4)], [(-1, 1, 2), (0, 0, 2)]),
        ([(-1, 0, 1), (0, -1, 1)], [(0, 0, 4), (0, -1, 4)]),
        ([(-1, 0, 1), (0, 0, 1)], [(0, 1, 2), (0, 0, 2)]),
        ([(-1, 0, 1), (0, 1, 4), (1, 0, 2)], [(0, 0, 2), (-1, 1, 1), (1, 0, 4)]),
        ([(0, -1, 1), (0, 1, 2), (-1, 0, 4)], [(0, -1, 4), (0, 0, 1), (-1, 1, 2)]),
        ([(-1, 0, 2), (-2, 1, 1), (0, 1, 2), (0, -1, 1)], [(-2, 0, 1), (-1, 1, 4), (0, 0, 1), (0, -1, 4)]),
        ([(-1, 0, 4), (0, 1, 2), (1, -1, 4), (0, -1, 2)], [(-1, 1, 2), (0, 0, 1), (1, -1, 2), (-1, -1, 1)]),
        ([(-1, 0, 4), (-1, 1, 1), (1, 0, 4), (0, -1, 1)], [(-1, 1, 2), (0, 1, 4), (1, 0, 2), (0, -1, 4)]),
    ]
    start = T.Dimers(t).reshape(M, M)
    seen = {start.tobytes()}
    frontier = [start]
    while frontier:
        nxt = []
        for D in frontier:
            for half_a, half_b in cycles:
                for a in range(2, M - 2):
                    for b in range(2, M - 2):
                        has = [all(D[a + da, b + db] & bit for da, db, bit in h) for h in (half_a, half_b)]
                        if not any(has):
                            continue
                        U = D.copy()
                        for da, db, bit in half_a + half_b:
                            U[a + da, b + db] ^= bit
                        k = U.tobytes()
                        if k not in seen:
                            seen.add(k)
                            nxt.append(U)
        frontier = nxt
    return seen


def test_oracle_matches_reference_vectors(orc):
    for hc in GOLD["host_cases"]:
        assert np.array_equal(orc.td_icecream(hc["n"], hc["m"]), hc["tiling"])
    for case in GOLD["cases"]:
        t = np.array(case["start"], np.int32)
        orc.td_walk_tinymt(t, case["N"], case["steps"], case["seed"], params=case.get("params"))
        assert np.array_equal(t, case["expected"]), case["name"]


def test_host_utilities_match_reference_vectors(rt):
    T = rt.TriangleDimerTiler
    for hc in GOLD["host_cases"]:
        t = T.IceCreamCone(hc["n"], hc["m"])
        assert np.array_equal(t, hc["tiling"])
        assert np.array_equal(T.FromDimers(T.Dimers(t), hc["N"]), t)
    ex = GOLD["example"]
    assert np.array_equal(T.IceCreamCone(ex["n"], ex["m"]), ex["tiling"])  # DimerStart.txt
    assert np.array_equal(T.TilingToDomain(ex["tiling"])[: len(ex["domain"])], ex["domain"])  # Domain.txt
    for case in GOLD["cases"]:
        c0, c1 = cover(rt, np.array(case["start"])), cover(rt, np.array(case["expected"]))
        assert c0.max() == 1 and np.array_equal(c0, c1)
        assert int(T.TilingToVertices(case["expected"]).sum()) == int(c1.sum())


def test_derived_move_states_match_reference_vectors(rt):
    T = rt.TriangleDimerTiler
    for hc in GOLD["host_cases"]:
        assert np.array_equal(T.TilingToTriangleFlips(hc["tiling"]), hc["triangle_flips"])
        assert np.array_equal(T.TilingToButterflyFlips(hc["tiling"]), hc["butterfly_flips"])
    for tb in GOLD["test_butterflies"]:
        t = T.TestButterfly(tb["type"])
        assert np.array_equal(t, tb["tiling"])
        assert np.array_equal(T.TilingToButterflyFlips(t), tb["butterfly_flips"])
        assert np.array_equal(T.TilingToTriangleFlips(t), tb["triangle_flips"])
    # a test butterfly is flippable: its state at the centre is 85 or 170
    for typ, (i, j) in ((0, (6, 7)), (1, (7, 6)), (2, (7, 7))):
        assert T.TilingToButterflyFlips(T.TestButterfly(typ)).reshape(16, 16)[i, j] in (85, 170)


def test_rhombus_brick_is_a_covering_of_the_rhombus(rt):
    T = rt.TriangleDimerTiler
    t = T.RhombusBrick(6, 8)
    c = cover(rt, t)
    assert c.max() == 1 and int(c.sum()) == 48
    assert np.array_equal(np.argwhere(c == 1).min(0), [3, 3]) and np.array_equal(np.argwhere(c == 1).max(0), [8, 10])
    with pytest.raises(rt.RTError):
        T.RhombusBrick(4, 5)


def test_walk_rejects_states_that_are_not_dimers_on_the_host(rt):
    T = rt.TriangleDimerTiler
    t = T.IceCreamCone(4, 1)
    t[7 * int(np.sqrt(t.size)) + 7] ^= 2
    with pytest.raises(rt.RTError):
        T().Walk(t, 3, 1)


@pytest.mark.parametrize("n,m", [(3, 0), (4, 1), (5, 2), (6, 0)])
def test_moves_connect_every_covering(rt, n, m):
    t = rt.TriangleDimerTiler.IceCreamCone(n, m)
    c = cover(rt, t)
    reach = flip_all(rt, t)
    assert len(reach) == count_coverings({(int(a), int(b)) for a, b in np.argwhere(c == 1)})


def test_oracle_fast_walks_keep_coverings(rt, orc):
    for n, m, steps in ((7, 0, 500), (11, 3, 300)):
        t = orc.td_icecream(n, m)
        N = int(np.sqrt(t.size))
        u = t.copy()
        orc.td_walk_fast(u, N, 0, steps, 2024, 5)
        assert np.array_equal(cover(rt, u), cover(rt, t)) and not np.array_equal(u, t)


@pytest.mark.gpu
def test_walk_matches_reference_vectors(rt):
    for case in GOLD["cases"]:
        T = rt.TriangleDimerTiler()
        if "params" in case:  # LoadTinyMT's per-generator table (TriangleDimerTiler.cpp:24-27)
            T.LoadTinyMT(case["params"])
        t = np.array(case["start"], np.int32)
        T.Walk(t, case["steps"], case["seed"])
        assert np.array_equal(t, case["expected"]), case["name"]


@pytest.mark.gpu
def test_walks_match_oracle(rt, orc):
    T = rt.TriangleDimerTiler
    for n, m, steps, seed, stream in ((4, 1, 40, 3, 0), (9, 1, 700, -8, 1), (16, 6, 400, 12345, 777), (30, 2, 250, 5, 65535)):
        start = orc.td_icecream(n, m)
        N = int(np.sqrt(start.size))
        for mode in ("tinymt", "fast"):
            a, b = start.copy(), start.copy()
            T(rng=mode, fast_stream=stream).Walk(a, steps, seed)
            if mode == "tinymt":
                orc.td_walk_tinymt(b, N, steps, seed)
            else:
                orc.td_walk_fast(b, N, 0, steps, seed, stream)
            assert np.array_equal(a, b), (n, m, mode)
    r = T.RhombusBrick(40, 40)
    a, b = r.copy(), r.copy()
    T(rng="fast", fast_stream=3).Walk(a, 600, 9)
    orc.td_walk_fast(b, int(np.sqrt(r.size)), 0, 600, 9, 3)
    assert np.array_equal(a, b) and not np.array_equal(a, r)


@pytest.mark.gpu
def test_rhombus_512_from_brick_stays_a_covering(rt):
    T = rt.TriangleDimerTiler
    t = T.RhombusBrick(512, 512)
    c0 = cover(rt, t)
    stats = T(rng="fast").Walk(t, 3000, 1)
    c1 = cover(rt, t)
    assert c0.max() == 1 and np.array_equal(c0, c1)
    assert stats["flip_attempts"] > 0 and stats["total_steps"] == 3000


@pytest.mark.gpu
def test_fast_chain_is_uniform_over_the_coverings_of_a_small_domain(rt):
    from scipy.stats import chi2

    T = rt.TriangleDimerTiler
    start = T.IceCreamCone(5, 2)
    reach = sorted(flip_all(rt, start))
    index = {k: i for i, k in enumerate(reach)}
    counts = np.zeros(len(reach))
    N = int(np.sqrt(start.size))
    for s in range(3000):
        t = start.copy()
        T(rng="fast", fast_stream=s % 65536).Walk(t, 300, 1 + s // 65536)
        counts[index[T.Dimers(t).reshape(N // 2, N // 2).tobytes()]] += 1
    exp = counts.sum() / len(reach)
    stat = float(((counts - exp) ** 2 / exp).sum())
    assert chi2.sf(stat, len(reach) - 1) > 1e-3

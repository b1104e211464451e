"""q-weighted lozenge tilings (the reference's qlozengekernel.cl, q a runtime argument and its
down-move rescaling corrected).

For q <= 1 the corrected rule makes the reference's decisions, so TinyMT walks at the compiled
q = 0.99 are pinned bit-exactly against the reference's own kernel (tests/golden). For any q
the chain's law is q^volume: the enumeration of all tilings of small hexagons reproduces
MacMahon's q-product, and CFTP samples (q < 1 and q > 1, where the reference's rescaling
would be wrong) pass a chi-square test against it."""
import json
import math
from pathlib import Path

import numpy as np
import pytest

from tests.test_lozenge import _lz_flip, enumerate_lozenge

GOLD = json.loads((Path(__file__).parent / "golden/lozenge_ref_cases.json").read_text())


def volumes(tilings, seen):
    """Cubes of each tiling: the rank in the flip graph, +1 for every 25 -> 38 rotation."""
    rank = {0: 0}
    frontier = [0]
    while frontier:
        nxt = []
        for x in frontier:
            T = tilings[x]
            for i, j in zip(*np.nonzero((T == 25) | (T == 38))):
                y = seen[_lz_flip(T, i, j).tobytes()]
                if y not in rank:
                    rank[y] = rank[x] + (1 if T[i, j] == 25 else -1)
                    nxt.append(y)
        frontier = nxt
    v = np.array([rank[k] for k in range(len(tilings))])
    return v - v.min()


def macmahon(n: int, q: float) -> float:
    z = 1.0
    for i in range(1, n + 1):
        for j in range(1, n + 1):
            for k in range(1, n + 1):
                z *= (1 - q ** (i + j + k - 1)) / (1 - q ** (i + j + k - 2))
    return z


def test_oracle_matches_the_reference_q_kernel(orc):
    for case in GOLD["q_cases"]:
        t = np.array(case["start"], np.int32)
        with orc.lz_rule(case["q"]):
            orc.lz_walk_tinymt(t, case["N"], case["steps"], case["seed"])
        assert np.array_equal(t, case["expected"]), case["name"]


@pytest.mark.parametrize("n", [2, 3])
def test_volume_generating_function_is_macmahons(rt, n):
    _, _, tilings, seen = enumerate_lozenge(rt, n)
    v = volumes(tilings, seen)
    assert v.max() == n ** 3
    for q in (0.3, 0.77, 1.9):
        assert float(np.sum(q ** v)) == pytest.approx(macmahon(n, q), rel=1e-12)


def test_q_rule_is_rejected_for_non_positive_q(rt):
    L = rt.LozengeTiler
    d = L.Hexagon(2)
    t = L.MaxTiling(d)
    with pytest.raises(rt.RTError):
        L(q=0.0).Walk(t, 1, 1)


@pytest.mark.gpu
def test_tinymt_q_walk_matches_the_reference_q_kernel(rt):
    for case in GOLD["q_cases"]:
        t = np.array(case["start"], np.int32)
        rt.LozengeTiler(q=case["q"]).Walk(t, case["steps"], case["seed"])
        assert np.array_equal(t, case["expected"]), case["name"]


@pytest.mark.gpu
@pytest.mark.parametrize("q", [0.5, 1.7])
def test_q_walks_match_oracle(rt, orc, q):
    L = rt.LozengeTiler
    for n, steps, seed in ((3, 300, 4), (12, 200, 99)):
        d = L.Hexagon(n)
        start = L.MaxTiling(d)
        N = int(np.sqrt(start.size))
        for mode in ("tinymt", "fast"):
            a, b = start.copy(), start.copy()
            L(rng=mode, fast_stream=6, q=q).Walk(a, steps, seed)
            with orc.lz_rule(q):
                if mode == "tinymt":
                    orc.lz_walk_tinymt(b, N, steps, seed)
                else:
                    orc.lz_walk_fast(b, N, 0, steps, seed, 6)
            assert np.array_equal(a, b), (n, mode, q)
            assert not np.array_equal(a, start)


@pytest.mark.gpu
@pytest.mark.parametrize("q", [0.6, 1.8])
def test_q_cftp_samples_follow_q_to_the_volume(rt, q):
    from scipy.stats import chi2

    d, N, tilings, seen = enumerate_lozenge(rt, 2)
    v = volumes(tilings, seen)
    pi = q ** v / np.sum(q ** v)
    L = rt.LozengeTiler
    tmax, tmin = L.MaxTiling(d), L.MinTiling(d)
    counts = np.zeros(len(tilings))
    for k in range(3000):
        out, _ = L(rng="fast", fast_stream=k, q=q).cftp(tmax, tmin, 500 + k, first_steps=8, max_attempts=20)
        counts[seen[out.reshape(N, N).tobytes()]] += 1
    exp = pi * counts.sum()
    stat = float(((counts - exp) ** 2 / exp).sum())
    assert chi2.sf(stat, len(tilings) - 1) > 1e-3

"""Rectangle-triangle tilings: host utilities and the three-colour sweep.

CPU: the oracle and the library's host utilities against vectors made from the reference's
own src/RectTriangle code (tests/golden/recttri_ref_cases.json, whose generator also pins
the reference's committed Examples/ExampleOuts/RectTriangle fixtures).  GPU: TinyMT-mode
walks bit-exact with those vectors, weighted walks in both random modes bit-exact with the
oracle, and at larger sizes the triangle-consistency invariant of every state."""
import json
from pathlib import Path

import numpy as np
import pytest

GOLD = json.loads((Path(__file__).parent / "golden/recttri_ref_cases.json").read_text())


def inconsistent_triangles(t) -> int:
    """Triangles whose code differs between the three vertices around it: an up triangle at
    (i, c) is digit 0 of (i, c), digit 2 of (i, c+1) and digit 4 of (i+1, c); a down triangle
    is digit 1 of (i, c+1), digit 3 of (i+1, c) and digit 5 of (i+1, c+1)."""
    t = np.asarray(t)
    n = int(np.sqrt(t.size))
    T = t.reshape(n, n)
    d = [(T >> (4 * k)) & 15 for k in range(6)]
    up = (d[0][:-1, :-1] != d[2][:-1, 1:]) | (d[0][:-1, :-1] != d[4][1:, :-1])
    dn = (d[1][:-1, 1:] != d[3][1:, :-1]) | (d[1][:-1, 1:] != d[5][1:, 1:])
    return int(up.sum() + dn.sum())


def random_weights(rng) -> np.ndarray:
    return rng.uniform(0.3, 2.5, size=9)


def test_oracle_matches_reference_recttri_vectors(orc):
    for hc in GOLD["host_cases"]:
        assert np.array_equal(orc.rt_hex(hc["n"], True), hc["max"])
        assert np.array_equal(orc.rt_hex(hc["n"], False), hc["min"])
    for case in GOLD["cases"]:
        t = np.array(case["start"], np.int32)
        orc.rt_walk_tinymt(t, case["N"], case["steps"], case["seed"], params=case.get("params"))
        assert np.array_equal(t, case["expected"]), case["name"]
        assert inconsistent_triangles(t) == 0


def test_host_utilities_match_reference_recttri_vectors(rt):
    R = rt.RectTriangleTiler
    for hc in GOLD["host_cases"]:
        assert np.array_equal(R.maxHex(hc["n"]), hc["max"])
        assert np.array_equal(R.minHex(hc["n"]), hc["min"])
        assert np.array_equal(R.slopeHex(hc["n"]), hc["slope"])
        assert inconsistent_triangles(R.slopeHex(hc["n"])) == 0 or hc["n"] == 2  # slopeHex(2) is not a tiling
        assert int(np.sqrt(len(hc["max"]))) == hc["N"] and hc["N"] % 3 == 0
    for cv in GOLD["from_lozenge"]:
        out = R.LozengeToRectTriangle(np.array(cv["lozenge"], np.int32), np.array(cv["domain"], np.int32))
        assert np.array_equal(out, cv["expected"])
        assert inconsistent_triangles(out) == 0


def test_oracle_weighted_walks_stay_consistent(orc):
    rng = np.random.default_rng(5)
    for n, steps in ((4, 300), (9, 200)):
        w = random_weights(rng)
        t = orc.rt_hex(n, False)
        N = int(np.sqrt(t.size))
        orc.rt_walk_tinymt(t, N, steps, 11, w)
        assert inconsistent_triangles(t) == 0
        u = orc.rt_hex(n, True)
        orc.rt_walk_fast(u, N, 0, steps, 12345, 3, w)
        assert inconsistent_triangles(u) == 0 and not np.array_equal(u, orc.rt_hex(n, True))


def test_walk_rejects_bad_arguments_before_any_device_work(rt):
    R = rt.RectTriangleTiler
    with pytest.raises(rt.RTError):
        R().Walk(np.zeros(10 * 10, np.int32), 5, 1)  # side not a multiple of 3
    t = R.minHex(3)
    t[0] = 0x1000000  # seven hex digits
    with pytest.raises(rt.RTError):
        R().Walk(t, 5, 1)
    with pytest.raises(ValueError):
        R(weights=[1.0] * 8)


@pytest.mark.gpu
def test_walk_matches_reference_vectors(rt):
    for case in GOLD["cases"]:
        R = rt.RectTriangleTiler()
        if "params" in case:  # LoadTinyMT's per-generator table (RectTriangleTiler.cpp:22-25)
            R.LoadTinyMT(case["params"])
        t = np.array(case["start"], np.int32)
        R.Walk(t, case["steps"], case["seed"])
        assert np.array_equal(t, case["expected"]), case["name"]


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["tinymt", "fast"])
def test_weighted_walk_matches_oracle(rt, orc, mode):
    rng = np.random.default_rng(17 if mode == "tinymt" else 18)
    for n, steps, seed in ((2, 50, 3), (5, 400, -9), (11, 300, 2024), (30, 120, 7)):
        w = random_weights(rng)
        for top in (False, True):
            start = orc.rt_hex(n, top)
            N = int(np.sqrt(start.size))
            a, b = start.copy(), start.copy()
            rt.RectTriangleTiler(rng=mode, fast_stream=5, weights=w).Walk(a, steps, seed)
            if mode == "tinymt":
                orc.rt_walk_tinymt(b, N, steps, seed, w)
            else:
                orc.rt_walk_fast(b, N, 0, steps, seed, 5, w)
            assert np.array_equal(a, b), (mode, n, top)
            assert not np.array_equal(a, start)


@pytest.mark.gpu
def test_large_hexagon_stays_consistent_and_moves(rt, orc):
    # hexagon of side 600 (N = 1209): every state is a tiling, and the fast-mode walk equals
    # the oracle's.  From the extremal tiling only the corner moves at first (about 2000
    # vertices changed after 600 steps).
    start = rt.RectTriangleTiler.minHex(600)
    N = int(np.sqrt(start.size))
    a = start.copy()
    rt.RectTriangleTiler(rng="fast").Walk(a, 600, 99)
    assert inconsistent_triangles(a) == 0
    assert int((a != start).sum()) > 1000
    b = start.copy()
    orc.rt_walk_fast(b, N, 0, 600, 99)
    assert np.array_equal(a, b)

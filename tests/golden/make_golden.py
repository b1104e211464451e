"""Generates tests/golden/{domino,lozenge,recttri,bibone}_ref_cases.json from the reference's own code.

Runs where the reference tree exists (it is not on the GPU machine): builds oracle/_ref
(`make -C oracle ref`), which compiles the reference's domino .cl kernel files and its host
code (src/Domino/DominoTiler.cpp) from the reference tree, and records for a set of small
cases the start tiling and the tiling after the reference's own sweep code ran (TinyMT
generators with the default parameter set, or with a seeded synthetic parameter table where
noted; the reference's own table file is absent from its tree).  Also pins the committed
fixture Examples/ExampleOuts/WeightedAztecDiamond/TilingStart.txt against the reference's
MinTiling(AztecDiamond(16)).

    python tests/golden/make_golden.py --ref <reference tree>
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
RULES = ["plain", "CFTP", "twoperiodic", "CFTPtwoperiodic"]


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="path of the reference tree (its src/ and Examples/)")
    args = ap.parse_args()
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "ref", f"REF={args.ref}"], check=True)
    host = C.CDLL(str(ROOT / "oracle/_ref/libref_domino_host.so"))
    cl = C.CDLL(str(ROOT / "oracle/_ref/libref_domino_cl.so"))
    P = lambda a: None if a is None else a.ctypes.data_as(C.c_void_p)

    def domain(n):
        buf = np.zeros((2 * n + 6) ** 2, np.int32)
        side = host.refh_dm_aztec_rectangle(n, None, 0, P(buf), buf.size)
        return buf[: side * side].copy(), side

    def extremal(n, which):
        d, m = domain(n)
        out = np.zeros((m + 1) ** 2, np.int32)
        getattr(host, f"refh_dm_{which}_tiling")(P(d), m, P(out))
        return out, m + 1

    for nm in RULES:
        for suffix in ("_walk", "_walk_epochs"):
            f = getattr(cl, f"ref_{nm}{suffix}")
            f.restype = C.c_int
        getattr(cl, f"ref_{nm}_walk").argtypes = [C.c_void_p, C.c_int, C.c_long, C.c_long, C.c_void_p, C.c_long]
        getattr(cl, f"ref_{nm}_walk_epochs").argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                                         C.c_void_p, C.c_long]

    def walk(nm, t, n, steps, seed, params=None):
        t = t.copy()
        getattr(cl, f"ref_{nm}_walk")(P(t), n, steps, seed, P(params), 0 if params is None else params.shape[0])
        return t

    def walk_epochs(nm, t, n, steps, seeds, params=None):
        t = t.copy()
        st = np.asarray(steps, np.int64)
        sd = np.asarray(seeds, np.int64)
        getattr(cl, f"ref_{nm}_walk_epochs")(P(t), n, P(st), P(sd), len(st), P(params),
                                             0 if params is None else params.shape[0])
        return t

    cases = []

    def add(name, kind, rule, start, n, expected, **kw):
        cases.append({"name": name, "kind": kind, "rule": rule, "N": n, "start": start.tolist(),
                      "expected": expected.tolist(), **kw})

    # Single walks, every rule, from the max and the min tiling.
    for r, nm in enumerate(RULES):
        for order, which, steps, seed in [(6, "max", 57, 34893), (11, "min", 131, 1)]:
            start, n = extremal(order, which)
            add(f"walk_{nm}_aztec{order}_{which}", "walk", r, start, n, walk(nm, start, n, steps, seed),
                steps=steps, seed=seed)
    # Epoch walks (the vector overload).
    for r, nm in enumerate(RULES):
        start, n = extremal(7, "min")
        steps, seeds = [40, 23, 17], [11, 2024, 4294967295]
        add(f"epochs_{nm}_aztec7", "epochs", r, start, n, walk_epochs(nm, start, n, steps, seeds),
            steps=steps, seeds=seeds)
    # A per-generator parameter table (synthetic, seeded) in place of the missing file.
    start, n = extremal(5, "max")
    rng = np.random.default_rng(20261203)
    params = rng.integers(0, 2**32, size=(n * n // 2, 3), dtype=np.uint64).astype(np.uint32)
    add("walk_plain_aztec5_paramtable", "walk", 0, start, n, walk("plain", start, n, 73, 99, params),
        steps=73, seed=99, params=params.tolist())
    # The MinimalDomino example tiling (Examples/MinimalDominoEx.cpp:33-42, 10 x 10), 100 steps, seed 34893.
    t10 = np.zeros(100, np.int32)
    rows = {2: {4: 2}, 3: {2: 8, 3: 4, 4: 1, 5: 8, 6: 4}, 4: {3: 8, 4: 12, 5: 4}, 5: {2: 8, 3: 4, 4: 2, 5: 8, 6: 4},
            6: {4: 1}}
    for i, row in rows.items():
        for j, v in row.items():
            t10[i * 10 + j] = v
    add("walk_plain_minimal_domino", "walk", 0, t10, 10, walk("plain", t10, 10, 100, 34893), steps=100, seed=34893)
    # The CFTP example (Examples/AztecDiamondCftpEx.cpp:13,51-77): order 5, driver seed 345903,
    # first epoch 128 steps, epochs prepended at 2 * steps.back(); both chains through the
    # reference's epoch walk.
    tmax, n = extremal(5, "max")
    tmin, _ = extremal(5, "min")
    drv = np.random.RandomState(345903)
    draw = lambda: int(drv.randint(0, 2**32, dtype=np.uint32))
    steps, seeds = [128], [draw()]
    attempts = 0
    while True:
        attempts += 1
        top = walk_epochs("CFTP", tmax, n, steps, seeds)
        bot = walk_epochs("CFTP", tmin, n, steps, seeds)
        if np.array_equal(top, bot):
            break
        steps.insert(0, steps[-1] * 2)
        seeds.insert(0, draw())
        assert attempts < 30
    cases.append({"name": "cftp_example_aztec5", "kind": "cftp", "rule": 1, "N": n, "tmax": tmax.tolist(),
                  "tmin": tmin.tolist(), "driver_seed": 345903, "first_steps": 128, "schedule": 0,
                  "attempts": attempts, "expected": top.tolist()})

    # Pin: the committed start tiling of the weighted example equals MinTiling(AztecDiamond(16)).
    fixture = np.loadtxt(Path(args.ref) / "Examples/ExampleOuts/WeightedAztecDiamond/TilingStart.txt", dtype=np.int32)
    mint, _ = extremal(16, "min")
    assert np.array_equal(fixture.ravel(), mint), "reference MinTiling differs from its committed fixture"
    pins = {"min_tiling_aztec16": mint.tolist()}
    # Reference host utilities on a few domains for the host-side restatement.
    host_cases = []
    for order in (1, 2, 3, 9):
        d, m = domain(order)
        tmx = np.zeros((m + 1) ** 2, np.int32)
        tmn = np.zeros((m + 1) ** 2, np.int32)
        host.refh_dm_max_tiling(P(d), m, P(tmx))
        host.refh_dm_min_tiling(P(d), m, P(tmn))
        hf = np.zeros((m + 1) ** 2, np.int32)
        host.refh_dm_tiling_to_heightfunc(P(tmx), P(d), m + 1, P(hf))
        host_cases.append({"order": order, "domain": d.tolist(), "max": tmx.tolist(), "min": tmn.tolist(),
                           "hf_max": hf.tolist()})
    rect = np.zeros(30 * 30, np.int32)
    side = host.refh_dm_rectangle(6, 9, P(rect), rect.size)
    pins["rectangle_6x9"] = rect[: side * side].tolist()
    out = {"generator": "tests/golden/make_golden.py", "cases": cases, "pins": pins, "host_cases": host_cases}
    (HERE / "domino_ref_cases.json").write_text(json.dumps(out, separators=(",", ":")))
    print(f"wrote {len(cases)} sweep cases, {len(host_cases)} host cases")
    lozenge(args.ref)


def lozenge(ref: str) -> None:
    """Lozenge vectors from the reference-compiled src/Lozenge code (oracle/_ref/libref_lozenge.so)."""
    lz = C.CDLL(str(ROOT / "oracle/_ref/libref_lozenge.so"))
    P = lambda a: None if a is None else a.ctypes.data_as(C.c_void_p)
    lz.ref_lz_walk.argtypes = [C.c_void_p, C.c_int, C.c_long, C.c_long, C.c_void_p, C.c_long]

    def domain(n, m):
        buf = np.zeros(2 * (2 * n + 9) ** 2, np.int32)
        rows = lz.refh_lz_almost_hex_domain(n, m, P(buf), buf.size)
        return buf[: 2 * rows * rows].copy(), rows

    def extremal(d, rows, which):
        out = np.zeros((rows + 1) ** 2, np.int32)
        getattr(lz, f"refh_lz_{which}_tiling")(P(d), rows, P(out))
        return out

    def walk(t, n, steps, seed, params=None):
        t = t.copy()
        lz.ref_lz_walk(P(t), n, steps, seed, P(params), 0 if params is None else params.shape[0])
        return t

    cases, host = [], []
    for n, m in [(2, 0), (3, 1), (5, 0), (10, 2)]:
        d, rows = domain(n, m)
        tmax, tmin = extremal(d, rows, "max"), extremal(d, rows, "min")
        hf = np.zeros((rows + 1) ** 2, np.int32)
        lz.refh_lz_tiling_to_heightfunc(P(tmax), P(d), rows + 1, P(hf))
        v = np.zeros((rows + 1) ** 2, np.int32)
        lz.refh_lz_domain_to_vertices(P(d), rows, P(v))
        host.append({"n": n, "m": m, "domain": d.tolist(), "max": tmax.tolist(), "min": tmin.tolist(),
                     "hf_max": hf.tolist(), "vertices": v.tolist()})
        for which, start, steps, seed in [("max", tmax, 97, 34893), ("min", tmin, 250, -17)]:
            cases.append({"name": f"lz_walk_hex{n}_{m}_{which}", "kind": "walk", "N": rows + 1, "start": start.tolist(),
                          "steps": steps, "seed": seed, "expected": walk(start, rows + 1, steps, seed).tolist()})
    # The MinimalLozenge example shape (Examples/MinimalLozengeEx.cpp:15-16): AlmostHexDomain(10, 2),
    # MaxTiling start, 1000 steps; a fixed seed replaces its random_device.
    d, rows = domain(10, 2)
    start = extremal(d, rows, "max")
    cases.append({"name": "lz_walk_minimal_lozenge", "kind": "walk", "N": rows + 1, "start": start.tolist(),
                  "steps": 1000, "seed": 2018, "expected": walk(start, rows + 1, 1000, 2018).tolist()})
    # A per-generator parameter table (synthetic, seeded; LoadTinyMT's buffer, one triple per
    # generator of the N x N/3 grid) in place of the missing parameter file.
    d, rows = domain(5, 0)
    start = extremal(d, rows, "min")
    params = np.random.default_rng(20261204).integers(0, 2**32, size=((rows + 1) * ((rows + 1) // 3), 3),
                                                      dtype=np.uint64).astype(np.uint32)
    cases.append({"name": "lz_walk_hex5_0_paramtable", "kind": "walk", "N": rows + 1, "start": start.tolist(),
                  "steps": 180, "seed": 4321, "params": params.tolist(),
                  "expected": walk(start, rows + 1, 180, 4321, params).tolist()})
    # CFTP from the reference's Walk: epochs of Walk(t, steps_k, seed_k) on both chains,
    # seeds from mt19937(driver seed), prepending 2 * steps.back().
    d, rows = domain(3, 0)
    tmax, tmin = extremal(d, rows, "max"), extremal(d, rows, "min")
    drv = np.random.RandomState(777)
    draw = lambda: int(drv.randint(0, 2**32, dtype=np.uint32))
    steps, seeds, attempts = [16], [draw()], 0
    while True:
        attempts += 1
        top, bot = tmax.copy(), tmin.copy()
        for st, sd in zip(steps, seeds):
            top, bot = walk(top, rows + 1, st, sd), walk(bot, rows + 1, st, sd)
        if np.array_equal(top, bot):
            break
        steps.insert(0, steps[-1] * 2)
        seeds.insert(0, draw())
        assert attempts < 40
    cases.append({"name": "lz_cftp_hex3", "kind": "cftp", "N": rows + 1, "tmax": tmax.tolist(), "tmin": tmin.tolist(),
                  "driver_seed": 777, "first_steps": 16, "schedule": 0, "attempts": attempts,
                  "expected": top.tolist()})
    # the q-weighted kernel (qlozengekernel.cl, q = 0.99 as compiled; oracle/_ref/libref_qlozenge.so)
    qlz = C.CDLL(str(ROOT / "oracle/_ref/libref_qlozenge.so"))
    qlz.ref_qlz_walk.argtypes = [C.c_void_p, C.c_int, C.c_long, C.c_long, C.c_void_p, C.c_long]
    qcases = []
    for n, m, steps, seed in [(2, 0, 200, 1), (5, 1, 500, 77), (10, 2, 300, -5)]:
        d, rows = domain(n, m)
        start = extremal(d, rows, "max")
        t = start.copy()
        qlz.ref_qlz_walk(P(t), rows + 1, steps, seed, None, 0)
        qcases.append({"name": f"qlz_walk_hex{n}_{m}", "kind": "walk", "N": rows + 1, "q": 0.99, "start": start.tolist(),
                       "steps": steps, "seed": seed, "expected": t.tolist()})
    (HERE / "lozenge_ref_cases.json").write_text(json.dumps({"generator": "tests/golden/make_golden.py", "cases": cases,
                                                             "host_cases": host, "q_cases": qcases},
                                                            separators=(",", ":")))
    print(f"wrote {len(cases)} lozenge sweep cases, {len(host)} lozenge host cases")
    recttri(ref)


def _read_matrix(path: Path) -> np.ndarray:
    return np.array([int(x) for x in path.read_text().split()], np.int32)


def recttri(ref: str) -> None:
    """Rectangle-triangle vectors from the reference-compiled src/RectTriangle code
    (oracle/_ref/libref_recttri.so); pins the committed fixtures
    Examples/ExampleOuts/RectTriangle/{Max,Min,Slope}Tiling.txt (RectTriangleEx.cpp, N = 5)
    against the reference's maxHex / minHex / slopeHex."""
    rl = C.CDLL(str(ROOT / "oracle/_ref/libref_recttri.so"))
    lz = C.CDLL(str(ROOT / "oracle/_ref/libref_lozenge.so"))
    P = lambda a: None if a is None else a.ctypes.data_as(C.c_void_p)
    rl.ref_rt_walk.argtypes = [C.c_void_p, C.c_int, C.c_long, C.c_long, C.c_void_p, C.c_long]
    rl.refh_rt_hex.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_long]
    rl.refh_rt_from_lozenge.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p]

    def hexagon(n, which):
        buf = np.zeros((2 * n + 9) ** 2, np.int32)
        side = rl.refh_rt_hex(n, which, P(buf), buf.size)
        return buf[: side * side].copy(), side

    def walk(t, n, steps, seed, params=None):
        t = t.copy()
        rl.ref_rt_walk(P(t), n, steps, seed, P(params), 0 if params is None else params.shape[0])
        return t

    fixtures = Path(ref) / "Examples/ExampleOuts/RectTriangle"
    for name, which in (("MaxTiling", 1), ("MinTiling", 0), ("SlopeTiling", 2)):
        assert np.array_equal(_read_matrix(fixtures / f"{name}.txt"), hexagon(5, which)[0]), name
    # the exact bytes SaveMatrix wrote for maxHex(5), the format pin of rt_save_matrix
    format_pin = {"file": "Examples/ExampleOuts/RectTriangle/MaxTiling.txt", "n": 5,
                  "text": (fixtures / "MaxTiling.txt").read_text()}
    host, cases = [], []
    for n in (2, 3, 5, 8, 13):
        (tmax, side), (tmin, _) = hexagon(n, 1), hexagon(n, 0)
        host.append({"n": n, "N": side, "max": tmax.tolist(), "min": tmin.tolist(), "slope": hexagon(n, 2)[0].tolist()})
    for n, which, steps, seed in [(2, 0, 40, 1), (3, 1, 333, 99), (5, 0, 1000, 2018), (5, 1, 517, -5), (8, 0, 300, 77),
                                  (13, 1, 200, 4242)]:
        start, side = hexagon(n, which)
        cases.append({"name": f"rt_walk_hex{n}_{'max' if which else 'min'}_{steps}", "N": side, "start": start.tolist(),
                      "steps": steps, "seed": seed, "expected": walk(start, side, steps, seed).tolist()})
    # a per-generator parameter table (synthetic, seeded), one triple per generator of the
    # N x N/3 grid, in place of the missing parameter file
    start, side = hexagon(5, 0)
    params = np.random.default_rng(20261205).integers(0, 2**32, size=(side * (side // 3), 3),
                                                      dtype=np.uint64).astype(np.uint32)
    cases.append({"name": "rt_walk_hex5_min_paramtable", "N": side, "start": start.tolist(), "steps": 400,
                  "seed": 606, "params": params.tolist(), "expected": walk(start, side, 400, 606, params).tolist()})
    # the reference's own end state of RectTriangleEx (1000 steps from minHex(5), seed not
    # recorded) as a start state
    end = _read_matrix(fixtures / "EndTiling.txt")
    side = int(np.sqrt(end.size))
    cases.append({"name": "rt_walk_example_end_state", "N": side, "start": end.tolist(), "steps": 250, "seed": 31337,
                  "expected": walk(end, side, 250, 31337).tolist()})
    # LozengeToRectTriangle on lozenge extremal tilings of AlmostHexDomain(n, m)
    conv = []
    for n, m in ((3, 0), (4, 1), (6, 2)):
        buf = np.zeros(2 * (2 * n + 9) ** 2, np.int32)
        rows = lz.refh_lz_almost_hex_domain(n, m, P(buf), buf.size)
        d = buf[: 2 * rows * rows].copy()
        for which in ("max", "min"):
            t = np.zeros((rows + 1) ** 2, np.int32)
            getattr(lz, f"refh_lz_{which}_tiling")(P(d), rows, P(t))
            out = np.zeros_like(t)
            rl.refh_rt_from_lozenge(P(t), rows + 1, P(d), rows, P(out))
            conv.append({"n": n, "m": m, "which": which, "domain": d.tolist(), "lozenge": t.tolist(),
                         "expected": out.tolist()})
    (HERE / "recttri_ref_cases.json").write_text(json.dumps(
        {"generator": "tests/golden/make_golden.py", "fixtures_pinned": ["MaxTiling.txt", "MinTiling.txt",
                                                                         "SlopeTiling.txt"],
         "host_cases": host, "cases": cases, "from_lozenge": conv, "format_pin": format_pin}, separators=(",", ":")))
    print(f"wrote {len(cases)} rectangle-triangle sweep cases, {len(host)} host cases, {len(conv)} conversions")
    bibone(ref)


def bibone(ref: str) -> None:
    """Bibone (triangular-lattice dimer) vectors from the reference-compiled src/TriangleDimer
    code (oracle/_ref/libref_tdimer.so: its .cl kernels run by the Walk host loop, and its
    IceCreamCone).  Pins the committed Examples/ExampleOuts/TriangleDimer/DimerStart.txt
    (SaveMatrix of IceCreamCone(6, 0), TriangleDimerEx.cpp:31-34) against the reference's
    IceCreamCone, and records its Domain.txt beside it: SaveMatrix writes floor(sqrt(size))^2
    entries, so the file holds the first 196 of the 10 x 20 entries of TilingToDomain."""
    td = C.CDLL(str(ROOT / "oracle/_ref/libref_tdimer.so"))
    P = lambda a: None if a is None else a.ctypes.data_as(C.c_void_p)
    td.refh_td_icecream.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_long]
    td.ref_td_walk.argtypes = [C.c_void_p, C.c_int, C.c_long, C.c_long, C.c_void_p, C.c_long]

    def cone(n, m):
        buf = np.zeros(4 * (n + 8) ** 2, np.int32)
        side = td.refh_td_icecream(n, m, P(buf), buf.size)
        return buf[: side * side].copy(), side

    def walk(t, n, steps, seed, params=None):
        t = t.copy()
        td.ref_td_walk(P(t), n, steps, seed, P(params), 0 if params is None else params.shape[0])
        return t

    fixtures = Path(ref) / "Examples/ExampleOuts/TriangleDimer"
    start = _read_matrix(fixtures / "DimerStart.txt")
    assert np.array_equal(start, cone(6, 0)[0]), "DimerStart.txt"
    example = {"n": 6, "m": 0, "tiling": start.tolist(), "domain": _read_matrix(fixtures / "Domain.txt").tolist()}
    td.refh_td_tri_flips.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    td.refh_td_bfly_flips.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    td.refh_td_test_butterfly.argtypes = [C.c_int, C.c_void_p, C.c_long]

    def derived(t, side):
        tri, bf = np.zeros((side // 2) * side, np.int32), np.zeros(side * side, np.int32)
        td.refh_td_tri_flips(P(t), side, P(tri))
        td.refh_td_bfly_flips(P(t), side, P(bf))
        return tri.tolist(), bf.tolist()

    host, cases = [], []
    for n, m in [(3, 0), (4, 1), (6, 0), (8, 2), (11, 3), (20, 4)]:
        t, side = cone(n, m)
        tri, bf = derived(t, side)
        host.append({"n": n, "m": m, "N": side, "tiling": t.tolist(), "triangle_flips": tri, "butterfly_flips": bf})
    butterflies = []
    for typ in (0, 1, 2, 3):
        buf = np.zeros(256, np.int32)
        td.refh_td_test_butterfly(typ, P(buf), buf.size)
        tri, bf = derived(buf, 16)
        butterflies.append({"type": typ, "tiling": buf.tolist(), "triangle_flips": tri, "butterfly_flips": bf})
    for n, m, steps, seed in [(4, 1, 1, 5), (4, 1, 50, 1), (7, 0, 400, 77), (8, 2, 1000, -3), (11, 3, 2000, 2018),
                              (20, 4, 1500, 99)]:
        t, side = cone(n, m)
        cases.append({"name": f"td_walk_cone{n}_{m}_{steps}", "N": side, "start": t.tolist(), "steps": steps, "seed": seed,
                      "expected": walk(t, side, steps, seed).tolist()})
    # a per-generator parameter table (synthetic, seeded), one triple per generator of the
    # M x M grid, in place of the missing parameter file
    t, side = cone(7, 0)
    params = np.random.default_rng(20261206).integers(0, 2**32, size=((side // 2) ** 2, 3),
                                                      dtype=np.uint64).astype(np.uint32)
    cases.append({"name": "td_walk_cone7_0_paramtable", "N": side, "start": t.tolist(), "steps": 600, "seed": 515,
                  "params": params.tolist(), "expected": walk(t, side, 600, 515, params).tolist()})
    (HERE / "bibone_ref_cases.json").write_text(json.dumps(
        {"generator": "tests/golden/make_golden.py", "example": example, "host_cases": host, "cases": cases,
         "test_butterflies": butterflies},
        separators=(",", ":")))
    print(f"wrote {len(cases)} bibone sweep cases, {len(host)} host cases")


if __name__ == "__main__":
    main()

"""Pins the MTGP mode's decision logic to the reference's own CUDA kernels.

oracle/Makefile (`make ref`) compiles the rotate kernels of the reference's CUDA build
(src/Domino/dominokernel*.cu, src/Lozenge/lozengekernel.cu,
src/RectTriangle/recttrianglekernel.cu, src/TriangleDimer/triangledimerkernel.cu) as host C++
under oracle/ref_cu_shim.h, and
oracle/ref_cu_driver.cpp runs them over the reference's launch grid with the draws supplied per
thread.  Here they rotate random colour arrays with random draws (threshold neighbourhoods
included), and the oracle's CUDA-path rotations, and the library's MTGP acceptance intervals,
must give the same arrays.  Runs where the reference tree was available to build oracle/_ref."""
import ctypes as C

import numpy as np
import pytest

from tests.oracle_py import REF_DIR

LIB = REF_DIR / "libref_cu.so"
pytestmark = pytest.mark.skipif(not LIB.exists(), reason="oracle/_ref not built here")

# The weights compiled into dominokerneltwoperiodic.cu:7-8 and dominokernelCFTPtwoperiodic.cu:6-7.
REF_A, REF_B = 0.7, 1.0
# The hexagon states recttrianglekernel.cu:45-130 moves between.
RT_STATES = [0x122133, 0x331221, 0x8EBBE8, 0xFC99CF, 0xA7DD7A, 0x47D47A, 0xD22A33, 0xA74D74, 0x33A22D, 0x8EB558,
             0x331EB1, 0x855BE8, 0x1BE133, 0x6699CF, 0xCF1221, 0xFC9966, 0x1221FC]


@pytest.fixture(scope="module")
def ref():
    h = C.CDLL(str(LIB))
    h.ref_cu_domino_rotate.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p]
    h.ref_cu_lozenge_rotate.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    h.ref_cu_recttri_flip.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    return h


def _draws(rng, shape, thresholds):
    """Uniform floats in (0, 1], with a fifth of the entries at or next to the thresholds."""
    d = rng.random(shape, dtype=np.float32)
    d[d == 0] = np.float32(1.0)
    edges = []
    for x in thresholds:
        f = np.float32(x)
        edges += [f, np.nextafter(f, np.float32(0)), np.nextafter(f, np.float32(2))]
    edges += [np.float32(1.0), np.float32(2.0**-32)]
    pick = rng.random(shape) < 0.2
    d[pick] = rng.choice(np.array(edges, np.float32), int(pick.sum()))
    return d


@pytest.mark.parametrize("variant", [0, 1, 2, 3])
def test_domino_cuda_rotations_equal_the_oracle_and_the_mtgp_tables(ref, orc, rt, variant):
    rng = np.random.default_rng(300 + variant)
    table = np.zeros(16, np.uint32)
    assert rt.lib().rt_domino_rule_table(variant, rt.RNG_MODES["mtgp"], REF_A, REF_B, table.ctypes.data) == 0
    f = orc.lib().orc_dm_rotate_cuda_grid
    f.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_double, C.c_double]
    for N in (18, 26, 40, 66):
        H, rows, cols = N // 2, N - 2, N // 2 - 2
        for t in (0, 1):
            colour = rng.choice(np.array([0, 3, 12, 5, 10, 15], np.uint8), size=N * H, p=[.1, .35, .35, .1, .05, .05])
            draws = _draws(rng, (rows, cols), [0.8, 0.5, 0.4, 0.25, 0.75, 0.625, 0.9])
            mine = colour.copy()
            assert ref.ref_cu_domino_rotate(variant, mine.ctypes.data, N, t, draws.ctypes.data) == 0
            theirs = colour.copy()
            f(theirs.ctypes.data, N, t, draws.ctypes.data, variant, REF_A, REF_B)
            assert np.array_equal(mine, theirs), (variant, N, t)
            # the library's MTGP intervals over the draw's bit pattern
            lib_out = colour.copy().reshape(N, H)
            bits = draws.view(np.uint32).astype(np.uint64)
            for i in range(1, N - 1):
                c = (i & 1) | (t << 1)
                lo_up, w_up, lo_dn, w_dn = (int(x) for x in table[4 * c: 4 * c + 4])
                row = lib_out[i, 1:cols + 1]
                u = bits[i - 1]
                up = (row == 3) & (((u - lo_up) % 2**32) < w_up)
                dn = (row == 12) & (((u - lo_dn) % 2**32) < w_dn)
                row[up] = 12
                row[dn] = 3
            assert np.array_equal(lib_out.ravel(), mine), (variant, N, t)
            assert (mine != colour).sum() > 0


def test_lozenge_cuda_rotation_equals_the_oracle(ref, orc):
    rng = np.random.default_rng(77)
    f = orc.lib().orc_lz_rotate_cuda_grid
    f.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    orc.lz_lib()
    for N in (12, 30, 51):
        M = N // 3
        colour = rng.choice(np.array([25, 38, 0, 9, 63], np.uint8), size=N * M, p=[.4, .4, .1, .05, .05])
        draws = _draws(rng, (N, M), [0.4, 0.8])
        mine, theirs = colour.copy(), colour.copy()
        assert ref.ref_cu_lozenge_rotate(mine.ctypes.data, N, draws.ctypes.data) == 0
        f(theirs.ctypes.data, N, draws.ctypes.data)
        assert np.array_equal(mine, theirs), N
        assert (mine != colour).sum() > 0


def test_recttri_cuda_flip_equals_the_oracle(ref, orc):
    rng = np.random.default_rng(91)
    f = orc.rt_lib().orc_rt_flip_grid
    f.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    unit = np.ones(9, np.float64)
    for N in (12, 30, 51):
        M = N // 3
        pool = np.array(RT_STATES + [0, 0x111111, 0x123456], np.int32)
        colour = rng.choice(pool, size=N * M).astype(np.int32)
        draws = _draws(rng, (N, M), [0.9, 0.225, 0.45, 0.675])
        mine, theirs = colour.copy(), colour.copy()
        assert ref.ref_cu_recttri_flip(mine.ctypes.data, N, draws.ctypes.data) == 0
        f(theirs.ctypes.data, N, draws.ctypes.data, unit.ctypes.data)
        assert np.array_equal(mine, theirs), N
        assert (mine != colour).sum() > 0


@pytest.mark.parametrize("move_type", [0, 1, 2])
def test_bibone_cuda_rotations_flip_exactly_the_oracle_class(ref, orc, move_type):
    """RotateLozenges/Triangles/ButterflysKernel flip a site's state (5 <-> 10, 45 <-> 54,
    85 <-> 170) exactly when its draw is below 0.5 and the site is in the oracle's step class
    (in_class of oracle/bibone_oracle.cpp, which the library's td_in_class restates)."""
    ref.ref_cu_td_rotate.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]
    in_class = orc.td_lib().orc_td_in_class
    in_class.argtypes = [C.c_int] * 7
    pair = {0: (5, 10), 1: (45, 54), 2: (85, 170)}[move_type]
    rng = np.random.default_rng(500 + move_type)
    for M in (11, 24, 37):
        for _ in range(4):
            r1, r2, p1, p2 = int(rng.integers(3)), int(rng.integers(2)), int(rng.integers(3)), int(rng.integers(2))
            states = rng.choice(np.array([pair[0], pair[1], 0, 7, 63], np.int32), size=M * M, p=[.4, .4, .1, .05, .05])
            states = states.astype(np.int32)
            draws = _draws(rng, (M, M), [0.5])
            mine = states.copy()
            assert ref.ref_cu_td_rotate(move_type, mine.ctypes.data, M, r1, r2, p1, p2, draws.ctypes.data) == 0
            want = states.copy()
            for a in range(M):
                for b in range(M):
                    k = a * M + b
                    if draws[a, b] < 0.5 and want[k] in pair and in_class(move_type, r1, r2, p1, p2, a, b):
                        want[k] = pair[1] if want[k] == pair[0] else pair[0]
            assert np.array_equal(mine, want), (move_type, M, r1, r2, p1, p2)
            assert (mine != states).sum() > 0

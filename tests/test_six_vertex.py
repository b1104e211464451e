"""Six-vertex model with domain-wall boundary (no reference counterpart; validated from the
mathematics).

CPU: host utilities equal to the oracle's; exhaustive enumeration of the domain-wall height
functions (the alternating sign matrices: 1, 2, 7, 42, 429), the 2-enumeration
sum_ASM 2^(#-1) = 2^(n(n-1)/2) through the vertex weights at a = b = 1, c = sqrt(2), and
chi-square tests of the oracle's CFTP samples against the enumerated Gibbs law.
GPU: walks and CFTP bit-exact with the oracle, chi-square of the library's CFTP samples, and
the refined ASM enumeration (the law of the 1 in the first row of a uniform ASM) at n = 8."""
import math
from fractions import Fraction

import numpy as np
import pytest

ASM_COUNTS = {1: 1, 2: 2, 3: 7, 4: 42, 5: 429}


def vertex_counts(h, n):
    """(#a, #b, #c) of the configuration with height function h ((n+1)^2)."""
    H = np.asarray(h).reshape(n + 1, n + 1)
    nw, ne, sw, se = H[:-1, :-1], H[:-1, 1:], H[1:, :-1], H[1:, 1:]
    c = (ne == sw) & (nw == se)
    a = (ne == sw) & (nw != se)
    b = (nw == se) & (ne != sw)
    assert int((a | b | c).sum()) == n * n
    return int(a.sum()), int(b.sum()), int(c.sum())


def enumerate_dwbc(n, hmin):
    """All height functions reachable from hmin by single-point moves h' +- 1."""
    L = n + 1
    start = np.asarray(hmin, np.int32).reshape(L, L)
    seen = {start.tobytes(): 0}
    states, frontier = [start], [start]
    while frontier:
        nxt = []
        for H in frontier:
            for y in range(1, n):
                for x in range(1, n):
                    nb = (H[y, x - 1], H[y, x + 1], H[y - 1, x], H[y + 1, x])
                    if nb.count(nb[0]) != 4:
                        continue
                    U = H.copy()
                    U[y, x] = nb[0] * 2 - H[y, x]
                    k = U.tobytes()
                    if k not in seen:
                        seen[k] = len(states)
                        states.append(U)
                        nxt.append(U)
        frontier = nxt
    return states, seen


def gibbs(states, n, a, b, c):
    w = np.array([a ** va * b ** vb * c ** vc for va, vb, vc in (vertex_counts(s, n) for s in states)])
    return w / w.sum()


def chi_square_p(counts, probs):
    from scipy.stats import chi2

    exp = probs * counts.sum()
    stat = float(((counts - exp) ** 2 / exp).sum())
    return float(chi2.sf(stat, len(probs) - 1))


def test_host_utilities_match_oracle(rt, orc):
    S = rt.SixVertexTiler
    for abc in [(1, 1, 1), (1, 1, 1.5), (0.7, 1.3, 2.0), (2.0, 0.5, 0.3), (1e-3, 1.0, 1e3)]:
        assert np.array_equal(S.Thresholds(*abc), orc.sv_thresholds(*abc))
    assert S.Thresholds(1, 1, 1.5)[4] == 2 ** 31  # k1 = k2 = 1: P = 1/2
    for n in (1, 2, 5, 16):
        assert np.array_equal(S.MaxHeight(n), orc.sv_dwbc(n, True))
        assert np.array_equal(S.MinHeight(n), orc.sv_dwbc(n, False))
        ident = S.HeightToASM(S.MinHeight(n)).reshape(n, n)
        assert np.array_equal(ident, np.eye(n, dtype=np.int32))
        assert np.array_equal(S.HeightToASM(S.MaxHeight(n)).reshape(n, n), np.eye(n, dtype=np.int32)[::-1])
        assert np.array_equal(S.ASMToHeight(ident), S.MinHeight(n))


def test_enumeration_counts_and_two_enumeration(rt):
    S = rt.SixVertexTiler
    for n, count in ASM_COUNTS.items():
        states, _ = enumerate_dwbc(n, S.MinHeight(n))
        assert len(states) == count
        # every state is an ASM whose height function round-trips
        for st in states[:50]:
            A = S.HeightToASM(st.ravel())
            assert np.array_equal(S.ASMToHeight(A), st.ravel())
        # a = b = 1, c = sqrt 2: Z = 2^(n/2) * 2^(n(n-1)/2)
        Z = sum(math.sqrt(2) ** vertex_counts(s, n)[2] for s in states)
        assert Z == pytest.approx(2 ** (n / 2) * 2 ** (n * (n - 1) / 2), rel=1e-12)


def test_invalid_inputs_rejected_on_host(rt):
    S = rt.SixVertexTiler
    h = S.MinHeight(4)
    h[7] += 2
    with pytest.raises(rt.RTError):
        S.HeightToASM(h)
    bad = np.eye(3, dtype=np.int32)
    bad[0, 0] = 2
    with pytest.raises(rt.RTError):
        S.ASMToHeight(bad)
    with pytest.raises(rt.RTError):
        S.Thresholds(1.0, 0.0, 1.0)


@pytest.mark.parametrize("abc", [(1.0, 1.0, 1.5), (0.8, 1.2, 1.5)])
def test_oracle_cftp_samples_follow_the_gibbs_law(rt, orc, abc):
    n = 4
    S = rt.SixVertexTiler
    states, index = enumerate_dwbc(n, S.MinHeight(n))
    probs = gibbs(states, n, *abc)
    hmax, hmin = orc.sv_dwbc(n, True), orc.sv_dwbc(n, False)
    counts = np.zeros(len(states))
    for seed in range(3000):
        out, att, _ = orc.sv_cftp(hmax, hmin, n, 1000 + seed, 0, 2, 20, *abc)
        assert att > 0
        counts[index[out.reshape(n + 1, n + 1).tobytes()]] += 1
    assert chi_square_p(counts, probs) > 1e-3


@pytest.mark.gpu
@pytest.mark.parametrize("engine", [1, 2])
@pytest.mark.parametrize("abc", [(1.0, 1.0, 1.0), (1.0, 1.0, 1.5), (0.6, 1.7, 0.9), (2.5, 0.4, 1.1)])
def test_walk_matches_oracle(rt, orc, abc, engine):
    S = rt.SixVertexTiler
    for n, sweeps, seed, stream in ((2, 3, 1, 0), (3, 10, 5, 1), (7, 40, -3, 2), (33, 25, 99, 7), (64, 20, 2026, 65535),
                                    (101, 12, 7, 3), (190, 6, 11, 12)):
        for top in (False, True):
            start = S.MaxHeight(n) if top else S.MinHeight(n)
            a = start.copy()
            stats = S(*abc, fast_stream=stream, engine=engine).Walk(a, sweeps, seed)
            b = start.copy()
            orc.sv_walk(b, n, 0, 4 * sweeps, seed, stream, *abc)
            assert np.array_equal(a, b), (n, top, abc)
            assert stats["flip_attempts"] == (n - 1) ** 2 * sweeps
            if n >= 7 and max(abc) / min(abc) < 3:  # strongly a-weighted chains may stay at the maximum
                assert not np.array_equal(a, start)


@pytest.mark.gpu
def test_walk_from_a_non_dwbc_boundary_keeps_its_boundary(rt, orc):
    # a flat boundary (heights 0/1, not domain-wall) on a 40 x 40 grid, started from its
    # minimal height function: the boundary stays fixed and the result equals the oracle's
    S = rt.SixVertexTiler
    n = 40
    H = np.zeros((n + 1, n + 1), np.int32)
    H[0, :] = np.arange(n + 1) % 2
    H[:, 0] = np.arange(n + 1) % 2
    H[-1, :] = (n + np.arange(n + 1)) % 2
    H[:, -1] = (n + np.arange(n + 1)) % 2
    # rebuild a valid interior: the minimal height function for this boundary (Lipschitz)
    B = [(y, x) for y in range(n + 1) for x in range(n + 1) if y in (0, n) or x in (0, n)]
    Hm = np.array([[max(H[by, bx] - abs(by - y) - abs(bx - x) for by, bx in B) for x in range(n + 1)]
                   for y in range(n + 1)], np.int32)
    a = Hm.ravel().copy()
    S(1.0, 1.0, 1.5, fast_stream=4).Walk(a, 60, 12)
    b = Hm.ravel().copy()
    orc.sv_walk(b, n, 0, 240, 12, 4, 1.0, 1.0, 1.5)
    assert np.array_equal(a, b)
    A = a.reshape(n + 1, n + 1)
    assert np.array_equal(A[0], Hm[0]) and np.array_equal(A[:, 0], Hm[:, 0]) and not np.array_equal(A, Hm)


@pytest.mark.gpu
@pytest.mark.parametrize("engine", [1, 2])
@pytest.mark.parametrize("abc", [(1.0, 1.0, 1.5), (0.9, 0.5, 1.0)])
def test_cftp_matches_oracle(rt, orc, abc, engine):
    S = rt.SixVertexTiler
    for n, seed in ((6, 1), (10, 2), (17, 3)):
        hmax, hmin = S.MaxHeight(n), S.MinHeight(n)
        out, stats = S(*abc, fast_stream=9, engine=engine).cftp(hmax, hmin, seed, first_sweeps=4, max_attempts=16)
        ref, att, used = orc.sv_cftp(hmax, hmin, n, seed, 9, 4, 16, *abc)
        assert att == stats["attempts"] and 4 * used == stats["final_steps"]
        assert np.array_equal(out, ref)


def test_cftp_rejects_non_monotone_weights_before_any_device_work(rt):
    S = rt.SixVertexTiler
    with pytest.raises(rt.RTError):
        S(1.0, 1.0, 0.5).cftp(S.MaxHeight(4), S.MinHeight(4), 1)


@pytest.mark.gpu
def test_cftp_samples_follow_the_gibbs_law(rt):
    n, abc = 4, (0.8, 1.2, 1.5)
    S = rt.SixVertexTiler
    states, index = enumerate_dwbc(n, S.MinHeight(n))
    probs = gibbs(states, n, *abc)
    hmax, hmin = S.MaxHeight(n), S.MinHeight(n)
    counts = np.zeros(len(states))
    sampler = S(*abc, fast_stream=1)
    for seed in range(3000):
        out, _ = sampler.cftp(hmax, hmin, 50_000 + seed, first_sweeps=2, max_attempts=20)
        counts[index[out.reshape(n + 1, n + 1).tobytes()]] += 1
    assert chi_square_p(counts, probs) > 1e-3


def refined_asm(n):
    """A(n, k): ASMs of size n with the first row's 1 in column k (Zeilberger's refined
    alternating sign matrix theorem)."""
    prod = Fraction(1)
    for j in range(n - 1):
        prod *= Fraction(math.factorial(3 * j + 1), math.factorial(n + j))
    return [Fraction(math.comb(n + k - 2, k - 1) * math.factorial(2 * n - k - 1), math.factorial(n - k)) * prod
            for k in range(1, n + 1)]


def test_refined_enumeration_formula_matches_enumeration(rt):
    S = rt.SixVertexTiler
    for n in (3, 4, 5):
        states, _ = enumerate_dwbc(n, S.MinHeight(n))
        first = np.zeros(n, int)
        for st in states:
            first[int(np.argmax(S.HeightToASM(st.ravel())[:n]))] += 1
        assert [int(v) for v in refined_asm(n)] == first.tolist()


@pytest.mark.gpu
def test_engines_agree_at_the_benchmark_size(rt):
    # n = 512, a = b = 1, c = 1.5: the cluster-resident and per-sub-sweep engines give the
    # same heights after 300 sweeps, and the result is a valid domain-wall height function
    S = rt.SixVertexTiler
    n = 512
    a, b = S.MaxHeight(n), S.MaxHeight(n)
    sa = S(1.0, 1.0, 1.5, engine=2).Walk(a, 300, 5)
    S(1.0, 1.0, 1.5, engine=1).Walk(b, 300, 5)
    assert np.array_equal(a, b) and not np.array_equal(a, S.MaxHeight(n))
    asm = S.HeightToASM(a).reshape(n, n)
    assert np.array_equal(asm.sum(0), np.ones(n)) and np.array_equal(asm.sum(1), np.ones(n))
    assert sa["flip_attempts"] == 511 * 511 * 300


@pytest.mark.gpu
def test_uniform_asm_first_row_law_at_n8(rt):
    n = 8
    S = rt.SixVertexTiler
    A = refined_asm(n)
    assert sum(A) == 10_850_216  # the number of 8 x 8 alternating sign matrices
    probs = np.array([float(v / sum(A)) for v in A])
    hmax, hmin = S.MaxHeight(n), S.MinHeight(n)
    counts = np.zeros(n)
    sampler = S(1.0, 1.0, 1.0, fast_stream=2)
    for seed in range(1500):
        out, _ = sampler.cftp(hmax, hmin, seed, first_sweeps=8, max_attempts=20)
        counts[int(np.argmax(S.HeightToASM(out)[:n]))] += 1
    assert chi_square_p(counts, probs) > 1e-3

"""Edge densities and the mean height function of exact samples on larger Aztec diamonds,
and lozenge placement frequencies on a larger hexagon, against exactly computed values.

Exact edge-placement probabilities come from the Kasteleyn matrix (tests/test_edge_densities.py:
uniform and two-periodic weights) up to Aztec order 44, and from generalized domino shuffling
(shuffling_edge_probs below, equal to the Kasteleyn values where both hold) beyond.  The height function (TilingToHeightfunc,
DominoTiler.cpp:555-593) changes along a lattice edge u -> w by s (1 - 4 x), where
s = +-1 is the step of the reference's walk (its axis and the colour of u) and x = 1 when a
domino covers the edge (each square has exactly one covered side, so the three free sides'
steps and the covered side's -3 s close up).  The height is therefore linear in the
edge-covering indicators, and its exact mean is the path sum of s (1 - 4 P(e)).  On CPU the
path formula is checked against TilingToHeightfunc on concrete tilings; on the GPU, batched
CFTP samples (8000 per case) are compared with both exact quantities: every edge by its exact
binomial tail (Bonferroni, family-wise level 1e-3), every vertex's mean height within |z| < 5
where the height moves often enough for the normal approximation, and by a bound on the
count of moves elsewhere."""
import os
from collections import deque

import numpy as np
import pytest

from tests.test_edge_densities import kasteleyn_edge_probs

DIRS = ((1, 0), (-1, 0), (0, 1), (0, -1))  # down, up, right, left (the reference's order)


def _walk_order(d):
    """Base vertex and BFS tree of the domain's lattice: (vertex, parent, direction) rows."""
    M = int(np.sqrt(d.size))
    N = M + 1
    F = d.reshape(M, M)

    def face(i, j):
        return 0 <= i < M and 0 <= j < M and F[i, j] == 1

    def touches(i, j, k):  # lattice edge from vertex (i, j) in direction k borders a domain face
        if k == 0:
            return face(i, j - 1) or face(i, j)
        if k == 1:
            return face(i - 1, j - 1) or face(i - 1, j)
        if k == 2:
            return face(i - 1, j) or face(i, j)
        return face(i - 1, j - 1) or face(i, j - 1)

    def in_domain(i, j):
        return any(face(i - a, j - b) for a in (0, 1) for b in (0, 1))

    def boundary(i, j):
        return in_domain(i, j) and not all(face(i - a, j - b) for a in (0, 1) for b in (0, 1))

    base = next((i, j) for i in range(N) for j in range(N) if boundary(i, j))
    seen = {base}
    order = []
    q = deque([base])
    while q:
        i0, j0 = q.popleft()
        for k, (di, dj) in enumerate(DIRS):
            i, j = i0 + di, j0 + dj
            if (i, j) in seen or not (0 <= i < N and 0 <= j < N) or not touches(i0, j0, k):
                continue
            seen.add((i, j))
            order.append(((i, j), (i0, j0), k))
            q.append((i, j))
    return N, base, order


def heights_from_edges(d, cover):
    """Height function from edge-covering values in the [2][N][N] layout of
    rt_domino_edge_indicators (0: the edge below a vertex, 1: the edge to its right), exact
    0/1 for one tiling or probabilities for the mean; NaN outside the domain."""
    N, base, order = _walk_order(d)
    c = np.asarray(cover, np.float64).reshape(2, N, N)
    h = np.full((N, N), np.nan)
    h[base] = 0.0
    for (i, j), (i0, j0), k in order:
        if k == 0:
            x = c[0, i0, j0]
        elif k == 1:
            x = c[0, i, j]
        elif k == 2:
            x = c[1, i0, j0]
        else:
            x = c[1, i, j]
        s = (1 if k >= 2 else -1) * (1 if (i0 + j0) % 2 == 0 else -1)
        h[i, j] = h[i0, j0] + s * (1 - 4 * x)
    return h


def shuffling_edge_probs(d, a, b, dtype=np.float64):
    """Exact placement probabilities of the two-periodic weighted Aztec diamond d (the weights
    of kasteleyn_edge_probs) by generalized domino shuffling (J. Propp, "Generalized
    domino-shuffling", Theoret. Comput. Sci. 303 (2003) 267-301), in the same [2][N][N] layout.

    Cells of the order-n diamond are the lattice points (R, C) inside it with R + C + n odd.
    In the rotated coordinates s = R + C, t = R - C they form an n x n grid, and a cell's four
    edges (the grid segments meeting at its point, each crossed by one domino position) fill a
    2 x 2 block of a 2n x 2n array: up (0, 0), left (0, 1), right (1, 0), down (1, 1), so that
    opposite edges sit diagonally opposite.  Urban renewal at every cell gives each edge its
    opposite's weight over D = w00 w11 + w01 w10; dropping the array's outer rows and columns
    leaves the weights of the order n-1 diamond, whose cells are the other parity of points.
    Probabilities go back up the way the shuffling builds a tiling: a domino of the order
    k-1 tiling slides across its cell to the opposite edge, and the cell's complement (1 minus
    its four order k-1 probabilities, the array padded by zeros) is filled by a pair, up and
    down in the proportion w00 w11 / D, left and right w01 w10 / D.  The complement is not a
    probability (a cell holding two dominoes, which the shuffling removes, counts twice; it
    is negative for two-periodic weights), but the values stay accurate at any order (at order
    256 double and extended precision agree to 1e-14), where the Kasteleyn inverse loses all
    digits beyond order 48."""
    M = int(np.sqrt(d.size))
    F = np.asarray(d).reshape(M, M)
    rows = np.flatnonzero(F.any(axis=1))
    cols = np.flatnonzero(F.any(axis=0))
    n = len(rows) // 2
    r0, c0 = int(rows[0]), int(cols[0])
    i, j = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    R = (2 * i + 2 * j + 2) // 2 + r0  # s = 2i + n + 1, t = 2j - n + 1 in the diamond's frame
    C = (2 * i - 2 * j + 2 * n) // 2 + c0
    ref = np.zeros((M, M), np.int8)
    ref[r0:r0 + 2 * n, c0:c0 + 2 * n] = [[1 if abs(r - n + 0.5) + abs(c - n + 0.5) <= n else 0
                                          for c in range(2 * n)] for r in range(2 * n)]
    assert np.array_equal(F, ref), "not an Aztec diamond"
    W = np.empty((2 * n, 2 * n), dtype)
    h = np.where((C - 1) % 2 == 1, a, b)  # horizontal domino: a when its left face's column is odd
    v = np.where((R - 1) % 2 == 0, a, b)  # vertical domino: a when its top face's row is even
    W[0::2, 0::2] = W[1::2, 1::2] = h
    W[0::2, 1::2] = W[1::2, 0::2] = v
    levels = [W]
    for _ in range(n - 1):
        w00, w01, w10, w11 = W[0::2, 0::2], W[0::2, 1::2], W[1::2, 0::2], W[1::2, 1::2]
        D = w00 * w11 + w01 * w10
        X = np.empty_like(W)
        X[0::2, 0::2], X[1::2, 1::2], X[0::2, 1::2], X[1::2, 0::2] = w11 / D, w00 / D, w10 / D, w01 / D
        W = X[1:-1, 1:-1].copy()
        levels.append(W)
    P = np.zeros((0, 0), dtype)
    for W in reversed(levels):
        Q = np.zeros(W.shape, dtype)
        Q[1:-1, 1:-1] = P
        w00, w01, w10, w11 = W[0::2, 0::2], W[0::2, 1::2], W[1::2, 0::2], W[1::2, 1::2]
        D = w00 * w11 + w01 * w10
        q00, q01, q10, q11 = Q[0::2, 0::2], Q[0::2, 1::2], Q[1::2, 0::2], Q[1::2, 1::2]
        empty = 1 - (q00 + q01 + q10 + q11)
        P = np.empty_like(Q)
        P[0::2, 0::2] = q11 + w00 * w11 / D * empty
        P[1::2, 1::2] = q00 + w00 * w11 / D * empty
        P[0::2, 1::2] = q10 + w01 * w10 / D * empty
        P[1::2, 0::2] = q01 + w01 * w10 / D * empty
    out = np.zeros((2, M + 1, M + 1), dtype)
    out[0, R - 1, C] = P[0::2, 0::2]  # up: horizontal domino on faces (R-1, C-1), (R-1, C)
    out[0, R, C] = P[1::2, 1::2]      # down: faces (R, C-1), (R, C)
    out[1, R, C - 1] = P[0::2, 1::2]  # left: vertical domino on faces (R-1, C-1), (R, C-1)
    out[1, R, C] = P[1::2, 0::2]      # right: faces (R-1, C), (R, C)
    return out.ravel()


def face_cover(d, p):
    """Per face of d, the summed probabilities of its four domino positions (exactly one
    covers it in every tiling)."""
    M = int(np.sqrt(d.size))
    q = np.asarray(p).reshape(2, M + 1, M + 1)
    return q[0, :M, 1:] + q[0, :M, :M] + q[1, 1:, :M] + q[1, :M, :M]


@pytest.mark.parametrize("a,b", [(1.0, 1.0), (1.0, 0.8), (1.0, 0.5), (0.3, 1.0)])
def test_shuffling_probabilities_equal_kasteleyn(rt, a, b):
    from tests.test_edge_densities import kasteleyn_edge_probs

    # The difference at order 24 (a few 1e-11) is the Kasteleyn inverse's rounding, which
    # grows with the order; a misplaced edge or weight would differ by O(1).
    for order in (1, 2, 3, 5, 8, 13, 24):
        d = rt.DominoTiler.AztecDiamond(order)
        assert np.abs(shuffling_edge_probs(d, a, b) - kasteleyn_edge_probs(d, a, b)).max() < 1e-9


@pytest.mark.parametrize("order", [128, 256])
def test_shuffling_probabilities_hold_at_large_orders(rt, order):
    d = rt.DominoTiler.AztecDiamond(order)
    M = int(np.sqrt(d.size))
    F = d.reshape(M, M) == 1
    for a, b in ((1.0, 1.0), (1.0, 0.8)):
        p = shuffling_edge_probs(d, a, b)
        assert np.abs(p - shuffling_edge_probs(d, a, b, np.longdouble)).max() < 1e-12
        assert p.min() >= 0 and p.max() <= 1 + 1e-15
        cover = face_cover(d, p)
        assert np.abs(cover[F] - 1).max() < 1e-12 and not cover[~F].any()
        assert abs(p.sum() - order * (order + 1)) < 1e-9


def test_device_exact_probabilities_reject_bad_arguments(rt):
    lib = rt.lib()
    out = np.zeros(2 * 12 * 12)
    for order, a, b in ((0, 1.0, 1.0), (3, 1.0, 0.0), (3, -1.0, 1.0), (3, float("nan"), 1.0), (3, 1.0, float("inf"))):
        assert lib.rt_domino_aztec_edge_probs(order, a, b, out.ctypes.data, out.size, None) == rt.RT_ERR_INVALID_ARGUMENT
    assert lib.rt_domino_aztec_edge_probs(4, 1.0, 1.0, out.ctypes.data, out.size, None) == rt.RT_ERR_BUFFER_TOO_SMALL


@pytest.mark.gpu
@pytest.mark.parametrize("a,b", [(1.0, 1.0), (1.0, 0.8), (1.0, 0.5), (0.3, 1.0), (2.0, 0.7)])
def test_device_exact_probabilities_equal_the_restatement(rt, a, b):
    """rt_domino_aztec_edge_probs (one launch per level on the device) against
    shuffling_edge_probs, odd and even orders, up to one past the batched kernels' CTA size."""
    for order in (1, 2, 3, 7, 16, 33, 100, 257):
        d = rt.DominoTiler.AztecDiamond(order)
        got = rt.aztec_edge_probs(order, a, b)
        assert got.shape == shuffling_edge_probs(d, a, b).shape
        assert np.abs(got - shuffling_edge_probs(d, a, b)).max() < 1e-12, order


@pytest.mark.gpu
def test_device_exact_probabilities_at_order_2048(rt):
    """Every face of the order-2048 diamond is covered with probability 1, the probabilities
    sum to the domino count, and the uniform ones are symmetric under the diamond's mirror."""
    order = 2048
    d = rt.DominoTiler.AztecDiamond(order)
    M = int(np.sqrt(d.size))
    F = d.reshape(M, M) == 1
    for a, b in ((1.0, 1.0), (1.0, 0.5)):
        p = rt.aztec_edge_probs(order, a, b)
        assert p.min() >= 0 and p.max() <= 1 + 1e-12
        cover = face_cover(d, p)
        assert np.abs(cover[F] - 1).max() < 1e-10 and not cover[~F].any()
        assert abs(p.sum() - order * (order + 1)) < 1e-6 * order
    q = rt.aztec_edge_probs(order, 1.0, 1.0).reshape(2, M + 1, M + 1)
    # the diamond's faces fill columns 2 .. M - 3: the left-right mirror takes a vertical
    # domino in face column C to face column M - 2 - C
    assert np.abs(q[1][:, :M - 1] - q[1][:, M - 2::-1]).max() < 1e-12


@pytest.mark.parametrize("order", [6, 20])
def test_height_path_formula_equals_tiling_to_heightfunc(rt, order):
    D = rt.DominoTiler
    d = D.AztecDiamond(order)
    for t in (D.MaxTiling(d), D.MinTiling(d)):
        n = rt.side_of(t)
        ref = D.TilingToHeightfunc(t, d).reshape(n, n).astype(np.float64)
        got = heights_from_edges(d, rt.edge_indicators(t))
        live = ~np.isnan(got)
        assert live.sum() > 0
        assert np.array_equal(got[live], ref[live])


def test_exact_values_are_exact_at_the_tested_sizes(rt):
    """The exact reference values are double-precision inverses of Kasteleyn matrices, whose
    entries grow exponentially between the frozen regions: at Aztec order 48 the edge
    probabilities already sum to the domino count only within 1e-4, at order 64 within 40.
    The tests therefore stop at order 44 and hexagon side 48, where the sums hold to 1e-5 and
    1e-11 and no probability leaves [0, 1]."""
    from tests.test_edge_densities import kasteleyn_edge_probs

    for order, a, b in ((44, 1.0, 1.0), (44, 1.0, 0.8)):
        p = kasteleyn_edge_probs(rt.DominoTiler.AztecDiamond(order), a, b)
        assert abs(p.sum() - order * (order + 1)) < 1e-4 and p.min() > -1e-9 and p.max() < 1 + 1e-9
    d = rt.LozengeTiler.Hexagon(48)
    P = lozenge_dimer_probs(d)
    assert abs(P.sum() - d.sum() / 2) < 1e-8 and P.min() > -1e-9 and P.max() < 1 + 1e-9


@pytest.mark.gpu
@pytest.mark.parametrize("order,rule,a,b", [(32, "cftp", 1.0, 1.0), (32, "cftp_twoperiodic", 1.0, 0.8),
                                            (44, "cftp", 1.0, 1.0), (44, "cftp_twoperiodic", 1.0, 0.8)])
def test_cftp_edges_and_mean_height_match_exact_values(rt, order, rule, a, b):
    d = rt.DominoTiler.AztecDiamond(order)
    check_domino_cftp_samples(rt, d, order, rule, a, b, 8000, kasteleyn_edge_probs(d, a, b))


@pytest.mark.gpu
@pytest.mark.parametrize("order,samples", [(16, 4000), (24, 2000)])
def test_cftp_at_the_benchmark_weights_matches_exact_values(rt, order, samples):
    """The two-periodic rule at the benchmark's weights (a = 1, b = 0.5), whose coupled chains
    coalesce far more slowly than at b = 0.8, against the shuffling probabilities."""
    d = rt.DominoTiler.AztecDiamond(order)
    check_domino_cftp_samples(rt, d, order, "cftp_twoperiodic", 1.0, 0.5, samples, shuffling_edge_probs(d, 1.0, 0.5))


@pytest.mark.gpu
@pytest.mark.skipif(not os.environ.get("RT_LONG_TESTS"), reason="long test: set RT_LONG_TESTS=1")
def test_cftp_at_the_benchmark_weights_matches_exact_values_at_order_32(rt):
    """As above at order 32 (2000 samples; the coupled chains need 2^20 - 2^22 half-sweeps of
    look-back here, so up to 20 doublings from 64 sweeps)."""
    d = rt.DominoTiler.AztecDiamond(32)
    check_domino_cftp_samples(rt, d, 32, "cftp_twoperiodic", 1.0, 0.5, 2000, shuffling_edge_probs(d, 1.0, 0.5),
                              max_attempts=20)


@pytest.mark.gpu
def test_cftp_edges_and_mean_height_match_exact_values_at_order_128_short(rt):
    """The order-128 check below with 400 uniform samples (about 25 s on one GB300): every
    edge frequency and vertex mean height against the shuffling probabilities."""
    d = rt.DominoTiler.AztecDiamond(128)
    check_domino_cftp_samples(rt, d, 128, "cftp", 1.0, 1.0, 400, shuffling_edge_probs(d, 1.0, 1.0))


@pytest.mark.gpu
@pytest.mark.skipif(not os.environ.get("RT_LONG_TESTS"), reason="long test: set RT_LONG_TESTS=1")
@pytest.mark.parametrize("order,rule,a,b", [(128, "cftp", 1.0, 1.0), (128, "cftp_twoperiodic", 1.0, 0.8)])
def test_cftp_edges_and_mean_height_match_exact_values_at_order_128(rt, order, rule, a, b):
    """2000 exact samples of the order-128 diamond (66 k domino positions) against the
    shuffling probabilities.  The coupled chains coalesce after 131 K - 524 K half-sweeps of
    look-back here, so each case takes minutes of the whole GPU."""
    d = rt.DominoTiler.AztecDiamond(order)
    check_domino_cftp_samples(rt, d, order, rule, a, b, 2000, shuffling_edge_probs(d, a, b))


def check_domino_cftp_samples(rt, d, order, rule, a, b, samples, p, max_attempts=16):
    """Batched CFTP samples of the Aztec diamond d against its exact placement probabilities
    p: every edge frequency, and every vertex's mean height."""
    D = rt.DominoTiler
    tmax, tmin = D.MaxTiling(d), D.MinTiling(d)
    n = rt.side_of(tmax)
    jobs = [{"model": "domino", "tmax": tmax, "tmin": tmin, "seed": 31000 + 100000 * order + k, "stream": k,
             "rule": rule, "a": a, "b": b, "first_steps": 64, "max_attempts": max_attempts} for k in range(samples)]
    outs, attempts, _ = rt.cftp_batch(jobs)
    assert min(attempts) > 0
    counts = np.zeros(2 * n * n, np.uint32)
    hsum = np.zeros((n, n))
    hsq = np.zeros((n, n))
    for o in outs:
        rt.edge_indicators(o, counts)
        h = D.TilingToHeightfunc(o, d).reshape(n, n).astype(np.float64)
        hsum += h
        hsq += h * h
    freq = counts / samples
    live = (p > 1e-12) & (p < 1 - 1e-12)
    # Exact two-sided binomial tails (edges near the frozen regions have tiny or near-one
    # probabilities, where the normal approximation understates the tails), Bonferroni over
    # the edges at a family-wise level of 1e-3.
    from scipy.stats import binom

    k, q = counts[live].astype(np.int64), p[live]
    tail = 2 * np.minimum(binom.cdf(k, samples, q), binom.sf(k - 1, samples, q))
    assert tail.min() * live.sum() > 1e-3, (float(tail.min()), int(live.sum()))
    assert np.array_equal(freq[~live], np.round(p[~live]))
    mean_exact = heights_from_edges(d, p)
    mean = hsum / samples
    var = hsq / samples - mean * mean
    known = ~np.isnan(mean_exact)
    # A vertex's height moves in steps of 4; where it moves in at least about 20 samples
    # (var >= 16 * 20 / samples) the sample mean is close to normal and its z is tested.
    # Vertices that rarely or never move (the boundary, the frozen regions) are bounded by
    # the count of moves instead: fewer than ~25 expected, so a count off by more than 50
    # (a mean off by 200 / samples) has a Poisson probability far below 1e-9.
    often = known & (var * samples / 16 >= 20)
    zh = (mean[often] - mean_exact[often]) / np.sqrt(var[often] / samples)
    assert often.sum() > min(1000, known.sum() // 4)
    assert np.abs(zh).max() < 5.0, float(np.abs(zh).max())
    rare = known & ~often
    assert np.abs(mean[rare] - mean_exact[rare]).max() < 200 / samples


def lozenge_dimer_probs(d):
    """Exact lozenge placement probabilities of a simply connected region of triangles
    (M x 2M, even columns one colour class, odd the other), in the layout [3][N][N] of the
    vertex bits 1, 2 and 8 (LozengeTiler.cpp:514-556: bit 1 of vertex (i, j) pairs triangles
    (i-1, 2j-1) and (i-1, 2j), bit 2 pairs (i-1, 2j) and (i-1, 2j+1), bit 8 pairs (i-1, 2j+1)
    and (i, 2j)).  Every inner face of the triangles' adjacency graph is a hexagon, so the
    plain adjacency matrix is a Kasteleyn matrix and P(b, w) = K^-1(w, b)."""
    M = int(np.sqrt(d.size // 2))
    F = np.asarray(d).reshape(M, 2 * M)
    N = M + 1
    black = [(r, c) for r in range(M) for c in range(0, 2 * M, 2) if F[r, c] == 1]
    white = [(r, c) for r in range(M) for c in range(1, 2 * M, 2) if F[r, c] == 1]
    bi = {t: k for k, t in enumerate(black)}
    wi = {t: k for k, t in enumerate(white)}
    K = np.zeros((len(black), len(white)))
    edges = []
    for (r, c) in black:
        for w, kind, vi, vj in (((r, c - 1), 0, r + 1, c // 2), ((r, c + 1), 1, r + 1, c // 2), ((r - 1, c + 1), 2, r, c // 2)):
            if w in wi:
                K[bi[(r, c)], wi[w]] = 1.0
                edges.append(((r, c), w, kind, vi, vj))
    Kinv = np.linalg.inv(K)
    P = np.zeros((3, N, N))
    for b, w, kind, vi, vj in edges:
        P[kind, vi, vj] = Kinv[wi[w], bi[b]]
    return P


def lozenge_indicators(t):
    n = int(np.sqrt(t.size))
    x = np.asarray(t).reshape(n, n)
    return np.stack([(x & 1) != 0, (x & 2) != 0, (x & 8) != 0]).astype(np.float64)


@pytest.mark.parametrize("side", [3, 8])
def test_lozenge_dimers_of_extremal_tilings_cover_each_triangle_once(rt, side):
    L = rt.LozengeTiler
    d = L.Hexagon(side)
    M = int(np.sqrt(d.size // 2))
    F = d.reshape(M, 2 * M)
    p = lozenge_dimer_probs(d)
    assert p.sum() == pytest.approx(F.sum() / 2, rel=1e-9)  # lozenges per tiling
    for t in (L.MaxTiling(d), L.MinTiling(d)):
        cover = np.zeros((M, 2 * M), int)
        x = lozenge_indicators(t)
        for kind in range(3):
            for i, j in np.argwhere(x[kind] > 0):
                pair = {0: ((i - 1, 2 * j - 1), (i - 1, 2 * j)), 1: ((i - 1, 2 * j), (i - 1, 2 * j + 1)),
                        2: ((i - 1, 2 * j + 1), (i, 2 * j))}[kind]
                for r, c in pair:
                    cover[r, c] += 1
                assert p[kind, i, j] > 0  # every placed lozenge is an edge of the exact model
        assert np.array_equal(cover, F)


@pytest.mark.gpu
@pytest.mark.parametrize("side", [12, 32, 48])
def test_lozenge_cftp_edge_frequencies_match_exact_probabilities(rt, side):
    from scipy.stats import binom

    L = rt.LozengeTiler
    samples = 8000
    d = L.Hexagon(side)
    tmax, tmin = L.MaxTiling(d), L.MinTiling(d)
    jobs = [{"model": "lozenge", "tmax": tmax, "tmin": tmin, "seed": 52000 + 100000 * side + k, "stream": k,
             "first_steps": 64, "max_attempts": 20} for k in range(samples)]
    outs, attempts, _ = rt.cftp_batch(jobs)
    assert min(attempts) > 0
    p = lozenge_dimer_probs(d)
    counts = np.zeros_like(p)
    for o in outs:
        counts += lozenge_indicators(o)
    live = (p > 1e-12) & (p < 1 - 1e-12)
    k, q = counts[live].astype(np.int64), p[live]
    tail = 2 * np.minimum(binom.cdf(k, samples, q), binom.sf(k - 1, samples, q))
    assert live.sum() > 300
    assert tail.min() * live.sum() > 1e-3, (float(tail.min()), int(live.sum()))
    assert np.array_equal(counts[~live] / samples, np.round(p[~live]))

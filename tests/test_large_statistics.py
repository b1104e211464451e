"""Edge densities and the mean height function of exact samples on larger Aztec diamonds,
and lozenge placement frequencies on a larger hexagon, against exactly computed values.

Exact edge-placement probabilities come from the Kasteleyn matrix (tests/test_edge_densities.py:
uniform and two-periodic weights).  The height function (TilingToHeightfunc,
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
    D = rt.DominoTiler
    samples = 8000
    d = D.AztecDiamond(order)
    tmax, tmin = D.MaxTiling(d), D.MinTiling(d)
    n = rt.side_of(tmax)
    jobs = [{"model": "domino", "tmax": tmax, "tmin": tmin, "seed": 31000 + 100000 * order + k, "stream": k,
             "rule": rule, "a": a, "b": b, "first_steps": 64, "max_attempts": 16} for k in range(samples)]
    outs, attempts, _ = rt.cftp_batch(jobs)
    assert min(attempts) > 0
    p = kasteleyn_edge_probs(d, a, b)
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
    assert often.sum() > 1000
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

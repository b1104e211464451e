"""Edge-placement statistics of domino tilings against exactly computed values.

Exact placement probabilities come from the Kasteleyn matrix of the domain's faces
(horizontal adjacencies weight w, vertical ones i w; P(domino) = |K(b, w) K^-1(w, b)|, Kenyon
1997).  The two-periodic chain of the reference (dominokernelCFTPtwoperiodic.cl:72-101,
acceptance wFin / wInit) is reversible for the product of per-domino weights: a horizontal
domino weighs a when its left face is in an odd column and b otherwise, a vertical domino a
when its top face is in an even row and b otherwise.  CPU: that model and the Kasteleyn
probabilities equal the edge marginals of the chain's own stationary law on every tiling of
small Aztec diamonds.  GPU: edge frequencies of batched CFTP samples at order 10 match the
exact values within binomial z-scores, and the device-side accumulator equals host counting."""
import numpy as np
import pytest

from tests.test_cftp_exactness import enumerate_tilings, stationary


def kasteleyn_edge_probs(d: np.ndarray, a: float, b: float) -> np.ndarray:
    """Placement probabilities in the counter layout of rt_domino_edge_indicators
    ([2][N][N], N = M + 1 for the M x M face array d)."""
    M = int(np.sqrt(d.size))
    N = M + 1
    F = d.reshape(M, M)
    faces = [tuple(f) for f in np.argwhere(F == 1)]
    black = [f for f in faces if (f[0] + f[1]) % 2 == 0]
    white = [f for f in faces if (f[0] + f[1]) % 2 == 1]
    bi = {f: k for k, f in enumerate(black)}
    wi = {f: k for k, f in enumerate(white)}
    K = np.zeros((len(black), len(white)), complex)
    edges = []
    for (r, c) in black:
        for dr, dc in ((0, 1), (0, -1), (1, 0), (-1, 0)):
            f2 = (r + dr, c + dc)
            if f2 not in wi:
                continue
            if dr == 0:
                left = min(c, c + dc)
                K[bi[(r, c)], wi[f2]] = a if left % 2 == 1 else b
                edges.append(((r, c), f2, 0, r, left + 1))
            else:
                top = min(r, r + dr)
                K[bi[(r, c)], wi[f2]] = 1j * (a if top % 2 == 0 else b)
                edges.append(((r, c), f2, 1, top + 1, c))
    Kinv = np.linalg.inv(K)
    P = np.zeros((2, N, N))
    for fb, fw, kind, i, j in edges:
        P[kind, i, j] = abs(K[bi[fb], wi[fw]] * Kinv[wi[fw], bi[fb]])
    return P.ravel()


def kasteleyn_edge_probs_sparse(d: np.ndarray, a: float, b: float, block: int = 2048) -> np.ndarray:
    """The same probabilities for large domains: the Kasteleyn matrix has four entries per
    row, so a sparse LU factorisation solved block by block against unit columns gives the
    entries of K^-1 at the edges without forming the dense inverse."""
    from scipy.sparse import csc_matrix
    from scipy.sparse.linalg import splu

    M = int(np.sqrt(d.size))
    N = M + 1
    F = d.reshape(M, M)
    faces = [tuple(f) for f in np.argwhere(F == 1)]
    black = [f for f in faces if (f[0] + f[1]) % 2 == 0]
    white = [f for f in faces if (f[0] + f[1]) % 2 == 1]
    bi = {f: k for k, f in enumerate(black)}
    wi = {f: k for k, f in enumerate(white)}
    rows, cols, vals, edges = [], [], [], []
    for (r, c) in black:
        for dr, dc in ((0, 1), (0, -1), (1, 0), (-1, 0)):
            f2 = (r + dr, c + dc)
            if f2 not in wi:
                continue
            if dr == 0:
                left = min(c, c + dc)
                v = a if left % 2 == 1 else b
                edges.append((bi[(r, c)], wi[f2], v, 0, r, left + 1))
            else:
                top = min(r, r + dr)
                v = 1j * (a if top % 2 == 0 else b)
                edges.append((bi[(r, c)], wi[f2], v, 1, top + 1, c))
            rows.append(bi[(r, c)])
            cols.append(wi[f2])
            vals.append(v)
    n = len(black)
    lu = splu(csc_matrix((np.array(vals, complex), (rows, cols)), shape=(n, n)))
    # K^-1(w, b) = column b of K^-1 at row w: solve K X = E_b for blocks of unit columns b.
    by_b = {}
    for e in edges:
        by_b.setdefault(e[0], []).append(e)
    P = np.zeros((2, N, N))
    for b0 in range(0, n, block):
        b1 = min(n, b0 + block)
        E = np.zeros((n, b1 - b0), complex)
        E[np.arange(b0, b1), np.arange(b1 - b0)] = 1.0
        X = lu.solve(E)
        for bb in range(b0, b1):
            for _, w, v, kind, i, j in by_b.get(bb, ()):
                P[kind, i, j] = abs(v * X[w, bb - b0])
    return P.ravel()


@pytest.mark.parametrize("order,a,b", [(6, 1.0, 1.0), (9, 1.0, 0.8), (12, 0.7, 1.0)])
def test_sparse_kasteleyn_equals_dense(rt, order, a, b):
    d = rt.DominoTiler.AztecDiamond(order)
    assert np.allclose(kasteleyn_edge_probs_sparse(d, a, b, block=37), kasteleyn_edge_probs(d, a, b), atol=1e-10)


@pytest.mark.parametrize("order,a,b", [(3, 1.0, 1.0), (3, 1.0, 0.5), (4, 0.6, 1.0), (4, 1.0, 0.3)])
def test_kasteleyn_equals_the_chains_stationary_edge_marginals(rt, order, a, b):
    d, n, tilings, seen = enumerate_tilings(rt, order)
    rule = 1 if a == b == 1.0 else 3
    pi = stationary(rt, tilings, seen, n, rule, 1, a, b, colour_mix=False)
    marg = np.zeros(2 * n * n)
    for p, T in zip(pi, tilings):
        marg += p * rt.edge_indicators(T.ravel()).astype(float)
    exact = kasteleyn_edge_probs(d, a, b)
    assert exact.sum() == pytest.approx(order * (order + 1), rel=1e-9)  # dominoes per tiling
    assert np.abs(marg - exact).max() < 1e-6


def test_host_edge_indicators_count_each_domino_once(rt):
    D = rt.DominoTiler
    for order in (1, 5, 12):
        d = D.AztecDiamond(order)
        for t in (D.MaxTiling(d), D.MinTiling(d)):
            assert int(rt.edge_indicators(t).sum()) == order * (order + 1)


@pytest.mark.gpu
@pytest.mark.parametrize("rule,a,b", [("cftp", 1.0, 1.0), ("cftp_twoperiodic", 1.0, 0.8)])
def test_cftp_edge_frequencies_match_exact_probabilities(rt, rule, a, b):
    D = rt.DominoTiler
    order, samples = 10, 4000
    d = D.AztecDiamond(order)
    tmax, tmin = D.MaxTiling(d), D.MinTiling(d)
    jobs = [{"model": "domino", "tmax": tmax, "tmin": tmin, "seed": 9000 + k, "stream": k, "rule": rule, "a": a,
             "b": b, "first_steps": 16, "max_attempts": 16} for k in range(samples)]
    outs, attempts, _ = rt.cftp_batch(jobs)
    assert min(attempts) > 0
    counts = np.zeros(2 * int(np.sqrt(tmax.size)) ** 2, np.uint32)
    for o in outs:
        rt.edge_indicators(o, counts)
    exact = kasteleyn_edge_probs(d, a, b)
    freq = counts / samples
    live = (exact > 1e-12) & (exact < 1 - 1e-12)
    z = (freq[live] - exact[live]) / np.sqrt(exact[live] * (1 - exact[live]) / samples)
    assert np.abs(z).max() < 5.0, float(np.abs(z).max())
    assert np.array_equal(freq[~live], np.round(exact[~live]))


@pytest.mark.gpu
def test_device_accumulator_equals_host_counting(rt):
    torch = pytest.importorskip("torch")
    D = rt.DominoTiler
    d = D.AztecDiamond(40)
    tmax = D.MaxTiling(d)
    n = int(np.sqrt(tmax.size))
    tiler = rt.DominoTiler(rule="cftp", rng="fast", fast_stream=1)
    s = rt.DominoSampler(n, 1, tiler)
    s.load(0, tmax)
    counts = torch.zeros(2 * n * n, dtype=torch.int32, device="cuda")
    host = np.zeros(2 * n * n, np.uint32)
    for k in range(20):
        s.run_fast(77, 64 * k, 64)
        s.accumulate_edges(0, counts.data_ptr())
        t = s.store(0)
        rt.edge_indicators(t, host)
    s.sync()
    torch.cuda.synchronize()
    assert np.array_equal(counts.cpu().numpy().astype(np.uint32), host)
    s.close()

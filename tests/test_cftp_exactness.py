"""CFTP returns exact samples: chi-square tests against exhaustive enumeration.

Every domino tiling of a small Aztec diamond is enumerated by walking the flip graph from
the maximal tiling (it is connected for simply connected regions, Thurston 1990).  The exact
distribution CFTP must return is the stationary distribution of the chain the kernels run:
built here as the transition matrix of one black half-sweep and one white half-sweep over
all tilings, with each site's acceptance probability taken from the rule table the kernels
use (interval width / 2^23 for TinyMT draws, / 2^32 for fast draws; the table itself is
checked against the reference's decisions for every draw in test_host_api.py).  Samples from
independent CFTP runs are then binned and tested with Pearson's chi-square.
"""
import itertools

import numpy as np
import pytest

from tests.test_domino_gpu import _is_valid_tiling

scipy_stats = pytest.importorskip("scipy.stats")


def _flip(T: np.ndarray, i: int, j: int) -> np.ndarray:
    """Rotates the 2x2 block around vertex (i, j): state 3 <-> 12 and the four neighbours'
    shared edge bits."""
    U = T.copy()
    U[i, j] ^= 15
    U[i - 1, j] ^= 2
    U[i + 1, j] ^= 1
    U[i, j - 1] ^= 8
    U[i, j + 1] ^= 4
    return U


def enumerate_tilings(rt, order: int):
    D = rt.DominoTiler
    d = D.AztecDiamond(order)
    t0 = D.MaxTiling(d)
    n = int(np.sqrt(t0.size))
    start = t0.reshape(n, n)
    seen = {start.tobytes(): 0}
    tilings = [start]
    frontier = [start]
    while frontier:
        nxt = []
        for T in frontier:
            ii, jj = np.nonzero((T == 3) | (T == 12))
            for i, j in zip(ii, jj):
                U = _flip(T, i, j)
                k = U.tobytes()
                if k not in seen:
                    seen[k] = len(tilings)
                    tilings.append(U)
                    nxt.append(U)
        frontier = nxt
    return d, n, tilings, seen


def stationary(rt, tilings, seen, n: int, rule: int, rng_mode: int, a: float, b: float, colour_mix: bool):
    table = np.zeros(16, np.uint32)
    assert rt.lib().rt_domino_rule_table(rule, rng_mode, a, b, table.ctypes.data) == 0
    scale = float(2**23 if rng_mode == 0 else 2**32)
    S = len(tilings)

    def half_sweep_matrix(colour: int) -> np.ndarray:
        M = np.zeros((S, S))
        for x, T in enumerate(tilings):
            ii, jj = np.nonzero(((T == 3) | (T == 12)) & ((np.add.outer(np.arange(n), np.arange(n)) % 2 == 0) == (colour == 1)))
            probs = []
            for i, j in zip(ii, jj):
                c = (i & 1) | (colour << 1)  # colour-array row i is the tiling row
                lo_up, w_up, lo_dn, w_dn = table[4 * c: 4 * c + 4]
                p = (w_up if T[i, j] == 3 else w_dn) / scale
                probs.append(p)
            for subset in itertools.product((0, 1), repeat=len(probs)):
                U = T
                p = 1.0
                for (i, j), s, q in zip(zip(ii, jj), subset, probs):
                    if s:
                        U = _flip(U, i, j)
                        p *= q
                    else:
                        p *= 1.0 - q
                M[x, seen[U.tobytes()]] += p
        return M

    Mb, Mw = half_sweep_matrix(1), half_sweep_matrix(0)
    P = 0.5 * (Mb + Mw) if colour_mix else Mb @ Mw
    w, v = np.linalg.eig(P.T)
    pi = np.real(v[:, np.argmin(np.abs(w - 1))])
    return pi / pi.sum()


def chi_square_p(counts: np.ndarray, pi: np.ndarray) -> float:
    exp = counts.sum() * pi
    order = np.argsort(exp)
    # merge the smallest expected bins until each holds >= 5
    obs_m, exp_m, acc_o, acc_e = [], [], 0.0, 0.0
    for k in order:
        acc_o += counts[k]
        acc_e += exp[k]
        if acc_e >= 5:
            obs_m.append(acc_o)
            exp_m.append(acc_e)
            acc_o = acc_e = 0.0
    if acc_e > 0:
        obs_m[-1] += acc_o
        exp_m[-1] += acc_e
    obs_m, exp_m = np.array(obs_m), np.array(exp_m)
    stat = float(((obs_m - exp_m) ** 2 / exp_m).sum())
    return float(scipy_stats.chi2.sf(stat, len(obs_m) - 1))


@pytest.mark.gpu
@pytest.mark.parametrize("rng,rule,a,b,order,samples", [
    ("fast", "cftp", 1.0, 1.0, 3, 3000),
    ("fast", "cftp_twoperiodic", 1.0, 0.5, 3, 3000),
    ("fast", "cftp_twoperiodic", 0.6, 1.0, 4, 6000),
    ("tinymt", "cftp_twoperiodic", 1.0, 0.5, 3, 2000),
])
def test_cftp_samples_pass_chi_square_against_enumeration(rt, rng, rule, a, b, order, samples):
    d, n, tilings, seen = enumerate_tilings(rt, order)
    assert len(tilings) == 2 ** (order * (order + 1) // 2)  # Aztec diamond tiling count
    rules = {"cftp": 1, "cftp_twoperiodic": 3}
    pi = stationary(rt, tilings, seen, n, rules[rule], 0 if rng == "tinymt" else 1, a, b, colour_mix=(rng == "tinymt"))
    D = rt.DominoTiler
    tmax, tmin = D.MaxTiling(d), D.MinTiling(d)
    counts = np.zeros(len(tilings))
    for k in range(samples):
        if rng == "fast":
            tiler = rt.DominoTiler(rule=rule, rng="fast", a=a, b=b, fast_stream=k & 0xFFFF)
            out, _ = tiler.cftp(tmax, tmin, driver_seed=1000 + k, first_steps=4, max_attempts=20)
        else:
            tiler = rt.DominoTiler(rule=rule, rng="tinymt", a=a, b=b)
            out, _ = tiler.cftp(tmax, tmin, driver_seed=1000 + k, first_steps=16, schedule=1, max_attempts=20)
        counts[seen[out.reshape(n, n).tobytes()]] += 1
    assert _is_valid_tiling(rt, out, d)
    p = chi_square_p(counts, pi)
    assert p > 1e-3, (p, counts[:10], (samples * pi)[:10])


def test_enumeration_counts_and_stationary_is_uniform_for_uniform_weights(rt):
    """CPU check of the test machinery: Aztec counts 2^(n(n+1)/2) and a uniform stationary law
    for the unweighted monotone rule."""
    for order in (1, 2, 3):
        d, n, tilings, seen = enumerate_tilings(rt, order)
        assert len(tilings) == 2 ** (order * (order + 1) // 2)
    pi = stationary(rt, tilings, seen, n, 1, 1, 1.0, 1.0, colour_mix=False)
    assert np.allclose(pi, 1.0 / len(tilings), atol=1e-9)

"""Batched CFTP (rt_cftp_batch): every instance of a mixed batch equals the single-instance
fast-mode CFTP with the same seed and stream, and batched samples pass the chi-square test
against the enumerated stationary law."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _jobs(rt, count, seed0=0):
    D, L = rt.DominoTiler, rt.LozengeTiler
    rng = np.random.default_rng(20261203)
    jobs = []
    cache = {}
    for k in range(count):
        if k % 2 == 0:
            order = int(rng.integers(2, 12))
            key = ("d", order)
            if key not in cache:
                d = D.AztecDiamond(order)
                cache[key] = (D.MaxTiling(d), D.MinTiling(d))
            tmax, tmin = cache[key]
            weighted = k % 4 == 0
            jobs.append({"model": "domino", "tmax": tmax, "tmin": tmin, "seed": seed0 + k, "stream": k,
                         "rule": "cftp_twoperiodic" if weighted else "cftp", "a": 1.0,
                         "b": float(rng.uniform(0.3, 1.0)) if weighted else 1.0, "first_steps": 8})
        else:
            side = int(rng.integers(2, 7))
            key = ("l", side)
            if key not in cache:
                d = L.Hexagon(side)
                cache[key] = (L.MaxTiling(d), L.MinTiling(d))
            tmax, tmin = cache[key]
            jobs.append({"model": "lozenge", "tmax": tmax, "tmin": tmin, "seed": seed0 + k, "stream": k, "first_steps": 8})
    return jobs


def test_batch_equals_single_instance_cftp(rt):
    jobs = _jobs(rt, 48)
    outs, attempts, stats = rt.cftp_batch(jobs)
    assert stats["instances"] == 48 and stats["coalesced"] == 48
    for job, out, att in zip(jobs, outs, attempts):
        if job["model"] == "domino":
            tiler = rt.DominoTiler(rule=job["rule"], rng="fast", a=job["a"], b=job["b"], fast_stream=job["stream"])
        else:
            tiler = rt.LozengeTiler(rng="fast", fast_stream=job["stream"])
        ref, st = tiler.cftp(job["tmax"], job["tmin"], job["seed"], first_steps=8, schedule=1, max_attempts=20)
        assert att == st["attempts"] and np.array_equal(out, ref), job["model"]


def test_batched_domino_samples_pass_chi_square(rt):
    from tests.test_cftp_exactness import chi_square_p, enumerate_tilings, stationary

    d, n, tilings, seen = enumerate_tilings(rt, 3)
    pi = stationary(rt, tilings, seen, n, 3, 1, 1.0, 0.5, colour_mix=False)
    D = rt.DominoTiler
    tmax, tmin = D.MaxTiling(d), D.MinTiling(d)
    jobs = [{"model": "domino", "tmax": tmax, "tmin": tmin, "seed": 77, "stream": k, "rule": "cftp_twoperiodic",
             "a": 1.0, "b": 0.5, "first_steps": 4} for k in range(8000)]
    outs, attempts, stats = rt.cftp_batch(jobs)
    assert stats["coalesced"] == len(jobs)
    counts = np.zeros(len(tilings))
    for out in outs:
        counts[seen[out.reshape(n, n).tobytes()]] += 1
    assert chi_square_p(counts, pi) > 1e-3


def test_batch_rejects_bad_instances(rt):
    D = rt.DominoTiler
    d = D.AztecDiamond(3)
    tmax, tmin = D.MaxTiling(d), D.MinTiling(d)
    with pytest.raises(rt.RTError):
        rt.cftp_batch([{"model": "domino", "tmax": tmax, "tmin": tmin, "seed": 1, "stream": 1, "rule": "plain"}])
    with pytest.raises(rt.RTError):
        rt.cftp_batch([{"model": "domino", "tmax": tmax, "tmin": tmin, "seed": 1, "stream": 70000}])

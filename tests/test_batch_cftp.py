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


def _plain(rt, job):
    """The single-instance entry point called directly, so that a run that did not coalesce
    still returns its sample and attempt count."""
    import ctypes as C

    if job["model"] == "domino":
        tiler = rt.DominoTiler(rule=job["rule"], rng="fast", a=job["a"], b=job["b"], fast_stream=job["stream"])
        fn = rt.lib().rt_domino_cftp
    else:
        tiler = rt.LozengeTiler(rng="fast", fast_stream=job["stream"])
        fn = rt.lib().rt_lozenge_cftp
    a, b = np.ascontiguousarray(job["tmax"], np.int32), np.ascontiguousarray(job["tmin"], np.int32)
    out = np.zeros_like(a)
    st = rt.CftpStats()
    o = tiler.opts()
    status = fn(rt._ptr(a), rt._ptr(b), rt.side_of(a), int(job["seed"]), int(job["first_steps"]), 1,
                int(job.get("max_attempts", 20)), C.byref(o), rt._ptr(out), C.byref(st))
    return status, out, st.attempts


def test_oversized_instances_run_on_the_single_instance_path(rt):
    """Instances whose two chains exceed one CTA's shared memory (an order-168 Aztec diamond,
    a side-170 hexagon) run through the single-instance entry points inside the batch; every
    instance of the mixed batch still equals its single-instance result, coalesced or not."""
    D, L = rt.DominoTiler, rt.LozengeTiler
    jobs = _jobs(rt, 6)
    d = D.AztecDiamond(168)
    jobs.append({"model": "domino", "tmax": D.MaxTiling(d), "tmin": D.MinTiling(d), "seed": 9, "stream": 7,
                 "rule": "cftp", "a": 1.0, "b": 1.0, "first_steps": 1 << 18, "max_attempts": 2})
    h = L.Hexagon(170)
    jobs.append({"model": "lozenge", "tmax": L.MaxTiling(h), "tmin": L.MinTiling(h), "seed": 10, "stream": 8,
                 "first_steps": 64, "max_attempts": 1})
    outs, attempts, stats = rt.cftp_batch(jobs)
    assert stats["instances"] == 8
    assert attempts[-1] == -1  # 64 sweeps do not coalesce a side-170 hexagon
    assert stats["coalesced"] == 8 - sum(a < 0 for a in attempts)
    for job, out, att in zip(jobs, outs, attempts):
        status, ref, ref_att = _plain(rt, job)
        assert status in (rt.RT_OK, rt.RT_ERR_NOT_COALESCED)
        assert abs(att) == ref_att and (att > 0) == (status == rt.RT_OK), job["model"]
        assert np.array_equal(out, ref), (job["model"], rt.side_of(job["tmax"]))

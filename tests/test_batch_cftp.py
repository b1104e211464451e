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


def _smem_limit():
    import torch

    return torch.cuda.get_device_properties(0).shared_memory_per_block_optin - 1024


def _placement(rt, job, limit):
    """Where rt_cftp_batch runs an instance: 1 (one CTA), the cluster size (2..16), or 0 (the
    single-instance path), from the shared memory its chains need."""
    n = rt.side_of(job["tmax"])
    ncol = 2 if job["model"] == "domino" else 3
    pitch = ((n // ncol) + 15) // 16 * 16
    if 2 * ncol * n * pitch <= limit:
        return 1
    rows = n - 2 if job["model"] == "domino" else n
    for c in range(2, 17):
        if 2 * ncol * ((rows + c - 1) // c + 2) * pitch <= limit:
            return c
    return 0


def test_oversized_instances_run_in_clusters(rt):
    """Instances whose two chains exceed one CTA's shared memory (an order-168 Aztec diamond,
    a side-170 hexagon) run on thread-block clusters inside the batch; every instance of the
    mixed batch still equals its single-instance result, coalesced or not."""
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
    assert [_placement(rt, j, _smem_limit()) for j in jobs[-2:]] == [2, 2]
    assert stats["cluster_instances"] == 2 and stats["single_instances"] == 0
    assert attempts[-1] == -1  # 64 sweeps do not coalesce a side-170 hexagon
    assert stats["coalesced"] == 8 - sum(a < 0 for a in attempts)
    for job, out, att in zip(jobs, outs, attempts):
        status, ref, ref_att = _plain(rt, job)
        assert status in (rt.RT_OK, rt.RT_ERR_NOT_COALESCED)
        assert abs(att) == ref_att and (att > 0) == (status == rt.RT_OK), job["model"]
        assert np.array_equal(out, ref), (job["model"], rt.side_of(job["tmax"]))


def test_cluster_sizes_up_to_sixteen_ctas_and_the_single_instance_path(rt):
    """Aztec diamonds of orders 240-700 and hexagons of sides 300-640 beside small instances:
    clusters of 2 to 16 CTAs (non-power-of-two sizes included), and an order-700 diamond that
    no 16-CTA cluster holds, which runs on the single-instance path.  Short look-backs (the
    samples need not coalesce): every output and attempt count equals the single-instance
    entry point's."""
    D, L = rt.DominoTiler, rt.LozengeTiler
    jobs = _jobs(rt, 4, seed0=500)
    for k, (order, rule, b) in enumerate(((240, "cftp_twoperiodic", 0.7), (400, "cftp", 1.0), (520, "cftp", 1.0),
                                          (640, "cftp_twoperiodic", 0.9), (700, "cftp", 1.0))):
        d = D.AztecDiamond(order)
        jobs.append({"model": "domino", "tmax": D.MaxTiling(d), "tmin": D.MinTiling(d), "seed": 40 + k,
                     "stream": 900 + k, "rule": rule, "a": 1.0, "b": b, "first_steps": 3, "max_attempts": 3})
    for k, side in enumerate((300, 440, 640)):
        h = L.Hexagon(side)
        jobs.append({"model": "lozenge", "tmax": L.MaxTiling(h), "tmin": L.MinTiling(h), "seed": 70 + k,
                     "stream": 950 + k, "first_steps": 2, "max_attempts": 3})
    where = [_placement(rt, j, _smem_limit()) for j in jobs]
    assert where[4:] == [where[4], where[5], where[6], where[7], 0, where[9], where[10], where[11]]
    assert all(2 <= c <= 16 for c in where[4:8] + where[9:])
    assert len(set(where[4:8] + where[9:])) >= 4 and max(where) >= 15
    outs, attempts, stats = rt.cftp_batch(jobs)
    assert stats["cluster_instances"] == 7 and stats["single_instances"] == 1, (stats, where)
    for job, out, att in zip(jobs, outs, attempts):
        status, ref, ref_att = _plain(rt, job)
        assert status in (rt.RT_OK, rt.RT_ERR_NOT_COALESCED)
        assert abs(att) == ref_att and (att > 0) == (status == rt.RT_OK), job["model"]
        assert np.array_equal(out, ref), (job["model"], rt.side_of(job["tmax"]))

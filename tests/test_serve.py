"""Continuous-batching server: results are the same alone and in the mix (and equal the
batch path), requests arriving in waves after the kernel went idle are still served, and
admission refuses requests over the budget or without a free slot."""
import time

import numpy as np
import pytest

from tests.test_batch_cftp import _jobs

pytestmark = pytest.mark.gpu


def test_server_results_equal_batch_and_alone(rt):
    jobs = _jobs(rt, 40, seed0=300)
    ref, ref_att, _ = rt.cftp_batch(jobs)
    srv = rt.Server(slots=64, max_side=80, idle_seconds=0.05)
    try:
        # all at once (in the mix)
        tickets = [srv.submit(j) for j in jobs]
        for t, r, a in zip(tickets, ref, ref_att):
            out, att, _ = srv.wait(t)
            assert att == a and np.array_equal(out, r)
        # one at a time, with pauses long enough for the kernel to go idle and be relaunched
        for k in (0, 7, 13):
            time.sleep(0.2)
            t = srv.submit(jobs[k])
            out, att, _ = srv.wait(t)
            assert att == ref_att[k] and np.array_equal(out, ref[k])
        # waves: submit while earlier requests are still running
        pending = []
        for wave in range(4):
            pending += [(srv.submit(jobs[k]), k) for k in range(wave * 10, wave * 10 + 10)]
            time.sleep(0.01)
        for t, k in pending:
            out, att, _ = srv.wait(t)
            assert np.array_equal(out, ref[k])
    finally:
        srv.close()


def test_server_admission(rt):
    jobs = _jobs(rt, 6, seed0=900)
    srv = rt.Server(slots=2, max_side=80, idle_seconds=0.05)
    try:
        t0 = srv.submit(jobs[0])
        t1 = srv.submit(jobs[1])
        with pytest.raises(rt.RTError) as e:
            srv.submit(jobs[2])  # both slots taken until collected
        assert e.value.status == rt.RT_ERR_BUSY
        srv.wait(t0)
        srv.wait(t1)
        srv.wait(srv.submit(jobs[2]))
    finally:
        srv.close()
    tiny = rt.Server(slots=8, max_side=80, memory_budget_bytes=1000, idle_seconds=0.05)
    try:
        with pytest.raises(rt.RTError) as e:
            tiny.submit(jobs[0])
        assert e.value.status == rt.RT_ERR_BUSY
    finally:
        tiny.close()


def _mid_jobs(rt):
    """Two mid-size requests (an Aztec diamond of order 60, tiling side 126, 2-periodic b=0.9,
    and a hexagon of side 30) at the look-back the serving benchmark uses."""
    D, L = rt.DominoTiler, rt.LozengeTiler
    d = D.AztecDiamond(60)
    h = L.Hexagon(30)
    return [{"model": "domino", "tmax": D.MaxTiling(d), "tmin": D.MinTiling(d), "seed": 6060, "stream": 60,
             "rule": "cftp_twoperiodic", "a": 1.0, "b": 0.9, "first_steps": 16, "max_attempts": 14},
            {"model": "lozenge", "tmax": L.MaxTiling(h), "tmin": L.MinTiling(h), "seed": 3030, "stream": 30,
             "first_steps": 16, "max_attempts": 14}]


def test_server_mid_size_requests_alone_and_in_the_mix(rt):
    mid = _mid_jobs(rt)
    small = _jobs(rt, 30, seed0=1200)
    ref, ref_att, _ = rt.cftp_batch(mid)
    assert all(a > 0 for a in ref_att)
    # the plain one-instance entry points give the same samples
    dm = rt.DominoTiler(rule="cftp_twoperiodic", rng="fast", a=1.0, b=0.9, fast_stream=60)
    out, _ = dm.cftp(mid[0]["tmax"], mid[0]["tmin"], 6060, first_steps=16, schedule=1, max_attempts=14)
    assert np.array_equal(out, ref[0])
    lz = rt.LozengeTiler(rng="fast", fast_stream=30)
    out, _ = lz.cftp(mid[1]["tmax"], mid[1]["tmin"], 3030, first_steps=16, schedule=1, max_attempts=14)
    assert np.array_equal(out, ref[1])
    srv = rt.Server(slots=128, max_side=134, idle_seconds=0.05)
    try:
        for k, job in enumerate(mid):  # alone
            out, att, _ = srv.wait(srv.submit(job))
            assert att == ref_att[k] and np.array_equal(out, ref[k])
        # in a mix with small requests arriving before, between and after them
        tickets = [srv.submit(j) for j in small[:10]]
        tickets.append(srv.submit(mid[0]))
        tickets += [srv.submit(j) for j in small[10:20]]
        tickets.append(srv.submit(mid[1]))
        tickets += [srv.submit(j) for j in small[20:]]
        got = [srv.wait(t) for t in tickets]
        assert np.array_equal(got[10][0], ref[0]) and got[10][1] == ref_att[0]
        assert np.array_equal(got[21][0], ref[1]) and got[21][1] == ref_att[1]
        small_ref, _, _ = rt.cftp_batch(small)
        for g, r in zip(got[:10] + got[11:21] + got[22:], small_ref):
            assert np.array_equal(g[0], r)
    finally:
        srv.close()

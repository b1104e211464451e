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

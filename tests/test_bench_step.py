"""The benchmark's own step, checked against the oracle at full size.

bench.py times one step of the headline workload (weighted Aztec diamond of order 1024,
a = 1, b = 0.5, rule cftp_twoperiodic, coupled max/min chains, one epoch of 2048
half-sweeps) through DominoSampler: copy_chain -> seed -> run.  These tests run exactly that
path (bench.headline_sampler / bench.headline_step) and compare both swept chains bit for
bit with the oracle's restatement of the reference's epoch (DominoTiler.cpp:125-231), and
pin the digest bench.py checks its first timed step against.
"""
import json
import os
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = json.loads((ROOT / "tests/golden/bench_check.json").read_text())


def test_bench_check_digest_is_the_golden_one():
    import bench

    assert int(bench.timed_seeds(0, 1)[0]) == GOLDEN["seed"]
    assert bench.BENCH_CHECK_SHA256 == GOLDEN["sha256"]


@pytest.mark.gpu
@pytest.mark.parametrize("engine", [0, 2, 4])
def test_bench_step_tinymt_equals_oracle(rt, orc, engine):
    import torch

    import bench
    from tests.golden.make_bench_check import oracle_step

    tiler = rt.DominoTiler(rule="cftp_twoperiodic", rng="tinymt", a=bench.WEIGHT_A, b=bench.WEIGHT_B, engine=engine)
    stream = torch.cuda.Stream()
    s, tmax, tmin, _ = bench.headline_sampler(rt, tiler, stream.cuda_stream)
    assert s.engine_info()["engine"] in ((2, 4) if engine == 0 else (engine,)), "the bench step runs resident"
    # A first step on other seeds, as the bench's warm-up does, then the checked one.
    bench.headline_step(rt, s, int(bench.warmup_seeds(0, 1)[0]), "tinymt")
    bench.headline_step(rt, s, GOLDEN["seed"], "tinymt")
    top, bottom = s.store(1), s.store(0)
    s.close()
    seed, otop, obottom = oracle_step(orc, os.cpu_count() or 1)
    assert seed == GOLDEN["seed"]
    assert np.array_equal(top, otop), "top chain differs from the oracle"
    assert np.array_equal(bottom, obottom), "bottom chain differs from the oracle"
    assert bench.chains_sha256(top, bottom) == GOLDEN["sha256"]


@pytest.mark.gpu
def test_bench_step_fast_equals_oracle(rt, orc):
    import torch

    import bench

    tiler = rt.DominoTiler(rule="cftp_twoperiodic", rng="fast", a=bench.WEIGHT_A, b=bench.WEIGHT_B)
    stream = torch.cuda.Stream()
    s, tmax, tmin, _ = bench.headline_sampler(rt, tiler, stream.cuda_stream)
    assert s.engine_info()["engine"] == 2
    seed = GOLDEN["seed"]
    bench.headline_step(rt, s, seed, "fast")
    top, bottom = s.store(1), s.store(0)
    s.close()
    n = int(np.sqrt(tmax.size))
    for got, start in ((top, tmax), (bottom, tmin)):
        want = start.copy()
        orc.walk_fast(want, n, -bench.HALF_SWEEPS, bench.HALF_SWEEPS, seed, 0, rule=3, a=bench.WEIGHT_A,
                      b=bench.WEIGHT_B, threads=os.cpu_count() or 1)
        assert np.array_equal(got, want)

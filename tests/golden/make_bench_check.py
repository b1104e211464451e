"""Writes tests/golden/bench_check.json: the oracle's result of the benchmark's first timed
step on rank 0 in TinyMT mode, as a digest bench.py checks its own first step against.

The step (bench.py headline_step): the weighted Aztec diamond of order 1024 (a = 1, b = 0.5,
rule cftp_twoperiodic), the bottom chain reset to the minimal tiling and the top chain to
the maximal one, then one epoch of 2048 half-sweeps seeded with the first draw of
mt19937(1): generator k seeded seed + k, colours from mt19937(seed) - the reference's
Walk(t, steps[], seeds[]) epoch (src/Domino/DominoTiler.cpp:125-231), which the oracle
restates (oracle/domino_oracle.cpp).  Digest: sha256 of the top chain's int32 tiling followed
by the bottom chain's.

    python tests/golden/make_bench_check.py [--threads N]
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))


def oracle_step(orc, threads: int):
    import bench

    _, tmax, tmin, _ = bench.headline_domain_oracle(orc)
    n = int(round(tmax.size ** 0.5))
    seed = int(bench.timed_seeds(0, 1)[0])
    top, bottom = tmax.copy(), tmin.copy()
    for t in (top, bottom):
        orc.walk_epochs_tinymt(t, n, [bench.HALF_SWEEPS], [seed], rule=3, a=bench.WEIGHT_A, b=bench.WEIGHT_B,
                               threads=threads)
    return seed, top, bottom


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    args = ap.parse_args()
    import bench
    from tests import oracle_py as orc

    t0 = time.perf_counter()
    seed, top, bottom = oracle_step(orc, args.threads)
    out = {"workload": f"aztec{bench.ORDER}_twoperiodic_a1.0_b0.5, {bench.HALF_SWEEPS} TinyMT half-sweeps, "
                       "top chain from the maximal tiling then bottom chain from the minimal one",
           "seed": seed, "sha256": bench.chains_sha256(top, bottom),
           "oracle_seconds": round(time.perf_counter() - t0, 1), "threads": args.threads}
    (HERE / "bench_check.json").write_text(json.dumps(out, indent=1) + "\n")
    print(json.dumps(out))


if __name__ == "__main__":
    main()

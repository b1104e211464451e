"""Benchmark: flip attempts/s of coupled-from-the-past domino chains on one GB300.

Workload: the weighted Aztec diamond of order 1024 (tiling side N = 2054) with 2x2-periodic
weights a = 1.0, b = 0.5 (fp32 values), the monotone two-periodic CFTP rule, coupled max and
min chains on one shared random stream.  One step is one CFTP attempt at the first look-back
of 2^10 sweeps: both chains reset to the extremal tilings, 2048 half-sweeps, then the device
XOR-popcount coalescence test.  In TinyMT mode (the default) each step is an epoch of the
reference's CFTP driver (generators seeded from the epoch seed, colours from mt19937 of it).

`value` times steps on chains resident in HBM; `e2e` times the same attempt through the C ABI
(rt_domino_cftp) from pinned host buffers, copies included.  The CPU baseline and the
`--impl reference` arm run the reference's sweep logic (the oracle's restatement of its
OpenCL kernels) on all host threads over a bounded sample of the same attempt.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

ORDER = 1024
WEIGHT_A, WEIGHT_B = 1.0, 0.5
HALF_SWEEPS = 2048  # look-back of 2^10 sweeps
DRIVER_SEED = 1
METRIC = "flip attempts/sec/GPU (coupled CFTP chains, weighted Aztec diamond n=1024)"
L2_FLUSH_BYTES = 256 << 20


def _peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def _interior_by_colour(v: np.ndarray) -> tuple[int, int]:
    """Interior vertices (value 1 of DomainToVertices) of each colour: (white, black)."""
    n = int(np.sqrt(v.size))
    ii, jj = np.divmod(np.arange(v.size), n)
    inter = v == 1
    black = int(np.count_nonzero(inter & ((ii + jj) % 2 == 0)))
    return int(np.count_nonzero(inter)) - black, black  # (white, black)


def _attempts(colours: np.ndarray, interior: tuple[int, int], chains: int = 2) -> int:
    nb = int(np.count_nonzero(colours))
    return chains * (nb * interior[1] + (colours.size - nb) * interior[0])


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()

    def summary(self):
        if not self.proc or not self.path:
            return None
        rows = []
        for line in Path(self.path).read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                rows.append(f)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, name in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": float(rows[0][2]) if rows[0][2].replace(".", "").isdigit() else None,
                "samples": len(rows), "reasons": sorted(reasons)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, 0, None
    import torch
    import torch.distributed as dist

    rank, local = int(os.environ["RANK"]), int(os.environ.get("LOCAL_RANK", "0"))
    backend = "nccl" if torch.cuda.is_available() else "gloo"
    if backend == "nccl":
        torch.cuda.set_device(local)
    dist.init_process_group(backend)
    return rank, ws, local, dist


def _max_over_ranks(x: float, dist, device) -> float:
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _sum_over_ranks(x: float, dist, device) -> float:
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def cpu_leg(orc, tmax, tmin, interior, steps_per_sample: int, samples: int, threads: int):
    """Oracle (the reference's sweep logic restated) on `threads` host threads: `samples`
    coupled attempts of `steps_per_sample` TinyMT steps each; returns attempts/s per sample.
    Uses the oracle alone (its own mt19937), so no library of this repository is loaded."""
    n = int(np.sqrt(tmax.size))
    rates = []
    drv = orc.mt19937(DRIVER_SEED, samples)
    for k in range(samples):
        driver = int(drv[k]) ^ 0x5EED
        epoch_seed = int(orc.mt19937(driver, 1)[0])  # the driver's first draw seeds the epoch
        cols = (orc.mt19937(epoch_seed, steps_per_sample) % 2).astype(np.uint8)
        t0 = time.perf_counter()
        # One attempt (max_attempts=1) at a look-back of steps_per_sample: the same work
        # pattern as a GPU step, shortened.
        orc.cftp_tinymt(tmax, tmin, n, driver, steps_per_sample, 0, 1, rule=3, a=WEIGHT_A,
                        b=WEIGHT_B, threads=threads)
        dt = time.perf_counter() - t0
        rates.append(_attempts(cols, interior) / dt)
    return rates


def headline_domain_oracle(orc):
    """The headline workload's domain, extremal tilings and interior counts from the oracle."""
    d = orc.aztec_rectangle(ORDER)
    rc1, tmax = orc.max_tiling(d)
    rc2, tmin = orc.min_tiling(d)
    assert rc1 == 0 and rc2 == 0
    return d, tmax, tmin, _interior_by_colour(orc.domain_to_vertices(d))


# Batched form (config 4's shape): 8192 instances, half Aztec diamonds and half hexagons,
# half of the diamonds 2-periodic.  The config's full size ranges (orders up to 512, sides up
# to 256) and its b down to 0.3 would take hours for any implementation of the reference's
# chain: the coalescence look-back grows like the order squared and, at b <= 0.6, by 8-16x per
# doubling of the order.  The sizes are therefore truncated to orders U[16, 64] and sides
# U[8, 32], b to U[0.8, 1.0], and the look-back capped at BATCH_ATTEMPTS doublings from
# BATCH_FIRST sweeps (2 x 16 x 2^13 half-sweeps for dominoes).
BATCH_INSTANCES = 8192
BATCH_ORDERS = (16, 64)   # Aztec diamond orders, uniform
BATCH_SIDES = (8, 32)     # hexagon sides, uniform
BATCH_B = (0.8, 1.0)      # 2-periodic b of the weighted half (a = 1)
BATCH_FIRST, BATCH_ATTEMPTS = 16, 14
PLAIN_SAMPLES = 64        # instances drawn across the mix for the one-at-a-time baseline


def _batch_job(rt, cache, rng, k: int, log_sizes: bool = False) -> dict:
    """Instance k of the mix: even k an Aztec diamond (every other one 2-periodic), odd k a
    hexagon; sizes uniform (log-uniform for the served stream) in the ranges above."""
    D, L = rt.DominoTiler, rt.LozengeTiler

    def draw(lo, hi):
        if log_sizes:
            return int(np.exp(rng.uniform(np.log(lo), np.log(hi + 1))))
        return int(rng.integers(lo, hi + 1))

    if k % 2 == 0:
        order = draw(*BATCH_ORDERS)
        if ("d", order) not in cache:
            d = D.AztecDiamond(order)
            cache[("d", order)] = (D.MaxTiling(d), D.MinTiling(d))
        tmax, tmin = cache[("d", order)]
        weighted = (k // 2) % 2 == 1
        return {"model": "domino", "tmax": tmax, "tmin": tmin, "seed": k, "stream": k & 0xFFFF,
                "rule": "cftp_twoperiodic" if weighted else "cftp", "a": 1.0,
                "b": float(rng.uniform(*BATCH_B)) if weighted else 1.0, "first_steps": BATCH_FIRST,
                "max_attempts": BATCH_ATTEMPTS}
    side = draw(*BATCH_SIDES)
    if ("l", side) not in cache:
        d = L.Hexagon(side)
        cache[("l", side)] = (L.MaxTiling(d), L.MinTiling(d))
    tmax, tmin = cache[("l", side)]
    return {"model": "lozenge", "tmax": tmax, "tmin": tmin, "seed": k, "stream": k & 0xFFFF,
            "first_steps": BATCH_FIRST, "max_attempts": BATCH_ATTEMPTS}


def _plain_cftp(rt, job):
    """The one-at-a-time path: rt_domino_cftp / rt_lozenge_cftp on one instance, fast mode."""
    tiler = (rt.DominoTiler(rule=job["rule"], rng="fast", a=job["a"], b=job["b"], fast_stream=job["stream"])
             if job["model"] == "domino" else rt.LozengeTiler(rng="fast", fast_stream=job["stream"]))
    try:
        out, _ = tiler.cftp(job["tmax"], job["tmin"], job["seed"], first_steps=job["first_steps"], schedule=1,
                            max_attempts=job["max_attempts"])
        return out
    except rt.RTError as e:
        if e.status != rt.RT_ERR_NOT_COALESCED:
            raise
        return None


def batched_leg(rt, instances: int = BATCH_INSTANCES) -> dict:
    """Batched fast-mode CFTP (rt_cftp_batch) on the mix above, against the same kind of
    instances run one at a time through the plain entry points (PLAIN_SAMPLES instances drawn
    across the mix).  Samples/s count coalesced instances; every batched sample equals the
    plain result of its instance (tests/test_batch_cftp.py)."""
    rng = np.random.default_rng(20261203)
    cache = {}
    jobs = [_batch_job(rt, cache, rng, k) for k in range(instances)]
    rt.cftp_batch(jobs[:64])  # warm-up
    t0 = time.perf_counter()
    outs, attempts, stats = rt.cftp_batch(jobs)
    wall = time.perf_counter() - t0
    pick = np.random.default_rng(7).choice(len(jobs), size=min(PLAIN_SAMPLES, len(jobs)), replace=False)
    lat, same = [], 0
    for k in pick:
        t1 = time.perf_counter()
        out = _plain_cftp(rt, jobs[k])
        lat.append(time.perf_counter() - t1)
        same += out is not None and attempts[k] > 0 and np.array_equal(out, outs[k])
    lat = np.array(lat)
    plain_rate = 1.0 / lat.mean()
    return {"workload": f"{instances} CFTP instances (config 4's count and mix, sizes truncated): Aztec orders "
                        f"U{list(BATCH_ORDERS)} and hexagon sides U{list(BATCH_SIDES)}, half of the diamonds 2-periodic "
                        f"(a=1, b~U{list(BATCH_B)}), seeds and streams k, look-back {BATCH_FIRST} sweeps doubling, at "
                        f"most {BATCH_ATTEMPTS} attempts",
            "samples_per_s": stats["coalesced"] / wall, "coalesced": stats["coalesced"], "kernel_s": stats["seconds"],
            "wall_s": wall, "ctas": stats["ctas"],
            "plain_samples_per_s": plain_rate, "plain_sampled_instances": len(pick),
            "plain_equal_to_batched": int(same),
            "plain_latency_p50_s": float(np.percentile(lat, 50)), "plain_latency_p99_s": float(np.percentile(lat, 99)),
            "batched_over_plain": (stats["coalesced"] / wall) / plain_rate,
            "api": "rt_cftp_batch vs rt_domino_cftp / rt_lozenge_cftp, fast RNG mode, identical samples"}


SERVE_RATES = (2000.0, 8000.0, 32000.0)  # offered Poisson arrival rates, per second
SERVE_SECONDS = 3.0                       # per rate
SERVE_SLOTS = 16384                       # ring slots: requests admitted and not yet collected
SERVE_POLL_WINDOW = 4096                  # oldest outstanding requests polled per client loop


def serving_leg(rt) -> dict:
    """Continuous-batching server under Poisson request streams at increasing offered rates
    (SERVE_RATES, SERVE_SECONDS each): requests alternate domino / lozenge, sizes log-uniform
    in the batched leg's ranges, weights as there.  Latency = completion time - arrival time;
    samples/s = completions / (time until the last completes).  A request that finds every
    slot holding an uncollected one is refused (RT_ERR_BUSY) and counted as rejected.  Where
    the achieved rate stops following the offered one the server is saturated: that rate is
    its capacity."""
    rng = np.random.default_rng(20261203)
    cache = {}
    srv = rt.Server(slots=SERVE_SLOTS, max_side=max(2 * BATCH_ORDERS[1] + 6, 3 * ((2 * BATCH_SIDES[1] + 9) // 3 + 1)),
                    memory_budget_bytes=120 << 30, idle_seconds=0.5)
    levels = []
    try:
        srv.wait(srv.submit(_batch_job(rt, cache, rng, 0, True)))  # warm-up
        base = 1
        for rate in SERVE_RATES:
            arrivals = np.cumsum(rng.exponential(1.0 / rate, size=int(rate * SERVE_SECONDS * 1.2) + 16))
            arrivals = arrivals[arrivals < SERVE_SECONDS]
            reqs = [_batch_job(rt, cache, rng, base + k, True) for k in range(len(arrivals))]
            base += len(reqs)
            lat, rejected = [], 0
            tickets = [0] * len(reqs)
            outstanding = []  # submitted, not yet collected, oldest first
            submit_s = 0.0
            t0 = time.perf_counter()
            k = 0
            while k < len(reqs) or outstanding:
                now = time.perf_counter() - t0
                while k < len(reqs) and arrivals[k] <= now:
                    ts = time.perf_counter()
                    try:
                        tickets[k] = srv.submit(reqs[k])
                        outstanding.append(k)
                    except rt.RTError as e:  # admission refused: every slot holds an uncollected request
                        if e.status != rt.RT_ERR_BUSY:
                            raise
                        rejected += 1
                    submit_s += time.perf_counter() - ts
                    k += 1
                # collect the finished ones among the oldest SERVE_POLL_WINDOW outstanding requests
                keep = []
                for q in outstanding[:SERVE_POLL_WINDOW]:
                    if srv.poll(tickets[q]):
                        srv.wait(tickets[q])
                        lat.append(time.perf_counter() - t0 - arrivals[q])
                    else:
                        keep.append(q)
                outstanding = keep + outstanding[SERVE_POLL_WINDOW:]
            wall = time.perf_counter() - t0
            lat = np.array(lat)
            levels.append({"offered_per_s": rate, "requests": len(reqs), "served": int(len(lat)), "rejected": rejected,
                           "achieved_per_s": len(lat) / wall, "seconds": wall, "drain_s": wall - SERVE_SECONDS,
                           "latency_p50_s": float(np.percentile(lat, 50)), "latency_p99_s": float(np.percentile(lat, 99)),
                           "client_submit_us": 1e6 * submit_s / max(1, len(reqs))})
    finally:
        srv.close()
    capacity = max(x["achieved_per_s"] for x in levels)
    # saturated: admissions refused, or the median request waiting more than a second
    saturated = [x["offered_per_s"] for x in levels if x["rejected"] > 0 or x["latency_p50_s"] > 1.0]
    return {"workload": f"Poisson arrivals at {', '.join(f'{r:.0f}' for r in SERVE_RATES)}/s, {SERVE_SECONDS:.0f} s each: "
                        f"Aztec orders log-U{list(BATCH_ORDERS)} (half 2-periodic, b~U{list(BATCH_B)}) and hexagon "
                        f"sides log-U{list(BATCH_SIDES)}; config 5's 60 s at log-U[16,512] truncated as the batched leg",
            "levels": levels, "capacity_samples_per_s": capacity,
            "saturated_at_offered_per_s": saturated[0] if saturated else None,
            "samples_per_s": levels[0]["achieved_per_s"], "latency_p50_s": levels[0]["latency_p50_s"],
            "latency_p99_s": levels[0]["latency_p99_s"],
            "api": "rt_server_submit / rt_server_poll / rt_server_wait (continuous batching)"}


MID_ORDER, MID_INSTANCES, MID_SWEEPS = 200, 152, 1024  # thread-block-cluster leg
MID_PLAIN = 4  # of its instances also run one at a time


def mid_batch_leg(rt) -> dict:
    """Instances too large for one CTA (Aztec diamonds of order 200, N = 402), each held by a
    thread-block cluster inside rt_cftp_batch: MID_INSTANCES uniform instances with a fixed
    look-back of MID_SWEEPS sweeps (one attempt each, coalesced or not), against MID_PLAIN of
    them run one at a time through rt_domino_cftp on the whole GPU.  Both in fast mode; the
    samples are identical (checked here)."""
    import ctypes as C

    D = rt.DominoTiler
    d = D.AztecDiamond(MID_ORDER)
    tmax, tmin = D.MaxTiling(d), D.MinTiling(d)
    n = rt.side_of(tmax)
    jobs = [{"model": "domino", "tmax": tmax, "tmin": tmin, "seed": 7000 + k, "stream": k, "rule": "cftp", "a": 1.0,
             "b": 1.0, "first_steps": MID_SWEEPS, "max_attempts": 1} for k in range(MID_INSTANCES)]
    rt.cftp_batch(jobs[:2])  # warm-up
    t0 = time.perf_counter()
    outs, attempts, stats = rt.cftp_batch(jobs)
    wall = time.perf_counter() - t0
    half_sweeps = 2 * MID_SWEEPS
    plain_s, plain_dev, same, flips = [], [], 0, 0
    for k in range(MID_PLAIN):
        job = jobs[k]
        tiler = rt.DominoTiler(rule="cftp", rng="fast", fast_stream=job["stream"])
        a_, b_ = np.ascontiguousarray(tmax, np.int32), np.ascontiguousarray(tmin, np.int32)
        out = np.zeros_like(a_)
        st = rt.CftpStats()
        o = tiler.opts()
        t1 = time.perf_counter()
        status = rt.lib().rt_domino_cftp(rt._ptr(a_), rt._ptr(b_), n, int(job["seed"]), MID_SWEEPS, 1, 1, C.byref(o),
                                         rt._ptr(out), C.byref(st))
        plain_s.append(time.perf_counter() - t1)
        if status not in (rt.RT_OK, rt.RT_ERR_NOT_COALESCED):
            raise rt.RTError(status, rt.lib().rt_last_error().decode())
        same += np.array_equal(out, outs[k])
        plain_dev.append(st.seconds)
        flips = st.flip_attempts  # both chains, every half-sweep of the attempt
    per_instance_half_sweep_us = 1e6 * stats["seconds"] / (MID_INSTANCES * half_sweeps)
    plain_us = 1e6 * statistics.median(plain_dev) / half_sweeps
    out = {"workload": f"{MID_INSTANCES} uniform Aztec diamonds of order {MID_ORDER} (N = {n}), one CFTP attempt of "
                       f"{MID_SWEEPS} sweeps each, fast mode",
           "cluster_instances": stats["cluster_instances"], "ctas": stats["ctas"], "kernel_s": stats["seconds"],
           "wall_s": wall, "us_per_instance_half_sweep": per_instance_half_sweep_us,
           "plain_us_per_half_sweep": plain_us, "plain_call_s": statistics.median(plain_s),
           "plain_instances": MID_PLAIN, "plain_equal_to_batched": int(same),
           "batched_over_plain": plain_us / per_instance_half_sweep_us,
           "flip_attempts_per_s": flips * MID_INSTANCES / stats["seconds"],
           "plain_flip_attempts_per_s": flips / statistics.median(plain_dev),
           "api": "rt_cftp_batch (thread-block clusters) vs rt_domino_cftp one at a time"}
    return out


# Config 4's full size ranges, at a fixed look-back: 8192 instances, Aztec orders U[16, 512]
# (half of them 2-periodic, a = 1, b ~ U[0.3, 1]) and hexagon sides U[8, 256], each run for
# one coupled attempt of FULL_SWEEPS sweeps from the extremal tilings (coalesced or not).
# Exact samples at these sizes take hours for any implementation of the reference's chain
# (the look-back grows like the order squared, and 8-16x per doubling of the order at
# b <= 0.6), so this leg measures the batch's flip-attempt throughput over the real size
# mix, against the same attempts made one instance at a time.
FULL_ORDERS, FULL_SIDES, FULL_B = (16, 512), (8, 256), (0.3, 1.0)
FULL_SWEEPS = 32
FULL_PLAIN = 64  # instances drawn across the mix for the one-at-a-time baseline


def full_range_leg(rt, instances: int = BATCH_INSTANCES) -> dict:
    """rt_cftp_batch over config 4's full size ranges (dominoes in clusters of CTAs where one
    CTA is too small), one attempt per instance; against rt_domino_cftp / rt_lozenge_cftp
    one instance at a time (FULL_PLAIN of them).  Rates count flip attempts over both chains:
    2 x FULL_SWEEPS x the instance's interior vertices."""
    import ctypes as C

    D, L = rt.DominoTiler, rt.LozengeTiler
    rng = np.random.default_rng(20261204)
    cache, jobs, flips = {}, [], []
    for k in range(instances):
        if k % 2 == 0:
            n = int(rng.integers(FULL_ORDERS[0], FULL_ORDERS[1] + 1))
            if ("d", n) not in cache:
                d = D.AztecDiamond(n)
                cache[("d", n)] = (D.MaxTiling(d), D.MinTiling(d))
            weighted = (k // 2) % 2 == 1
            b = float(rng.uniform(*FULL_B)) if weighted else 1.0
            jobs.append({"model": "domino", "tmax": cache[("d", n)][0], "tmin": cache[("d", n)][1], "seed": k,
                         "stream": k & 0xFFFF, "rule": "cftp_twoperiodic" if weighted else "cftp", "a": 1.0, "b": b,
                         "first_steps": FULL_SWEEPS, "max_attempts": 1})
            flips.append(2 * FULL_SWEEPS * (2 * n * n - 2 * n + 1))
        else:
            sd = int(rng.integers(FULL_SIDES[0], FULL_SIDES[1] + 1))
            if ("l", sd) not in cache:
                d = L.Hexagon(sd)
                cache[("l", sd)] = (L.MaxTiling(d), L.MinTiling(d))
            jobs.append({"model": "lozenge", "tmax": cache[("l", sd)][0], "tmin": cache[("l", sd)][1], "seed": k,
                         "stream": k & 0xFFFF, "first_steps": FULL_SWEEPS, "max_attempts": 1})
            flips.append(2 * FULL_SWEEPS * (3 * sd * sd - 3 * sd + 1))
    rt.cftp_batch(jobs[:2])  # warm-up
    t0 = time.perf_counter()
    outs, attempts, stats = rt.cftp_batch(jobs)
    wall = time.perf_counter() - t0
    pick = np.random.default_rng(8).choice(len(jobs), size=min(FULL_PLAIN, len(jobs)), replace=False)
    plain_dev, plain_wall, plain_flips, same = 0.0, 0.0, 0, 0
    for k in pick:
        job = jobs[int(k)]
        a_, b_ = np.ascontiguousarray(job["tmax"], np.int32), np.ascontiguousarray(job["tmin"], np.int32)
        out, st = np.zeros_like(a_), rt.CftpStats()
        n = rt.side_of(a_)
        t1 = time.perf_counter()
        if job["model"] == "domino":
            o = rt.DominoTiler(rule=job["rule"], rng="fast", a=job["a"], b=job["b"], fast_stream=job["stream"]).opts()
            status = rt.lib().rt_domino_cftp(rt._ptr(a_), rt._ptr(b_), n, int(job["seed"]), FULL_SWEEPS, 1, 1,
                                             C.byref(o), rt._ptr(out), C.byref(st))
        else:
            o = rt.LozengeTiler(rng="fast", fast_stream=job["stream"]).opts()
            status = rt.lib().rt_lozenge_cftp(rt._ptr(a_), rt._ptr(b_), n, int(job["seed"]), FULL_SWEEPS, 1, 1,
                                              C.byref(o), rt._ptr(out), C.byref(st))
        plain_wall += time.perf_counter() - t1
        if status not in (rt.RT_OK, rt.RT_ERR_NOT_COALESCED):
            raise rt.RTError(status, rt.lib().rt_last_error().decode())
        plain_dev += st.seconds
        plain_flips += flips[int(k)]
        same += np.array_equal(out, outs[int(k)])
    rate = float(np.sum(flips)) / stats["seconds"]
    plain_rate = plain_flips / plain_dev
    return {"workload": f"{instances} CFTP instances over config 4's full size ranges: Aztec orders "
                        f"U{list(FULL_ORDERS)} (half 2-periodic, a=1, b~U{list(FULL_B)}) and hexagon sides "
                        f"U{list(FULL_SIDES)}; one coupled attempt of {FULL_SWEEPS} sweeps each (fixed look-back: "
                        "exact samples at these sizes take hours for any implementation), fast mode",
            "flip_attempts": int(np.sum(flips)), "flip_attempts_per_s": rate, "kernel_s": stats["seconds"],
            "wall_s": wall, "wall_flip_attempts_per_s": float(np.sum(flips)) / wall,
            "plain_wall_flip_attempts_per_s": plain_flips / plain_wall, "cluster_instances": stats["cluster_instances"],
            "single_instances": stats["single_instances"], "ctas": stats["ctas"],
            "plain_flip_attempts_per_s": plain_rate, "plain_instances": len(pick), "plain_equal_to_batched": int(same),
            "batched_over_plain": rate / plain_rate,
            "api": "rt_cftp_batch vs rt_domino_cftp / rt_lozenge_cftp one at a time (device time both)"}


def single_instance_leg(rt) -> dict:
    """The other single-instance workloads: one coupled max/min CFTP attempt on the lozenge
    hexagon of side 512, 10^5 sweeps of bibone tilings of the 512 x 512 rhombus from the brick
    start, and 10^5 sweeps of the six-vertex model with domain-wall boundary at n = 512,
    a = b = 1, c = 1.5.  Fast (Philox) mode; rates from the device time of the sweeps."""
    out = {}
    L = rt.LozengeTiler(rng="fast")
    d = L.Hexagon(512)
    tmax, tmin = L.MaxTiling(d), L.MinTiling(d)
    look_back = 4096  # sweeps of the single attempt (3 steps each)
    o = L.opts()
    stats = rt.CftpStats()
    res = np.zeros_like(tmax)
    rt.lib().rt_lozenge_cftp(tmax.ctypes.data, tmin.ctypes.data, int(np.sqrt(tmax.size)), 11, 4, 0, 1, C.byref(o),
                             res.ctypes.data, C.byref(stats))  # warm-up: kernel loading outside the timed call
    status = rt.lib().rt_lozenge_cftp(tmax.ctypes.data, tmin.ctypes.data, int(np.sqrt(tmax.size)), 11, look_back, 0, 1,
                                      C.byref(o), res.ctypes.data, C.byref(stats))
    if status not in (rt.RT_OK, rt.RT_ERR_NOT_COALESCED):
        raise rt.RTError(status, rt.lib().rt_last_error().decode())
    out["lozenge_hexagon512_cftp_attempt"] = {
        "value": stats.flip_attempts / stats.seconds, "unit": "flip attempts/s", "look_back_sweeps": look_back,
        "coalesced": status == rt.RT_OK, "device_seconds": stats.seconds,
        "us_per_sweep": stats.seconds / look_back * 1e6, "interior_vertices": 3 * 512 * 512 - 3 * 512 + 1}
    T = rt.TriangleDimerTiler(rng="fast")
    t = T.RhombusBrick(512, 512)
    sweeps = 100_000
    st = T.Walk(t, 3 * sweeps, 7)
    out["bibone_rhombus512_walk"] = {
        "value": st["flip_attempts"] / st["seconds"], "unit": "flip attempts/s", "sweeps": sweeps,
        "steps": 3 * sweeps, "sweep": "3 steps (each step one move class)", "device_seconds": st["seconds"],
        "us_per_step": st["seconds"] / (3 * sweeps) * 1e6}
    S = rt.SixVertexTiler(1.0, 1.0, 1.5)
    h = S.MaxHeight(512)
    st = S.Walk(h, sweeps, 7)
    out["six_vertex_dwbc512_walk"] = {
        "value": st["flip_attempts"] / st["seconds"], "unit": "flip attempts/s", "sweeps": sweeps,
        "weights": [1.0, 1.0, 1.5], "device_seconds": st["seconds"], "us_per_sweep": st["seconds"] / sweeps * 1e6}
    out["domino_aztec1024_mtgp_reference_design"] = mtgp_leg(rt)
    return out


def mtgp_leg(rt, half_sweeps: int = 512) -> dict:
    """The headline workload (coupled max/min chains, two-periodic CFTP rule, order 1024) in
    the MTGP mode, which runs the reference CUDA build's own kernel design: one thread per
    site in 8 x 8 blocks, one cuRAND MTGP32 generator per block, a rotate and an update launch
    per half-sweep.  Device time of the half-sweeps (CUDA events on the sampler's stream); the
    host seeding of the 33,153 generators is reported apart, as the reference creates them
    once per Walk."""
    import time

    import torch

    D = rt.DominoTiler
    d = D.AztecDiamond(ORDER)
    tmax, tmin = D.MaxTiling(d), D.MinTiling(d)
    n = int(np.sqrt(tmax.size))
    interior = _interior_by_colour(D.DomainToVertices(d))
    stream = torch.cuda.Stream()
    tiler = rt.DominoTiler(rule="cftp_twoperiodic", rng="mtgp", a=WEIGHT_A, b=WEIGHT_B)
    s = rt.DominoSampler(n, 2, tiler, cuda_stream=stream.cuda_stream)
    s.load(0, tmin)
    s.load(1, tmax)
    s.sync()
    t0 = time.perf_counter()
    s.seed(DRIVER_SEED)
    s.sync()
    seeding = time.perf_counter() - t0
    cols = rt.mt19937_colours(DRIVER_SEED, 64 + half_sweeps)
    s.run(cols[:64])  # warm-up
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    s.run(cols[64:])
    e1.record(stream)
    stream.synchronize()
    sec = e0.elapsed_time(e1) / 1e3
    s.close()
    attempts = _attempts(cols[64:], interior)
    gens = ((n - 2 + 7) // 8) * ((n // 2 - 2 + 7) // 8)
    return {"value": attempts / sec, "unit": "flip attempts/s", "half_sweeps": half_sweeps,
            "us_per_half_sweep": sec / half_sweeps * 1e6, "generators": gens, "seeding_s": seeding,
            "api": "DominoSampler in rng='mtgp' (rt_dm_sampler_seed / rt_dm_sampler_run)"}


def run_reference(args) -> None:
    rank, ws, local, dist = _dist()
    if rank != 0:
        return
    from tests import oracle_py as orc  # the oracle alone: no library of this repository

    _, tmax, tmin, interior = headline_domain_oracle(orc)
    threads = os.cpu_count() or 1
    sample = 32
    cpu_leg(orc, tmax, tmin, interior, sample, max(args.warmup, 1), threads)
    t0 = time.perf_counter()
    rates = cpu_leg(orc, tmax, tmin, interior, sample, args.steps, threads)
    wall = time.perf_counter() - t0
    value = statistics.mean(rates)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "flip attempts/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * wall / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": {"workload": f"aztec{ORDER}_twoperiodic_a1.0_b0.5_cftp_coupled_maxmin",
                   "sample": f"{sample} of the {HALF_SWEEPS} half-sweeps of one attempt per step",
                   "l2": "n/a (host)"},
        "cpu_baseline": {"value": value, "unit": "flip attempts/s", "cores": threads, "kind": "port",
                         "sample": f"{sample} TinyMT half-sweeps of the coupled max/min chains per step, "
                                   f"order {ORDER}, {threads} host threads"},
        "e2e": {"value": value, "unit": "flip attempts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def headline_sampler(rt, tiler, cuda_stream):
    """The sampler a headline step runs on: chains 0 (bottom) and 1 (top) are swept, chains 2
    and 3 keep the min and max start states; returns (sampler, tmax, tmin, interior)."""
    D = rt.DominoTiler
    d = D.AztecDiamond(ORDER)
    tmax, tmin = D.MaxTiling(d), D.MinTiling(d)
    n = int(np.sqrt(tmax.size))
    s = rt.DominoSampler(n, 4, tiler, cuda_stream=cuda_stream)
    s.load(0, tmin)
    s.load(1, tmax)
    s.load(2, tmin)
    s.load(3, tmax)
    s.sync()
    s.set_active(2)
    return s, tmax, tmin, _interior_by_colour(D.DomainToVertices(d))


def headline_step(rt, s, seed: int, mode: str, before_run=None) -> np.ndarray:
    """One step of the headline workload: both chains reset to the extremal tilings, then one
    epoch of HALF_SWEEPS half-sweeps seeded `seed` (TinyMT: generators seeded seed + k and
    colours from mt19937(seed), the reference's epoch protocol; fast: half-sweeps -2048..-1
    keyed by seed).  Returns the colour of each half-sweep."""
    s.copy_chain(0, 2)
    s.copy_chain(1, 3)
    if mode == "tinymt":
        cols = rt.mt19937_colours(seed, HALF_SWEEPS)
        s.seed(seed)
        if before_run:
            before_run()
        s.run(cols)
    else:
        cols = np.array([1, 0] * (HALF_SWEEPS // 2), np.uint8)
        if before_run:
            before_run()
        s.run_fast(seed, -HALF_SWEEPS, HALF_SWEEPS)
    return cols


def timed_seeds(rank: int, steps: int) -> np.ndarray:
    """Seed of timed step k on a rank: draw k of mt19937(DRIVER_SEED + 7919 rank), so the
    first timed step's chains do not depend on the warm-up count."""
    return mt19937_host(DRIVER_SEED + 7919 * rank, steps)


def warmup_seeds(rank: int, steps: int) -> np.ndarray:
    return mt19937_host(DRIVER_SEED + 7919 * rank + 1, steps)


def mt19937_host(seed: int, count: int) -> np.ndarray:
    """First `count` outputs of std::mt19937(seed) (numpy's legacy MT19937 seeds and draws
    the same way)."""
    return np.random.RandomState(seed & 0xFFFFFFFF).randint(0, 2**32, size=count, dtype=np.uint32)


def chains_sha256(top: np.ndarray, bottom: np.ndarray) -> str:
    """Digest of a step's result: the top chain's int32 tiling, then the bottom chain's."""
    import hashlib

    h = hashlib.sha256()
    h.update(np.ascontiguousarray(top, np.int32).tobytes())
    h.update(np.ascontiguousarray(bottom, np.int32).tobytes())
    return h.hexdigest()


# The first timed step on rank 0 in TinyMT mode (seed 1791095845), as the oracle computes it:
# tests/golden/make_bench_check.py writes it to tests/golden/bench_check.json, and
# tests/test_bench_step.py checks both the GPU's result and this digest against the oracle.
BENCH_CHECK_SHA256 = "b363844c09336dfecba5a174eb2a1a6b93f0091e55872316ca600e0238604f67"

# DRAM bytes per launch of the resident sweep kernel (dram__bytes_read.sum +
# dram__bytes_write.sum), from one ncu capture of the same launch of this workload
# (profiles/k_bits_aztec1024.md, profiles/k_runs_aztec1024.md, profiles/k_persist_aztec1024.md):
#   ncu --set full --clock-control none -k regex:<kernel> -s 3 -c 1 \
#       python bench.py --no-cpu --no-batch --no-single --steps 2 --warmup 3 [--mode fast] [--engine 3]
# Keyed by (rng mode, kernel name).  None where no capture of that kernel exists.
NCU_TRAFFIC_BYTES = {
    ("tinymt", "k_bits"): 23_789_312 + 7_424,
    ("tinymt", "k_runs"): 25_105_664 + 44_288,
    ("tinymt", "k_persist"): 23_068_672,
    ("fast", "k_persist"): 6_047_744,
}


TUNE_TABLE = ROOT / "randomtilingspublic_gb300" / "tune" / "gb300.txt"


def run_ours(args) -> None:
    import torch

    rank, ws, local, dist = _dist()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    import randomtilingspublic_gb300 as rt

    # The autotuner's measured launch shapes (randomtilingspublic_gb300/autotune.py), when a
    # table for this GPU is present and not switched off.
    tune = None
    if not args.no_tune and TUNE_TABLE.exists():
        rt.tune_load(TUNE_TABLE)
        tune = str(TUNE_TABLE.relative_to(ROOT))

    tiler = rt.DominoTiler(rule="cftp_twoperiodic", rng=args.mode, a=WEIGHT_A, b=WEIGHT_B, fast_stream=rank,
                           engine=args.engine)
    stream = torch.cuda.Stream(device=dev)
    s, tmax, tmin, interior = headline_sampler(rt, tiler, stream.cuda_stream)
    n = int(np.sqrt(tmax.size))
    lib = rt.lib()
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    seeds = timed_seeds(rank, args.steps)
    wseeds = warmup_seeds(rank, args.warmup)
    info = s.engine_info()

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    kev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for k in range(args.warmup):
        headline_step(rt, s, int(wseeds[k]), args.mode)
        s.diff(0, 1)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    attempts = 0
    launches = 0
    check = None
    with Clocks(local) as clk:
        for k in range(args.steps):
            flush.zero_()  # L2 flush between timed steps (outside the events)
            torch.cuda.current_stream(dev).synchronize()
            with torch.cuda.stream(stream):
                ev[k][0].record(stream)
                l0 = s.launches
                cols = headline_step(rt, s, int(seeds[k]), args.mode, before_run=lambda: kev[k][0].record(stream))
                launches += s.launches - l0  # this library's kernels inside the events
                kev[k][1].record(stream)
                ev[k][1].record(stream)
            attempts += _attempts(cols, interior)
            s.diff(0, 1)
            if k == 0:
                # Self-check of the first timed step (outside the events): the digest of both
                # chains, against the oracle's value where one is recorded.
                digest = chains_sha256(s.store(1), s.store(0))
                expected = BENCH_CHECK_SHA256 if (args.mode == "tinymt" and rank == 0) else None
                check = {"step": 0, "seed": int(seeds[0]), "sha256": digest, "expected": expected,
                         "ok": None if expected is None else digest == expected}
        torch.cuda.synchronize()
    ms = sum(e0.elapsed_time(e1) for e0, e1 in ev)
    sec = _max_over_ranks(ms / 1e3, dist, dev)
    total_attempts = _sum_over_ranks(attempts, dist, dev)
    value = total_attempts / sec
    clocks = clk.summary()

    # Roofline of the sweep kernel.  Algorithmic bytes: 3 B per flip attempt (read and write
    # the active u8 site, write the passive one), plus TinyMT generator state where it moves
    # through memory: 32 B per generator per half-sweep on the per-half-sweep engine (every
    # generator of the grid), 32 B per flip-candidate generator per launch on the resident
    # engine (loaded once, stored once).
    kms = sum(e0.elapsed_time(e1) for e0, e1 in kev)
    half_sweeps = args.steps * HALF_SWEEPS
    cells = (n - 2) * (n // 2 - 2)
    tiling_bytes_per_half = 3 * (attempts / half_sweeps)
    peaks = _peaks()
    if info["engine"] in (2, 3, 4):
        kernel = {2: "k_runs (run-resident cooperative sweep, one launch per step)",
                  3: "k_persist (resident cooperative sweep exchanging band rows every half-sweep, one launch per step)",
                  4: "k_bits (bit-plane cooperative sweep: edge planes in shared memory, ballot-packed draws, one "
                     "launch per step)"}[info["engine"]]
        launches_timed = args.steps
        gen = 32 * info["units"] if args.mode == "tinymt" else 0
        algo_bytes = tiling_bytes_per_half * HALF_SWEEPS + gen
        limiter = ("on chip: integer issue and the neighbour-exchange latency; the chains stay in shared "
                   "memory for the whole launch, so the HBM copy bandwidth is a yardstick, not the limit")
    else:
        kernel = "k_rotate_tmt + k_update_w (one pair per half-sweep)"
        launches_timed = half_sweeps
        gen = 32 * cells if args.mode == "tinymt" else 0
        algo_bytes = tiling_bytes_per_half + gen
        limiter = "L2 and launch latency"
    t_launch = (kms / 1e3) / launches_timed
    achieved = algo_bytes / t_launch / 1e9
    traffic = NCU_TRAFFIC_BYTES.get((args.mode, kernel.split(" ")[0]))
    roofline = {"bound": "hbm", "limiter": limiter, "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / peaks["hbm_gbs"], "traffic": traffic,
                "traffic_source": "ncu capture of the same launch (bench.py NCU_TRAFFIC_BYTES)" if traffic else None,
                "peak_source": peaks["source"], "kernel": kernel, "algorithmic_bytes_per_launch": algo_bytes,
                "launch_us": t_launch * 1e6, "half_sweep_us": (kms / 1e3) / half_sweeps * 1e6, "engine": info}

    # e2e: one attempt through the C ABI from pinned host buffers, copies included.
    pin_max = torch.from_numpy(tmax).pin_memory()
    pin_min = torch.from_numpy(tmin).pin_memory()
    pin_out = torch.empty_like(pin_max).pin_memory()
    o = tiler.opts()
    stats = rt.CftpStats()
    e2e_rates = []
    for k in range(max(2, min(args.steps, 3))):
        t0 = time.perf_counter()
        st = lib.rt_domino_cftp(pin_max.data_ptr(), pin_min.data_ptr(), n, int(seeds[k]), HALF_SWEEPS, 0, 1,
                                C.byref(o), pin_out.data_ptr(), C.byref(stats))
        dt = time.perf_counter() - t0
        if st not in (rt.RT_OK, rt.RT_ERR_NOT_COALESCED):
            raise rt.RTError(st, lib.rt_last_error().decode())
        e2e_rates.append(stats.flip_attempts / dt)
    nbytes = n * n * 4
    e2e = {"value": _sum_over_ranks(statistics.median(e2e_rates[1:]), dist, dev), "unit": "flip attempts/s",
           # the max and min tilings (the min start state is copied on the device) and the
           # colour sequence in; the top chain and the coalescence count out
           "h2d_bytes_per_step": 2 * nbytes + HALF_SWEEPS, "d2h_bytes_per_step": nbytes + 8,
           "api": "rt_domino_cftp (one attempt, look-back 2048 half-sweeps)"}

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        from tests import oracle_py as orc

        threads = os.cpu_count() or 1
        sample = 32
        rates = cpu_leg(orc, tmax, tmin, interior, sample, 2, threads)
        cpu = {"value": statistics.mean(rates), "unit": "flip attempts/s", "cores": threads, "kind": "port",
               "sample": f"{sample} TinyMT half-sweeps of the coupled max/min chains (order {ORDER}) per attempt, "
                         f"2 attempts, {threads} host threads"}
    s.close()
    batched = serving = single = None
    mid = full = None
    if rank == 0 and not args.no_batch:
        batched = batched_leg(rt, args.batch_instances)
        serving = None if args.no_serve else serving_leg(rt)
        mid = mid_batch_leg(rt)
        full = None if args.no_full else full_range_leg(rt, args.batch_instances)
    if rank == 0 and not args.no_single:
        single = single_instance_leg(rt)
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "flip attempts/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "config": {"workload": f"aztec{ORDER}_twoperiodic_a1.0_b0.5_cftp_coupled_maxmin",
                       "rng": args.mode, "engine": args.engine, "half_sweeps_per_step": HALF_SWEEPS,
                       "l2": "flushed between timed steps (256 MiB write)", "parallelism": f"replicas{ws}",
                       "launch": {"tune_table": tune, "tuned": info.get("tuned"), "engine": info["engine"],
                                  "bands": info["bands"], "threads_per_band": info.get("threads"),
                                  "units_per_thread": info["units_per_thread"]}},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches, "clocks": clocks,
            "check": check, "batched_cftp": batched, "served_cftp": serving, "batched_cftp_clusters": mid,
            "batched_cftp_full_range": full,
            "single_instance": single,
        }
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--mode", choices=["tinymt", "fast"], default="tinymt")
    ap.add_argument("--engine", type=int, default=0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-full", action="store_true", help="skip the full-size-range batch leg")
    ap.add_argument("--batch-instances", type=int, default=BATCH_INSTANCES)
    ap.add_argument("--no-single", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="ignore the autotuner's table")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

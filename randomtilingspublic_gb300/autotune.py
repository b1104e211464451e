"""Measured launch-shape search for the domino sampler (the autotuner).

The reference launches every kernel with one compile-time block shape (BLOCK_DIM 8,
src/Domino/dominokernel.cuh:4).  Here the shape of the resident sweep is a choice: which
resident kernel (the bit-plane kernel, the run kernel, k_persist, or the per-half-sweep
kernels), how many bands (CTAs, each a strip of rows - the tile) and, for the run kernel,
how many threads per band (so how many column quads, four sites each, per thread).  For each Aztec-diamond order, chain count and random
mode asked for, every candidate shape is timed on the GPU (CUDA-synchronised wall time of a
fixed number of half-sweeps, best of a few repetitions) and the fastest is written to a
table the library reads (rt_tune_load, or the RT_TUNE_FILE environment variable).  Entries
cover tiling sides between the midpoints of the measured ones.  The shape never changes a
result: every draw is keyed by its site, whichever thread makes it.

    python -m randomtilingspublic_gb300.autotune --orders 32 128 512 1024 --chains 1 2 \\
        --rng tinymt fast --out randomtilingspublic_gb300/tune/gb300.txt
"""
from __future__ import annotations

import argparse
import time
from pathlib import Path

THREADS = (512, 640, 768, 896, 960, 992, 1024)


def candidates(sms: int) -> list[tuple[int, int, int]]:
    """(engine, bands, threads): the per-half-sweep kernels, k_persist, the run kernel over
    bands and threads per band, and the bit-plane kernel (TinyMT only; its threads follow from
    its plan) over bands."""
    out = [(1, 0, 0), (3, 0, 0)]
    for bands in sorted({sms, (3 * sms) // 4, sms // 2}, reverse=True):
        out.append((4, bands, 0))
        for threads in THREADS:
            out.append((2, bands, threads))
    return out


def _sampler(rt, n, chains, rng, tmax, tmin):
    tiler = rt.DominoTiler(rule="cftp_twoperiodic", rng=rng, a=1.0, b=0.5)
    s = rt.DominoSampler(n, chains, tiler)
    for c in range(chains):
        s.load(c, tmax if c % 2 == 0 else tmin)
    s.sync()
    return s


def measure(rt, n, chains, rng, tmax, tmin, shape, half_sweeps: int = 256, reps: int = 3):
    """(microseconds per half-sweep, the shape the sampler used) for `shape` on this domain,
    or None when the sampler does not take it (no such plan, e.g. too many quads per thread
    for register generators).  A plan has at most one band per row, so on small domains the
    bands used can be fewer than asked."""
    s = _sampler(rt, n, chains, rng, tmax, tmin)
    try:
        s.set_launch(*shape)
        try:
            info = s.engine_info()
        except rt.RTError:
            return None
        engine, bands, threads = shape
        if info["engine"] != engine or (engine == 2 and info["threads"] != threads):
            return None
        used = (engine, info["bands"], threads) if engine in (2, 4) else shape
        cols = rt.mt19937_colours(12345, half_sweeps)

        def run():
            if rng == "tinymt":
                s.run(cols)
            else:
                s.run_fast(7, 0, half_sweeps)

        if rng == "tinymt":
            s.seed(99)
        run()
        s.sync()
        best = float("inf")
        for _ in range(reps):
            t0 = time.perf_counter()
            run()
            s.sync()
            best = min(best, time.perf_counter() - t0)
        return best / half_sweeps * 1e6, used
    finally:
        s.close()


def tune_domino(rt, orders, chains_list=(2,), rngs=("tinymt",), half_sweeps: int = 256, log=print) -> list[dict]:
    """Times every candidate for each (order, chains, rng); returns the table's entries."""
    sms = _sm_count()
    D = rt.DominoTiler
    measured = []
    for order in orders:
        d = D.AztecDiamond(int(order))
        tmax, tmin = D.MaxTiling(d), D.MinTiling(d)
        n = rt.side_of(tmax)
        for chains in chains_list:
            for rng in rngs:
                results, used_shapes = [], set()
                for shape in candidates(sms):
                    got = measure(rt, n, chains, rng, tmax, tmin, shape, half_sweeps)
                    if got is not None and got[1] not in used_shapes:
                        used_shapes.add(got[1])
                        results.append(got)
                results.sort()
                us, shape = results[0]
                log(f"order {order} (N={n}) chains {chains} {rng}: best {shape} {us:.3f} us/half-sweep "
                    f"({len(results)} shapes timed; slowest {results[-1][0]:.3f})")
                measured.append({"N": n, "order": int(order), "chains": chains, "rng": rng, "engine": shape[0],
                                 "bands": shape[1], "threads": shape[2], "us": us})
    # Entries cover the tiling sides between midpoints of the measured ones, per (chains, rng).
    entries = []
    for chains in chains_list:
        for rng in rngs:
            ms = sorted((m for m in measured if m["chains"] == chains and m["rng"] == rng), key=lambda m: m["N"])
            for k, m in enumerate(ms):
                lo = 6 if k == 0 else (ms[k - 1]["N"] + m["N"]) // 2 + 1
                hi = 32768 if k == len(ms) - 1 else (m["N"] + ms[k + 1]["N"]) // 2
                entries.append(dict(m, n_lo=lo, n_hi=hi))
    return entries


def _sm_count() -> int:
    """Streaming multiprocessors of the current GPU (through torch, which the GPU tools of
    this repository use for device queries)."""
    import torch

    return torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count


def write_table(entries, path) -> None:
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    lines = ["# rt_tilings launch shapes measured by randomtilingspublic_gb300.autotune",
             "# model n_lo n_hi chains rng engine bands threads us_per_half_sweep (measured at order, N)"]
    for e in entries:
        lines.append(f"domino {e['n_lo']} {e['n_hi']} {e['chains']} {e['rng']} {e['engine']} {e['bands']} "
                     f"{e['threads']} {e['us']:.3f}  # order {e['order']}, N {e['N']}")
    path.write_text("\n".join(lines) + "\n")


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--orders", type=int, nargs="+", default=[32, 128, 512, 1024])
    ap.add_argument("--chains", type=int, nargs="+", default=[1, 2])
    ap.add_argument("--rng", nargs="+", default=["tinymt", "fast"])
    ap.add_argument("--half-sweeps", type=int, default=256)
    ap.add_argument("--out", required=True)
    args = ap.parse_args()
    import randomtilingspublic_gb300 as rt

    rt.tune_clear()  # measure the shapes themselves, not a loaded table's choice
    entries = tune_domino(rt, args.orders, args.chains, args.rng, args.half_sweeps)
    write_table(entries, args.out)
    print(f"wrote {len(entries)} entries to {args.out}")


if __name__ == "__main__":
    main()

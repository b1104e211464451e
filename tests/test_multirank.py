"""The multi-process path of bench.py on CPU (gloo, world size 2): the rank reductions that
turn per-rank times and counts into the job's numbers, and the reference arm under torchrun,
where rank 0 alone measures and prints one line and the other ranks exit 0.  The data path
itself has no collective: ranks run independent replicas (stream = rank)."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _reduce_worker(rank: int, port: int, out) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2",
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import torch

    import bench

    r, ws, local, dist = bench._dist()
    assert (r, ws) == (rank, 2)
    dev = torch.device("cpu")
    out.put((rank, bench._max_over_ranks(1.5 + rank, dist, dev), bench._sum_over_ranks(10.0 * (rank + 1), dist, dev)))
    dist.destroy_process_group()


def test_rank_reductions_over_gloo():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.SimpleQueue()
    port = _free_port()
    procs = [ctx.Process(target=_reduce_worker, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get() for _ in range(2))
    assert got == [(0, 2.5, 30.0), (1, 2.5, 30.0)]


@pytest.mark.timeout(600)
def test_reference_arm_under_torchrun_prints_one_line_from_rank_0():
    env = dict(os.environ, PYTHONPATH=str(ROOT), OMP_NUM_THREADS="1")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(_free_port()), "bench.py", "--impl", "reference", "--gpus", "2",
           "--steps", "1", "--warmup", "1"]
    res = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=580)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [json.loads(l) for l in res.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"


@pytest.mark.timeout(600)
def test_reference_arm_loads_no_library_of_this_repository():
    """The reference arm times the oracle alone: after it ran, the process has mapped the
    oracle's library and not librt_tilings.so."""
    code = (
        "import sys, argparse; sys.path.insert(0, '.'); import bench\n"
        "bench.run_reference(argparse.Namespace(gpus=1, steps=1, warmup=1))\n"
        "maps = open('/proc/self/maps').read()\n"
        "print('MAPS', 'librt_tilings' in maps, 'liboracle' in maps)\n"
    )
    res = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=580,
                         env=dict(os.environ, WORLD_SIZE="1"))
    assert res.returncode == 0, res.stderr[-2000:]
    assert "MAPS False True" in res.stdout

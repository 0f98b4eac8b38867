"""Multi-process (replicas-only) harness of bench.py, on CPU with the gloo backend.

The propagation path does not shard: under torchrun every rank propagates its
own replica, the ranks meet only at barriers around the timed region, and
rank 0 prints one line whose value is the total work over the slowest rank's
time. These tests run two ranks on the host (no GPU): the rendezvous, the
max-over-ranks reduction and the barrier of bench.py's harness, and the
reference arm launched the way the two-GPU bench is launched, where rank 0
alone runs and prints.
"""
import json
import os
import socket
import subprocess
import sys
from argparse import Namespace

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench

    w, r, local, pg = bench.dist_setup(Namespace(impl="reference"))
    assert (w, r, local) == (world, rank, rank) and pg is not None
    bench.barrier(pg)
    # each rank reports its own time; every rank must see the slowest one
    slowest = bench.max_over_ranks(pg, 10.0 + rank)
    bench.barrier(pg)
    with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
        f.write(repr(slowest))
    pg.destroy_process_group()


def test_gloo_two_ranks_max_over_ranks(tmp_path):
    world, port = 2, _free_port()
    mp.start_processes(_rank_main, args=(world, port, str(tmp_path)), nprocs=world, join=True, start_method="spawn")
    got = [float((tmp_path / f"rank{r}.txt").read_text()) for r in range(world)]
    assert got == [11.0, 11.0]


def test_single_process_needs_no_rendezvous():
    sys.path.insert(0, ROOT)
    import bench

    env = {k: os.environ.pop(k) for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK") if k in os.environ}
    try:
        w, r, local, pg = bench.dist_setup(Namespace(impl="own"))
        assert (w, r, local, pg) == (1, 0, 0, None)
        assert bench.max_over_ranks(pg, 3.5) == 3.5
        bench.barrier(pg)
    finally:
        os.environ.update(env)


def test_reference_arm_two_ranks_prints_once():
    """Launched like the two-GPU bench: rank 0 runs the host reference arm, rank 1 exits 0 without work."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "1"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(s) for s in r.stdout.splitlines() if s.startswith("{")]
    assert len(lines) == 1
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["value"] > 0 and line["e2e"]["value"] == line["value"]

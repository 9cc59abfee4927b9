"""The multi-rank side of bench.py on the CPU (gloo, world size 2).

The path does not shard: every rank renders its own replica and the only
collective is the max of the timed region over ranks.  The reference arm runs
on rank 0 alone and the other ranks exit without work.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, values, out_path):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    got = bench.max_over_ranks(values[rank], world)
    dist.barrier()
    dist.destroy_process_group()
    with open(f"{out_path}.{rank}", "w") as f:
        f.write(repr(got))


def test_max_over_ranks_gloo(tmp_path):
    import torch.multiprocessing as mp

    values = [3.25, 7.5]
    out = str(tmp_path / "res")
    mp.spawn(_rank_main, args=(2, _free_port(), values, out), nprocs=2, join=True)
    assert [float(open(f"{out}.{r}").read()) for r in range(2)] == [7.5, 7.5]


def test_max_over_ranks_single_process():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(1.5, 1) == 1.5


def test_reference_arm_under_torchrun(built, tmp_path):
    """`bench.py --impl reference` launched like the multi-GPU run: rank 0 prints
    one JSON line, the other rank exits 0 without work."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0

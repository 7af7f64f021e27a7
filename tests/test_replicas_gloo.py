"""The N > 1 path of bench.py is replicas only (independent FDTD runs, no
exchange step): two gloo ranks on CPU check the max-over-ranks timing, the
whole-job aggregate, and that the reference arm does its work on rank 0 only."""
import json
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

from tests.conftest import ROOT


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, ws, port, times, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    sys.path.insert(0, ROOT)
    import bench
    m = bench._barrier_max(times[rank], ws)
    out[rank] = (m, bench.aggregate_rate(1000.0, m, ws))
    dist.barrier()
    dist.destroy_process_group()


def test_barrier_max_and_aggregate():
    ws, port = 2, _free_port()
    times = [0.25, 0.5]
    with mp.Manager() as man:
        out = man.dict()
        mp.spawn(_rank, args=(ws, port, times, out), nprocs=ws, join=True)
        res = dict(out)
    for r in range(ws):
        m, rate = res[r]
        assert m == 0.5  # the slowest rank sets the time
        assert rate == pytest.approx(1000.0 * ws / 0.5)


def test_reference_arm_only_rank0_prints(tmp_path):
    """Under torchrun the reference arm's rank 1 exits 0 without output."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--gpus", "2", "--steps", "1", "--warmup", "0"],
                       env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""


def test_reference_arm_rank0_line():
    env = dict(os.environ, RANK="0", WORLD_SIZE="1", LOCAL_RANK="0", CEV_CPU_PROCS="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "0"],
                       env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["cores"] >= 1

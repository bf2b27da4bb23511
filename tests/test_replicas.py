"""The multi-GPU form of the bench is replicas: one independent program per
rank, whole-job throughput = all ranks' lattice updates over the slowest
rank's time.  Checked here with world_size 2 on CPU (gloo, 127.0.0.1); the
reference arm runs on rank 0 only."""
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(ws))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=ws)
    # rank r is slower on the device leg, rank 0 slower end to end
    dev = [2.0, 3.0][rank]
    e2e = [5.0, 4.0][rank]
    v, e, d, t = bench.aggregate_replicas(dev, e2e, 1e9, ws, device="cpu")
    out.put((rank, v, e, d, t))
    dist.destroy_process_group()


def test_replica_aggregation_takes_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, v, e, d, t in res:
        assert d == 3.0 and t == 5.0
        assert v == pytest.approx(2 * 1e9 / 3.0 / 1e9)
        assert e == pytest.approx(2 * 1e9 / 5.0 / 1e9)


def test_reference_arm_other_ranks_exit_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "0"], cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == ""

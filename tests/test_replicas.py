"""The multi-GPU path of bench.py is replicas only: every rank steps its own
box, the job is timed by the slowest rank, and the throughput is the sum over
ranks.  Checked here on CPU with two gloo ranks (no GPU): the max-over-ranks
reduction, the whole-job aggregation, and that a non-zero rank of the
reference arm exits quietly."""
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    ms = [12.5, 17.25][rank]
    m = bench.max_over_ranks(ms, ws, device="cpu")
    v = bench.whole_job_mlups(1000, 10, m / 1e3, ws)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, m, v))


def test_max_over_ranks_and_whole_job_throughput():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, m, v in out:
        assert m == 17.25  # the slowest rank times the job
        assert v == pytest.approx(1000 * 10 / 17.25e-3 / 1e6 * 2)


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert bench.whole_job_mlups(2_000_000, 5, 0.5, 1) == pytest.approx(20.0)


def test_reference_arm_nonzero_rank_exits_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == ""


def test_metric_names_follow_the_scheme_and_storage():
    import argparse
    sys.path.insert(0, ROOT)
    import bench
    assert bench.metric_name(argparse.Namespace(scheme="fused", storage="f16")) == bench.METRIC
    assert "FP32-storage plain" in bench.metric_name(argparse.Namespace(scheme="plain", storage="f32"))

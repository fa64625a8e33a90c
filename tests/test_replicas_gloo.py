"""The multi-GPU path of bench.py on CPU: two gloo ranks.

Every workload fits one GPU, so N GPUs run N independent replicas and the only
cross-rank steps are the barrier and the max-over-ranks of the timed region.
These tests run those steps with two gloo processes on 127.0.0.1: the job's
time is the slowest rank's, the whole-job rate counts every rank's particles,
and the reference arm prints nothing on ranks other than 0.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, times, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    dist.barrier()
    ms = bench.max_over_ranks(times[rank], "cpu")
    rate = bench.whole_job_rate(1000, world, 5, ms)
    out.put((rank, ms, rate))
    dist.destroy_process_group()


def test_max_over_ranks_and_whole_job_rate_with_two_gloo_ranks():
    world = 2
    times = [12.5, 20.0]  # rank 1 is the slow replica
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, times, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, rate in got:
        assert ms == max(times)
        assert rate == pytest.approx(1000 * world * 5 / (max(times) / 1e3))


def test_max_over_ranks_without_a_process_group_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.25, "cpu") == 3.25
    assert bench.whole_job_rate(10, 1, 4, 2.0) == pytest.approx(20000.0)


def test_reference_arm_prints_only_on_rank_zero():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""


def test_reference_arm_line_on_rank_zero_small_sample():
    env = dict(os.environ, RANK="0", WORLD_SIZE="1", LOCAL_RANK="0", OMP_NUM_THREADS="2")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--cpu-cells", "8",
                        "--cpu-steps", "1"], cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["unit"] == "particle-steps/s" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] == 2
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0

"""The multi-rank logic of bench.py on CPU: world_size-2 gloo process
groups (127.0.0.1), no GPU.

bench.py runs one full replica of the workload per rank (the transforms of
different batch items never exchange data, so there is no data-path
collective): the job's time is the slowest rank's, taken by an all-reduce
MAX, and the whole-job value counts every rank's bytes.  The reference arm
runs on rank 0 only; the other ranks leave without output.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402

torch = pytest.importorskip("torch")
dist = pytest.importorskip("torch.distributed")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = [12.5, 40.0][rank]  # rank 1 is the slow one
        worst = bench.max_over_ranks(ms, dist, torch.device("cpu"))
        dist.barrier()
        q.put((rank, worst, bench.whole_job_gbs(1e9, world, 10, worst / 1e3)))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_whole_job_value_gloo():
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in procs)
    for rank, worst, gbs in got:
        assert worst == 40.0  # every rank sees the slowest rank's time
        assert gbs == pytest.approx(1e9 * 2 * 10 / 0.040 / 1e9)  # both ranks' bytes over the slowest time
    assert bench.max_over_ranks(3.0, None, None) == 3.0


def test_reference_arm_under_torchrun_prints_once():
    # two ranks of the reference arm: rank 0 prints one JSON line, rank 1
    # exits 0 without work (the golden torch.fft path on the CPU)
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2", "--master-addr",
           "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"), "--impl", "reference",
           "--workload", "cfg1", "--gpus", "2", "--steps", "1", "--warmup", "1"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "reference" and d["config"]["same_config"]


def test_gpus_flag_self_launches_ranks():
    """`bench.py --gpus 2` outside a launcher starts two ranks itself; a
    launcher whose WORLD_SIZE disagrees with --gpus is refused."""
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "cfg1", "--gpus", "2",
           "--steps", "1", "--warmup", "1"]
    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1 and json.loads(lines[0])["n_gpus"] == 2
    env.update(WORLD_SIZE="1", RANK="0", LOCAL_RANK="0")
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT, env=env)
    assert r.returncode != 0 and "WORLD_SIZE=1" in r.stderr

"""bench.py's multi-GPU form is N independent replicas (one scene per rank, no collective on the
data path): the job rate is N x steps / the slowest rank's time.  Checked with world_size-2 gloo
ranks on the CPU, and the reference arm's rank handling (rank 0 alone prints)."""
import json
import os
import subprocess
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench
    local = [2.0, 3.0][rank]  # the second rank is slower
    rate, elapsed = bench.job_rate(local, 10, world, dist, "cpu")
    out[rank] = (rate, elapsed)
    dist.barrier()
    dist.destroy_process_group()


def test_job_rate_takes_the_slowest_replica():
    world = 2
    port = 29611
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for r in range(world):
        rate, elapsed = res[r]
        assert elapsed == 3.0
        assert rate == pytest.approx(2 * 10 / 3.0)


def test_job_rate_single_rank():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.job_rate(4.0, 8, 1) == (2.0, 4.0)


def test_reference_arm_other_ranks_exit_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode == 0
    assert r.stdout.strip() == ""


def test_reference_arm_line_on_rank0():
    """The reference arm (the oracle's CPU step on the host cores) prints one JSON line with the
    bench contract's keys; a tiny bounded sample (8^3 steps scaled to 16^3) keeps it quick."""
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0", "--res", "16", "--cpu-res", "8"],
                       capture_output=True, text=True, env=dict(os.environ, RANK="0", WORLD_SIZE="1"), timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [x for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "steps/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 1 and d["warmup"] == 0 and d["n_gpus"] == 1
    assert d["ms_per_step"] == pytest.approx(1e3 / d["value"])
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    assert d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert "16^3" in d["config"]["workload"]

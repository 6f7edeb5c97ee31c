"""The N > 1 path on CPU: replicas joined by a gloo process group (world size 2).

The render path does not shard (views are independent), so N GPUs run N replicas; the only
cross-rank traffic is the barrier around the timed region and the MAX over ranks of its
elapsed time.  These tests run that host logic as two gloo ranks, and the CPU arm of the
benchmark under the torch launcher with two ranks.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import PKG_DIR as PKG, REPO

sys.path.insert(0, PKG)

from gs300.replicas import Replicas  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, PKG)
    from gs300.replicas import Replicas

    g = Replicas("gloo").init()
    g.barrier()
    # rank r claims (r + 1) seconds for 10 frames: the job is as slow as rank 1
    rate, slowest = g.job_rate(10, float(rank + 1))
    peak = g.max_over_ranks(100.0 * rank - 7.0)
    res = {"rank": g.rank, "world": g.world, "leader": g.leader, "seed": g.scene_seed(6),
           "rate": rate, "slowest": slowest, "peak": peak}
    g.barrier()
    g.close()
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump(res, f)


def test_replicas_world2_gloo(tmp_path):
    import torch.multiprocessing as mp

    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(2)]
    for r, x in enumerate(res):
        assert x["rank"] == r and x["world"] == 2
        assert x["leader"] == (r == 0)
        assert x["slowest"] == 2.0  # MAX over ranks, seen by every rank
        assert x["rate"] == pytest.approx(2 * 10 / 2.0)
        assert x["peak"] == 93.0
    assert res[0]["seed"] != res[1]["seed"]  # each replica renders its own scene


def test_replicas_single_process():
    g = Replicas(env={}).init()  # world 1: no process group is created
    assert (g.rank, g.world, g.local, g.leader) == (0, 1, 0, True)
    g.barrier()
    assert g.job_rate(30, 0.5) == (60.0, 0.5)
    assert g.scene_seed(6) == 6
    with pytest.raises(ValueError):
        g.job_rate(1, 0.0)
    g.close()


def test_replicas_bad_env():
    with pytest.raises(ValueError):
        Replicas(env={"RANK": "2", "WORLD_SIZE": "2"})


def test_bench_reference_arm_two_ranks():
    """bench.py --impl reference under the launcher: rank 0 alone prints one line, all exit 0."""
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr=127.0.0.1", f"--master-port={port}", os.path.join(REPO, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "2", "--warmup", "1",
           "--splats", "3000", "--width", "64", "--height", "48"]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    p = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=REPO, env=env)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [json.loads(x) for x in p.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["value"] > 0 and line["steps"] == 2
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"

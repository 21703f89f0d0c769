"""bench.py's host side without a GPU: the reference arm (the CPU path timed
on the host's cores) launched as two ranks over gloo prints exactly one
JSON line, from rank 0, with the contract's keys; the other rank exits 0
without work.  The GPU arm's barrier and max-over-ranks reduction
(bench.rank_sync, NCCL on the GPU) run here as two gloo ranks."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.timeout(600)
def test_reference_arm_two_ranks_over_gloo(tmp_path):
    env = dict(os.environ, OMP_NUM_THREADS="2", PYTHONPATH=ROOT)
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", "29533", "bench.py",
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "3"]
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == "cell-updates/s"
    for k in ("metric", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "dtype", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] in ("port",
                                                                                  "reference")


def _sync_rank(rank, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=2)
    barrier, max_over_ranks = bench.rank_sync(dist, "cpu")
    barrier()
    got = max_over_ranks(1.5 + 2.0 * rank)  # rank 0: 1.5 s, rank 1: 3.5 s
    barrier()
    with open(os.path.join(out, f"r{rank}"), "w") as f:
        f.write(repr(got))
    dist.destroy_process_group()


@pytest.mark.timeout(300)
def test_rank_sync_over_gloo(tmp_path):
    """The timed region's barrier and max-over-ranks reduction of the GPU arm
    (bench.rank_sync), run as two gloo ranks: every rank gets the slowest
    rank's time, which the whole-job rate divides by."""
    import torch.multiprocessing as mp
    mp.spawn(_sync_rank, args=(29541, str(tmp_path)), nprocs=2, join=True)
    for r in range(2):
        assert (tmp_path / f"r{r}").read_text() == "3.5"
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    import bench
    b, m = bench.rank_sync(None, "cpu")  # one process: identity, no barrier
    b()
    assert m(2.25) == 2.25

"""Multi-GPU runs are replicas only (a single IMS solve does not shard): each
rank solves its own copy of the step and the job time is the maximum over
ranks.  These CPU tests cover that host logic with world_size 2 on gloo."""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _rank_main(rank, ws, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    sys.path.insert(0, str(ROOT))
    import bench
    v = bench.max_over_ranks(1.5 + rank, ws)
    dist.barrier()
    dist.destroy_process_group()
    Path(out, f"r{rank}").write_text(repr(v))


def test_max_over_ranks_gloo(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = 29500 + (os.getpid() % 1000)
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    assert [float(Path(tmp_path, f"r{r}").read_text()) for r in range(2)] == [2.5, 2.5]


def test_reference_arm_prints_one_line_under_torchrun():
    """Under torchrun only rank 0 runs the reference arm and prints its line;
    the other ranks exit 0 without work."""
    pytest.importorskip("torch")
    port = 30500 + (os.getpid() % 1000)
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0", "--scale", "0.05"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["cpu_baseline"]["cores"] == 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0

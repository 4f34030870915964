"""The N > 1 host path of bench.py on CPU: ranks are independent replicas (no
data-path collective); the only exchange is the max over ranks of the timed
region, and rank 0 alone prints.  Two ranks over gloo on 127.0.0.1."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out_dir: str) -> None:
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ws, r, local = bench.dist_env()
        # per-rank timings differ; every rank must see the slowest
        slowest = bench.max_over_ranks(10.0 + rank, dist, device="cpu")
        none = bench.max_over_ranks(3.0, None)
        Path(out_dir, f"rank{rank}.json").write_text(
            json.dumps({"ws": ws, "rank": r, "local": local, "max": slowest, "none": none}))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    got = [json.loads(Path(tmp_path, f"rank{r}.json").read_text()) for r in range(2)]
    for r, g in enumerate(got):
        assert g == {"ws": 2, "rank": r, "local": r, "max": 11.0, "none": 3.0}


@pytest.mark.parametrize("rank", [0, 1])
def test_reference_arm_prints_on_rank0_only(rank):
    env = dict(os.environ, RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank),
               MASTER_ADDR="127.0.0.1", MASTER_PORT=str(_free_port()))
    res = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", "c1",
                          "--gpus", "2", "--steps", "3", "--warmup", "3"],
                         cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [ln for ln in res.stdout.splitlines() if ln.strip()]
    if rank == 0:
        assert len(lines) == 1
        line = json.loads(lines[0])
        assert line["impl"] == "reference" and line["value"] > 0 and line["n_gpus"] == 2
    else:
        assert lines == []

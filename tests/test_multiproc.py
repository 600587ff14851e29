"""The N > 1 host logic of bench.py on CPU with two gloo ranks: the max-over-ranks
timing reduction and the split of the independent lattices of the batch workload
(disjoint, covering, balanced), as torchrun would run them (127.0.0.1 rendezvous)."""
from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, ws: int, port: int, q) -> None:
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench

    worst = bench.max_over_ranks(10.0 * (rank + 1), ws)
    lats = bench.batch_lattices(bench.BATCH)
    mine = bench.shard(lats, rank, ws)
    dist.barrier()
    q.put((rank, worst, [l[3] for l in mine], len(lats)))
    dist.destroy_process_group()


def test_two_gloo_ranks_reduce_and_shard():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [20.0, 20.0]
    seeds0, seeds1 = set(res[0][2]), set(res[1][2])
    assert not seeds0 & seeds1
    assert len(seeds0) + len(seeds1) == res[0][3] == 64
    assert abs(len(seeds0) - len(seeds1)) <= 1


def test_gpus_flag_starts_ranks_under_torchrun():
    """`bench.py --gpus 2` outside torchrun relaunches itself with two ranks (127.0.0.1 rendezvous); the
    reference arm runs on rank 0 alone, which prints the one line with n_gpus = 2."""
    pytest.importorskip("torch")
    import json
    import subprocess

    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--gpus", "2", "--impl", "reference", "--workload",
                        "cg", "--steps", "1", "--warmup", "0"], capture_output=True, text=True, timeout=600, env=env,
                       cwd=str(ROOT))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2


def test_gpus_flag_refuses_a_mismatched_world():
    import subprocess

    env = dict(os.environ, WORLD_SIZE="1", RANK="0", LOCAL_RANK="0")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--gpus", "2", "--impl", "reference", "--workload",
                        "cg", "--steps", "1"], capture_output=True, text=True, timeout=120, env=env, cwd=str(ROOT))
    assert r.returncode != 0 and "WORLD_SIZE" in (r.stderr + r.stdout)

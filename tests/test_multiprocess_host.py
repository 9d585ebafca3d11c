"""The bench's multi-rank path on CPU (gloo, world size 2): every rank gets the max-over-ranks
time, barriers complete, and the batched workload gives each rank its own independent scenes
while single-scene workloads replicate one scene."""
import os
import socket
import sys
from types import SimpleNamespace

import pytest

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import bench
    from bullet3_gb300 import scenes
    r, w, local = bench.dist_info()
    dist = bench.dist_init(w)
    t = bench.dist_max(dist, 1.0 + rank)  # rank 1 is the slow one
    bench.dist_barrier(dist)
    args = SimpleNamespace(workload="batched", scenes=16)
    sc = bench.make_scene(args, r)
    pile = bench.scene_seed(SimpleNamespace(workload="pile"), r)
    with open(os.path.join(out_dir, f"rank{r}.txt"), "w") as f:
        f.write(f"{r} {w} {t} {bench.scene_seed(args, r)} {pile} {sc.num_bodies} {float(sc.pos[:, 0].sum())}\n")
    dist.destroy_process_group()


def test_two_ranks_max_time_and_scene_sharding(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = _free_port()
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    rows = [open(tmp_path / f"rank{r}.txt").read().split() for r in range(2)]
    for r, row in enumerate(rows):
        assert int(row[0]) == r and int(row[1]) == 2
        assert float(row[2]) == 2.0  # max over ranks
        assert int(row[3]) == r  # batched: own scene set per rank
        assert int(row[4]) == 0  # pile: replicas of one scene
    assert rows[0][6] != rows[1][6]  # the two ranks' scene sets differ

"""The multi-process layout of the ray-cast workload (lmgpu/dist.py, used by
bench.py under torchrun) with world_size-2 gloo ranks on the CPU: each rank
draws its own rays, traces them against its own copy of the scene (here
with the CPU oracle, the path has no data exchange), and the timing
reduction returns the slowest rank's time on every rank."""
import os
import socket
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, ws: int, port: int, out_dir: str) -> None:
    for p in (os.path.join(REPO, "lightmetrica-v2_gb300"), os.path.join(REPO, "oracle")):
        sys.path.insert(0, p)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(ws), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist

    import lmoracle
    from lmgpu import dist as ldist
    from lmgpu import scenes

    got_ws, got_rank, _ = ldist.dist_env()
    assert (got_ws, got_rank) == (ws, rank)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    tris = scenes.raycast_scene(2000, 8, seed=5)
    rays = scenes.raycast_rays(512, stream=ldist.ray_stream(rank))
    hits = lmoracle.OracleAccel(lmoracle.BVH_SAHBIN, tris).trace(rays, threads=1)
    # a per-rank "time": the slowest rank's value must come back on every rank
    local = [1.0 + rank, 10.0 - rank]
    red = ldist.max_over_ranks(local)
    np.save(os.path.join(out_dir, f"rank{rank}.npy"),
            {"rays": rays, "ids": hits["id"], "red": red}, allow_pickle=True)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_shard_rays_and_reduce_times(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    ws = 2
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, ws, port, str(tmp_path))) for r in range(ws)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    res = [np.load(tmp_path / f"rank{r}.npy", allow_pickle=True).item() for r in range(ws)]
    # disjoint, reproducible ray sets per rank
    assert not np.array_equal(res[0]["rays"], res[1]["rays"])
    sys.path.insert(0, os.path.join(REPO, "lightmetrica-v2_gb300"))
    from lmgpu import dist as ldist
    from lmgpu import scenes

    for r in range(ws):
        assert np.array_equal(res[r]["rays"], scenes.raycast_rays(512, stream=ldist.ray_stream(r)))
    # the reduction is the element-wise maximum on every rank
    for r in range(ws):
        assert res[r]["red"] == [2.0, 10.0]
    # each rank traced its own rays (some hit the shared scene)
    assert all((x["ids"] >= 0).any() for x in res)
    assert ldist.aggregate_rate(512, ws, 0.5) == 2048.0

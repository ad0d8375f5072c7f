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


def _film_rank_main(rank: int, ws: int, port: int, out_dir: str, golden: str) -> None:
    for p in (os.path.join(REPO, "lightmetrica-v2_gb300"), os.path.join(REPO, "oracle"),
              os.path.join(REPO, "tests")):
        sys.path.insert(0, p)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(ws), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist

    import lmoracle
    import ptscene
    from lmgpu import dist as ldist

    dist.init_process_group("gloo", rank=rank, world_size=ws)
    scene, z = ptscene.load_cornell(golden)
    scene["camera"].update(width=32, height=32)
    spp = 64 * (rank + 1)  # unequal shares: the weights must follow the sample counts
    r = lmoracle.render_pt(scene, 32 * 32 * spp, int(z["max_num_vertices"]), ldist.rank_seed(21, rank), 2)
    img, var, n = ldist.reduce_film(r["image"], r["variance"], spp)
    np.save(os.path.join(out_dir, f"film{rank}.npy"),
            {"img": r["image"], "var": r["variance"], "spp": spp, "red_img": img, "red_var": var, "n": n},
            allow_pickle=True)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_render_and_reduce_the_film(tmp_path, golden_dir):
    """Render sharding (lmgpu/dist.py): two ranks render independent sample
    sets of the same view (64 and 128 spp, seeds from rank_seed) with the
    oracle's renderer::pt, and reduce_film combines them as the reference's
    scheduler combines its workers' films (accumulate, rescale by the total
    sample count, scheduler.cpp:281-288).  Every rank gets the same film: the
    sample-weighted mean, with the variance of that mean, and it agrees with
    one 192-spp render."""
    mp = pytest.importorskip("torch.multiprocessing")
    ws = 2
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_film_rank_main, args=(r, ws, port, str(tmp_path), golden_dir)) for r in range(ws)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=600)
        assert p.exitcode == 0
    res = [np.load(tmp_path / f"film{r}.npy", allow_pickle=True).item() for r in range(ws)]
    n = res[0]["spp"] + res[1]["spp"]
    want = (res[0]["img"] * res[0]["spp"] + res[1]["img"] * res[1]["spp"]) / n
    want_var = (res[0]["var"] * res[0]["spp"] ** 2 + res[1]["var"] * res[1]["spp"] ** 2) / n ** 2
    for r in range(ws):
        assert res[r]["n"] == n == 192
        assert np.allclose(res[r]["red_img"], want, rtol=1e-12, atol=0)
        assert np.allclose(res[r]["red_var"], want_var, rtol=1e-12, atol=0)
    # the two shares are independent sample sets
    assert not np.array_equal(res[0]["img"], res[1]["img"])
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import imgcheck
    import lmoracle
    import ptscene

    scene, z = ptscene.load_cornell(golden_dir)
    scene["camera"].update(width=32, height=32)
    one = lmoracle.render_pt(scene, 32 * 32 * n, int(z["max_num_vertices"]), 99, 4)
    imgcheck.assert_same_aggregates(res[0]["red_img"], res[0]["red_var"], one["image"], one["variance"],
                                    "two-rank film vs one render")

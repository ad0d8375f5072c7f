"""lmgpu_trace_static_scene: the entry point for callers that cannot allocate
device memory (a plugin whose host owns all device memory through its own
pool, or a query path that must not pay the device-wide synchronisation of
cudaMalloc/cudaFree).  It keeps its scratch and the BVH in one fixed
library-owned device array, so its results must equal those of the
allocating path (lmgpu_accel_build_device + lmgpu_trace_device) on the same
inputs, call after call, although every call reuses the same memory: closest
hits exactly, any-hit queries on hit or miss (the blocking triangle an any-hit
query reports depends on the tree, and this path collapses its BVH greedily).
And it must not allocate: after a first call, further calls leave the
device's free memory unchanged.

This file is collected last on purpose: if it fails, a run that stops at the
first failure has already run every other test.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

T_REL_TOL = 1e-5  # hit t, relative (the tolerance of the other parity tests)


def _allocating_path(gpu_lib, dt, ntri, dr, nrays, anyhit, stream):
    import torch

    acc = gpu_lib.Accel()
    acc.build_device(dt.data_ptr(), ntri, stream)
    dh = torch.empty((nrays, 4), dtype=torch.float32, device="cuda")
    acc.trace_device(dr.data_ptr(), dh.data_ptr(), nrays, anyhit, stream)
    acc.check(stream)
    out = dh.cpu().numpy().view(gpu_lib.HIT_DTYPE).reshape(-1).copy()
    acc.close()
    return out


def test_static_scene_matches_allocating_path_two_calls(gpu_lib):
    import torch
    from lmgpu import scenes

    stream = torch.cuda.current_stream().cuda_stream
    # two calls in a row on different scenes (the larger first, so stale
    # contents of the shared scratch would show up in the second)
    cases = [(scenes.raycast_scene(14_000, 30, seed=101), 303), (scenes.random_soup(3_000, seed=202), 404)]
    for tris, ray_seed in cases:
        ntri = tris.shape[0]
        assert ntri <= gpu_lib.STATIC_MAX_TRIANGLES
        rays = scenes.raycast_rays(1 << 16, seed=ray_seed)
        dt = torch.from_numpy(tris).cuda()
        dr = torch.from_numpy(rays).cuda()
        for anyhit in (False, True):
            dh = torch.empty((rays.shape[0], 4), dtype=torch.float32, device="cuda")
            gpu_lib.trace_static_scene(dt.data_ptr(), ntri, dr.data_ptr(), dh.data_ptr(), rays.shape[0], anyhit,
                                       stream)
            got = dh.cpu().numpy().view(gpu_lib.HIT_DTYPE).reshape(-1)
            ref = _allocating_path(gpu_lib, dt, ntri, dr, rays.shape[0], anyhit, stream)
            if anyhit:
                assert np.array_equal(got["prim"] >= 0, ref["prim"] >= 0)
                continue
            assert np.array_equal(got["prim"], ref["prim"])
            hit = ref["prim"] >= 0
            assert hit.any()
            rel = np.abs(got["t"][hit] - ref["t"][hit]) / np.abs(ref["t"][hit])
            assert rel.max() <= T_REL_TOL
            assert np.allclose(got["b1"][hit], ref["b1"][hit], atol=1e-6)
            assert np.allclose(got["b2"][hit], ref["b2"][hit], atol=1e-6)


def test_static_scene_allocates_nothing(gpu_lib):
    """After one call (which looks up the library's array), more calls on
    scenes up to the size limit leave cudaMemGetInfo's free bytes as they
    were."""
    import torch
    from lmgpu import scenes

    stream = torch.cuda.current_stream().cuda_stream
    tris = scenes.random_soup(gpu_lib.STATIC_MAX_TRIANGLES, seed=505)
    rays = scenes.raycast_rays(1 << 16, seed=506)
    dt = torch.from_numpy(tris).cuda()
    dr = torch.from_numpy(rays).cuda()
    dh = torch.empty((rays.shape[0], 4), dtype=torch.float32, device="cuda")
    gpu_lib.trace_static_scene(dt.data_ptr(), tris.shape[0], dr.data_ptr(), dh.data_ptr(), rays.shape[0], False,
                               stream)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for anyhit in (False, True, False):
        gpu_lib.trace_static_scene(dt.data_ptr(), tris.shape[0], dr.data_ptr(), dh.data_ptr(), rays.shape[0],
                                   anyhit, stream)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)


def test_static_scene_rejects_oversize(gpu_lib):
    import torch

    n = gpu_lib.STATIC_MAX_TRIANGLES + 1
    dt = torch.zeros((n, 9), dtype=torch.float32, device="cuda")
    dr = torch.zeros((4, 8), dtype=torch.float32, device="cuda")
    dh = torch.empty((4, 4), dtype=torch.float32, device="cuda")
    with pytest.raises(gpu_lib.LmgpuError) as e:
        gpu_lib.trace_static_scene(dt.data_ptr(), n, dr.data_ptr(), dh.data_ptr(), 4, False,
                                   torch.cuda.current_stream().cuda_stream)
    assert e.value.code == 1
    assert "static limit" in str(e.value)

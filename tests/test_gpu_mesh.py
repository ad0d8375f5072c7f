"""Mesh ingestion on the GPU (lmgpu_flatten_meshes_device,
lmgpu_accel_build_meshes): the triangles equal the reference's own
flattening bit for bit (tests/golden/surface.npz, and the numpy restatement
pinned to it on random meshes), out-of-range face indices are rejected, and an
accel built from meshes answers queries exactly as one built from the
host-flattened triangles."""
import os

import numpy as np
import pytest

import meshflat

pytestmark = pytest.mark.gpu


def gpu_flatten(gpu_lib, meshes):
    import torch

    dm = [(torch.from_numpy(np.ascontiguousarray(p, np.float32)).cuda(),
           torch.from_numpy(np.ascontiguousarray(f, np.uint32).view(np.int32)).cuda(), t) for p, f, t in meshes]
    nf = sum(int(np.asarray(f).size // 3) for _, f, _ in meshes)
    d_tris = torch.empty((max(nf, 1), 9), dtype=torch.float32, device="cuda")
    d_prim = torch.empty(max(nf, 1), dtype=torch.int32, device="cuda")
    gpu_lib.flatten_meshes_device(dm, d_tris.data_ptr(), d_prim.data_ptr())
    torch.cuda.synchronize()
    return d_tris.cpu().numpy()[:nf], d_prim.cpu().numpy()[:nf]


def test_flatten_matches_reference_triangles(gpu_lib, golden_dir):
    z = np.load(os.path.join(golden_dir, "surface.npz"))
    tris, prim = gpu_flatten(gpu_lib, meshflat.fixture_meshes(z))
    assert np.array_equal(tris.view(np.uint32), z["tris32"].view(np.uint32))
    _, ref_prim = meshflat.flatten(meshflat.fixture_meshes(z))
    assert np.array_equal(prim, ref_prim)


def test_flatten_random_meshes_bitexact(gpu_lib):
    """Shared vertices, empty meshes between others, large index ranges."""
    meshes = meshflat.random_meshes(77, [(1000, 3000), (0, 0), (5, 1), (70000, 200000), (3, 0), (17, 40)])
    tris, prim = gpu_flatten(gpu_lib, meshes)
    ref, ref_prim = meshflat.flatten(meshes)
    assert np.array_equal(tris.view(np.uint32), ref.view(np.uint32))
    assert np.array_equal(prim, ref_prim)


def test_out_of_range_face_is_rejected(gpu_lib):
    meshes = meshflat.random_meshes(5, [(10, 20), (10, 20)])
    bad = meshes[1][1].copy()
    bad[7, 2] = 10  # one past the last vertex
    meshes[1] = (meshes[1][0], bad, meshes[1][2])
    with pytest.raises(gpu_lib.LmgpuError):
        gpu_flatten(gpu_lib, meshes)
    acc = gpu_lib.Accel()
    with pytest.raises(gpu_lib.LmgpuError):
        acc.build_meshes(meshes)
    acc.close()


def test_build_meshes_equals_build_of_flattened(gpu_lib):
    from lmgpu import scenes

    meshes = meshflat.random_meshes(9, [(20000, 60000), (500, 900), (0, 0), (3000, 2000)])
    ref, _ = meshflat.flatten(meshes)
    rays = scenes.raycast_rays(50000, seed=3, lo=-30.0, hi=30.0)
    a = gpu_lib.Accel()
    a.build_meshes(meshes)
    b = gpu_lib.Accel()
    b.build(ref)
    ha, hb = a.trace(rays), b.trace(rays)
    assert a.info()["num_triangles"] == ref.shape[0]
    assert np.array_equal(ha["prim"], hb["prim"]) and np.array_equal(ha["t"], hb["t"])
    assert (ha["prim"] >= 0).sum() > 1000
    a.close()
    b.close()

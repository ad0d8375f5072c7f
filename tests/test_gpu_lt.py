"""renderer::ltdirect on the GPU (lmgpu_render_ltdirect: light tracing with a
sensor connection at every vertex) against the reference's own
renderer::ltdirect (double-precision build, tests/golden/cornell_ltdirect.npz)
and the oracle, per pixel within the statistical bar of tests/imgcheck.py."""
import os

import numpy as np
import pytest

import imgcheck
import ptscene

pytestmark = pytest.mark.gpu


def test_ltdirect_matches_reference_film(gpu_lib, golden_dir):
    scene, z = ptscene.load_scene(golden_dir, "cornell_ltdirect")
    sc = gpu_lib.Scene(scene)
    img, var = sc.render_ltdirect(16384, int(z["max_num_vertices"]), 5)
    sc.close()
    a, va = ptscene.downsample(img, var, 2)
    b, vb = ptscene.downsample(z["ref64_image"], z["ref64_variance"], 2)
    print(imgcheck.assert_same_image(a, va, b, vb, "gpu vs ref64 (ltdirect)"))
    print("relMSE vs FP64 reference", imgcheck.relmse(img, z["ref64_image"]))


def test_ltdirect_matches_oracle_on_variant_scene(gpu_lib, oracle_lib, golden_dir):
    """Glass and conductor boxes (no environment), non-square film, shorter
    paths: GPU vs oracle."""
    scene, _ = ptscene.load_scene(golden_dir, "materials_ptmis")
    scene["camera"].update(width=48, height=32, fov=55.0)
    sc = gpu_lib.Scene(scene)
    img, var = sc.render_ltdirect(16384, 6, 13)
    sc.close()
    r = oracle_lib.render_ltdirect(scene, 48 * 32 * 8192, 6, 77, os.cpu_count() or 4)
    a, va = ptscene.downsample(img, var, 2)
    b, vb = ptscene.downsample(r["image"], r["variance"], 2)
    print(imgcheck.assert_same_image(a, va, b, vb, "gpu vs oracle (ltdirect)"))


def test_ltdirect_boundaries_and_device_entry(gpu_lib, golden_dir):
    """max_num_vertices 1 renders nothing, 2 only the directly seen light;
    environment-lit and light-less scenes are rejected; the device entry
    equals the host entry."""
    import torch

    scene, _ = ptscene.load_scene(golden_dir, "cornell_ltdirect")
    sc = gpu_lib.Scene(scene)
    img1, _ = sc.render_ltdirect(64, 1, 1)
    assert not img1.any()
    img2, _ = sc.render_ltdirect(256, 2, 1)
    lit = img2.sum(axis=2) > 0
    assert 0 < lit.sum() < 0.2 * lit.size  # the light's pixels only
    a, va = sc.render_ltdirect(64, 9, 21)
    d_img = torch.empty(a.shape, dtype=torch.float32, device="cuda")
    d_var = torch.empty(a.shape, dtype=torch.float32, device="cuda")
    sc.render_ltdirect_device(d_img.data_ptr(), d_var.data_ptr(), 64, 9, 21)
    torch.cuda.synchronize()
    assert np.array_equal(d_img.cpu().numpy(), a) and np.array_equal(d_var.cpu().numpy(), va)
    sc.close()
    env_scene = dict(scene)
    env_scene["env"] = (1.0, 1.0, 1.0)
    sc = gpu_lib.Scene(env_scene)
    with pytest.raises(gpu_lib.LmgpuError):
        sc.render_ltdirect(4, 9, 1)
    sc.close()
    dark = dict(scene)
    dark["prims"] = [dict(p, light=False) for p in scene["prims"]]
    sc = gpu_lib.Scene(dark)
    with pytest.raises(gpu_lib.LmgpuError):
        sc.render_ltdirect(4, 9, 1)
    sc.close()

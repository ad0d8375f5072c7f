"""renderer::ptmis on the GPU (lmgpu_render_ptmis: next-event estimation,
balance heuristic) and renderer::ptdirect (lmgpu_render_ptdirect) against the reference's own renderer::ptmis
(double-precision build, tests/golden/*_ptmis.npz) and the oracle, per pixel
within the statistical bar of tests/imgcheck.py."""
import os

import numpy as np
import pytest

import imgcheck
import ptscene

pytestmark = pytest.mark.gpu


def render(gpu_lib, scene, spp, max_nv, seed):
    sc = gpu_lib.Scene(scene)
    img, var = sc.render_ptmis(spp, max_nv, seed)
    sc.close()
    return img, var


@pytest.mark.parametrize("name", ["cornell_ptmis", "materials_ptmis"])
def test_ptmis_matches_reference_film(gpu_lib, golden_dir, name):
    scene, z = ptscene.load_scene(golden_dir, name)
    img, var = render(gpu_lib, scene, 16384, int(z["max_num_vertices"]), 7)
    s64 = imgcheck.assert_same_image(img, var, z["ref64_image"], z["ref64_variance"], f"gpu vs ref64 ({name})")
    t = img.astype(np.float64).sum(axis=(0, 1))
    t32 = z["ref_image"].astype(np.float64).sum(axis=(0, 1))
    assert np.all(np.abs(t / t32 - 1.0) < 5e-3), (t, t32)
    print("vs f64", s64, "\nrelMSE vs FP64 reference", imgcheck.relmse(img, z["ref64_image"]))


def test_ptdirect_matches_reference_film(gpu_lib, golden_dir):
    """renderer::ptdirect (light samples only) against the reference's film."""
    scene, z = ptscene.load_scene(golden_dir, "cornell_ptdirect")
    sc = gpu_lib.Scene(scene)
    img, var = sc.render_ptdirect(16384, int(z["max_num_vertices"]), 7)
    sc.close()
    s64 = imgcheck.assert_same_image(img, var, z["ref64_image"], z["ref64_variance"], "gpu vs ref64 (ptdirect)")
    print("vs f64", s64, "\nrelMSE vs FP64 reference", imgcheck.relmse(img, z["ref64_image"]))


def test_ptmis_matches_oracle_on_variant_scene(gpu_lib, oracle_lib, golden_dir):
    """Non-square film, other fov and light colour, shorter paths: GPU vs oracle."""
    scene, _ = ptscene.load_scene(golden_dir, "materials_ptmis")
    scene["camera"].update(width=48, height=32, fov=55.0)
    for p in scene["prims"]:
        if p.get("light"):
            p["Le"] = (4.0, 9.0, 20.0)
    img, var = render(gpu_lib, scene, 16384, 5, 11)
    r = oracle_lib.render_ptmis(scene, 48 * 32 * 8192, 5, 99, os.cpu_count() or 4)
    print(imgcheck.assert_same_image(img, var, r["image"], r["variance"], "gpu vs oracle"))


def test_ptmis_agrees_with_gpu_pt(gpu_lib, golden_dir):
    """Both estimators converge to the same image (16,384 spp, 2 x 2 blocks)."""
    scene, _ = ptscene.load_scene(golden_dir, "cornell_ptmis")
    sc = gpu_lib.Scene(scene)
    a, va = sc.render_ptmis(16384, 9, 3)
    b, vb = sc.render_pt(16384, 9, 4)
    sc.close()
    a, va = ptscene.downsample(a.astype(np.float64), va.astype(np.float64), 2)
    b, vb = ptscene.downsample(b.astype(np.float64), vb.astype(np.float64), 2)
    print(imgcheck.assert_same_image(a, va, b, vb, "ptmis vs pt"))


def test_ptmis_has_lower_variance_than_pt(gpu_lib, golden_dir):
    scene, _ = ptscene.load_scene(golden_dir, "cornell_ptmis")
    sc = gpu_lib.Scene(scene)
    _, va = sc.render_ptmis(1024, 9, 5)
    _, vb = sc.render_pt(1024, 9, 6)
    sc.close()
    assert va.sum() < 0.5 * vb.sum(), (va.sum(), vb.sum())


def test_ptmis_rejects_environment_and_lightless_scenes(gpu_lib, golden_dir):
    scene, _ = ptscene.load_scene(golden_dir, "cornell_ptmis")
    env = dict(scene, env=(0.2, 0.3, 0.5))
    sc = gpu_lib.Scene(env)
    with pytest.raises(gpu_lib.LmgpuError):
        sc.render_ptmis(4, 9, 1)
    sc.close()
    for p in scene["prims"]:
        p["light"] = False
    sc = gpu_lib.Scene(scene)
    with pytest.raises(gpu_lib.LmgpuError):
        sc.render_ptmis(4, 9, 1)
    sc.close()


def test_ptmis_device_entry_matches_host_entry(gpu_lib, golden_dir):
    import torch

    scene, _ = ptscene.load_scene(golden_dir, "cornell_ptmis")
    sc = gpu_lib.Scene(scene)
    a, va = sc.render_ptmis(128, 9, 21)
    di = torch.empty((64, 64, 3), dtype=torch.float32, device="cuda")
    dv = torch.empty((64, 64, 3), dtype=torch.float32, device="cuda")
    sc.render_ptmis_device(di.data_ptr(), dv.data_ptr(), 128, 9, 21, torch.cuda.current_stream().cuda_stream)
    sc.close()
    assert np.allclose(di.cpu().numpy(), a, rtol=1e-4, atol=1e-5)
    assert np.allclose(dv.cpu().numpy(), va, rtol=1e-3, atol=1e-5)

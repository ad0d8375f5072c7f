"""renderer::bdpt on the GPU (lmgpu_render_bdpt) against the reference's own
renderer::bdpt (double-precision build, tests/golden/*_bdpt.npz) and the
oracle, per pixel within the statistical bar of tests/imgcheck.py."""
import os

import numpy as np
import pytest

import imgcheck
import ptscene

pytestmark = pytest.mark.gpu


def render(gpu_lib, scene, spp, max_nv, seed):
    sc = gpu_lib.Scene(scene)
    img, var = sc.render_bdpt(spp, max_nv, seed)
    sc.close()
    return img, var


@pytest.mark.parametrize("name", ["cornell_bdpt", "materials_bdpt"])
def test_bdpt_matches_reference_film(gpu_lib, golden_dir, name):
    """Per pixel against the reference film (32,768 spp, double precision),
    and the image totals against the single-precision film."""
    scene, z = ptscene.load_scene(golden_dir, name)
    img, var = render(gpu_lib, scene, 32768, int(z["max_num_vertices"]), 7)
    s64 = imgcheck.assert_same_image(img, var, z["ref64_image"], z["ref64_variance"], f"gpu vs ref64 ({name})")
    s32 = imgcheck.compare(img, var, z["ref_image"], z["ref_variance"])
    assert max(abs(x) for x in s32["total_z"]) < 4.0, s32
    print("vs f64", s64, "\nvs f32", s32, "\nrelMSE vs FP64 reference", imgcheck.relmse(img, z["ref64_image"]))


def test_bdpt_matches_oracle_on_variant_scene(gpu_lib, oracle_lib, golden_dir):
    """A non-square film, other fov and light colour, shorter paths: GPU vs oracle."""
    scene, _ = ptscene.load_scene(golden_dir, "materials_bdpt")
    scene["camera"].update(width=48, height=32, fov=55.0)
    for p in scene["prims"]:
        if p.get("light"):
            p["Le"] = (4.0, 9.0, 20.0)
    img, var = render(gpu_lib, scene, 16384, 6, 11)
    r = oracle_lib.render_bdpt(scene, 48 * 32 * 4096, 6, 99, os.cpu_count() or 4)
    print(imgcheck.assert_same_image(img, var, r["image"], r["variance"], "gpu vs oracle"))


def test_bdpt_agrees_with_gpu_pt_totals_only_with_reuse_bias(gpu_lib, golden_dir):
    """Sanity of the transport: the GPU BDPT and GPU PT images are both
    non-negative and finite and of the same total order of magnitude (they
    differ by the light-sample reuse of light::area, see the oracle tests)."""
    scene, z = ptscene.load_scene(golden_dir, "cornell_bdpt")
    sc = gpu_lib.Scene(scene)
    b, _ = sc.render_bdpt(1024, 10, 5)
    p, _ = sc.render_pt(1024, 10, 5)
    sc.close()
    assert np.isfinite(b).all() and (b >= 0).all()
    ratio = b.sum() / p.sum()
    assert 0.7 < ratio < 1.3, ratio


def test_bdpt_deterministic_and_seeded(gpu_lib, golden_dir):
    scene, _ = ptscene.load_scene(golden_dir, "cornell_bdpt")
    sc = gpu_lib.Scene(scene)
    a, _ = sc.render_bdpt(256, 10, 3)
    b, _ = sc.render_bdpt(256, 10, 3)
    c, _ = sc.render_bdpt(256, 10, 4)
    sc.close()
    # film sums are float atomics: equal up to summation order
    assert np.allclose(a, b, rtol=1e-4, atol=1e-5)
    assert not np.allclose(a, c)


def test_bdpt_two_vertices_only_lights(gpu_lib, golden_dir):
    scene, _ = ptscene.load_scene(golden_dir, "cornell_bdpt")
    img, _ = render(gpu_lib, scene, 256, 2, 1)
    lit = img.sum(axis=2) > 0
    assert 0 < lit.sum() < 0.08 * lit.size


def test_bdpt_without_light_is_rejected(gpu_lib, golden_dir):
    scene, _ = ptscene.load_scene(golden_dir, "cornell_bdpt")
    for p in scene["prims"]:
        p["light"] = False
    sc = gpu_lib.Scene(scene)
    with pytest.raises(gpu_lib.LmgpuError):
        sc.render_bdpt(4, 10, 1)
    sc.close()


def test_bdpt_device_entry_matches_host_entry(gpu_lib, golden_dir):
    import torch

    scene, _ = ptscene.load_scene(golden_dir, "cornell_bdpt")
    sc = gpu_lib.Scene(scene)
    a, va = sc.render_bdpt(128, 10, 21)
    di = torch.empty((32, 32, 3), dtype=torch.float32, device="cuda")
    dv = torch.empty((32, 32, 3), dtype=torch.float32, device="cuda")
    sc.render_bdpt_device(di.data_ptr(), dv.data_ptr(), 128, 10, 21, torch.cuda.current_stream().cuda_stream)
    sc.close()
    assert np.allclose(di.cpu().numpy(), a, rtol=1e-4, atol=1e-5)
    assert np.allclose(dv.cpu().numpy(), va, rtol=1e-3, atol=1e-5)


def test_bdpt_simple_weight_matches_reference_film(gpu_lib, golden_dir):
    """mis: simple against the reference's own film with that weight.  (It is
    not the power heuristic's image: the strategies that start on the light
    carry the light::area sample-reuse bias, light_area.cpp:73-80, so
    weighting them differently converges elsewhere, in the reference too.)"""
    scene, z = ptscene.load_scene(golden_dir, "cornell_bdpt_simple")
    sc = gpu_lib.Scene(scene)
    img, var = sc.render_bdpt(32768, int(z["max_num_vertices"]), 9, mis="simple")
    sc.close()
    print(imgcheck.assert_same_image(img, var, z["ref64_image"], z["ref64_variance"], "gpu vs ref64 (simple)"))
    print("relMSE vs FP64 reference", imgcheck.relmse(img, z["ref64_image"]))


def test_bdpt_caustic_room_matches_reference_film(gpu_lib, golden_dir):
    """The bidirectional configuration's own scene (a level-5 glass
    icosphere on the floor of a closed 20-triangle room, a 0.05-radius sphere
    light hidden from the camera by a thin panel), max_num_vertices 11, power
    heuristic, on a 48 x 27 film: per pixel against the reference's own
    renderer::bdpt (double precision, 16,384 samples per pixel), and the image
    totals against its single-precision film."""
    scene, z = ptscene.load_scene(golden_dir, "caustic_bdpt")
    assert int(z["max_num_vertices"]) == 11
    img, var = render(gpu_lib, scene, 65536, 11, 23)
    s64 = imgcheck.assert_same_image(img, var, z["ref64_image"], z["ref64_variance"], "gpu vs ref64 (caustic room)")
    s32 = imgcheck.compare(img, var, z["ref_image"], z["ref_variance"])
    assert max(abs(x) for x in s32["total_z"]) < 4.0, s32
    print("vs f64", s64, "\nvs f32", s32, "\nrelMSE vs FP64 reference", imgcheck.relmse(img, z["ref64_image"]))


def test_bdpt_caustic_room_matches_oracle(gpu_lib, oracle_lib, golden_dir):
    """The same scene on a 24 x 14 film with another camera aim: the GPU
    against the oracle's renderer::bdpt (aggregates: the oracle's sample
    count keeps per-pixel statistics short of normal)."""
    scene, _ = ptscene.load_scene(golden_dir, "caustic_bdpt")
    scene["camera"].update(width=24, height=14, center=(0.1, 0.35, 0.2))
    img, var = render(gpu_lib, scene, 32768, 11, 29)
    r = oracle_lib.render_bdpt(scene, 24 * 14 * 2048, 11, 31, os.cpu_count() or 4)
    print(imgcheck.assert_same_aggregates(img, var, r["image"], r["variance"], "gpu vs oracle (caustic room)"))

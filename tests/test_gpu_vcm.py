"""renderer::vcm on the GPU (lmgpu_render_vcm: vertex connection and merging
with a hashed photon grid) against the reference's own renderer::vcm
(tests/golden/cornell_vcm.npz, cornell_bdpm.npz) and the oracle, per pixel
within the statistical bar of tests/imgcheck.py.  The GPU runs each
fixture's radius schedule and photon count (they set the expected image)
with more eye samples per pass."""
import os

import numpy as np
import pytest

import imgcheck
import ptscene
from test_oracle_vcm import VCM_BLOCK_LIMIT, vcm_kw

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["cornell_vcm", "cornell_bdpm"])
def test_vcm_matches_reference_film(gpu_lib, golden_dir, name):
    scene, z = ptscene.load_scene(golden_dir, name)
    sc = gpu_lib.Scene(scene)
    img, var = sc.render_vcm(seed=11, **vcm_kw(z, num_eye_trace_samples=32 * 32 * 4))
    sc.close()
    a, va = ptscene.downsample(img, var, 2)
    b, vb = ptscene.downsample(z["ref_image"], z["ref_variance"], 2)
    print(imgcheck.assert_same_image(a, va, b, vb, f"gpu vs ref ({name})", block_limit=VCM_BLOCK_LIMIT))
    c, vc = ptscene.downsample(z["ref64_image"], z["ref64_variance"], 2)
    print(imgcheck.assert_same_aggregates(a, va, c, vc, f"gpu vs ref64 ({name})", block_limit=VCM_BLOCK_LIMIT))


@pytest.mark.parametrize("mode", ["vcm", "bdpt", "bdpm"])
def test_vcm_matches_oracle_on_variant_scene(gpu_lib, oracle_lib, golden_dir, mode):
    """Glass and conductor boxes (glass vertices are never merged: delta
    direction), non-square film, shorter paths, a minimum path length:
    GPU vs oracle in each mode."""
    scene, _ = ptscene.load_scene(golden_dir, "materials_ptmis")
    scene["camera"].update(width=48, height=32, fov=55.0)
    kw = dict(max_num_vertices=7, min_num_vertices=3, num_iteration_pass=64, num_photon_trace_samples=4096,
              initial_radius=0.04, alpha=0.75, mode=mode)
    sc = gpu_lib.Scene(scene)
    img, var = sc.render_vcm(seed=3, num_eye_trace_samples=48 * 32 * 16, **kw)
    sc.close()
    r = oracle_lib.render_vcm(scene, 7, os.cpu_count() or 4, num_eye_trace_samples=48 * 32 * 2, **kw)
    a, va = ptscene.downsample(img, var, 2)
    b, vb = ptscene.downsample(r["image"], r["variance"], 2)
    print(imgcheck.assert_same_image(a, va, b, vb, f"gpu vs oracle (vcm mode {mode})", block_limit=VCM_BLOCK_LIMIT))


def test_vcm_uniform_raster_positions(gpu_lib, oracle_lib, golden_dir):
    """An eye-sample count that is not a multiple of W x H: raster positions
    uniform over the film, as the reference draws them."""
    scene, z = ptscene.load_scene(golden_dir, "cornell_vcm")
    sc = gpu_lib.Scene(scene)
    img, var = sc.render_vcm(seed=5, **vcm_kw(z, num_eye_trace_samples=32 * 32 * 32 + 77))
    sc.close()
    a, va = ptscene.downsample(img, var, 2)
    c, vc = ptscene.downsample(z["ref64_image"], z["ref64_variance"], 2)
    print(imgcheck.assert_same_aggregates(a, va, c, vc, "gpu (uniform raster) vs ref64", block_limit=VCM_BLOCK_LIMIT))


def test_vcm_boundaries_and_device_entry(gpu_lib, golden_dir):
    """max_num_vertices 1 renders nothing, 2 only the directly seen light
    (bdpm: nothing); unbounded subpaths, an unknown mode, environment-lit and
    light-less scenes are rejected; the device entry renders the host
    entry's image."""
    import torch

    scene, z = ptscene.load_scene(golden_dir, "cornell_vcm")
    sc = gpu_lib.Scene(scene)
    small = dict(num_iteration_pass=4, num_photon_trace_samples=2048, num_eye_trace_samples=4096,
                 initial_radius=0.05)
    img1, _ = sc.render_vcm(max_num_vertices=1, **small)
    assert not img1.any()
    img2, _ = sc.render_vcm(max_num_vertices=2, **small)
    lit = img2.sum(axis=2) > 0
    assert 0 < lit.sum() < 0.2 * lit.size
    img2m, _ = sc.render_vcm(max_num_vertices=2, mode="bdpm", **small)
    assert not img2m.any()
    for bad in (dict(max_num_vertices=-1), dict(max_num_vertices=17), dict(mode="sppm"),
                dict(initial_radius=0.0)):
        with pytest.raises((gpu_lib.LmgpuError, KeyError)):
            sc.render_vcm(**dict(small, **bad))
    a, va = sc.render_vcm(max_num_vertices=6, seed=21, **small)
    d_img = torch.empty(a.shape, dtype=torch.float32, device="cuda")
    d_var = torch.empty(a.shape, dtype=torch.float32, device="cuda")
    sc.render_vcm_device(d_img.data_ptr(), d_var.data_ptr(), max_num_vertices=6, seed=21, **small)
    torch.cuda.synchronize()
    np.testing.assert_allclose(d_img.cpu().numpy(), a, rtol=1e-4, atol=1e-6)
    sc.close()
    env_scene = dict(scene)
    env_scene["env"] = (1.0, 1.0, 1.0)
    sc = gpu_lib.Scene(env_scene)
    with pytest.raises(gpu_lib.LmgpuError):
        sc.render_vcm(**small)
    sc.close()
    dark = dict(scene)
    dark["prims"] = [dict(p, light=False) for p in scene["prims"]]
    sc = gpu_lib.Scene(dark)
    with pytest.raises(gpu_lib.LmgpuError):
        sc.render_vcm(**small)
    sc.close()


def test_vcm_several_eye_waves_per_pass(gpu_lib, golden_dir):
    """At max_num_vertices 8 a wave holds ~355,000 eye samples: 1,048,576
    per pass take three waves, 262,144 one.  Same seed, so both renders share
    their photon subpaths and the first 262,144 eye samples (random numbers
    are keyed by global index); the expected images are equal."""
    scene, _ = ptscene.load_scene(golden_dir, "cornell_vcm")
    common = dict(max_num_vertices=8, num_iteration_pass=8, num_photon_trace_samples=8192, initial_radius=0.05,
                  alpha=0.7, seed=17)
    sc = gpu_lib.Scene(scene)
    a, va = sc.render_vcm(num_eye_trace_samples=32 * 32 * 256, **common)
    b, vb = sc.render_vcm(num_eye_trace_samples=32 * 32 * 1024, **common)
    sc.close()
    print(imgcheck.assert_same_aggregates(a, va, b, vb, "one wave vs three waves per pass",
                                          block_limit=VCM_BLOCK_LIMIT))
    assert np.isfinite(b).all() and (b >= 0).all()

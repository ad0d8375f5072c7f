"""Batched path tracing on the GPU (lmgpu_batch_*): several scenes of their
own resolution rendered by one wavefront with graph-replayed bounces.  Each
view must equal what renderer::pt gives for that scene alone: the reference's
own films (tests/golden/*_pt.npz) per pixel, and lmgpu_render_pt."""
import numpy as np
import pytest

import imgcheck
import ptscene

pytestmark = pytest.mark.gpu


def test_batch_views_match_reference_films(gpu_lib, golden_dir):
    """The Cornell box and the materials box (glass, GGX, environment) in one
    batch, roulette after 3 segments: each view against the reference's
    double-precision film (16,384 spp)."""
    s1, z1 = ptscene.load_cornell(golden_dir)
    s2, z2 = ptscene.load_scene(golden_dir, "materials_pt")
    scs = [gpu_lib.Scene(s1), gpu_lib.Scene(s2)]
    b = gpu_lib.Batch(scs)
    out = b.render_pt(16384, int(z1["max_num_vertices"]), 5, rr_depth=3)
    for (img, var), z, name in zip(out, (z1, z2), ("cornell", "materials")):
        s = imgcheck.assert_same_image(img, var, z["ref64_image"], z["ref64_variance"], f"batch vs ref64 ({name})")
        print(name, s, "relMSE", imgcheck.relmse(img, z["ref64_image"]))
    b.close()
    for sc in scs:
        sc.close()


def test_batch_matches_single_scene_renders(gpu_lib, golden_dir):
    """Mixed resolutions and scenes (a small sphere grid with every BSDF kind
    and an environment, and the Cornell box), reference roulette: each view
    agrees with lmgpu_render_pt of the same scene."""
    from lmgpu import scenes

    grid = scenes.sphere_grid_scene(7, 0, 48, 27, grid=4)
    cb, _ = ptscene.load_cornell(golden_dir)
    cb["camera"].update(width=40, height=40)
    scs = [gpu_lib.Scene(grid), gpu_lib.Scene(cb)]
    b = gpu_lib.Batch(scs)
    out = b.render_pt(8192, 9, 11, rr_depth=0)
    for (img, var), sc in zip(out, scs):
        ref, rvar = sc.render_pt(8192, 9, 12)
        a, va = ptscene.downsample(img.astype(np.float64), var.astype(np.float64), 1)
        print(imgcheck.assert_same_aggregates(a, va, ref.astype(np.float64), rvar.astype(np.float64), "batch vs pt"))
    b.close()
    for sc in scs:
        sc.close()


def test_batch_result_does_not_depend_on_tuning(gpu_lib, golden_dir):
    """Refill / postpone thresholds and the wave size change scheduling only:
    the same seed gives the same film (up to the order of the film sums)."""
    s1, _ = ptscene.load_cornell(golden_dir)
    sc = gpu_lib.Scene(s1)
    b = gpu_lib.Batch([sc])
    a = b.render_pt(64, 9, 3, rr_depth=3)[0][0]
    b.set_tuning(2, 0, 1 << 14)
    c = b.render_pt(64, 9, 3, rr_depth=3)[0][0]
    assert b.tuning()["wave_paths"] == 1 << 14
    assert np.allclose(a, c, rtol=1e-5, atol=1e-6)
    b.close()
    sc.close()


def test_batch_autotune_and_device_entry(gpu_lib, golden_dir):
    import torch

    s1, _ = ptscene.load_cornell(golden_dir)
    s2, _ = ptscene.load_scene(golden_dir, "materials_pt")
    scs = [gpu_lib.Scene(s1), gpu_lib.Scene(s2)]
    b = gpu_lib.Batch(scs)
    t = b.autotune(16, 9, 1, rr_depth=3)
    assert 1 <= t["refill"] <= 32 and 0 <= t["postpone"] <= 32 and t["probe_ms"] > 0
    assert b.tuning()["refill"] == t["refill"]
    host = b.render_pt(32, 9, 21, rr_depth=3)
    n0 = b.launch_count()
    npx = sum(s.width * s.height for s in scs)
    di = torch.empty(3 * npx, dtype=torch.float32, device="cuda")
    dv = torch.empty(3 * npx, dtype=torch.float32, device="cuda")
    b.render_pt_device(di.data_ptr(), dv.data_ptr(), 32, 9, 21, 3, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert b.launch_count() > n0
    flat = np.concatenate([h[0].ravel() for h in host])
    assert np.allclose(di.cpu().numpy(), flat, rtol=1e-4, atol=1e-5)
    b.close()
    for sc in scs:
        sc.close()


def test_sphere_grid_view_matches_reference_film(gpu_lib, golden_dir):
    """One view of the batched configuration (a 4 x 4 grid of level-4
    icospheres in Lambertian, GGX-for-Phong and glass BSDFs on a ground
    plane, an icosphere light and a constant environment; 96 x 54, paths of
    up to 16 segments) batched with the Cornell box: the batched renderer
    (roulette after 3 segments) and lmgpu_render_pt (the reference's
    roulette) each against the reference's own renderer::pt film (double
    precision, 16,384 samples per pixel)."""
    grid, z = ptscene.load_scene(golden_dir, "grid_pt")
    mnv = int(z["max_num_vertices"])
    assert mnv == 17
    cb, _ = ptscene.load_cornell(golden_dir)
    cb["camera"].update(width=40, height=24)
    scs = [gpu_lib.Scene(grid), gpu_lib.Scene(cb)]
    b = gpu_lib.Batch(scs)
    (img, var), _ = b.render_pt(32768, mnv, 41, rr_depth=3)
    s = imgcheck.assert_same_image(img, var, z["ref64_image"], z["ref64_variance"], "batch vs ref64 (sphere grid)")
    print("batch", s, "relMSE", imgcheck.relmse(img, z["ref64_image"]))
    b.close()
    img, var = scs[0].render_pt(32768, mnv, 43)
    s = imgcheck.assert_same_image(img, var, z["ref64_image"], z["ref64_variance"], "pt vs ref64 (sphere grid)")
    print("pt", s, "relMSE", imgcheck.relmse(img, z["ref64_image"]))
    for sc in scs:
        sc.close()

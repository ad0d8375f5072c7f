"""The traversal instrumentation of a scene's and a batch's renders
(lmgpu_scene_set_trace_profile / lmgpu_scene_read_trace_profile and the
lmgpu_batch_* pair): the counting
mode runs the counting traversal, the timing mode the production one with
events; neither changes the image, and the counts agree with the renders'
own arithmetic."""
import numpy as np
import pytest

import ptscene

pytestmark = pytest.mark.gpu


def _images_match(a, b):
    # the film sums splats in FP64 with atomics: the order of additions, not
    # the values, may differ between two renders of the same seed
    assert np.allclose(a, b, rtol=1e-6, atol=1e-7)


@pytest.mark.parametrize("renderer", ["pt", "ptmis", "bdpt", "ltdirect"])
def test_trace_profile_counts_and_times_without_changing_the_image(gpu_lib, golden_dir, renderer):
    scene, _ = ptscene.load_cornell(golden_dir)
    scene["camera"].update(width=64, height=48)
    spp, max_nv, seed = 16, 6, 5
    sc = gpu_lib.Scene(scene)
    render = getattr(sc, "render_" + renderer)
    img0, _ = render(spp, max_nv, seed)

    sc.set_trace_profile(gpu_lib.TRACE_PROFILE_COUNT)
    img1, _ = render(spp, max_nv, seed)
    c = sc.read_trace_profile()
    sc.set_trace_profile(gpu_lib.TRACE_PROFILE_TIME)
    img2, _ = render(spp, max_nv, seed)
    t = sc.read_trace_profile()
    sc.set_trace_profile(gpu_lib.TRACE_PROFILE_OFF)
    img3, _ = render(spp, max_nv, seed)
    off = sc.read_trace_profile()
    sc.close()

    for im in (img1, img2, img3):
        _images_match(im, img0)
    n = 64 * 48 * spp
    # every sample traces its camera (or light) ray; later bounces trace fewer
    assert c["rays"] >= n
    assert 0 < c["hits"] <= c["rays"]
    assert c["node_fetches"] >= c["rays"]
    assert c["triangle_fetches"] >= c["hits"]
    assert c["device_ms"] == 0.0 and c["timed_launches"] == 0
    # the same launches in both modes, every one of them timed
    assert c["launches"] == t["launches"] > 0
    assert t["timed_launches"] == t["launches"]
    assert t["device_ms"] > 0.0
    assert t["rays"] == 0 and t["node_fetches"] == 0
    assert off == {k: 0 for k in off} | {"device_ms": 0.0}


def test_trace_profile_rays_of_one_bounce(gpu_lib, golden_dir):
    """With max_num_vertices 2 a path-tracer sample traces exactly its camera ray."""
    scene, _ = ptscene.load_cornell(golden_dir)
    scene["camera"].update(width=32, height=32)
    sc = gpu_lib.Scene(scene)
    sc.set_trace_profile(gpu_lib.TRACE_PROFILE_COUNT)
    sc.render_pt(8, 2, 3)
    c = sc.read_trace_profile()
    sc.close()
    assert c["launches"] == 1
    assert c["rays"] == 32 * 32 * 8


def test_batch_trace_profile(gpu_lib, golden_dir):
    """The batch renderer's profile: bounces launched one by one instead of
    through the captured graphs give the same films; with max_num_vertices 2
    each sample traces exactly its camera ray, in one traversal launch."""
    from lmgpu import scenes

    cb, _ = ptscene.load_cornell(golden_dir)
    cb["camera"].update(width=40, height=30)
    grid = scenes.sphere_grid_scene(7, 0, 48, 27, grid=4)
    scs = [gpu_lib.Scene(cb), gpu_lib.Scene(grid)]
    b = gpu_lib.Batch(scs)
    spp, seed = 8, 9
    base = b.render_pt(spp, 9, seed, rr_depth=3)

    b.set_trace_profile(gpu_lib.TRACE_PROFILE_COUNT)
    counted = b.render_pt(spp, 9, seed, rr_depth=3)
    c = b.read_trace_profile()
    b.set_trace_profile(gpu_lib.TRACE_PROFILE_TIME)
    timed = b.render_pt(spp, 9, seed, rr_depth=3)
    t = b.read_trace_profile()
    b.set_trace_profile(gpu_lib.TRACE_PROFILE_COUNT)
    b.render_pt(spp, 2, seed, rr_depth=3)
    one = b.read_trace_profile()
    b.set_trace_profile(gpu_lib.TRACE_PROFILE_OFF)
    after = b.render_pt(spp, 9, seed, rr_depth=3)
    b.close()
    for sc in scs:
        sc.close()

    for out in (counted, timed, after):
        for (img, _), (ref, _) in zip(out, base):
            _images_match(img, ref)
    n = (40 * 30 + 48 * 27) * spp
    assert c["rays"] >= n and 0 < c["hits"] <= c["rays"]
    assert c["node_fetches"] >= c["rays"] and c["triangle_fetches"] >= c["hits"]
    assert c["launches"] == t["launches"] == t["timed_launches"] > 0
    assert t["device_ms"] > 0.0 and t["rays"] == 0
    assert one["launches"] == 1 and one["rays"] == n


@pytest.mark.parametrize("mode", ["vcm", "bdpt"])
def test_vcm_merge_profile(gpu_lib, golden_dir, mode):
    """renderer::vcm's photon merges in the profile: the counting merge and
    the timed one leave the image as it was (up to the order of the float
    sums of the merges), the counts hold together, and mode bdpt merges
    nothing."""
    scene, _ = ptscene.load_scene(golden_dir, "materials_ptmis")
    scene["camera"].update(width=48, height=32)
    kw = dict(max_num_vertices=7, num_iteration_pass=4, num_photon_trace_samples=4096,
              num_eye_trace_samples=48 * 32 * 4, initial_radius=0.04, alpha=0.75, mode=mode, seed=5)
    sc = gpu_lib.Scene(scene)
    img0, _ = sc.render_vcm(**kw)
    sc.set_trace_profile(gpu_lib.TRACE_PROFILE_COUNT)
    img1, _ = sc.render_vcm(**kw)
    c = sc.read_trace_profile()
    sc.set_trace_profile(gpu_lib.TRACE_PROFILE_TIME)
    img2, _ = sc.render_vcm(**kw)
    t = sc.read_trace_profile()
    sc.set_trace_profile(gpu_lib.TRACE_PROFILE_OFF)
    sc.close()

    for im in (img1, img2):
        assert np.allclose(im, img0, rtol=1e-4, atol=1e-6)
    assert c["launches"] == t["launches"] > 0 and c["rays"] > 0
    if mode == "bdpt":
        assert c["merge_launches"] == t["merge_launches"] == 0
        assert c["merge_queries"] == 0 and t["merge_ms"] == 0.0
        return
    assert c["merge_launches"] == t["merge_launches"] == t["merge_timed_launches"] > 0
    assert c["merge_queries"] > 0
    # a query at eye vertex t reads the t vertices of its eye subpath, t >= 2
    assert c["merge_eye_vertices"] >= 2 * c["merge_queries"]
    assert 0 < c["merges"] <= c["merge_entries"]
    assert c["merge_ms"] == 0.0 and c["merge_timed_launches"] == 0
    assert t["merge_ms"] > 0.0 and t["merge_queries"] == 0

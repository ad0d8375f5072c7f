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

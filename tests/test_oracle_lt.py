"""Pins the oracle's renderer::ltdirect restatement (oracle/lmoracle_bdpt.c,
light tracing with a sensor connection at every vertex) against the film of
the reference's own renderer::ltdirect (tests/golden/cornell_ltdirect.npz:
64x64x16,384 light paths, made by tests/golden/make_golden.py from the
compiled reference sources)."""
import os

import imgcheck
import ptscene


def test_oracle_ltdirect_matches_reference(oracle_lib, golden_dir):
    scene, z = ptscene.load_scene(golden_dir, "cornell_ltdirect")
    W, H = scene["camera"]["width"], scene["camera"]["height"]
    r = oracle_lib.render_ltdirect(scene, W * H * 4096, int(z["max_num_vertices"]), 2468, os.cpu_count() or 4)
    a, va = ptscene.downsample(r["image"], r["variance"], 2)
    b, vb = ptscene.downsample(z["ref64_image"], z["ref64_variance"], 2)
    print(imgcheck.assert_same_image(a, va, b, vb, "oracle vs ref64 (ltdirect)"))


def test_light_sample_reuse_is_the_ltdirect_pt_difference(oracle_lib, golden_dir):
    """The reference's renderer::ltdirect, like its renderer::bdpt, converges
    to a different image than renderer::pt: light::area draws the emission
    direction from the same 2D sample as the emission point
    (light_area.cpp:73-80).  With that one line changed (the oracle's
    diagnostic variant) the light tracer agrees with the path-tracing film;
    the reference's own ltdirect film does not."""
    scene, zl = ptscene.load_scene(golden_dir, "cornell_ltdirect")
    _, zp = ptscene.load_cornell(golden_dir)
    W, H = scene["camera"]["width"], scene["camera"]["height"]
    a, va = ptscene.downsample(zp["ref64_image"], zp["ref64_variance"], 2)
    indep = oracle_lib.render_ltdirect(scene, W * H * 4096, int(zl["max_num_vertices"]), 31,
                                       os.cpu_count() or 4, independent_light_dir=True)
    b, vb = ptscene.downsample(indep["image"], indep["variance"], 2)
    print(imgcheck.assert_same_aggregates(b, vb, a, va, "ltdirect (independent) vs pt"))
    c, vc = ptscene.downsample(zl["ref64_image"], zl["ref64_variance"], 2)
    s = imgcheck.compare(c, vc, a, va)
    assert s["block_max_abs_z"] > 10.0, s

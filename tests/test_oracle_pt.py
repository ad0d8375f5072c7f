"""Pins the oracle's renderer::pt restatement (oracle/lmoracle_pt.c) against
the film of the reference's own renderer::pt (tests/golden/cornell_pt.npz,
made by tests/golden/make_golden.py from the compiled reference sources).

Path tracing is compared statistically: per-pixel z-scores with the
variance of both estimates (tests/imgcheck.py)."""
import os

import numpy as np

import imgcheck
import ptscene


def test_reference_single_and_double_precision_agree(golden_dir):
    _, z = ptscene.load_cornell(golden_dir)
    imgcheck.assert_same_image(z["ref_image"], z["ref_variance"], z["ref64_image"], z["ref64_variance"], "ref f32/f64")


def test_oracle_pt_matches_reference(oracle_lib, golden_dir):
    scene, z = ptscene.load_cornell(golden_dir)
    W, H = scene["camera"]["width"], scene["camera"]["height"]
    # 4096 samples per pixel, compared on 2 x 2 pixel blocks (16K samples per block)
    r = oracle_lib.render_pt(scene, W * H * 4096, int(z["max_num_vertices"]), 1234, os.cpu_count() or 4)
    a, va = ptscene.downsample(r["image"], r["variance"], 2)
    b, vb = ptscene.downsample(z["ref_image"].astype(np.float64), z["ref_variance"].astype(np.float64), 2)
    s = imgcheck.assert_same_image(a, va, b, vb, "oracle vs ref")
    print(s)


def test_oracle_pt_max_vertices_two_sees_only_lights(oracle_lib, golden_dir):
    """max_num_vertices = 2: sensor + one surface vertex, so only directly
    seen emitters contribute (renderer_pt.cpp:120-123)."""
    scene, _ = ptscene.load_cornell(golden_dir)
    W, H = scene["camera"]["width"], scene["camera"]["height"]
    r = oracle_lib.render_pt(scene, W * H * 64, 2, 5, 4)
    lit = r["image"].sum(axis=2) > 0
    assert 0 < lit.sum() < 0.05 * W * H


def test_oracle_pt_materials_match_reference(oracle_lib, golden_dir):
    """Glass (bsdf::flesnel), GGX conductor (bsdf::cook_torrance) and a
    constant environment light, against the reference's film."""
    scene, z = ptscene.load_scene(golden_dir, "materials_pt")
    W, H = scene["camera"]["width"], scene["camera"]["height"]
    imgcheck.assert_same_image(z["ref_image"], z["ref_variance"], z["ref64_image"], z["ref64_variance"], "ref f32/f64")
    r = oracle_lib.render_pt(scene, W * H * 4096, int(z["max_num_vertices"]), 4321, os.cpu_count() or 4)
    a, va = ptscene.downsample(r["image"], r["variance"], 2)
    b, vb = ptscene.downsample(z["ref_image"].astype(np.float64), z["ref_variance"].astype(np.float64), 2)
    print(imgcheck.assert_same_image(a, va, b, vb, "oracle vs ref (materials)"))


def test_oracle_pt_matches_reference_on_sphere_grid(oracle_lib, golden_dir):
    """A view of the batched configuration's sphere grid (every BSDF kind,
    an icosphere light, the environment; paths of up to 16 segments): the
    oracle's renderer::pt against the reference's own film (aggregates at the
    oracle's 256 samples per pixel)."""
    scene, z = ptscene.load_scene(golden_dir, "grid_pt")
    W, H = scene["camera"]["width"], scene["camera"]["height"]
    r = oracle_lib.render_pt(scene, W * H * 256, int(z["max_num_vertices"]), 77, os.cpu_count() or 4)
    print(imgcheck.assert_same_aggregates(r["image"], r["variance"], z["ref64_image"], z["ref64_variance"],
                                          "oracle vs ref64 (sphere grid)"))

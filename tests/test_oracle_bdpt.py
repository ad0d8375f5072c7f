"""Pins the oracle's renderer::bdpt restatement (oracle/lmoracle_bdpt.c)
against the films of the reference's own renderer::bdpt
(tests/golden/cornell_bdpt.npz, materials_bdpt.npz; 32x32, 32,768 samples
per pixel, made by tests/golden/make_golden.py from the compiled reference
sources).

The double-precision reference build is the pin.  The single-precision
build agrees with it in the image totals but not per pixel: its light
subpath connections near sharp edges differ by up to ~16 sigma in 4 x 4
blocks (the float build's approximate vector normalisation), so per-pixel
comparisons use the double-precision film."""
import os

import numpy as np
import pytest

import imgcheck
import ptscene

SCENES = ["cornell_bdpt", "materials_bdpt"]


@pytest.mark.parametrize("name", SCENES)
def test_reference_single_and_double_precision_totals_agree(golden_dir, name):
    _, z = ptscene.load_scene(golden_dir, name)
    s = imgcheck.compare(z["ref_image"], z["ref_variance"], z["ref64_image"], z["ref64_variance"])
    assert max(abs(x) for x in s["total_z"]) < 4.0, s


@pytest.mark.parametrize("name", SCENES)
def test_oracle_bdpt_matches_reference(oracle_lib, golden_dir, name):
    scene, z = ptscene.load_scene(golden_dir, name)
    W, H = scene["camera"]["width"], scene["camera"]["height"]
    r = oracle_lib.render_bdpt(scene, W * H * 4096, int(z["max_num_vertices"]), 1234, os.cpu_count() or 4)
    print(imgcheck.assert_same_image(r["image"], r["variance"], z["ref64_image"], z["ref64_variance"],
                                     f"oracle vs ref64 ({name})"))


def test_light_sample_reuse_is_the_bdpt_pt_difference(oracle_lib, golden_dir):
    """renderer::bdpt and renderer::pt of the reference converge to different
    images: light::area draws the emitted direction from the same 2D sample as
    the emission point (light_area.cpp:73-80), which correlates the two and
    biases every strategy that starts on the light.  With that one line
    changed (the oracle's diagnostic variant) BDPT agrees with the
    path-tracing film; as the reference has it, it does not."""
    scene, _ = ptscene.load_scene(golden_dir, "cornell_bdpt")
    _, zp = ptscene.load_cornell(golden_dir)
    W, H = scene["camera"]["width"], scene["camera"]["height"]
    a, va = ptscene.downsample(zp["ref64_image"], zp["ref64_variance"], 2)
    indep = oracle_lib.render_bdpt(scene, W * H * 4096, 9, 77, os.cpu_count() or 4, independent_light_dir=True)
    print(imgcheck.assert_same_aggregates(indep["image"], indep["variance"], a, va, "bdpt (independent) vs pt"))
    reuse = oracle_lib.render_bdpt(scene, W * H * 4096, 9, 77, os.cpu_count() or 4)
    s = imgcheck.compare(reuse["image"], reuse["variance"], a, va)
    assert s["block_max_abs_z"] > 10.0, s


def test_oracle_bdpt_no_light_is_black(oracle_lib, golden_dir):
    scene, _ = ptscene.load_scene(golden_dir, "cornell_bdpt")
    for p in scene["prims"]:
        if "light" in p:
            p["light"] = False
        else:
            p["kind"] = 0
    r = oracle_lib.render_bdpt(scene, 32 * 32 * 4, 10, 1, 2)
    assert not r["image"].any()


def test_oracle_bdpt_simple_weight_matches_reference(oracle_lib, golden_dir):
    """mis: simple (misweight::simple, one over the number of strategies that
    can sample the path) against the reference's own film with that weight."""
    scene, z = ptscene.load_scene(golden_dir, "cornell_bdpt_simple")
    W, H = scene["camera"]["width"], scene["camera"]["height"]
    r = oracle_lib.render_bdpt(scene, W * H * 4096, int(z["max_num_vertices"]), 4321, os.cpu_count() or 4,
                               mis="simple")
    print(imgcheck.assert_same_image(r["image"], r["variance"], z["ref64_image"], z["ref64_variance"],
                                     "oracle vs ref64 (bdpt, simple weight)"))


def test_oracle_bdpt_matches_reference_on_caustic_room(oracle_lib, golden_dir):
    """The bidirectional configuration's caustic room (glass icosphere,
    sphere light behind a panel), max_num_vertices 11, power heuristic: the
    oracle's renderer::bdpt against the reference's own film (aggregates at
    the oracle's 256 samples per pixel)."""
    scene, z = ptscene.load_scene(golden_dir, "caustic_bdpt")
    W, H = scene["camera"]["width"], scene["camera"]["height"]
    r = oracle_lib.render_bdpt(scene, W * H * 256, int(z["max_num_vertices"]), 78, os.cpu_count() or 4)
    print(imgcheck.assert_same_aggregates(r["image"], r["variance"], z["ref64_image"], z["ref64_variance"],
                                          "oracle vs ref64 (caustic room)"))

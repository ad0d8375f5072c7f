"""Pins the oracle's renderer::ptmis and renderer::ptdirect restatement (oracle/lmoracle_bdpt.c,
next-event estimation with the balance heuristic) against the films of the
reference's own renderer::ptmis (tests/golden/cornell_ptmis.npz,
materials_ptmis.npz; 64x64, 16,384 samples per pixel, made by
tests/golden/make_golden.py from the compiled reference sources)."""
import os

import numpy as np
import pytest

import imgcheck
import ptscene

SCENES = ["cornell_ptmis", "materials_ptmis"]


@pytest.mark.parametrize("name", SCENES)
def test_reference_single_and_double_precision_totals_agree(golden_dir, name):
    """The single-precision reference sums its film in FP32, which at 16,384
    samples per pixel drops small splats (the Cornell film's totals come out
    0.13 % low, 4.5 sigma): the two builds agree within 0.5 % relative, and
    per-pixel checks use the double-precision film."""
    _, z = ptscene.load_scene(golden_dir, name)
    t32 = z["ref_image"].astype(np.float64).sum(axis=(0, 1))
    t64 = z["ref64_image"].sum(axis=(0, 1))
    assert np.all(np.abs(t32 / t64 - 1.0) < 5e-3), (t32, t64)


@pytest.mark.parametrize("name", SCENES)
def test_oracle_ptmis_matches_reference(oracle_lib, golden_dir, name):
    scene, z = ptscene.load_scene(golden_dir, name)
    W, H = scene["camera"]["width"], scene["camera"]["height"]
    r = oracle_lib.render_ptmis(scene, W * H * 4096, int(z["max_num_vertices"]), 1234, os.cpu_count() or 4)
    a, va = ptscene.downsample(r["image"], r["variance"], 2)
    b, vb = ptscene.downsample(z["ref64_image"], z["ref64_variance"], 2)
    print(imgcheck.assert_same_image(a, va, b, vb, f"oracle vs ref64 ({name})"))


def test_oracle_ptdirect_matches_reference(oracle_lib, golden_dir):
    """renderer::ptdirect (light samples only, weight 1) against the
    reference's own ptdirect film."""
    scene, z = ptscene.load_scene(golden_dir, "cornell_ptdirect")
    W, H = scene["camera"]["width"], scene["camera"]["height"]
    r = oracle_lib.render_ptmis(scene, W * H * 4096, int(z["max_num_vertices"]), 4321, os.cpu_count() or 4,
                                direct_only=True)
    a, va = ptscene.downsample(r["image"], r["variance"], 2)
    b, vb = ptscene.downsample(z["ref64_image"], z["ref64_variance"], 2)
    print(imgcheck.assert_same_image(a, va, b, vb, "oracle vs ref64 (ptdirect)"))


def test_ptmis_and_pt_agree(golden_dir):
    """Next-event estimation changes the variance, not the image: the
    reference's ptmis and pt films of the Cornell box (both double precision,
    16,384 spp) agree in 2 x 2 blocks."""
    _, zm = ptscene.load_scene(golden_dir, "cornell_ptmis")
    _, zp = ptscene.load_cornell(golden_dir)
    a, va = ptscene.downsample(zm["ref64_image"], zm["ref64_variance"], 2)
    b, vb = ptscene.downsample(zp["ref64_image"], zp["ref64_variance"], 2)
    print(imgcheck.assert_same_aggregates(a, va, b, vb, "ptmis vs pt (reference)"))

"""Pins the oracle's renderer::vcm restatement (oracle/lmoracle_bdpt.c:
SubpathSampler subpaths, connections and merges, EvaluateMISWeight_VCM /
_BDPM) against the films of the reference's own renderer::vcm
(tests/golden/cornell_vcm.npz and cornell_bdpm.npz: 32x32, 256 passes of
8,192 photon subpaths and 8,192 eye samples, made by
tests/golden/make_golden.py from the compiled reference sources).  The
oracle runs the fixture's radius schedule and photon count, which set the
expected image, with fewer eye samples per pass."""
import os

import numpy as np
import pytest

import imgcheck
import ptscene


# Every eye sample of a pass merges with the same photon subpaths, so
# neighbouring pixels are correlated within a pass and the per-pixel
# variances understate the variance of 8 x 8 block means: the block bound is
# wider than imgcheck's default 4.5.
VCM_BLOCK_LIMIT = 6.0


def vcm_kw(z, **over):
    kw = {k: (float(z[k]) if k in ("initial_radius", "alpha") else int(z[k]))
          for k in ("max_num_vertices", "num_iteration_pass", "num_photon_trace_samples", "num_eye_trace_samples",
                    "initial_radius", "alpha")}
    kw["mode"] = str(z["mode"])
    kw.update(over)
    return kw


@pytest.mark.parametrize("name", ["cornell_vcm", "cornell_bdpm"])
def test_oracle_vcm_matches_reference(oracle_lib, golden_dir, name):
    scene, z = ptscene.load_scene(golden_dir, name)
    r = oracle_lib.render_vcm(scene, 1357, os.cpu_count() or 4, **vcm_kw(z, num_eye_trace_samples=1024))
    a, va = ptscene.downsample(r["image"], r["variance"], 2)
    b, vb = ptscene.downsample(z["ref_image"], z["ref_variance"], 2)
    print(imgcheck.assert_same_image(a, va, b, vb, f"oracle vs ref ({name})", block_limit=VCM_BLOCK_LIMIT))
    c, vc = ptscene.downsample(z["ref64_image"], z["ref64_variance"], 2)
    print(imgcheck.assert_same_aggregates(a, va, c, vc, f"oracle vs ref64 ({name})", block_limit=VCM_BLOCK_LIMIT))


def test_vcm_without_merges_is_its_bdpt_mode(oracle_lib, golden_dir):
    """mode bdpt (connections, EvaluateMISWeight_BDPT) and mode vcm converge
    to the same image: merging only redistributes weight (renderer_vcm.cpp
    :278-320); bdpm misses the paths no merge can make (those seen directly,
    and s = 0 paths in general) and is darker."""
    scene, z = ptscene.load_scene(golden_dir, "cornell_vcm")
    kw = vcm_kw(z, num_iteration_pass=32, num_eye_trace_samples=4096)
    b = oracle_lib.render_vcm(scene, 99, os.cpu_count() or 4, **dict(kw, mode="bdpt"))
    a, va = ptscene.downsample(b["image"], b["variance"], 2)
    c, vc = ptscene.downsample(z["ref64_image"], z["ref64_variance"], 2)
    print(imgcheck.assert_same_aggregates(a, va, c, vc, "oracle bdpt mode vs ref64 vcm", block_limit=VCM_BLOCK_LIMIT))
    _, zb = ptscene.load_scene(golden_dir, "cornell_bdpm")
    assert zb["ref64_image"].sum() < 0.8 * z["ref64_image"].sum()
    # the light itself is black in bdpm (no strategy samples a 2-vertex path)
    lit = z["ref64_image"].sum(axis=2) > 10.0
    assert lit.any() and np.all(zb["ref64_image"][lit].sum(axis=1) < 1.0)


def test_vcm_edge_parameters(oracle_lib, golden_dir):
    """max_num_vertices 1 renders nothing (no strategy has two vertices);
    zero passes render nothing."""
    scene, z = ptscene.load_scene(golden_dir, "cornell_vcm")
    r = oracle_lib.render_vcm(scene, 5, 2, **vcm_kw(z, max_num_vertices=1, num_iteration_pass=2,
                                                    num_eye_trace_samples=256))
    assert not r["image"].any()
    r = oracle_lib.render_vcm(scene, 5, 2, **vcm_kw(z, num_iteration_pass=0))
    assert not r["image"].any() and r["samples"] == 0

"""Pins the CPU oracle (oracle/) against fixtures produced by the reference
itself (tests/golden/make_golden.py runs the reference's accel sources).

The oracle must reproduce the reference bit for bit: same hit ids, hit
points and barycentrics for accel::naive, accel::bvh_sahbin and accel::qbvh
(the reference's fastest native accel, which the benchmark's CPU arm times).  The accel
test cases additionally check the analytic values the reference's own test
asserts (src/lightmetrica-test/test_accel3.cpp:272-345) within its 1e-3.
"""
import os

import numpy as np
import pytest

import hitcheck


def load(golden_dir, name):
    return dict(np.load(os.path.join(golden_dir, name + ".npz")))


@pytest.mark.parametrize("case", ["accel3_simple", "accel3_simple2", "soup_small"])
@pytest.mark.parametrize("kind,tag", [(0, "naive"), (1, "bvh_sahbin"), (2, "qbvh")])
def test_oracle_matches_reference_bitwise(oracle_lib, golden_dir, case, kind, tag):
    z = load(golden_dir, case)
    acc = oracle_lib.OracleAccel(kind, z["tris"])
    h = acc.trace(z["rays"], threads=4)
    assert np.array_equal(h["id"], z[f"{tag}_id"])
    hit = h["id"] >= 0
    assert np.array_equal(h["p"][hit], z[f"{tag}_p"][hit])
    assert np.array_equal(h["b0"][hit], z[f"{tag}_b"][hit, 0])
    assert np.array_equal(h["b1"][hit], z[f"{tag}_b"][hit, 1])


@pytest.mark.parametrize("case", ["accel3_simple", "accel3_simple2"])
def test_oracle_accel3_expected_values(oracle_lib, golden_dir, case):
    """The checks of Accel3Test.Simple / Simple2 applied to the oracle."""
    z = load(golden_dir, case)
    acc = oracle_lib.OracleAccel(0, z["tris"])
    h = acc.trace(z["rays"])
    tol = float(z["tolerance"])
    assert (h["id"] >= 0).all()
    for i in range(len(h)):
        r = z["rays"][i]
        p, gn, sn, uv = hitcheck.hit_geometry(z["positions"], z["normals"], z["texcoords"], z["faces"],
                                              int(h["id"][i]), float(h["b0"][i]), float(h["b1"][i]),
                                              r[0:3], r[4:7], float(h["t"][i]))
        assert np.allclose(p, z["expected_p"][i], atol=tol)
        assert np.allclose(h["p"][i], z["expected_p"][i], atol=tol)
        assert np.allclose(gn, z["expected_gn"][i], atol=tol)
        assert np.allclose(sn, z["expected_sn"][i], atol=tol)
        assert np.allclose(uv, z["expected_uv"][i], atol=tol)


def test_reference_accels_agree_up_to_classified_cases(oracle_lib, golden_dir):
    """The reference's own accels (naive, bvh_sahbin, qbvh) disagree only on
    the documented classes; this calibrates the classifier the GPU tests use."""
    z = load(golden_dir, "soup_small")
    for other in ("bvh_sahbin", "qbvh"):
        c = hitcheck.classify(z["tris"], z["rays"], z["naive_id"], z[f"{other}_id"])
        assert c["unexplained"] == [], (other, c)


def test_oracle_qbvh_matches_live_reference(oracle_lib):
    """accel::qbvh on a 100k-triangle soup and heightfield, 65,536 rays: the
    oracle against the reference's own qbvh compiled from its sources
    (oracle/_ref/ref_accel, built where the reference tree is present)."""
    import subprocess
    import tempfile

    from lmgpu import scenes

    if not os.access(oracle_lib.REF_ACCEL, os.X_OK):
        pytest.skip("reference harness oracle/_ref/ref_accel not built here")
    tris = scenes.raycast_scene(100_000, 96, seed=21)
    rays = scenes.raycast_rays(1 << 16, seed=22)
    with tempfile.TemporaryDirectory() as tmp:
        ps, pr, po = (os.path.join(tmp, x) for x in ("s.bin", "r.bin", "o.bin"))
        oracle_lib.write_ref_inputs(ps, pr, [tris], rays)
        subprocess.run([oracle_lib.REF_ACCEL, "accel::qbvh", ps, pr, po, "4"], check=True, capture_output=True)
        ref = oracle_lib.read_ref_output(po)
    h = oracle_lib.OracleAccel(oracle_lib.QBVH, tris).trace(rays, threads=4)
    assert np.array_equal(h["id"], ref["id"])
    hit = h["id"] >= 0
    assert hit.mean() > 0.3
    assert np.array_equal(h["p"][hit], ref["p"][hit])
    assert np.array_equal(h["b0"][hit], ref["b"][hit, 0])


def test_oracle_qbvh_coincident_centroids(oracle_lib):
    """Twenty copies of one triangle (every centroid equal: the reference's
    qbvh build divides 0 by 0 there) build and trace; the tie goes to one of
    the copies."""
    tri = np.array([0, 0, 0, 1, 0, 0, 0, 1, 0], dtype=np.float32)
    tris = np.tile(tri, (20, 1))
    rays = np.array([[0.25, 0.25, 1, 1e-4, 0, 0, -1, 3.4e38]], dtype=np.float32)
    h = oracle_lib.OracleAccel(2, tris).trace(rays)
    assert 0 <= h["id"][0] < 20 and abs(h["t"][0] - 1.0) < 1e-6


def test_oracle_empty_scene(oracle_lib):
    rays = np.array([[0, 0, 0, 1e-4, 0, 0, 1, 3.4e38]], dtype=np.float32)
    for kind in (0, 1, 2):
        h = oracle_lib.OracleAccel(kind, np.zeros((0, 9), np.float32)).trace(rays)
        assert h["id"][0] == -1


def test_oracle_tie_rule_highest_index(oracle_lib):
    """accel::naive keeps the last of equal-t candidates (triaccel.h:137)."""
    tri = np.array([0, 0, 0, 1, 0, 0, 0, 1, 0], dtype=np.float32)
    tris = np.stack([tri, tri, tri])
    rays = np.array([[0.25, 0.25, 1, 1e-4, 0, 0, -1, 3.4e38]], dtype=np.float32)
    h = oracle_lib.OracleAccel(0, tris).trace(rays)
    assert h["id"][0] == 2

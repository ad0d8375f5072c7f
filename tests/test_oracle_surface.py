"""The surface-geometry oracle (oracle/lmoracle_surface.c) against the
reference's own IntersectionUtils::CreateTriangleIntersection
(intersectionutils.h:59-135), compiled in double and single precision
(tests/golden/surface.npz, made by tests/golden/make_golden.py)."""
import os

import numpy as np

FIELDS = {"p": slice(0, 3), "gn": slice(3, 6), "sn": slice(6, 9), "dpdu": slice(9, 12), "dpdv": slice(12, 15),
          "dndu": slice(15, 18), "dndv": slice(18, 21), "uv": slice(21, 23)}


def golden(golden_dir):
    return dict(np.load(os.path.join(golden_dir, "surface.npz")))


def golden_rays_hits(g, dtype=np.float64):
    q = g["queries"]
    rays = np.zeros((q.shape[0], 8), dtype)
    rays[:, 0:3] = q[:, 2:5]
    rays[:, 4:7] = q[:, 5:8]
    rays[:, 7] = np.finfo(np.float32).max
    hits = np.stack([q[:, 8], g["global_id"].astype(np.float64), q[:, 9], q[:, 10]], 1)
    return rays, hits


def assert_close(a, b, rtol, atol, what):
    """Per field: NaN where the reference has NaN, else |a - b| <= atol + rtol |b|."""
    for name, sl in FIELDS.items():
        x, y = a[:, sl], b[:, sl]
        nan_ref = np.isnan(y)
        assert np.array_equal(np.isnan(x), nan_ref), (what, name, "NaN pattern differs")
        ok = ~nan_ref
        err = np.abs(x[ok] - y[ok])
        lim = atol + rtol * np.abs(y[ok])
        assert np.all(err <= lim), (what, name, float(err.max()), float((err - lim).max()))


def test_oracle_matches_reference_fp64(oracle_lib, golden_dir):
    g = golden(golden_dir)
    rays, hits = golden_rays_hits(g)
    out = oracle_lib.surface(g["tris64"], g["normals64"], g["texcoords64"], g["flags"], rays, hits)
    assert_close(out, g["geom64"], 1e-12, 1e-12, "oracle vs reference (double)")
    assert np.array_equal(g["face64"], g["queries"][:, 1].astype(np.int32))
    # the golden covers every branch: normals / none, texcoords / none, the NaN fallback
    assert set(np.unique(g["flags"])) == {0, 1, 2, 3}
    assert np.isnan(g["geom64"]).any()


def test_single_precision_reference_is_within_its_rsqrt_error(golden_dir):
    """The reference's single-precision build normalises with the SSE
    reciprocal square-root estimate (math.h:1872-1875, about 12 bits): its
    unit vectors sit within 1e-3 of the double build's.  The GPU path is
    therefore checked against the double build."""
    g = golden(golden_dir)
    a, b = g["geom32"], g["geom64"]
    assert np.array_equal(np.isnan(a), np.isnan(b))
    ok = ~np.isnan(b)
    unit = np.zeros(23, bool)
    unit[3:15] = True
    d = np.abs(a - b)
    assert np.all(d[:, unit][ok[:, unit]] < 1e-3)
    assert np.all(d[:, 0:3] <= 1e-6 * (1 + np.abs(b[:, 0:3])))

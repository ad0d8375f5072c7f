"""The numpy restatement of the reference's mesh flattening (tests/meshflat.py)
against the triangles the reference itself produced for the surface fixture's
four transformed primitives (tests/golden/surface.npz, tris32: the
single-precision reference build), bit for bit."""
import os

import numpy as np

import meshflat


def test_restatement_matches_reference_triangles(golden_dir):
    z = np.load(os.path.join(golden_dir, "surface.npz"))
    tris, prim = meshflat.flatten(meshflat.fixture_meshes(z))
    assert tris.dtype == np.float32 and tris.shape == z["tris32"].shape
    assert np.array_equal(tris.view(np.uint32), z["tris32"].view(np.uint32))
    assert np.array_equal(np.bincount(prim), [int(z[f"mesh{i}_faces"].shape[0]) for i in range(4)])

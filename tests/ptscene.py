"""Rebuilds the path-tracing scene stored in tests/golden/cornell_pt.npz."""
import os

import numpy as np


def load_cornell(golden_dir):
    z = dict(np.load(os.path.join(golden_dir, "cornell_pt.npz")))
    prims = []
    for i in range(int(z["nprims"])):
        prims.append({"kind": int(z[f"prim{i}_kind"]), "R": tuple(float(x) for x in z[f"prim{i}_R"]),
                      "Le": tuple(float(x) for x in z[f"prim{i}_Le"]), "tris": z[f"prim{i}_tris"]})
    cam = {"eye": tuple(z["cam_eye"]), "center": tuple(z["cam_center"]), "up": tuple(z["cam_up"]),
           "fov": float(z["cam_fov"]), "width": int(z["width"]), "height": int(z["height"])}
    return {"prims": prims, "camera": cam}, z


def downsample(img, var, f):
    """Block means of f x f pixels and the variance of those means."""
    H, W, C = img.shape
    a = img.reshape(H // f, f, W // f, f, C).mean(axis=(1, 3))
    v = var.reshape(H // f, f, W // f, f, C).sum(axis=(1, 3)) / (f * f) ** 2
    return a, v

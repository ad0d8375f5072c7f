"""Rebuilds the path-tracing scenes stored in tests/golden/*_pt.npz."""
import os

import numpy as np


def load_scene(golden_dir, name):
    z = dict(np.load(os.path.join(golden_dir, name + ".npz")))
    prims = []
    for i in range(int(z["nprims"])):
        if f"prim{i}_bsdf" in z:
            p = {"bsdf": int(z[f"prim{i}_bsdf"]), "light": bool(z[f"prim{i}_light"]), "tris": z[f"prim{i}_tris"]}
            for k in ("R", "Le", "ct_eta", "ct_k"):
                p[k] = tuple(float(x) for x in z[f"prim{i}_{k}"])
            for k in ("eta1", "eta2", "roughness"):
                p[k] = float(z[f"prim{i}_{k}"])
        else:
            p = {"kind": int(z[f"prim{i}_kind"]), "R": tuple(float(x) for x in z[f"prim{i}_R"]),
                 "Le": tuple(float(x) for x in z[f"prim{i}_Le"]), "tris": z[f"prim{i}_tris"]}
        prims.append(p)
    cam = {"eye": tuple(float(x) for x in z["cam_eye"]), "center": tuple(float(x) for x in z["cam_center"]),
           "up": tuple(float(x) for x in z["cam_up"]), "fov": float(z["cam_fov"]), "width": int(z["width"]),
           "height": int(z["height"])}
    scene = {"prims": prims, "camera": cam}
    if int(z.get("has_env", 0)):
        scene["env"] = tuple(float(x) for x in z["env_Le"])
    return scene, z


def load_cornell(golden_dir):
    return load_scene(golden_dir, "cornell_pt")


def downsample(img, var, f):
    """Block means of f x f pixels and the variance of those means."""
    H, W, C = img.shape
    a = img.reshape(H // f, f, W // f, f, C).mean(axis=(1, 3))
    v = var.reshape(H // f, f, W // f, f, C).sum(axis=(1, 3)) / (f * f) ** 2
    return a, v

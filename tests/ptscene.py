"""Rebuilds the path-tracing scenes stored in the render fixtures of tests/golden/."""
import os

import numpy as np


def prim_tris(z, i):
    """Triangles of primitive i: stored, or an instance of a stored unit mesh
    (scale, shift) regenerated with the generator's own arithmetic."""
    if f"prim{i}_tris" in z:
        return z[f"prim{i}_tris"]
    from lmgpu import scenes

    unit = z["mesh_" + str(z[f"prim{i}_inst_mesh"])]
    return scenes.instance_tris(unit, float(z[f"prim{i}_inst_scale"]), z[f"prim{i}_inst_shift"])


def load_scene(golden_dir, name):
    import hashlib

    z = dict(np.load(os.path.join(golden_dir, name + ".npz")))
    prims = []
    digest = hashlib.sha256()
    for i in range(int(z["nprims"])):
        tris = np.ascontiguousarray(prim_tris(z, i), np.float32)
        digest.update(tris.tobytes())
        if f"prim{i}_bsdf" in z:
            p = {"bsdf": int(z[f"prim{i}_bsdf"]), "light": bool(z[f"prim{i}_light"]), "tris": tris}
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
    if "tris_sha256" in z:
        assert digest.hexdigest() == str(z["tris_sha256"]), f"{name}: regenerated triangles differ from the fixture's"
    return scene, z


def load_cornell(golden_dir):
    return load_scene(golden_dir, "cornell_pt")


def downsample(img, var, f):
    """Block means of f x f pixels and the variance of those means."""
    H, W, C = img.shape
    a = img.reshape(H // f, f, W // f, f, C).mean(axis=(1, 3))
    v = var.reshape(H // f, f, W // f, f, C).sum(axis=(1, 3)) / (f * f) ** 2
    return a, v

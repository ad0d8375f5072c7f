"""The reference-side plugins (lightmetrica-v2_gb300/plugin/*.cpp) executed
through the reference's own component interfaces: each plugin is linked into
the reference harness (oracle/build_ref.sh: ref_plugin, ref_render_plugins),
registers itself by its static initialiser through ComponentFactory_Register
(include/lightmetrica/component.h:441), and is created by key and called
through the portable vtable as the reference's scene and CLI do
(Accel::Initialize / Build, Accel3::Intersect, Renderer::Initialize / Render).

The C ABI below the plugins is the CPU stand-in of include/lmgpu.h
(oracle/refharness/lmgpu_cpu_fake.cpp), because the reference tree, and so
the plugins' headers, exist only on this machine, which has no GPU; the GPU
tests call the real library through the same C ABI.  What runs here is the
plugins' own code: scene export from Scene3, mesh and transform hand-over,
the (primitive, face) back-mapping, Intersection filling through
IntersectionUtils::CreateTriangleIntersection, parameter parsing and the film
write.  Skipped where the reference harness is not built (no reference tree,
or not x86-64)."""
import json
import os
import subprocess
import tempfile

import numpy as np
import pytest

import imgcheck
import ptscene


def _need(path):
    if not os.access(path, os.X_OK):
        pytest.skip("reference plugin harness not built here (needs the reference tree on x86-64)")


def _prim_record(transform_cols, ps, ns, ts, fs) -> bytes:
    """One primitive in the harness's mesh layout (ref_plugin_cli.cpp)."""
    out = np.asarray(transform_cols, np.float32).reshape(16).tobytes()
    nv, nf = len(ps) // 3, len(fs) // 3
    out += np.array([nv, nf, 1 if ns is not None else 0, 1 if ts is not None else 0], np.uint32).tobytes()
    out += np.asarray(ps, np.float32).tobytes()
    if ns is not None:
        out += np.asarray(ns, np.float32).tobytes()
    if ts is not None:
        out += np.asarray(ts, np.float32).tobytes()
    return out + np.asarray(fs, np.uint32).tobytes()


IDENTITY = np.eye(4, dtype=np.float32).reshape(16)


@pytest.mark.parametrize("case", ["simple", "simple2"])
def test_accel_plugin_passes_reference_accel3_test(oracle_lib, golden_dir, case):
    """accel::cuda runs the checks of the reference's Accel3Test.Simple /
    Simple2 (src/lightmetrica-test/test_accel3.cpp:272-345) on the test's own
    stub meshes through Create<Accel3> -> Initialize -> Build -> Intersect,
    and the batch slots give the same hits."""
    _need(oracle_lib.REF_PLUGIN)
    z = dict(np.load(os.path.join(golden_dir, "accel3_" + case + ".npz")))
    with tempfile.TemporaryDirectory() as tmp:
        mp = os.path.join(tmp, "mesh.bin")
        with open(mp, "wb") as f:
            f.write(_prim_record(IDENTITY, z["positions"], z["normals"], z["texcoords"], z["faces"]))
        r = subprocess.run([oracle_lib.REF_PLUGIN, "accel3test", case, mp], capture_output=True, text=True)
    assert r.returncode == 0, (r.stdout, r.stderr)
    rec = json.loads(r.stdout.strip().splitlines()[-1])
    assert rec["rays"] == 81 and rec["failed"] == 0 and rec["batch_mismatch"] == 0 and rec["geometry_mismatch"] == 0


def _rot_y(deg):
    a = np.radians(deg)
    return np.array([[np.cos(a), 0, np.sin(a)], [0, 1, 0], [-np.sin(a), 0, np.cos(a)]])


def test_accel_plugin_maps_primitives_faces_and_transforms(oracle_lib):
    """Three primitives with indexed meshes and non-trivial transforms
    (scale, rotation, translation): the plugin's hits through Intersect and
    IntersectBatchGeometry name the same (primitive, face) as the oracle's
    accel::naive on the triangles transformed as the reference does, at the
    same points, and geometric normals agree with the transformed faces."""
    _need(oracle_lib.REF_PLUGIN)
    from lmgpu import scenes

    ico = scenes.closed_icosphere(2)  # (320, 9)
    # an indexed mesh: shared vertices
    v, inv = np.unique(ico.reshape(-1, 3), axis=0, return_inverse=True)
    fs = inv.reshape(-1).astype(np.uint32)
    mats = []
    for s, ang, t in ((0.3, 0.0, (0.2, 0.3, 0.5)), (0.25, 30.0, (0.7, 0.6, 0.4)), (0.2, -50.0, (0.45, 0.2, 0.8))):
        M = np.eye(4)
        M[:3, :3] = _rot_y(ang) * s
        M[:3, 3] = t
        mats.append(M)
    rays = scenes.raycast_rays(4096, seed=77, lo=0.0, hi=1.0)
    rays[:, 3] = 1e-4
    with tempfile.TemporaryDirectory() as tmp:
        sp, rp, op = (os.path.join(tmp, x) for x in ("s.bin", "r.bin", "o.bin"))
        with open(sp, "wb") as f:
            f.write(np.uint32(len(mats)).tobytes())
            for M in mats:
                f.write(_prim_record(M.T.reshape(16), v.reshape(-1), None, None, fs))
        with open(rp, "wb") as f:
            f.write(np.uint32(rays.shape[0]).tobytes())
            f.write(rays.tobytes())
        r = subprocess.run([oracle_lib.REF_PLUGIN, "trace", sp, rp, op], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        rec = np.fromfile(op, dtype=np.dtype([("hit", "<i4"), ("prim", "<i4"), ("face", "<i4"), ("p", "<f4", 3),
                                              ("gn", "<f4", 3), ("sn", "<f4", 3), ("uv", "<f4", 2)]))
    n = rays.shape[0]
    single, batch = rec[:n], rec[n:]
    # the triangles as the reference transforms them (float Mat4 x Vec4)
    tris = []
    for M in mats:
        Mf = M.astype(np.float32)
        P = v.astype(np.float32)
        q = [((Mf[k, 0] * P[:, 0] + Mf[k, 1] * P[:, 1]) + (Mf[k, 2] * P[:, 2] + Mf[k, 3])).astype(np.float32)
             for k in range(3)]
        tris.append(np.stack(q, axis=1)[fs].reshape(-1, 9))
    tris = np.concatenate(tris).astype(np.float32)
    h = oracle_lib.OracleAccel(oracle_lib.NAIVE, tris).trace(rays)
    nf = fs.size // 3
    hit = h["id"] >= 0
    assert 0.1 < hit.mean() < 0.9
    assert np.array_equal(single["hit"] == 1, hit)
    assert np.array_equal(single["prim"][hit], h["id"][hit] // nf)
    assert np.array_equal(single["face"][hit], h["id"][hit] % nf)
    assert np.allclose(single["p"][hit], h["p"][hit], atol=1e-5)
    for k in ("hit", "prim", "face"):
        assert np.array_equal(batch[k], single[k])
    assert np.allclose(batch["p"][hit], single["p"][hit], atol=1e-5)
    # normals within Math::EpsLarge (1e-3, the reference test's tolerance):
    # the single-ray path normalises with the reference's single-precision
    # SSE arithmetic, the batch path's geometry is computed in double
    assert np.allclose(batch["gn"][hit], single["gn"][hit], atol=1e-3)
    T = tris[h["id"][hit]].reshape(-1, 3, 3).astype(np.float64)
    gn = np.cross(T[:, 1] - T[:, 0], T[:, 2] - T[:, 0])
    gn /= np.linalg.norm(gn, axis=1, keepdims=True)
    assert np.allclose(single["gn"][hit], gn, atol=1e-3)
    assert np.allclose(batch["gn"][hit], gn, atol=1e-5)


@pytest.mark.parametrize("plugin,golden,params", [
    ("pt_cuda", "cornell_pt", {}),
    ("ptmis_cuda", "cornell_ptmis", {}),
    ("ptdirect_cuda", "cornell_ptdirect", {}),
    ("ltdirect_cuda", "cornell_ltdirect", {}),
    ("bdpt_cuda", "cornell_bdpt", {"mis": "powerheuristics"}),
    ("pt_guided_cuda", "cornell_pt", {"alpha": 0.5, "throughput_roulette": 1}),
])
def test_renderer_plugin_renders_through_renderer_interface(oracle_lib, golden_dir, plugin, golden, params):
    """renderer::<plugin> created by key in the reference's render harness:
    Initialize with the scene file's parameters, Render on the harness's
    Scene3 (BSDF, light and sensor components of the reference), the film
    written through Film::SetPixel.  Its image agrees with the reference's
    own renderer's film (aggregates, with the per-pixel variance scaled from
    the reference's to the plugin's sample count)."""
    _need(oracle_lib.REF_RENDER_PLUGINS)
    scene, z = ptscene.load_scene(golden_dir, golden)
    W, H = scene["camera"]["width"], scene["camera"]["height"]
    spp = 256
    r = oracle_lib.run_ref_render(scene, W * H * spp, int(z["max_num_vertices"]), 97, os.cpu_count() or 4,
                                  renderer=plugin, params=params, exe=oracle_lib.REF_RENDER_PLUGINS)
    assert r["info"]["renderer"] == "renderer::" + plugin
    img = r["image"].astype(np.float64)
    ref_spp = int(z["num_samples"]) // (W * H)
    var = z["ref64_variance"] * (ref_spp / spp)
    s = imgcheck.assert_same_aggregates(img, var, z["ref64_image"], z["ref64_variance"], f"{plugin} vs ref64")
    print(plugin, s)


def test_vcm_plugin_renders_through_renderer_interface(oracle_lib, golden_dir):
    """renderer::vcm_cuda with the reference's own vcm parameters."""
    _need(oracle_lib.REF_RENDER_PLUGINS)
    scene, z = ptscene.load_scene(golden_dir, "cornell_vcm")
    prm = {k: (float(z[k]) if k in ("initial_radius", "alpha") else int(z[k]))
           for k in ("num_iteration_pass", "num_photon_trace_samples", "num_eye_trace_samples", "initial_radius",
                     "alpha")}
    prm["num_iteration_pass"] = 16
    prm["mode"] = "vcm"
    W, H = scene["camera"]["width"], scene["camera"]["height"]
    # renderer::vcm takes its sample counts from its own parameters
    r = oracle_lib.run_ref_render(scene, W * H, int(z["max_num_vertices"]), 98, os.cpu_count() or 4,
                                  renderer="vcm_cuda", params=prm, exe=oracle_lib.REF_RENDER_PLUGINS)
    img = r["image"].astype(np.float64)
    assert np.isfinite(img).all() and img.min() >= 0
    ratio = img.sum() / z["ref64_image"].sum()
    assert 0.8 < ratio < 1.2, ratio

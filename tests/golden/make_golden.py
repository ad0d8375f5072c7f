"""Generates the golden fixtures of tests/golden/ from the reference itself.

Run in a checkout that has the reference tree (default: $LM_REFERENCE_ROOT, else
a `reference` directory beside the repository) and
the reference harness built by oracle/build_ref.sh (oracle/_ref/ref_accel):

    python tests/golden/make_golden.py [REFERENCE_ROOT] [--only NAME[,NAME...]]

Fixtures written:
  accel3_simple.npz, accel3_simple2.npz
      The two meshes of the reference's accel test (read from
      src/lightmetrica-test/test_accel3.cpp), its 9x9 ray grids with
      directions normalised by the reference's own Math::Normalize, the
      expected values that test asserts (p, gn, sn, uv), and the hits of the
      reference accels naive / bvh_sahbin / qbvh on those rays.
  cornell_pt.npz
      The Cornell-style box of the path-tracing configuration at 64x64: the
      scene, and the film and per-pixel variance of the reference's own
      renderer::pt (compiled from its sources) at 16,384 samples per pixel,
      in single precision and in double precision (LM_USE_DOUBLE_PRECISION).
  materials_pt.npz
      The same box with a glass box (bsdf::flesnel), a GGX conductor box
      (bsdf::cook_torrance) and a constant environment light (light::env),
      reference films likewise.
  cornell_bdpt.npz, materials_bdpt.npz
      The same two boxes (the materials box without the environment light,
      which renderer::bdpt does not sample) rendered by the reference's own
      renderer::bdpt at 32x32 with max_num_vertices 10: films and
      per-pixel variances in single and double precision.
  cornell_ptmis.npz, materials_ptmis.npz
      The same two boxes (no environment light) rendered by the reference's
      own renderer::ptmis (next-event estimation, balance heuristic) at
      64x64, 16,384 samples per pixel, max_num_vertices 9, single and double
      precision.
  cornell_ptdirect.npz
      The Cornell box rendered by the reference's own renderer::ptdirect
      (light samples only) at 64x64, 16,384 samples per pixel,
      max_num_vertices 9, single and double precision.
  cornell_bdpt_simple.npz
      The Cornell box rendered by the reference's own renderer::bdpt with
      mis: simple (misweight::simple, one over the number of strategies that
      can sample the path) at 32x32, 32,768 samples per pixel,
      max_num_vertices 10, single and double precision.
  cornell_pt_min3.npz, cornell_ptmis_min3.npz, cornell_bdpt_min3.npz
      The Cornell box with min_num_vertices 3 (paths of fewer vertices
      contribute nothing, so the directly seen light is black), rendered by
      the reference's own renderer::pt, renderer::ptmis (64x64) and
      renderer::bdpt (32x32, max_num_vertices 10), single and double precision.
  cornell_ltdirect.npz
      The Cornell box rendered by the reference's own renderer::ltdirect
      (light tracing, a sensor connection at every vertex) with 64x64x16,384
      light paths, max_num_vertices 9, single and double precision.
  cornell_vcm.npz, cornell_bdpm.npz
      The Cornell box rendered by the reference's own renderer::vcm (vertex
      connection and merging; SubpathSampler) at 32x32 with mode vcm and mode
      bdpm: max_num_vertices 8, 256 passes of 8,192 photon subpaths and
      8,192 eye samples, initial_radius 0.05, alpha 0.7; films in single and
      double precision with variances from the film's per-sample squares.
  surface.npz
      Surface geometry at hits from the reference's own
      IntersectionUtils::CreateTriangleIntersection (intersectionutils.h),
      compiled in single and double precision (oracle/_ref/ref_isect,
      ref_isect64): four primitives under non-uniform scale / rotation /
      translation transforms (a smooth icosphere with normals and texcoords,
      a quad with texcoords only, a face with all-zero normals, a bare mesh)
      and seeded queries (face, barycentrics including edges and vertices,
      ray origin, direction and t).  Also the meshes' single-precision
      inputs (mesh<i>_positions, _faces, _transform column-major), whose
      transformed triangles tris32 pin the GPU mesh flattening.  Per triangle: the vertices, normals and
      texcoords as the reference transforms them; per query: p, gn, sn,
      dpdu, dpdv, dndu, dndv, uv.
  soup_small.npz
      A seeded three-primitive scene (random triangle soup, heightfield,
      duplicated triangles for exact-t ties, zero-area triangles) and rays
      (random, axis-aligned, and finite segments), with the hits of the
      reference accels.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "lightmetrica-v2_gb300"))

import lmoracle as lo  # noqa: E402
from lmgpu import scenes  # noqa: E402

FLT_MAX = np.float32(np.finfo(np.float32).max)
ACCELS = ["accel::naive", "accel::bvh_sahbin", "accel::qbvh"]


def parse_mesh(src: str, cls: str) -> dict:
    """Reads the ps/ns/ts/fs initialisers of one stub mesh class."""
    start = src.index(f"class {cls} ")
    body = src[start:src.index("};\n\nclass", start) if "};\n\nclass" in src[start:] else len(src)]
    out = {}
    for name in ("ps", "ns", "ts", "fs"):
        m = re.search(r"std::vector<(?:Float|unsigned int)> " + name + r"\{([^}]*)\}", body)
        vals = [v.strip().replace("_f", "") for v in m.group(1).replace("\n", " ").split(",") if v.strip()]
        out[name] = np.array([float(v) for v in vals], dtype=np.float32 if name != "fs" else np.float64)
    out["fs"] = out["fs"].astype(np.uint32)
    return out


def ref_normalize(vs: np.ndarray, tmp: str) -> np.ndarray:
    vs = np.ascontiguousarray(vs, dtype=np.float32).reshape(-1, 3)
    pin, pout = os.path.join(tmp, "nin.bin"), os.path.join(tmp, "nout.bin")
    with open(pin, "wb") as f:
        f.write(np.uint32(vs.shape[0]).tobytes())
        f.write(vs.tobytes())
    subprocess.run([lo.REF_ACCEL, "--normalize", pin, pout], check=True)
    return np.fromfile(pout, dtype=np.float32).reshape(-1, 3)


def run_ref(meshes: list, rays: np.ndarray, tmp: str) -> dict:
    ps, pr = os.path.join(tmp, "scene.bin"), os.path.join(tmp, "rays.bin")
    lo.write_ref_inputs(ps, pr, meshes, rays)
    res = {}
    for key in ACCELS:
        po = os.path.join(tmp, "out.bin")
        subprocess.run([lo.REF_ACCEL, key, ps, pr, po, "8"], check=True, capture_output=True)
        o = lo.read_ref_output(po)
        tag = key.split("::")[1]
        res[f"{tag}_id"] = o["id"]
        res[f"{tag}_p"] = o["p"]
        res[f"{tag}_b"] = o["b"]
    return res


def accel3_case(src: str, cls: str, simple2: bool, tmp: str) -> dict:
    mesh = parse_mesh(src, cls)
    tris = mesh["ps"].reshape(-1, 3)[mesh["fs"].reshape(-1, 3)].reshape(-1, 9)
    steps = 10
    delta = np.float32(1.0) / np.float32(steps)
    rays, exp_p, exp_gn, exp_uv = [], [], [], []
    raw_dirs = []
    for i in range(1, steps):
        y = np.float32(delta * np.float32(i))
        for j in range(1, steps):
            x = np.float32(delta * np.float32(j))
            if simple2:
                o = np.array([x, y, 1], dtype=np.float32)
                raw_dirs.append(None)
                rays.append(np.array([o[0], o[1], o[2], 0, 0, 0, -1, FLT_MAX], dtype=np.float32))
                exp_p.append([x, y, -x])
            else:
                o = np.array([0, 0, 1], dtype=np.float32)
                raw_dirs.append(np.array([x, y, 0], dtype=np.float32) - o)
                rays.append(np.array([0, 0, 1, 0, 0, 0, 0, FLT_MAX], dtype=np.float32))
                exp_p.append([x, y, 0])
            exp_uv.append([x, y])
    rays = np.array(rays, dtype=np.float32)
    if not simple2:
        d = ref_normalize(np.array(raw_dirs), tmp)
        rays[:, 4:7] = d
        n = np.array([0, 0, 1], dtype=np.float32)
    else:
        n = ref_normalize(np.array([[1, 0, 1]], dtype=np.float32), tmp)[0]
    exp_gn = np.tile(n, (rays.shape[0], 1))
    out = dict(positions=mesh["ps"], normals=mesh["ns"], texcoords=mesh["ts"], faces=mesh["fs"], tris=tris,
               rays=rays, expected_p=np.array(exp_p, dtype=np.float32), expected_gn=exp_gn,
               expected_sn=exp_gn.copy(), expected_uv=np.array(exp_uv, dtype=np.float32),
               tolerance=np.float32(1e-3))
    out.update(run_ref([tris], rays, tmp))
    return out


def soup_case(tmp: str) -> dict:
    g = scenes.rng(0xC0FFEE, 7)
    soup = scenes.random_soup(3000, seed=0xC0FFEE, mu=np.log(0.03))
    hf = scenes.heightfield(24, seed=0xC0FFEE, amplitude=0.1, base=0.3)
    dup_src = soup[g.choice(soup.shape[0], 16, replace=False)]
    degenerate = np.array([
        [0.2, 0.2, 0.2, 0.2, 0.2, 0.2, 0.2, 0.2, 0.2],      # a point
        [0.1, 0.5, 0.5, 0.3, 0.5, 0.5, 0.6, 0.5, 0.5],      # collinear
        [0.5, 0.1, 0.5, 0.5, 0.4, 0.5, 0.5, 0.9, 0.5],      # collinear
        [0.7, 0.7, 0.1, 0.7, 0.7, 0.1, 0.7, 0.7, 0.9],      # two equal vertices
    ], dtype=np.float32)
    extra = np.concatenate([dup_src, degenerate], axis=0)
    meshes = [soup, hf, extra]
    r_rand = scenes.raycast_rays(3072, seed=0xC0FFEE, stream=9)
    # axis-aligned rays (zero direction components)
    o = g.uniform(-0.1, 1.1, size=(512, 3)).astype(np.float32)
    axis = g.integers(0, 3, size=512)
    sign = np.where(g.random(512) < 0.5, -1.0, 1.0)
    d = np.zeros((512, 3), dtype=np.float32)
    d[np.arange(512), axis] = sign
    r_axis = np.concatenate([o, np.full((512, 1), 1e-4, np.float32), d, np.full((512, 1), FLT_MAX, np.float32)], 1)
    # finite segments (shadow-ray style [1e-4, L(1 - 1e-4)])
    a = g.uniform(0.0, 1.0, size=(512, 3))
    b = g.uniform(0.0, 1.0, size=(512, 3))
    L = np.linalg.norm(b - a, axis=1)
    dd = (b - a) / L[:, None]
    r_seg = np.concatenate([a, np.full((512, 1), 1e-4), dd, (L * (1 - 1e-4))[:, None]], 1).astype(np.float32)
    # rays aimed exactly at the duplicated triangles' centroids (exact ties)
    cen = dup_src.reshape(-1, 3, 3).mean(axis=1)
    src = cen + np.array([0.0, 0.0, 0.5])
    dt = (cen - src) / np.linalg.norm(cen - src, axis=1, keepdims=True)
    r_tie = np.concatenate([src, np.full((16, 1), 1e-4), dt, np.full((16, 1), FLT_MAX)], 1).astype(np.float32)
    rays = np.concatenate([r_rand, r_axis, r_seg, r_tie], axis=0).astype(np.float32)
    out = dict(mesh_sizes=np.array([m.shape[0] for m in meshes], dtype=np.int64),
               tris=np.concatenate(meshes, axis=0), rays=rays,
               groups=np.array([3072, 512, 512, 16], dtype=np.int64))
    out.update(run_ref(meshes, rays, tmp))
    return out


INSTANCE_MESHES = {"ico4": lambda: scenes.closed_icosphere(4)}


def scene_arrays(sc: dict) -> dict:
    """A path-tracing scene as flat arrays (read back by tests/ptscene.py).
    Primitives made by scaling and shifting a unit mesh (the sphere grid's
    icospheres) are stored as that mesh once plus a scale and a shift each;
    tris_sha256 pins the regenerated triangles."""
    import hashlib

    out = {"nprims": np.int32(len(sc["prims"]))}
    digest = hashlib.sha256()
    for i, p0 in enumerate(sc["prims"]):
        p = scenes.prim_params(p0)
        tris = np.ascontiguousarray(p["tris"], np.float32)
        digest.update(tris.tobytes())
        inst = p0.get("instance")
        if inst is not None:
            name, scale, shift = inst
            unit = INSTANCE_MESHES[name]()
            assert np.array_equal(scenes.instance_tris(unit, scale, shift), tris)
            out[f"mesh_{name}"] = unit
            out[f"prim{i}_inst_mesh"] = np.array(name)
            out[f"prim{i}_inst_scale"] = np.float64(scale)
            out[f"prim{i}_inst_shift"] = np.array(shift, np.float64)
        else:
            out[f"prim{i}_tris"] = tris
        out[f"prim{i}_bsdf"] = np.int32(p["bsdf"])
        out[f"prim{i}_light"] = np.int32(1 if p["light"] else 0)
        for k in ("R", "Le", "ct_eta", "ct_k"):
            out[f"prim{i}_{k}"] = np.array(p[k], np.float32)
        for k in ("eta1", "eta2", "roughness"):
            out[f"prim{i}_{k}"] = np.float32(p[k])
    c = sc["camera"]
    out["cam_eye"], out["cam_center"], out["cam_up"] = (np.array(c[k], np.float32) for k in ("eye", "center", "up"))
    out["cam_fov"] = np.float32(c["fov"])
    out["width"], out["height"] = np.int32(c["width"]), np.int32(c["height"])
    out["has_env"] = np.int32(1 if sc.get("env") is not None else 0)
    out["env_Le"] = np.array(sc.get("env") or (0.0, 0.0, 0.0), np.float32)
    out["tris_sha256"] = np.array(digest.hexdigest())
    return out


def pt_case(sc: dict, spp: int, seed: int, renderer: str = "pt", max_num_vertices: int = 9,
            mis: str | None = None, min_num_vertices: int = 0, accel64: str | None = None) -> dict:
    """accel64: the accel of the double-precision run (default the harness's
    accel::bvh_sahbin).  accel::bvh_sahbin divides 0 by 0 when the centroids
    of a node's triangles coincide on its split axis
    (accel_bvh_sahbin.cpp:155-157) and crashes on such scenes (the caustic
    room, the sphere grid); accel::bvh_sah (sorted object splits) has no such
    case and returns the same closest hits."""
    W, H = sc["camera"]["width"], sc["camera"]["height"]
    N = W * H * spp
    extra = {"min_num_vertices": min_num_vertices} if min_num_vertices else None
    f = lo.run_ref_render(sc, N, max_num_vertices, seed, os.cpu_count() or 8, renderer=renderer, mis=mis,
                          params=extra)
    d = lo.run_ref_render(sc, N, max_num_vertices, seed + 1, os.cpu_count() or 8, double=True, renderer=renderer,
                          mis=mis, params=extra, accel=accel64)
    out = scene_arrays(sc)
    out.update({"num_samples": np.int64(N), "max_num_vertices": np.int32(max_num_vertices),
                "min_num_vertices": np.int32(min_num_vertices),
                "ref_image": f["image"].astype(np.float32), "ref_variance": f["variance"].astype(np.float32),
                "ref64_image": d["image"].astype(np.float64), "ref64_variance": d["variance"].astype(np.float64)})
    return out


VCM_FIXTURE = dict(max_num_vertices=8, num_iteration_pass=256, num_photon_trace_samples=8192,
                   num_eye_trace_samples=8192, initial_radius=0.05, alpha=0.7)


def vcm_case(mode: str, seed: int) -> dict:
    sc = scenes.cornell_box(32, 32)
    prm = dict(VCM_FIXTURE, mode=mode)
    f = lo.run_ref_vcm(sc, seed, os.cpu_count() or 8, **prm)
    d = lo.run_ref_vcm(sc, seed + 1, os.cpu_count() or 8, double=True, **prm)
    out = scene_arrays(sc)
    out.update({k: np.float64(v) if isinstance(v, float) else np.int64(v) for k, v in VCM_FIXTURE.items()})
    out.update({"mode": np.array(mode),
                "ref_image": f["image"].astype(np.float32), "ref_variance": f["variance"].astype(np.float32),
                "ref64_image": d["image"].astype(np.float64), "ref64_variance": d["variance"].astype(np.float64)})
    return out


def _rot(axis, ang):
    a = np.asarray(axis, np.float64) / np.linalg.norm(axis)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    return np.eye(3) + np.sin(ang) * K + (1 - np.cos(ang)) * K @ K


def _affine(scale, axis, ang, trans):
    m = np.eye(4)
    m[:3, :3] = _rot(axis, ang) @ np.diag(scale)
    m[:3, 3] = trans
    return m


def surface_case() -> dict:
    g = np.random.default_rng(20241215)
    ico = scenes.closed_icosphere(2, 1.0)  # (nf, 9), unshared vertices
    pos = ico.reshape(-1, 3)
    faces = np.arange(pos.shape[0], dtype=np.uint32).reshape(-1, 3)
    nrm = pos / np.linalg.norm(pos, axis=1, keepdims=True)
    tc = np.stack([0.5 + np.arctan2(nrm[:, 2], nrm[:, 0]) / (2 * np.pi), np.arccos(np.clip(nrm[:, 1], -1, 1)) / np.pi], 1)
    quad = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], np.float64)
    prims = [
        {"transform": _affine((1.0, 2.0, 0.5), (0.3, 1.0, 0.2), 0.7, (0.5, -0.2, 3.0)), "positions": pos,
         "faces": faces, "normals": nrm, "texcoords": tc},
        {"transform": _affine((2.0, 0.5, 1.0), (1.0, 0.0, 0.5), -1.1, (-1.0, 0.4, 0.0)), "positions": quad,
         "faces": np.array([[0, 1, 2], [0, 2, 3]], np.uint32), "normals": None,
         "texcoords": np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float64)},
        {"transform": _affine((1.0, 1.0, 1.0), (0.0, 1.0, 0.0), 0.4, (0.0, 0.0, -2.0)),
         "positions": np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0.5]], np.float64),
         "faces": np.array([[0, 1, 2], [1, 3, 2]], np.uint32),
         "normals": np.array([[0, 0, 0], [0, 0, 0], [0, 0, 0], [0, 0.3, 1.0]], np.float64), "texcoords": None},
        {"transform": _affine((0.7, 1.3, 1.0), (0.2, 0.2, 1.0), 2.0, (1.0, 1.0, 1.0)), "positions": quad + 0.25,
         "faces": np.array([[0, 1, 2], [0, 2, 3]], np.uint32), "normals": None, "texcoords": None},
    ]
    nf = [p["faces"].shape[0] for p in prims]
    base = np.concatenate([[0], np.cumsum(nf)[:-1]])
    qs = []
    for k in range(600):
        pi = int(g.integers(len(prims))) if k >= 8 else k % 4
        fi = int(g.integers(nf[pi]))
        c = g.integers(4)
        if c == 0:
            b = g.dirichlet([1, 1, 1])[1:]
        elif c == 1:
            b = np.array([0.0, g.uniform()])  # on edge v1 - v3
        elif c == 2:
            b = [np.array([0.0, 0.0]), np.array([1.0, 0.0]), np.array([0.0, 1.0])][int(g.integers(3))]
        else:
            u = g.uniform()
            b = np.array([u, 1.0 - u])  # on edge v2 - v3
        o = g.normal(size=3) * 4.0
        d = g.normal(size=3)
        d /= np.linalg.norm(d)
        t = float(g.uniform(0.1, 8.0))
        qs.append([pi, fi, *o, *d, t, b[0], b[1]])
    q = np.array(qs, np.float64)
    r64 = lo.run_ref_isect(prims, q, double=True)
    r32 = lo.run_ref_isect(prims, q, double=False)
    meshes = {}
    for i, p in enumerate(prims):
        # the harness's inputs in single precision: positions and the column-major transform m[c][r]
        meshes[f"mesh{i}_positions"] = np.asarray(p["positions"], np.float32)
        meshes[f"mesh{i}_faces"] = np.asarray(p["faces"], np.uint32)
        meshes[f"mesh{i}_transform"] = np.asarray(p["transform"], np.float64).reshape(4, 4).T.reshape(-1).astype(
            np.float32)
    return {**meshes, "num_meshes": np.int32(len(prims)),
            "queries": q, "global_id": (base[q[:, 0].astype(int)] + q[:, 1]).astype(np.int32),
            "tris64": r64["tris"], "normals64": r64["normals"], "texcoords64": r64["texcoords"],
            "flags": r64["flags"], "geom64": r64["geom"], "face64": r64["face"],
            "tris32": r32["tris"].astype(np.float32), "normals32": r32["normals"].astype(np.float32),
            "texcoords32": r32["texcoords"].astype(np.float32), "geom32": r32["geom"]}


def main() -> None:
    args = sys.argv[1:]
    only = None
    if "--only" in args:
        i = args.index("--only")
        only = set(args[i + 1].split(","))
        del args[i:i + 2]
    ref = args[0] if args else os.environ.get("LM_REFERENCE_ROOT", os.path.join(os.path.dirname(REPO), "reference"))
    want = lambda name: only is None or name in only  # noqa: E731
    if not (os.path.exists(lo.REF_ACCEL) and os.path.exists(lo.REF_RENDER) and os.path.exists(lo.REF_RENDER64)):
        subprocess.run([os.path.join(REPO, "oracle", "build_ref.sh"), ref], check=True)
    src = open(os.path.join(ref, "src", "lightmetrica-test", "test_accel3.cpp")).read()
    with tempfile.TemporaryDirectory() as tmp:
        if want("accel3_simple"):
            np.savez_compressed(os.path.join(HERE, "accel3_simple.npz"),
                                **accel3_case(src, "StubTriangleMesh_Simple", False, tmp))
        if want("accel3_simple2"):
            np.savez_compressed(os.path.join(HERE, "accel3_simple2.npz"),
                                **accel3_case(src, "StubTriangleMesh_Simple2", True, tmp))
        if want("soup_small"):
            np.savez_compressed(os.path.join(HERE, "soup_small.npz"), **soup_case(tmp))
    if want("surface"):
        np.savez_compressed(os.path.join(HERE, "surface.npz"), **surface_case())
    if want("cornell_pt"):
        np.savez_compressed(os.path.join(HERE, "cornell_pt.npz"),
                            **pt_case(scenes.cornell_box(64, 64), 16384, 20240601))
    if want("materials_pt"):
        np.savez_compressed(os.path.join(HERE, "materials_pt.npz"),
                            **pt_case(scenes.cornell_materials(64, 64), 16384, 20240701))
    if want("cornell_bdpt"):
        np.savez_compressed(os.path.join(HERE, "cornell_bdpt.npz"),
                            **pt_case(scenes.cornell_box(32, 32), 32768, 20240801, "bdpt", 10))
    if want("materials_bdpt"):
        sc = scenes.cornell_materials(32, 32)
        sc.pop("env", None)
        np.savez_compressed(os.path.join(HERE, "materials_bdpt.npz"),
                            **pt_case(sc, 32768, 20240901, "bdpt", 10))
    for name, make in (("cornell_ptmis", scenes.cornell_box), ("materials_ptmis", scenes.cornell_materials)):
        if want(name):
            sc = make(64, 64)
            sc.pop("env", None)
            np.savez_compressed(os.path.join(HERE, name + ".npz"),
                                **pt_case(sc, 16384, 20241001 if name.startswith("cornell") else 20241101, "ptmis", 9))
    if want("cornell_ptdirect"):
        np.savez_compressed(os.path.join(HERE, "cornell_ptdirect.npz"),
                            **pt_case(scenes.cornell_box(64, 64), 16384, 20241201, "ptdirect", 9))
    if want("cornell_bdpt_simple"):
        np.savez_compressed(os.path.join(HERE, "cornell_bdpt_simple.npz"),
                            **pt_case(scenes.cornell_box(32, 32), 32768, 20241401, "bdpt", 10, mis="simple"))
    for name, rend, spp, res, mnv in (("cornell_pt_min3", "pt", 16384, 64, 9), ("cornell_ptmis_min3", "ptmis", 8192, 64, 9),
                                      ("cornell_bdpt_min3", "bdpt", 16384, 32, 10)):
        if want(name):
            np.savez_compressed(os.path.join(HERE, name + ".npz"),
                                **pt_case(scenes.cornell_box(res, res), spp, 20241501 + len(name), rend, mnv,
                                          min_num_vertices=3))
    if want("cornell_ltdirect"):
        np.savez_compressed(os.path.join(HERE, "cornell_ltdirect.npz"),
                            **pt_case(scenes.cornell_box(64, 64), 16384, 20241301, "ltdirect", 9))
    for mode in ("vcm", "bdpm"):
        if want(f"cornell_{mode}"):
            np.savez_compressed(os.path.join(HERE, f"cornell_{mode}.npz"), **vcm_case(mode, 20241601))
    if want("caustic_bdpt"):
        # the bidirectional configuration's own scene on a 48 x 27 film
        np.savez_compressed(os.path.join(HERE, "caustic_bdpt.npz"),
                            **pt_case(scenes.caustic_room(48, 27), 16384, 20250101, "bdpt", 11,
                                      accel64="accel::bvh_sah"))
    if want("grid_pt"):
        # one view of the batched configuration: a 4 x 4 sphere grid (every
        # BSDF kind, icosphere light, constant environment), 96 x 54, paths of
        # up to 16 segments
        np.savez_compressed(os.path.join(HERE, "grid_pt.npz"),
                            **pt_case(scenes.sphere_grid_scene(7, 0, 96, 54, grid=4), 16384, 20250201, "pt", 17,
                                      accel64="accel::bvh_sah"))
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()

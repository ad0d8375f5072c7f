"""ctypes view of the CPU oracle (oracle/liblmoracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker and by bench.py
for its CPU-baseline leg.  The product path never imports this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblmoracle.so")
REF_ACCEL = os.path.join(HERE, "_ref", "ref_accel")

HIT_DTYPE = np.dtype([("id", "<i4"), ("t", "<f4"), ("b0", "<f4"), ("b1", "<f4"), ("p", "<f4", (3,))])

NAIVE = 0
BVH_SAHBIN = 1
QBVH = 2


def build() -> str:
    """Compiles liblmoracle.so with the host compiler (make)."""
    r = subprocess.run(["make", "-s", "-C", HERE], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB_PATH


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        vp, sz = ctypes.c_void_p, ctypes.c_size_t
        L.lmo_accel_build.argtypes = [ctypes.c_int, vp, sz]
        L.lmo_accel_build.restype = vp
        L.lmo_accel_free.argtypes = [vp]
        L.lmo_accel_free.restype = None
        L.lmo_accel_trace.argtypes = [vp, vp, sz, vp, ctypes.c_int]
        L.lmo_accel_trace.restype = None
        L.lmo_accel_stats.argtypes = [vp, ctypes.POINTER(sz), ctypes.POINTER(sz), ctypes.POINTER(ctypes.c_int)]
        L.lmo_accel_stats.restype = None
        L.lmo_plane_t_fp64.argtypes = [vp, vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
        L.lmo_plane_t_fp64.restype = ctypes.c_double
        L.lmo_render_pt.argtypes = [vp, vp, sz, vp, vp, vp, ctypes.c_uint64, ctypes.c_int, ctypes.c_uint64,
                                    ctypes.c_int, vp, vp]
        L.lmo_render_pt.restype = ctypes.c_uint64
        L.lmo_render_bdpt.argtypes = [vp, vp, sz, vp, ctypes.c_int, vp, ctypes.c_uint64, ctypes.c_int, ctypes.c_uint64,
                                      ctypes.c_int, vp, vp]
        L.lmo_render_bdpt.restype = ctypes.c_uint64
        L.lmo_render_bdpt_ex.argtypes = L.lmo_render_bdpt.argtypes + [ctypes.c_int]
        L.lmo_render_bdpt_ex.restype = ctypes.c_uint64
        L.lmo_render_bdpt_mis.argtypes = L.lmo_render_bdpt.argtypes + [ctypes.c_int, ctypes.c_int]
        L.lmo_render_bdpt_mis.restype = ctypes.c_uint64
        L.lmo_render_vcm.argtypes = [vp, vp, sz, vp, ctypes.c_int, vp, vp, ctypes.c_uint64, ctypes.c_int, vp, vp]
        L.lmo_render_vcm.restype = ctypes.c_uint64
        L.lmo_render_ptmis.argtypes = L.lmo_render_bdpt.argtypes
        L.lmo_render_ptmis.restype = ctypes.c_uint64
        L.lmo_render_ptdirect.argtypes = L.lmo_render_bdpt.argtypes
        L.lmo_render_ptdirect.restype = ctypes.c_uint64
        L.lmo_render_ltdirect.argtypes = L.lmo_render_bdpt.argtypes
        L.lmo_render_ltdirect.restype = ctypes.c_uint64
        L.lmo_surface.argtypes = [vp, vp, vp, vp, vp, vp, sz, vp]
        L.lmo_surface.restype = None
        _lib = L
    return _lib


class OracleAccel:
    """accel::naive (kind 0), accel::bvh_sahbin (kind 1) or accel::qbvh (kind 2), restated in C."""

    def __init__(self, kind: int, tris: np.ndarray):
        self.tris = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1, 9)
        self._h = lib().lmo_accel_build(kind, self.tris.ctypes.data, self.tris.shape[0])

    def trace(self, rays: np.ndarray, threads: int = 1) -> np.ndarray:
        r = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        out = np.empty(r.shape[0], dtype=HIT_DTYPE)
        lib().lmo_accel_trace(self._h, r.ctypes.data, r.shape[0], out.ctypes.data, threads)
        return out

    def stats(self) -> dict:
        n, l, d = ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_int()
        lib().lmo_accel_stats(self._h, ctypes.byref(n), ctypes.byref(l), ctypes.byref(d))
        return {"nodes": n.value, "leaves": l.value, "depth": d.value}

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().lmo_accel_free(self._h)
            self._h = None

    def __del__(self) -> None:
        try:
            self.close()
        except Exception:
            pass


def t_fp64(tris: np.ndarray, rays: np.ndarray, ids: np.ndarray) -> np.ndarray:
    """FP64 ray parameter of each ray on the plane of triangle ids[i] (vectorised)."""
    T = np.asarray(tris, dtype=np.float64).reshape(-1, 9)[ids]
    R = np.asarray(rays, dtype=np.float64).reshape(-1, 8)
    v0, e1, e2 = T[:, 0:3], T[:, 3:6] - T[:, 0:3], T[:, 6:9] - T[:, 0:3]
    o, d = R[:, 0:3], R[:, 4:7]
    n = np.cross(e1, e2)
    return np.einsum("ij,ij->i", n, v0 - o) / np.einsum("ij,ij->i", n, d)


def barycentrics_fp64(tris: np.ndarray, rays: np.ndarray, ids: np.ndarray) -> np.ndarray:
    """FP64 barycentrics (b1, b2) of the ray's plane hit in triangle ids[i]."""
    T = np.asarray(tris, dtype=np.float64).reshape(-1, 9)[ids]
    R = np.asarray(rays, dtype=np.float64).reshape(-1, 8)
    v0, e1, e2 = T[:, 0:3], T[:, 3:6] - T[:, 0:3], T[:, 6:9] - T[:, 0:3]
    o, d = R[:, 0:3], R[:, 4:7]
    pv = np.cross(d, e2)
    det = np.einsum("ij,ij->i", e1, pv)
    tv = o - v0
    u = np.einsum("ij,ij->i", tv, pv) / det
    qv = np.cross(tv, e1)
    v = np.einsum("ij,ij->i", d, qv) / det
    return np.stack([u, v], axis=1)


def write_ref_inputs(path_scene: str, path_rays: str, meshes: list[np.ndarray], rays: np.ndarray) -> None:
    """Writes the input files of oracle/_ref/ref_accel (see refharness/ref_accel_cli.cpp)."""
    with open(path_scene, "wb") as f:
        f.write(np.uint32(len(meshes)).tobytes())
        f.write(np.array([m.reshape(-1, 9).shape[0] for m in meshes], dtype=np.uint32).tobytes())
        for m in meshes:
            f.write(np.ascontiguousarray(m, dtype=np.float32).tobytes())
    r = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
    with open(path_rays, "wb") as f:
        f.write(np.uint32(r.shape[0]).tobytes())
        f.write(r.tobytes())


REF_OUT_DTYPE = np.dtype([("id", "<i4"), ("p", "<f4", (3,)), ("b", "<f4", (2,))])


def read_ref_output(path: str) -> np.ndarray:
    return np.fromfile(path, dtype=REF_OUT_DTYPE)


REF_RENDER = os.path.join(HERE, "_ref", "ref_render")
REF_RENDER64 = os.path.join(HERE, "_ref", "ref_render64")
REF_RENDER_PLUGINS = os.path.join(HERE, "_ref", "ref_render_plugins")
REF_PLUGIN = os.path.join(HERE, "_ref", "ref_plugin")


def _prim_full(p: dict) -> dict:
    import sys as _s

    _s.path.insert(0, os.path.join(os.path.dirname(HERE), "lightmetrica-v2_gb300"))
    from lmgpu.scenes import prim_params

    return prim_params(p)


def write_render_scene(path: str, scene: dict, num_samples: int, max_num_vertices: int, seed: int,
                       threads: int) -> None:
    """Writes the input file of oracle/_ref/ref_render (refharness/ref_render_cli.cpp), version 2."""
    cam = scene["camera"]
    with open(path, "wb") as f:
        f.write(np.array([0x53524D4C, 2, cam["width"], cam["height"]], dtype=np.uint32).tobytes())
        f.write(np.array(list(cam["eye"]) + list(cam["center"]) + list(cam["up"]) + [cam["fov"]],
                         dtype=np.float32).tobytes())
        f.write(np.uint32(len(scene["prims"])).tobytes())
        for p0 in scene["prims"]:
            p = _prim_full(p0)
            f.write(np.array([p["bsdf"], 1 if p["light"] else 0], dtype=np.int32).tobytes())
            f.write(np.array(list(p["R"]) + list(p["Le"]) + [p["eta1"], p["eta2"]] + list(p["ct_eta"]) +
                             list(p["ct_k"]) + [p["roughness"]], dtype=np.float32).tobytes())
            t = np.ascontiguousarray(p["tris"], dtype=np.float32).reshape(-1, 9)
            f.write(np.uint32(t.shape[0]).tobytes())
            f.write(t.tobytes())
        env = scene.get("env")
        f.write(np.int32(1 if env is not None else 0).tobytes())
        f.write(np.array(env if env is not None else (0.0, 0.0, 0.0), dtype=np.float32).tobytes())
        f.write(np.uint64(num_samples).tobytes())
        f.write(np.int32(max_num_vertices).tobytes())
        f.write(np.uint32(seed).tobytes())
        f.write(np.uint32(threads).tobytes())


def run_ref_render(scene: dict, num_samples: int, max_num_vertices: int, seed: int, threads: int,
                   double: bool = False, renderer: str = "pt", mis: str | None = None,
                   params: dict | None = None, accel: str | None = None, exe: str | None = None) -> dict:
    """Runs the reference renderer::pt or renderer::bdpt (compiled from its
    sources) and returns the film (H, W, 3), the per-pixel variance of that
    estimate and timing.  accel overrides the harness's accel component
    (accel::qbvh in single precision, accel::bvh_sahbin in double); every
    accel returns the same closest hits, so the film does not depend on it.
    exe: another build of the harness (the one with the renderer plugins)."""
    import json
    import tempfile

    cam = scene["camera"]
    W, H = cam["width"], cam["height"]
    env = dict(os.environ)
    if accel:
        env["LM_REF_ACCEL"] = accel
    with tempfile.TemporaryDirectory() as tmp:
        ps, po = os.path.join(tmp, "scene.bin"), os.path.join(tmp, "out.bin")
        write_render_scene(ps, scene, num_samples, max_num_vertices, seed, threads)
        exe = exe or (REF_RENDER64 if double else REF_RENDER)
        extra = dict(params or {})
        if mis:
            extra["mis"] = mis
        cmd = [exe, ps, po, renderer] + [f"{k}={v}" for k, v in extra.items()]
        out = subprocess.run(cmd, capture_output=True, text=True, check=True, env=env).stdout
        raw = open(po, "rb").read()
    n = W * H * 3
    img = np.frombuffer(raw[:4 * n], dtype=np.float32).reshape(H, W, 3)
    sumsq = np.frombuffer(raw[4 * n:12 * n], dtype=np.float64).reshape(H, W, 3)
    N = int(np.frombuffer(raw[12 * n:12 * n + 8], dtype=np.uint64)[0])
    return {"image": img, "variance": pixel_variance(img.astype(np.float64), sumsq, N, W * H), "samples": N,
            "raw_sumsq": sumsq, "info": json.loads(out.strip().splitlines()[-1])}


def pixel_variance(image: np.ndarray, sumsq: np.ndarray, num_samples: int, num_pixels: int) -> np.ndarray:
    """Variance of the film estimate I_p = (W H / N) sum_i C_i [i in p] with
    raster positions uniform over the film (renderer_pt.cpp:84-91,
    film_hdr.cpp:218-223, scheduler.cpp:281-288): with X_i = C_i [i in p],
    Var(I_p) = (W H)^2 Var(X) / N, Var(X) = E[X^2] - E[X]^2."""
    scale = num_pixels / num_samples
    ex = image / scale / num_samples          # E[X] = (sum_i X_i) / N
    ex2 = sumsq / num_samples                 # E[X^2]
    return (num_pixels ** 2) * np.maximum(ex2 - ex * ex, 0.0) / num_samples


class PtPrim(ctypes.Structure):
    _fields_ = [("bsdf", ctypes.c_int32), ("is_light", ctypes.c_int32), ("R", ctypes.c_float * 3),
                ("Le", ctypes.c_float * 3), ("eta1", ctypes.c_float), ("eta2", ctypes.c_float),
                ("ct_eta", ctypes.c_float * 3), ("ct_k", ctypes.c_float * 3), ("roughness", ctypes.c_float)]


class PtEnv(ctypes.Structure):
    _fields_ = [("enabled", ctypes.c_int32), ("Le", ctypes.c_float * 3)]


class PtCamera(ctypes.Structure):
    _fields_ = [("eye", ctypes.c_float * 3), ("center", ctypes.c_float * 3), ("up", ctypes.c_float * 3),
                ("fov_deg", ctypes.c_float), ("width", ctypes.c_int32), ("height", ctypes.c_int32)]


def scene_prims(scene: dict) -> "ctypes.Array":
    """Scene primitives in the oracle's layout (kind 0 = diffuse, 1 = light without BSDF)."""
    arr = (PtPrim * len(scene["prims"]))()
    for i, p0 in enumerate(scene["prims"]):
        p = _prim_full(p0)
        arr[i].bsdf = p["bsdf"]
        arr[i].is_light = 1 if p["light"] else 0
        for k in range(3):
            arr[i].R[k] = p["R"][k]
            arr[i].Le[k] = p["Le"][k]
            arr[i].ct_eta[k] = p["ct_eta"][k]
            arr[i].ct_k[k] = p["ct_k"][k]
        arr[i].eta1, arr[i].eta2, arr[i].roughness = p["eta1"], p["eta2"], p["roughness"]
    return arr


def scene_camera(scene: dict) -> PtCamera:
    c = scene["camera"]
    cam = PtCamera()
    for k in range(3):
        cam.eye[k], cam.center[k], cam.up[k] = c["eye"][k], c["center"][k], c["up"][k]
    cam.fov_deg, cam.width, cam.height = c["fov"], c["width"], c["height"]
    return cam


def render_pt(scene: dict, num_samples: int, max_num_vertices: int, seed: int, threads: int) -> dict:
    """The oracle's renderer::pt: film (H, W, 3) and per-pixel variance."""
    tris = np.ascontiguousarray(np.concatenate([p["tris"] for p in scene["prims"]]), dtype=np.float32)
    tri_prim = np.concatenate([np.full(p["tris"].shape[0], i, np.int32) for i, p in enumerate(scene["prims"])])
    W, H = scene["camera"]["width"], scene["camera"]["height"]
    s = np.zeros((H, W, 3), np.float64)
    q = np.zeros((H, W, 3), np.float64)
    prims = scene_prims(scene)
    cam = scene_camera(scene)
    env = PtEnv()
    if scene.get("env") is not None:
        env.enabled = 1
        for k in range(3):
            env.Le[k] = scene["env"][k]
    lib().lmo_render_pt(tris.ctypes.data, tri_prim.ctypes.data, tris.shape[0], ctypes.addressof(prims),
                        ctypes.addressof(env), ctypes.addressof(cam), num_samples, max_num_vertices, seed, threads,
                        s.ctypes.data, q.ctypes.data)
    img = s * (W * H / num_samples)
    return {"image": img, "variance": pixel_variance(img, q, num_samples, W * H), "samples": num_samples}


def render_bdpt(scene: dict, num_samples: int, max_num_vertices: int, seed: int, threads: int,
                independent_light_dir: bool = False, mis: str = "powerheuristics") -> dict:
    """The oracle's renderer::bdpt: film (H, W, 3) and per-pixel variance.
    independent_light_dir: the diagnostic variant of lmo_render_bdpt_ex;
    mis: the renderer's "mis" parameter, powerheuristics or simple."""
    tris = np.ascontiguousarray(np.concatenate([p["tris"] for p in scene["prims"]]), dtype=np.float32)
    tri_prim = np.concatenate([np.full(p["tris"].shape[0], i, np.int32) for i, p in enumerate(scene["prims"])])
    W, H = scene["camera"]["width"], scene["camera"]["height"]
    s = np.zeros((H, W, 3), np.float64)
    q = np.zeros((H, W, 3), np.float64)
    prims = scene_prims(scene)
    cam = scene_camera(scene)
    lib().lmo_render_bdpt_mis(tris.ctypes.data, tri_prim.ctypes.data, tris.shape[0], ctypes.addressof(prims),
                              len(scene["prims"]), ctypes.addressof(cam), num_samples, max_num_vertices, seed,
                              threads, s.ctypes.data, q.ctypes.data, 1 if independent_light_dir else 0,
                              {"powerheuristics": 0, "simple": 1}[mis])
    img = s * (W * H / num_samples)
    return {"image": img, "variance": pixel_variance(img, q, num_samples, W * H), "samples": num_samples}


VCM_MODES = {"vcm": 0, "bdpt": 1, "bdpm": 2}


class VcmParams(ctypes.Structure):
    _fields_ = [("max_num_vertices", ctypes.c_int32), ("min_num_vertices", ctypes.c_int32),
                ("num_iteration_pass", ctypes.c_uint64), ("num_photon_trace_samples", ctypes.c_uint64),
                ("num_eye_trace_samples", ctypes.c_uint64), ("initial_radius", ctypes.c_float),
                ("alpha", ctypes.c_float), ("mode", ctypes.c_int32), ("reserved", ctypes.c_int32)]


def vcm_variance(image: np.ndarray, sumsq: np.ndarray, passes: int, n_eye: int) -> np.ndarray:
    """Variance of renderer::vcm's film I = (1 / P) sum_i X_i over the M = P N_E
    eye samples of all passes, X_i a sample's splats on the pixel (already
    scaled by W H / N_E), treated as independent: Var(I) = M Var(X) / P^2."""
    M = passes * n_eye
    ex = image * passes / M
    ex2 = sumsq / M
    return M * np.maximum(ex2 - ex * ex, 0.0) / (passes * passes)


def render_vcm(scene: dict, seed: int, threads: int, max_num_vertices: int = 10, min_num_vertices: int = 0,
               num_iteration_pass: int = 100, num_photon_trace_samples: int = 10000,
               num_eye_trace_samples: int = 10000, initial_radius: float = 0.1, alpha: float = 0.7,
               mode: str = "vcm") -> dict:
    """The oracle's renderer::vcm (defaults: Renderer_VCM::Initialize,
    renderer_vcm.cpp:573-593): film (H, W, 3) and per-pixel variance."""
    tris = np.ascontiguousarray(np.concatenate([p["tris"] for p in scene["prims"]]), dtype=np.float32)
    tri_prim = np.concatenate([np.full(p["tris"].shape[0], i, np.int32) for i, p in enumerate(scene["prims"])])
    W, H = scene["camera"]["width"], scene["camera"]["height"]
    s = np.zeros((H, W, 3), np.float64)
    q = np.zeros((H, W, 3), np.float64)
    prims = scene_prims(scene)
    cam = scene_camera(scene)
    prm = VcmParams(max_num_vertices, min_num_vertices, num_iteration_pass, num_photon_trace_samples,
                    num_eye_trace_samples, initial_radius, alpha, VCM_MODES[mode], 0)
    n = lib().lmo_render_vcm(tris.ctypes.data, tri_prim.ctypes.data, tris.shape[0], ctypes.addressof(prims),
                             len(scene["prims"]), ctypes.addressof(cam), ctypes.addressof(prm), seed, threads,
                             s.ctypes.data, q.ctypes.data)
    P = max(num_iteration_pass, 1)
    img = s / P
    return {"image": img, "variance": vcm_variance(img, q, P, num_eye_trace_samples), "samples": int(n)}


def run_ref_vcm(scene: dict, seed: int, threads: int, double: bool = False, **params) -> dict:
    """The reference's own renderer::vcm (compiled from its sources): film and
    per-pixel variance (vcm_variance); params are renderer::vcm's
    (max_num_vertices, num_iteration_pass, num_photon_trace_samples, ...)."""
    prm = dict(params)
    mnv = int(prm.pop("max_num_vertices", 10))
    r = run_ref_render(scene, 1, mnv, seed, threads, double=double, renderer="vcm", params=prm)
    P = int(prm.get("num_iteration_pass", 100))
    NE = int(prm.get("num_eye_trace_samples", 10000))
    img = r["image"].astype(np.float64)
    # the film's own squares: per pass, per sample (ref_render writes the
    # sums of squares of the splats as splatted, W H / N_E included)
    sumsq = r["raw_sumsq"]
    return {"image": img, "variance": vcm_variance(img, sumsq, P, NE), "samples": P * NE, "info": r["info"]}


def render_ptmis(scene: dict, num_samples: int, max_num_vertices: int, seed: int, threads: int,
                 direct_only: bool = False) -> dict:
    """The oracle's renderer::ptmis (NEE + balance heuristic, area lights), or
    with direct_only renderer::ptdirect: film (H, W, 3) and per-pixel variance."""
    tris = np.ascontiguousarray(np.concatenate([p["tris"] for p in scene["prims"]]), dtype=np.float32)
    tri_prim = np.concatenate([np.full(p["tris"].shape[0], i, np.int32) for i, p in enumerate(scene["prims"])])
    W, H = scene["camera"]["width"], scene["camera"]["height"]
    s = np.zeros((H, W, 3), np.float64)
    q = np.zeros((H, W, 3), np.float64)
    prims = scene_prims(scene)
    cam = scene_camera(scene)
    fn = lib().lmo_render_ptdirect if direct_only else lib().lmo_render_ptmis
    fn(tris.ctypes.data, tri_prim.ctypes.data, tris.shape[0], ctypes.addressof(prims),
       len(scene["prims"]), ctypes.addressof(cam), num_samples, max_num_vertices, seed, threads,
       s.ctypes.data, q.ctypes.data)
    img = s * (W * H / num_samples)
    return {"image": img, "variance": pixel_variance(img, q, num_samples, W * H), "samples": num_samples}


def render_ptdirect(scene: dict, num_samples: int, max_num_vertices: int, seed: int, threads: int) -> dict:
    """The oracle's renderer::ptdirect (light samples only, weight 1)."""
    return render_ptmis(scene, num_samples, max_num_vertices, seed, threads, direct_only=True)


def render_ltdirect(scene: dict, num_samples: int, max_num_vertices: int, seed: int, threads: int,
                    independent_light_dir: bool = False) -> dict:
    """The oracle's renderer::ltdirect (light paths connected to the sensor at
    every vertex): film (H, W, 3) and per-pixel variance.
    independent_light_dir: the diagnostic variant that draws the emission
    direction from its own 2D sample."""
    tris = np.ascontiguousarray(np.concatenate([p["tris"] for p in scene["prims"]]), dtype=np.float32)
    tri_prim = np.concatenate([np.full(p["tris"].shape[0], i, np.int32) for i, p in enumerate(scene["prims"])])
    W, H = scene["camera"]["width"], scene["camera"]["height"]
    s = np.zeros((H, W, 3), np.float64)
    q = np.zeros((H, W, 3), np.float64)
    prims = scene_prims(scene)
    cam = scene_camera(scene)
    lib().lmo_render_bdpt_ex(tris.ctypes.data, tri_prim.ctypes.data, tris.shape[0], ctypes.addressof(prims),
                             len(scene["prims"]), ctypes.addressof(cam), num_samples, max_num_vertices, seed,
                             threads, s.ctypes.data, q.ctypes.data, -4 if independent_light_dir else -3)
    img = s * (W * H / num_samples)
    return {"image": img, "variance": pixel_variance(img, q, num_samples, W * H), "samples": num_samples}


SURFACE_FIELDS = ("p", "gn", "sn", "dpdu", "dpdv", "dndu", "dndv", "uv")


def surface(tris, normals, texcoords, flags, rays, hits) -> np.ndarray:
    """(n, 23) surface geometry of hits (t, prim, b1, b2) in FP64:
    p, gn, sn, dpdu, dpdv, dndu, dndv, uv (see lmo_surface)."""
    def d(a, w):
        return None if a is None else np.ascontiguousarray(np.asarray(a, np.float64).reshape(-1, w))

    t, r = d(tris, 9), d(rays, 8)
    nrm, tc = d(normals, 9), d(texcoords, 6)
    h = d(hits, 4)
    fl = None if flags is None else np.ascontiguousarray(np.asarray(flags, np.uint8))
    out = np.zeros((h.shape[0], 23), np.float64)
    ptr = lambda a: None if a is None else a.ctypes.data
    lib().lmo_surface(ptr(t), ptr(nrm), ptr(tc), ptr(fl), ptr(r), ptr(h), h.shape[0], out.ctypes.data)
    return out


def run_ref_isect(prims: list[dict], queries: np.ndarray, double: bool = True) -> dict:
    """Runs the reference's CreateTriangleIntersection (oracle/_ref/ref_isect,
    ref_isect64 for double) on primitives {"transform": (4, 4) row-major,
    "positions": (nv, 3), "faces": (nf, 3), "normals": (nv, 3) or None,
    "texcoords": (nv, 2) or None} and queries (n, 11) = prim, face, o[3],
    d[3], t, b[2].  Returns the per-triangle arrays in global order (tris,
    normals, texcoords, flags) and the per-query geometry (n, 23) and face
    indices."""
    import struct
    import subprocess
    import tempfile

    exe = os.path.join(os.path.dirname(LIB_PATH), "_ref", "ref_isect64" if double else "ref_isect")
    if not os.path.exists(exe):
        raise FileNotFoundError(exe)
    with tempfile.TemporaryDirectory() as td:
        pin, pout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        with open(pin, "wb") as f:
            f.write(struct.pack("<I", len(prims)))
            for p in prims:
                m = np.asarray(p["transform"], np.float64).reshape(4, 4)
                f.write(m.T.astype("<f8").tobytes())  # column-major m[c][r]
                pos = np.asarray(p["positions"], np.float64).reshape(-1, 3)
                faces = np.asarray(p["faces"], np.uint32).reshape(-1, 3)
                nrm, tc = p.get("normals"), p.get("texcoords")
                flags = (1 if nrm is not None else 0) | (2 if tc is not None else 0)
                f.write(struct.pack("<III", pos.shape[0], faces.shape[0], flags))
                f.write(pos.astype("<f8").tobytes())
                if nrm is not None:
                    f.write(np.asarray(nrm, np.float64).reshape(-1, 3).astype("<f8").tobytes())
                if tc is not None:
                    f.write(np.asarray(tc, np.float64).reshape(-1, 2).astype("<f8").tobytes())
                f.write(faces.astype("<u4").tobytes())
            q = np.asarray(queries, np.float64).reshape(-1, 11)
            f.write(struct.pack("<I", q.shape[0]))
            for row in q:
                f.write(struct.pack("<ii", int(row[0]), int(row[1])))
                f.write(row[2:].astype("<f8").tobytes())
        subprocess.run([exe, pin, pout], check=True)
        b = open(pout, "rb").read()
    ntri = struct.unpack_from("<I", b, 0)[0]
    rec = np.dtype([("v", "<f8", 24), ("flags", "<u4")])
    tri = np.frombuffer(b, rec, ntri, 4)
    off = 4 + ntri * rec.itemsize
    nq = struct.unpack_from("<I", b, off)[0]
    qrec = np.dtype([("g", "<f8", 23), ("face", "<i4")])
    qq = np.frombuffer(b, qrec, nq, off + 4)
    return {"tris": tri["v"][:, 0:9].copy(), "normals": tri["v"][:, 9:18].copy(),
            "texcoords": tri["v"][:, 18:24].copy(), "flags": tri["flags"].astype(np.uint8),
            "geom": qq["g"].copy(), "face": qq["face"].copy()}

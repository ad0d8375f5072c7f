"""Python view of the lmgpu C ABI (include/lmgpu.h), via ctypes.

Used by the tests and the benchmark; the product boundary is the C ABI
itself.  Loading fails loudly when liblmgpu.so has not been built: there is
no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .build import LIB_PATH

LMGPU_OK = 0
ERROR_NAMES = {1: "INVALID", 2: "CUDA", 3: "NOT_BUILT", 4: "OVERFLOW", 5: "NO_DEVICE"}


class LmgpuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"lmgpu error {code} ({ERROR_NAMES.get(code, '?')}): {msg}")
        self.code = code


class Hit(ctypes.Structure):
    _fields_ = [("t", ctypes.c_float), ("prim", ctypes.c_int32), ("b1", ctypes.c_float), ("b2", ctypes.c_float)]


# renderer::bdpt's "mis" parameter -> LMGPU_MIS_*
MIS_WEIGHTS = {"powerheuristics": 0, "simple": 1}
VCM_MODES = {"vcm": 0, "bdpt": 1, "bdpm": 2}

HIT_DTYPE = np.dtype([("t", "<f4"), ("prim", "<i4"), ("b1", "<f4"), ("b2", "<f4")])


class AccelInfo(ctypes.Structure):
    _fields_ = [
        ("num_triangles", ctypes.c_uint64),
        ("num_binary_nodes", ctypes.c_uint64),
        ("num_wide_nodes", ctypes.c_uint64),
        ("node_bytes", ctypes.c_uint64),
        ("triangle_bytes", ctypes.c_uint64),
        ("binary_depth", ctypes.c_int32),
        ("wide_depth", ctypes.c_int32),
        ("build_ms", ctypes.c_double),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class TraceProfile(ctypes.Structure):
    """lmgpu_trace_profile: a scene's (or batch's) traversal launches since the
    last read, and renderer::vcm's photon-merge launches."""
    _fields_ = [
        ("launches", ctypes.c_uint64),
        ("rays", ctypes.c_uint64),
        ("node_fetches", ctypes.c_uint64),
        ("triangle_fetches", ctypes.c_uint64),
        ("hits", ctypes.c_uint64),
        ("device_ms", ctypes.c_double),
        ("timed_launches", ctypes.c_uint64),
        ("merge_launches", ctypes.c_uint64),
        ("merge_queries", ctypes.c_uint64),
        ("merge_eye_vertices", ctypes.c_uint64),
        ("merge_entries", ctypes.c_uint64),
        ("merges", ctypes.c_uint64),
        ("merge_ms", ctypes.c_double),
        ("merge_timed_launches", ctypes.c_uint64),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


TRACE_PROFILE_OFF, TRACE_PROFILE_COUNT, TRACE_PROFILE_TIME = 0, 1, 2


class TraceStats(ctypes.Structure):
    _fields_ = [
        ("rays", ctypes.c_uint64),
        ("node_fetches", ctypes.c_uint64),
        ("triangle_fetches", ctypes.c_uint64),
        ("hits", ctypes.c_uint64),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def lib() -> ctypes.CDLL:
    """Loads liblmgpu.so (built in-tree by lmgpu.build)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it first (python -c 'import __graft_entry__ as g; g.build()')")
    L = ctypes.CDLL(LIB_PATH)
    vp, u64, i32 = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int
    L.lmgpu_version.restype = ctypes.c_char_p
    L.lmgpu_last_error.restype = ctypes.c_char_p
    L.lmgpu_accel_create.argtypes = [ctypes.POINTER(vp)]
    L.lmgpu_accel_destroy.argtypes = [vp]
    L.lmgpu_accel_destroy.restype = None
    L.lmgpu_accel_build.argtypes = [vp, vp, u64]
    L.lmgpu_accel_build_device.argtypes = [vp, vp, u64, vp]
    L.lmgpu_flatten_meshes_device.argtypes = [vp, ctypes.c_uint32, vp, vp, vp]
    L.lmgpu_accel_build_meshes.argtypes = [vp, vp, ctypes.c_uint32]
    L.lmgpu_accel_get_info.argtypes = [vp, ctypes.POINTER(AccelInfo)]
    L.lmgpu_trace.argtypes = [vp, vp, vp, u64, i32]
    L.lmgpu_trace_device.argtypes = [vp, vp, vp, u64, i32, vp]
    L.lmgpu_trace_stats_device.argtypes = [vp, vp, vp, u64, i32, vp, ctypes.POINTER(TraceStats)]
    L.lmgpu_accel_check.argtypes = [vp, vp]
    L.lmgpu_trace_static_scene.argtypes = [vp, u64, vp, vp, u64, i32, vp]
    L.lmgpu_accel_set_tuning.argtypes = [vp, i32, i32]
    L.lmgpu_accel_set_attributes.argtypes = [vp, vp, vp, vp, u64]
    L.lmgpu_surface.argtypes = [vp, vp, vp, u64, vp]
    L.lmgpu_surface_device.argtypes = [vp, vp, vp, u64, vp, vp]
    L.lmgpu_scene_create.argtypes = [vp, vp, u64, vp, ctypes.c_uint32, vp, ctypes.POINTER(vp)]
    L.lmgpu_scene_destroy.argtypes = [vp]
    L.lmgpu_scene_destroy.restype = None
    L.lmgpu_scene_set_environment.argtypes = [vp, vp]
    L.lmgpu_scene_accel.argtypes = [vp, ctypes.POINTER(vp)]
    L.lmgpu_render_pt.argtypes = [vp, vp, vp, vp]
    L.lmgpu_render_pt_device.argtypes = [vp, vp, vp, vp, vp]
    L.lmgpu_render_bdpt.argtypes = [vp, vp, vp, vp]
    L.lmgpu_render_ptmis.argtypes = [vp, vp, vp, vp]
    L.lmgpu_render_ptdirect.argtypes = [vp, vp, vp, vp]
    L.lmgpu_render_ltdirect.argtypes = [vp, vp, vp, vp]
    L.lmgpu_render_bdpt_mis.argtypes = [vp, vp, i32, vp, vp]
    L.lmgpu_render_bdpt_mis_device.argtypes = [vp, vp, i32, vp, vp, vp]
    L.lmgpu_render_ltdirect_device.argtypes = [vp, vp, vp, vp, vp]
    L.lmgpu_render_vcm.argtypes = [vp, vp, vp, vp]
    L.lmgpu_render_vcm_device.argtypes = [vp, vp, vp, vp, vp]
    L.lmgpu_guide_num_params.argtypes = [ctypes.POINTER(u64)]
    L.lmgpu_guide_create.argtypes = [vp, ctypes.c_uint32, ctypes.POINTER(vp)]
    L.lmgpu_guide_destroy.argtypes = [vp]
    L.lmgpu_guide_destroy.restype = None
    L.lmgpu_guide_get_params.argtypes = [vp, vp, u64]
    L.lmgpu_guide_set_params.argtypes = [vp, vp, u64]
    L.lmgpu_guide_forward.argtypes = [vp, vp, u64, vp]
    L.lmgpu_guide_gradient.argtypes = [vp, vp, vp, vp, u64, vp, vp]
    L.lmgpu_guide_train_step.argtypes = [vp, vp, vp, vp, u64, ctypes.c_float, vp]
    L.lmgpu_guide_forward_device.argtypes = [vp, vp, u64, vp, vp]
    L.lmgpu_guide_train_step_device.argtypes = [vp, vp, vp, vp, u64, ctypes.c_float, vp]
    L.lmgpu_render_pt_guided.argtypes = [vp, vp, vp, vp, vp, vp, vp]
    L.lmgpu_render_pt_guided_device.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp]
    L.lmgpu_batch_create.argtypes = [vp, ctypes.c_uint32, ctypes.POINTER(vp)]
    L.lmgpu_batch_destroy.argtypes = [vp]
    L.lmgpu_batch_destroy.restype = None
    L.lmgpu_batch_render_pt.argtypes = [vp, vp, vp, vp]
    L.lmgpu_batch_render_pt_device.argtypes = [vp, vp, vp, vp, vp]
    L.lmgpu_batch_autotune.argtypes = [vp, vp, vp]
    L.lmgpu_batch_set_tuning.argtypes = [vp, vp]
    L.lmgpu_batch_get_tuning.argtypes = [vp, vp]
    L.lmgpu_batch_launch_count.argtypes = [vp, ctypes.POINTER(u64)]
    L.lmgpu_render_ptdirect_device.argtypes = [vp, vp, vp, vp, vp]
    L.lmgpu_render_ptmis_device.argtypes = [vp, vp, vp, vp, vp]
    L.lmgpu_scene_launch_count.argtypes = [vp, ctypes.POINTER(u64)]
    L.lmgpu_scene_set_trace_profile.argtypes = [vp, ctypes.c_int]
    L.lmgpu_scene_read_trace_profile.argtypes = [vp, ctypes.POINTER(TraceProfile)]
    L.lmgpu_batch_set_trace_profile.argtypes = [vp, ctypes.c_int]
    L.lmgpu_batch_read_trace_profile.argtypes = [vp, ctypes.POINTER(TraceProfile)]
    L.lmgpu_render_bdpt_device.argtypes = [vp, vp, vp, vp, vp]
    for name in ("lmgpu_accel_create", "lmgpu_accel_build", "lmgpu_accel_build_device", "lmgpu_accel_get_info",
                 "lmgpu_trace", "lmgpu_trace_device", "lmgpu_trace_stats_device", "lmgpu_accel_check",
                 "lmgpu_trace_static_scene", "lmgpu_accel_set_tuning", "lmgpu_scene_create", "lmgpu_scene_accel",
                 "lmgpu_render_pt", "lmgpu_render_pt_device", "lmgpu_render_bdpt", "lmgpu_render_bdpt_device", "lmgpu_scene_launch_count",
                 "lmgpu_render_ptmis", "lmgpu_render_ptmis_device", "lmgpu_render_ptdirect",
                 "lmgpu_batch_create", "lmgpu_batch_render_pt", "lmgpu_batch_render_pt_device",
                 "lmgpu_batch_autotune", "lmgpu_batch_set_tuning", "lmgpu_batch_get_tuning",
                 "lmgpu_batch_launch_count", "lmgpu_guide_num_params", "lmgpu_guide_create",
                 "lmgpu_guide_get_params", "lmgpu_guide_set_params", "lmgpu_guide_forward", "lmgpu_guide_gradient",
                 "lmgpu_guide_train_step", "lmgpu_guide_forward_device", "lmgpu_guide_train_step_device",
                 "lmgpu_render_pt_guided", "lmgpu_render_pt_guided_device",
                 "lmgpu_render_ptdirect_device", "lmgpu_render_ltdirect", "lmgpu_render_ltdirect_device",
                 "lmgpu_render_bdpt_mis", "lmgpu_render_bdpt_mis_device", "lmgpu_render_vcm",
                 "lmgpu_flatten_meshes_device", "lmgpu_accel_build_meshes",
                 "lmgpu_render_vcm_device",
                 "lmgpu_accel_set_attributes", "lmgpu_surface", "lmgpu_surface_device",
                 "lmgpu_scene_set_environment", "lmgpu_scene_set_trace_profile",
                 "lmgpu_scene_read_trace_profile", "lmgpu_batch_set_trace_profile",
                 "lmgpu_batch_read_trace_profile"):
        getattr(L, name).restype = ctypes.c_int
    _lib = L
    return L


def _check(rc: int) -> None:
    if rc != LMGPU_OK:
        raise LmgpuError(rc, lib().lmgpu_last_error().decode())


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


class Mesh(ctypes.Structure):
    """lmgpu_mesh: an indexed triangle mesh with its column-major transform."""
    _fields_ = [("positions", ctypes.c_void_p), ("faces", ctypes.c_void_p), ("num_vertices", ctypes.c_uint32),
                ("num_faces", ctypes.c_uint32), ("transform", ctypes.c_float * 16)]


def _mesh_table(meshes, ptrs) -> ctypes.Array:
    """meshes: (positions, faces, transform) with ptrs giving the buffers' addresses."""
    table = (Mesh * max(1, len(meshes)))()
    for i, ((pos, faces, tr), (pp, fp)) in enumerate(zip(meshes, ptrs)):
        table[i].positions = pp
        table[i].faces = fp
        table[i].num_vertices = int(np.asarray(pos).size // 3) if not hasattr(pos, "numel") else int(pos.numel() // 3)
        table[i].num_faces = int(np.asarray(faces).size // 3) if not hasattr(faces, "numel") else int(faces.numel() // 3)
        t = np.asarray(tr, np.float32).reshape(-1)
        for k in range(16):
            table[i].transform[k] = float(t[k])
    return table


def flatten_meshes_device(meshes, d_triangles: int, d_tri_prim: int = 0, stream: int = 0) -> None:
    """lmgpu_flatten_meshes_device: meshes as (positions, faces, transform)
    with positions / faces CUDA tensors (float32 / int32 holding uint32
    indices) and transform 16 floats, column-major m[c][r]."""
    table = _mesh_table(meshes, [(p.data_ptr(), f.data_ptr()) for p, f, _ in meshes])
    _check(lib().lmgpu_flatten_meshes_device(ctypes.addressof(table), len(meshes), d_triangles, d_tri_prim or None,
                                             stream or None))


class Accel:
    """An accel::cuda instance: GPU-built binned-SAH BVH8 with watertight traversal."""

    def __init__(self) -> None:
        h = ctypes.c_void_p()
        _check(lib().lmgpu_accel_create(ctypes.byref(h)))
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().lmgpu_accel_destroy(self._h)
            self._h = None

    def __del__(self) -> None:
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def build(self, tris: np.ndarray) -> None:
        t = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1, 9)
        _check(lib().lmgpu_accel_build(self._h, _ptr(t), t.shape[0]))

    def build_device(self, d_tris_ptr: int, ntri: int, stream: int = 0) -> None:
        _check(lib().lmgpu_accel_build_device(self._h, d_tris_ptr, ntri, stream))

    def build_meshes(self, meshes) -> None:
        """lmgpu_accel_build_meshes: meshes as (positions (nv, 3) float32,
        faces (nf, 3) uint32, transform 16 floats column-major m[c][r])."""
        keep = [(np.ascontiguousarray(p, np.float32), np.ascontiguousarray(f, np.uint32), t) for p, f, t in meshes]
        table = _mesh_table(keep, [(_ptr(p), _ptr(f)) for p, f, _ in keep])
        _check(lib().lmgpu_accel_build_meshes(self._h, ctypes.addressof(table), len(keep)))

    def info(self) -> dict:
        i = AccelInfo()
        _check(lib().lmgpu_accel_get_info(self._h, ctypes.byref(i)))
        return i.as_dict()

    def trace(self, rays: np.ndarray, anyhit: bool = False, out: np.ndarray | None = None) -> np.ndarray:
        r = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        if out is None:
            out = np.empty(r.shape[0], dtype=HIT_DTYPE)
        _check(lib().lmgpu_trace(self._h, _ptr(r), _ptr(out), r.shape[0], int(anyhit)))
        return out

    def trace_ptr(self, rays_ptr: int, hits_ptr: int, n: int, anyhit: bool = False) -> None:
        """Host-pointer trace (pinned buffers from torch, for instance)."""
        _check(lib().lmgpu_trace(self._h, rays_ptr, hits_ptr, n, int(anyhit)))

    def trace_device(self, d_rays_ptr: int, d_hits_ptr: int, n: int, anyhit: bool = False, stream: int = 0) -> None:
        _check(lib().lmgpu_trace_device(self._h, d_rays_ptr, d_hits_ptr, n, int(anyhit), stream))

    def trace_stats_device(self, d_rays_ptr: int, d_hits_ptr: int, n: int, anyhit: bool = False,
                           stream: int = 0) -> dict:
        s = TraceStats()
        _check(lib().lmgpu_trace_stats_device(self._h, d_rays_ptr, d_hits_ptr, n, int(anyhit), stream,
                                              ctypes.byref(s)))
        return s.as_dict()

    def set_tuning(self, refill: int, postpone: int) -> None:
        _check(lib().lmgpu_accel_set_tuning(self._h, refill, postpone))

    def set_attributes(self, normals=None, texcoords=None, flags=None, ntri: int | None = None) -> None:
        """Per-triangle vertex normals (ntri, 9), texcoords (ntri, 6) and
        flags (ntri,) of lmgpu_surface (global triangle order)."""
        n = np.ascontiguousarray(normals, np.float32).reshape(-1, 9) if normals is not None else None
        t = np.ascontiguousarray(texcoords, np.float32).reshape(-1, 6) if texcoords is not None else None
        f = np.ascontiguousarray(flags, np.uint8) if flags is not None else None
        if ntri is None:
            ntri = next(a.shape[0] for a in (n, t, f) if a is not None)
        ptr = lambda a: None if a is None else a.ctypes.data  # noqa: E731
        _check(lib().lmgpu_accel_set_attributes(self._h, ptr(n), ptr(t), ptr(f), ntri))

    def surface(self, rays: np.ndarray, hits: np.ndarray) -> np.ndarray:
        """Surface geometry (n, 23) of hits: p, gn, sn, dpdu, dpdv, dndu,
        dndv, uv (IntersectionUtils::CreateTriangleIntersection)."""
        r = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        h = np.ascontiguousarray(hits)
        if h.dtype != HIT_DTYPE or h.shape != (r.shape[0],):
            raise ValueError("hits: one HIT_DTYPE record per ray")
        n = r.shape[0]
        out = np.empty((23, n), np.float32)
        _check(lib().lmgpu_surface(self._h, r.ctypes.data, h.ctypes.data, n, out.ctypes.data))
        return out.T.copy()

    def surface_device(self, d_rays_ptr: int, d_hits_ptr: int, n: int, d_out_ptr: int, stream: int = 0) -> None:
        _check(lib().lmgpu_surface_device(self._h, d_rays_ptr, d_hits_ptr, n, d_out_ptr, stream))

    def check(self, stream: int = 0) -> None:
        _check(lib().lmgpu_accel_check(self._h, stream))


STATIC_MAX_TRIANGLES = 16384  # LMGPU_STATIC_MAX_TRIANGLES


def trace_static_scene(d_tris_ptr: int, ntri: int, d_rays_ptr: int, d_hits_ptr: int, nrays: int,
                       anyhit: bool = False, stream: int = 0) -> None:
    """Allocation-free build + trace on device buffers (lmgpu_trace_static_scene)."""
    _check(lib().lmgpu_trace_static_scene(d_tris_ptr, ntri, d_rays_ptr, d_hits_ptr, nrays, int(anyhit), stream))


class Prim(ctypes.Structure):
    _fields_ = [("bsdf", ctypes.c_int32), ("is_light", ctypes.c_int32), ("R", ctypes.c_float * 3),
                ("Le", ctypes.c_float * 3), ("eta1", ctypes.c_float), ("eta2", ctypes.c_float),
                ("ct_eta", ctypes.c_float * 3), ("ct_k", ctypes.c_float * 3), ("roughness", ctypes.c_float)]


class Camera(ctypes.Structure):
    _fields_ = [("eye", ctypes.c_float * 3), ("center", ctypes.c_float * 3), ("up", ctypes.c_float * 3),
                ("fov_deg", ctypes.c_float), ("width", ctypes.c_int32), ("height", ctypes.c_int32)]


class PtParams(ctypes.Structure):
    _fields_ = [("spp", ctypes.c_uint64), ("max_num_vertices", ctypes.c_int32), ("seed", ctypes.c_uint32),
                ("min_num_vertices", ctypes.c_int32), ("reserved", ctypes.c_int32)]


BSDF_NULL, BSDF_DIFFUSE, BSDF_DIELECTRIC, BSDF_COOK_TORRANCE = 0, 1, 2, 3


class GuidingParams(ctypes.Structure):
    _fields_ = [("alpha", ctypes.c_float), ("learning_rate", ctypes.c_float), ("train", ctypes.c_uint32),
                ("batch", ctypes.c_uint32), ("max_steps_per_pass", ctypes.c_uint32), ("rr_mode", ctypes.c_uint32)]


class Scene:
    """A device-resident scene (lmgpu_scene): triangles, primitives, camera, BVH.

    `scene` is the dict of lmgpu.scenes (prims with kind 0 = diffuse,
    1 = area light without a BSDF; camera)."""

    def __init__(self, scene: dict) -> None:
        from .scenes import prim_params, scene_triangles

        tris, tri_prim = scene_triangles(scene)
        self.tris = np.ascontiguousarray(tris, dtype=np.float32)
        self.tri_prim = np.ascontiguousarray(tri_prim, dtype=np.int32)
        prims = (Prim * len(scene["prims"]))()
        for i, p0 in enumerate(scene["prims"]):
            p = prim_params(p0)
            prims[i].bsdf = p["bsdf"]
            prims[i].is_light = 1 if p["light"] else 0
            for k in range(3):
                prims[i].R[k] = p["R"][k]
                prims[i].Le[k] = p["Le"][k]
                prims[i].ct_eta[k] = p["ct_eta"][k]
                prims[i].ct_k[k] = p["ct_k"][k]
            prims[i].eta1, prims[i].eta2, prims[i].roughness = p["eta1"], p["eta2"], p["roughness"]
        c = scene["camera"]
        cam = Camera()
        for k in range(3):
            cam.eye[k], cam.center[k], cam.up[k] = c["eye"][k], c["center"][k], c["up"][k]
        cam.fov_deg, cam.width, cam.height = c["fov"], c["width"], c["height"]
        self.width, self.height = c["width"], c["height"]
        h = ctypes.c_void_p()
        _check(lib().lmgpu_scene_create(self.tris.ctypes.data, self.tri_prim.ctypes.data, self.tris.shape[0],
                                        ctypes.addressof(prims), len(scene["prims"]), ctypes.addressof(cam),
                                        ctypes.byref(h)))
        self._h = h
        if scene.get("env") is not None:
            le = (ctypes.c_float * 3)(*scene["env"])
            _check(lib().lmgpu_scene_set_environment(self._h, le))

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().lmgpu_scene_destroy(self._h)
            self._h = None

    def __del__(self) -> None:
        try:
            self.close()
        except Exception:
            pass

    def render_pt(self, spp: int, max_num_vertices: int = -1, seed: int = 0, min_num_vertices: int = 0) -> tuple[np.ndarray, np.ndarray]:
        """renderer::pt: film (H, W, 3) and per-pixel variance of the estimate."""
        img = np.empty((self.height, self.width, 3), np.float32)
        var = np.empty((self.height, self.width, 3), np.float32)
        prm = PtParams(spp, max_num_vertices, seed, min_num_vertices)
        _check(lib().lmgpu_render_pt(self._h, ctypes.byref(prm), img.ctypes.data, var.ctypes.data))
        return img, var

    def render_pt_device(self, d_image: int, d_variance: int, spp: int, max_num_vertices: int = -1,
                         seed: int = 0, stream: int = 0, min_num_vertices: int = 0) -> None:
        prm = PtParams(spp, max_num_vertices, seed, min_num_vertices)
        _check(lib().lmgpu_render_pt_device(self._h, ctypes.byref(prm), d_image, d_variance, stream))

    def render_ptmis(self, spp: int, max_num_vertices: int = -1, seed: int = 0, min_num_vertices: int = 0) -> tuple[np.ndarray, np.ndarray]:
        """renderer::ptmis: film (H, W, 3) and per-pixel variance of the estimate."""
        img = np.empty((self.height, self.width, 3), np.float32)
        var = np.empty((self.height, self.width, 3), np.float32)
        prm = PtParams(spp, max_num_vertices, seed, min_num_vertices)
        _check(lib().lmgpu_render_ptmis(self._h, ctypes.byref(prm), img.ctypes.data, var.ctypes.data))
        return img, var

    def render_ptmis_device(self, d_image: int, d_variance: int, spp: int, max_num_vertices: int = -1,
                            seed: int = 0, stream: int = 0, min_num_vertices: int = 0) -> None:
        prm = PtParams(spp, max_num_vertices, seed, min_num_vertices)
        _check(lib().lmgpu_render_ptmis_device(self._h, ctypes.byref(prm), d_image, d_variance, stream))

    def render_ptdirect(self, spp: int, max_num_vertices: int = -1, seed: int = 0, min_num_vertices: int = 0) -> tuple[np.ndarray, np.ndarray]:
        """renderer::ptdirect: film (H, W, 3) and per-pixel variance of the estimate."""
        img = np.empty((self.height, self.width, 3), np.float32)
        var = np.empty((self.height, self.width, 3), np.float32)
        prm = PtParams(spp, max_num_vertices, seed, min_num_vertices)
        _check(lib().lmgpu_render_ptdirect(self._h, ctypes.byref(prm), img.ctypes.data, var.ctypes.data))
        return img, var

    def render_ptdirect_device(self, d_image: int, d_variance: int, spp: int, max_num_vertices: int = -1,
                               seed: int = 0, stream: int = 0, min_num_vertices: int = 0) -> None:
        prm = PtParams(spp, max_num_vertices, seed, min_num_vertices)
        _check(lib().lmgpu_render_ptdirect_device(self._h, ctypes.byref(prm), d_image, d_variance, stream))

    def render_ltdirect(self, spp: int, max_num_vertices: int = -1, seed: int = 0, min_num_vertices: int = 0) -> tuple[np.ndarray, np.ndarray]:
        """renderer::ltdirect with spp x W x H light paths: film (H, W, 3) and
        per-pixel variance of the estimate."""
        img = np.empty((self.height, self.width, 3), np.float32)
        var = np.empty((self.height, self.width, 3), np.float32)
        prm = PtParams(spp, max_num_vertices, seed, min_num_vertices)
        _check(lib().lmgpu_render_ltdirect(self._h, ctypes.byref(prm), img.ctypes.data, var.ctypes.data))
        return img, var

    def render_ltdirect_device(self, d_image: int, d_variance: int, spp: int, max_num_vertices: int = -1,
                               seed: int = 0, stream: int = 0, min_num_vertices: int = 0) -> None:
        prm = PtParams(spp, max_num_vertices, seed, min_num_vertices)
        _check(lib().lmgpu_render_ltdirect_device(self._h, ctypes.byref(prm), d_image, d_variance, stream))

    def render_pt_guided(self, guide, spp: int, max_num_vertices: int = -1, seed: int = 0, alpha: float = 0.5,
                         learning_rate: float = 1e-3, train: bool = True, batch: int = 1 << 18,
                         max_steps_per_pass: int = 4, rr_mode: int = 1, min_num_vertices: int = 0) -> tuple[np.ndarray, np.ndarray, float]:
        """Guided renderer::pt: film, per-pixel variance, last training loss."""
        img = np.empty((self.height, self.width, 3), np.float32)
        var = np.empty((self.height, self.width, 3), np.float32)
        prm = PtParams(spp, max_num_vertices, seed, min_num_vertices)
        gp = GuidingParams(alpha, learning_rate, 1 if train else 0, batch, max_steps_per_pass, rr_mode)
        loss = ctypes.c_float()
        _check(lib().lmgpu_render_pt_guided(self._h, guide._h, ctypes.byref(prm), ctypes.byref(gp), img.ctypes.data,
                                            var.ctypes.data, ctypes.byref(loss)))
        return img, var, loss.value

    def render_pt_guided_device(self, guide, d_image: int, d_variance: int, spp: int, max_num_vertices: int = -1,
                                seed: int = 0, alpha: float = 0.5, learning_rate: float = 1e-3, train: bool = True,
                                batch: int = 1 << 18, max_steps_per_pass: int = 4, rr_mode: int = 1,
                                stream: int = 0, min_num_vertices: int = 0) -> float:
        prm = PtParams(spp, max_num_vertices, seed, min_num_vertices)
        gp = GuidingParams(alpha, learning_rate, 1 if train else 0, batch, max_steps_per_pass, rr_mode)
        loss = ctypes.c_float()
        _check(lib().lmgpu_render_pt_guided_device(self._h, guide._h, ctypes.byref(prm), ctypes.byref(gp), d_image,
                                                   d_variance, stream, ctypes.byref(loss)))
        return loss.value

    def launch_count(self) -> int:
        """Kernels launched by the renderers for this scene so far."""
        n = ctypes.c_uint64()
        _check(lib().lmgpu_scene_launch_count(self._h, ctypes.byref(n)))
        return n.value

    def set_trace_profile(self, mode: int) -> None:
        """Instruments the traversal launches of later renders: TRACE_PROFILE_COUNT
        (fetch counters), TRACE_PROFILE_TIME (device time per launch) or _OFF."""
        _check(lib().lmgpu_scene_set_trace_profile(self._h, mode))

    def read_trace_profile(self) -> dict:
        """The record since the last read or mode change (waits for the device)."""
        r = TraceProfile()
        _check(lib().lmgpu_scene_read_trace_profile(self._h, ctypes.byref(r)))
        return r.as_dict()

    def render_bdpt(self, spp: int, max_num_vertices: int = -1, seed: int = 0,
                    mis: str = "powerheuristics", min_num_vertices: int = 0) -> tuple[np.ndarray, np.ndarray]:
        """renderer::bdpt: film (H, W, 3) and per-pixel variance of the
        estimate; mis: the renderer's MIS weight, powerheuristics or simple."""
        img = np.empty((self.height, self.width, 3), np.float32)
        var = np.empty((self.height, self.width, 3), np.float32)
        prm = PtParams(spp, max_num_vertices, seed, min_num_vertices)
        _check(lib().lmgpu_render_bdpt_mis(self._h, ctypes.byref(prm), MIS_WEIGHTS[mis], img.ctypes.data,
                                           var.ctypes.data))
        return img, var

    def render_vcm(self, **params) -> tuple[np.ndarray, np.ndarray]:
        """renderer::vcm (keyword parameters as vcm_params): film (H, W, 3)
        and per-pixel variance of the estimate."""
        prm = vcm_params(**params)
        img = np.empty((self.height, self.width, 3), np.float32)
        var = np.empty((self.height, self.width, 3), np.float32)
        _check(lib().lmgpu_render_vcm(self._h, ctypes.byref(prm), img.ctypes.data, var.ctypes.data))
        return img, var

    def render_vcm_device(self, d_image: int, d_variance: int, stream: int = 0, **params) -> None:
        prm = vcm_params(**params)
        _check(lib().lmgpu_render_vcm_device(self._h, ctypes.byref(prm), d_image, d_variance, stream))

    def render_bdpt_device(self, d_image: int, d_variance: int, spp: int, max_num_vertices: int = -1,
                           seed: int = 0, stream: int = 0, min_num_vertices: int = 0) -> None:
        prm = PtParams(spp, max_num_vertices, seed, min_num_vertices)
        _check(lib().lmgpu_render_bdpt_device(self._h, ctypes.byref(prm), d_image, d_variance, stream))


class VcmParams(ctypes.Structure):
    """lmgpu_vcm_params: renderer::vcm's parameters (renderer_vcm.cpp:573-593)."""
    _fields_ = [("max_num_vertices", ctypes.c_int32), ("min_num_vertices", ctypes.c_int32),
                ("num_iteration_pass", ctypes.c_uint64), ("num_photon_trace_samples", ctypes.c_uint64),
                ("num_eye_trace_samples", ctypes.c_uint64), ("initial_radius", ctypes.c_float),
                ("alpha", ctypes.c_float), ("mode", ctypes.c_int32), ("seed", ctypes.c_uint32)]


def vcm_params(max_num_vertices: int = 10, min_num_vertices: int = 0, num_iteration_pass: int = 100,
               num_photon_trace_samples: int = 10000, num_eye_trace_samples: int = 10000,
               initial_radius: float = 0.1, alpha: float = 0.7, mode: str = "vcm", seed: int = 0) -> VcmParams:
    """renderer::vcm's parameters with the reference's defaults."""
    return VcmParams(max_num_vertices, min_num_vertices, num_iteration_pass, num_photon_trace_samples,
                     num_eye_trace_samples, initial_radius, alpha, VCM_MODES[mode], seed)


class BatchParams(ctypes.Structure):
    _fields_ = [("spp", ctypes.c_uint64), ("max_num_vertices", ctypes.c_int32), ("seed", ctypes.c_uint32),
                ("rr_depth", ctypes.c_int32)]


class BatchTuning(ctypes.Structure):
    _fields_ = [("refill", ctypes.c_int32), ("postpone", ctypes.c_int32), ("wave_paths", ctypes.c_uint64),
                ("probe_ms", ctypes.c_double)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class Batch:
    """Several scenes (views) rendered by one wavefront (lmgpu_batch).  The
    Scene objects must stay alive while the batch is used."""

    def __init__(self, scenes: list) -> None:
        self.scenes = list(scenes)
        arr = (ctypes.c_void_p * len(self.scenes))(*[s._h.value for s in self.scenes])
        h = ctypes.c_void_p()
        _check(lib().lmgpu_batch_create(ctypes.addressof(arr), len(self.scenes), ctypes.byref(h)))
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().lmgpu_batch_destroy(self._h)
            self._h = None

    def __del__(self) -> None:
        try:
            self.close()
        except Exception:
            pass

    def render_pt(self, spp: int, max_num_vertices: int = -1, seed: int = 0, rr_depth: int = 0) -> list:
        """Films and per-pixel variances of every view: [(img, var), ...]."""
        out = [(np.empty((s.height, s.width, 3), np.float32), np.empty((s.height, s.width, 3), np.float32))
               for s in self.scenes]
        imgs = (ctypes.c_void_p * len(out))(*[o[0].ctypes.data for o in out])
        vars_ = (ctypes.c_void_p * len(out))(*[o[1].ctypes.data for o in out])
        prm = BatchParams(spp, max_num_vertices, seed, rr_depth)
        _check(lib().lmgpu_batch_render_pt(self._h, ctypes.byref(prm), ctypes.addressof(imgs),
                                           ctypes.addressof(vars_)))
        return out

    def render_pt_device(self, d_images: int, d_variances: int, spp: int, max_num_vertices: int = -1,
                         seed: int = 0, rr_depth: int = 0, stream: int = 0) -> None:
        prm = BatchParams(spp, max_num_vertices, seed, rr_depth)
        _check(lib().lmgpu_batch_render_pt_device(self._h, ctypes.byref(prm), d_images, d_variances, stream))

    def autotune(self, spp: int, max_num_vertices: int = -1, seed: int = 0, rr_depth: int = 0) -> dict:
        prm = BatchParams(spp, max_num_vertices, seed, rr_depth)
        t = BatchTuning()
        _check(lib().lmgpu_batch_autotune(self._h, ctypes.byref(prm), ctypes.byref(t)))
        return t.as_dict()

    def set_tuning(self, refill: int, postpone: int, wave_paths: int) -> None:
        t = BatchTuning(refill, postpone, wave_paths, 0.0)
        _check(lib().lmgpu_batch_set_tuning(self._h, ctypes.byref(t)))

    def tuning(self) -> dict:
        t = BatchTuning()
        _check(lib().lmgpu_batch_get_tuning(self._h, ctypes.byref(t)))
        return t.as_dict()

    def launch_count(self) -> int:
        n = ctypes.c_uint64()
        _check(lib().lmgpu_batch_launch_count(self._h, ctypes.byref(n)))
        return n.value

    def set_trace_profile(self, mode: int) -> None:
        """Instruments the multi-scene traversal launches of later renders (as
        Scene.set_trace_profile); while on, bounces are launched one by one
        instead of through the captured graphs."""
        _check(lib().lmgpu_batch_set_trace_profile(self._h, mode))

    def read_trace_profile(self) -> dict:
        """The record since the last read or mode change (waits for the device)."""
        r = TraceProfile()
        _check(lib().lmgpu_batch_read_trace_profile(self._h, ctypes.byref(r)))
        return r.as_dict()


class Guide:
    """The path-guiding network (lmgpu_guide): 8-lobe vMF mixture from an MLP
    on the tensor cores.  box = (lo.x, lo.y, lo.z, hi.x, hi.y, hi.z)."""

    def __init__(self, box, seed: int = 0) -> None:
        b = (ctypes.c_float * 6)(*box)
        h = ctypes.c_void_p()
        _check(lib().lmgpu_guide_create(b, seed, ctypes.byref(h)))
        self._h = h

    @staticmethod
    def num_params() -> int:
        n = ctypes.c_uint64()
        _check(lib().lmgpu_guide_num_params(ctypes.byref(n)))
        return n.value

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().lmgpu_guide_destroy(self._h)
            self._h = None

    def __del__(self) -> None:
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> np.ndarray:
        p = np.empty(self.num_params(), np.float32)
        _check(lib().lmgpu_guide_get_params(self._h, p.ctypes.data, p.size))
        return p

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, np.float32)
        _check(lib().lmgpu_guide_set_params(self._h, p.ctypes.data, p.size))

    def forward(self, queries: np.ndarray) -> np.ndarray:
        q = np.ascontiguousarray(queries, np.float32).reshape(-1, 9)
        raw = np.empty((q.shape[0], 40), np.float32)
        _check(lib().lmgpu_guide_forward(self._h, q.ctypes.data, q.shape[0], raw.ctypes.data))
        return raw

    def gradient(self, queries, dirs, weights) -> tuple[float, np.ndarray]:
        q = np.ascontiguousarray(queries, np.float32).reshape(-1, 9)
        d = np.ascontiguousarray(dirs, np.float32).reshape(-1, 3)
        w = np.ascontiguousarray(weights, np.float32).reshape(-1)
        g = np.empty(self.num_params(), np.float32)
        loss = ctypes.c_float()
        _check(lib().lmgpu_guide_gradient(self._h, q.ctypes.data, d.ctypes.data, w.ctypes.data, q.shape[0],
                                          g.ctypes.data, ctypes.byref(loss)))
        return loss.value, g

    def forward_device(self, d_queries: int, n: int, d_raw: int, stream: int = 0) -> None:
        _check(lib().lmgpu_guide_forward_device(self._h, d_queries, n, d_raw, stream))

    def train_step_device(self, d_queries: int, d_dirs: int, d_weights: int, n: int, lr: float = 1e-3,
                          stream: int = 0) -> None:
        _check(lib().lmgpu_guide_train_step_device(self._h, d_queries, d_dirs, d_weights, n, lr, stream))

    def train_step(self, queries, dirs, weights, lr: float = 1e-3) -> float:
        q = np.ascontiguousarray(queries, np.float32).reshape(-1, 9)
        d = np.ascontiguousarray(dirs, np.float32).reshape(-1, 3)
        w = np.ascontiguousarray(weights, np.float32).reshape(-1)
        loss = ctypes.c_float()
        _check(lib().lmgpu_guide_train_step(self._h, q.ctypes.data, d.ctypes.data, w.ctypes.data, q.shape[0], lr,
                                            ctypes.byref(loss)))
        return loss.value


def version() -> str:
    return lib().lmgpu_version().decode()

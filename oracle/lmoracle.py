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
        _lib = L
    return _lib


class OracleAccel:
    """accel::naive (kind 0) or accel::bvh_sahbin (kind 1), restated in C."""

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

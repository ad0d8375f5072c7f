"""Helpers shared by the parity tests: hit-point geometry in the reference's
terms and the classification of documented disagreement classes.

A GPU hit id that differs from the oracle's is only accepted when FP32
rounding can explain it, and every test reports the counts.  The error
model: an FP32 ray/triangle test computes the hit point and the edge
functions with an absolute error of about one ulp of the coordinates
involved, amplified by 1 / |cos theta| at grazing incidence (the error in t
moves the point along the ray).  With s = max(1, |o|, |p|) (infinity norms
of the ray origin and the FP64 hit point) a candidate's tolerance is

    tol = 2^-23 s (4 + 1 / |cos theta|)      (world units)

and the classes, checked in this order, are:
  degen    a candidate triangle has zero area (TriAccel k == 3 never hits,
           triaccel.h:73-77);
  grazing  |d.n| < 1e-6 |d| |n| on a candidate;
  edge     on either candidate the FP64 plane hit lies within tol of an edge
           line, inside or outside (the reference's Wald test is inclusive
           but not watertight, triaccel.h:150; the GPU test is watertight);
  range    on either candidate the FP64 t lies within tol / |d| of the
           ray's tmin or tmax (the two sides round t differently);
  tie      both hit and their FP64 t differ by at most the sum of their
           tolerances (exact or FP32-unresolvable ties; the reference keeps
           the last accepted candidate, triaccel.h:137).
"""
from __future__ import annotations

import numpy as np


def tri_normals(tris: np.ndarray) -> np.ndarray:
    T = np.asarray(tris, dtype=np.float64).reshape(-1, 9)
    return np.cross(T[:, 3:6] - T[:, 0:3], T[:, 6:9] - T[:, 0:3])


def _candidate(T: np.ndarray, R: np.ndarray, ids: np.ndarray) -> dict:
    """FP64 plane hit of each ray on triangle ids[i] (ids < 0: no candidate):
    t, signed world distance to the nearest edge line (> 0 inside), |cos|,
    the error-model tolerance, and whether the triangle has zero area."""
    ok = ids >= 0
    v = T[np.where(ok, ids, 0)].reshape(-1, 3, 3)
    o, d = R[:, 0:3], R[:, 4:7]
    n = np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0])
    nn = np.linalg.norm(n, axis=1)
    dl = np.linalg.norm(d, axis=1)
    dn = np.einsum("ij,ij->i", n, d)
    with np.errstate(divide="ignore", invalid="ignore"):
        t = np.einsum("ij,ij->i", n, v[:, 0] - o) / dn
        p = o + t[:, None] * d
        cos = np.abs(dn) / (nn * dl)
        edge = np.full(len(ids), np.inf)
        for i in range(3):
            a, b, c = v[:, i], v[:, (i + 1) % 3], v[:, (i + 2) % 3]
            m = np.cross(n, b - a)
            m /= np.linalg.norm(m, axis=1, keepdims=True)
            m *= np.sign(np.einsum("ij,ij->i", m, c - a))[:, None]
            edge = np.minimum(edge, np.einsum("ij,ij->i", p - a, m))
        s = np.maximum(1.0, np.maximum(np.abs(o).max(axis=1), np.abs(p).max(axis=1)))
        tol = 2.0 ** -23 * s * (4.0 + 1.0 / np.maximum(cos, 1e-12))
    return {"ok": ok, "t": t, "edge": edge, "cos": cos, "tol": tol, "degen": ok & (nn == 0.0), "dl": dl}


def classify(tris: np.ndarray, rays: np.ndarray, id_a: np.ndarray, id_b: np.ndarray) -> dict:
    """Classifies rays where id_a != id_b.  Returns counts and the indices of
    unexplained disagreements."""
    id_a = np.asarray(id_a)
    id_b = np.asarray(id_b)
    mism = np.nonzero(id_a != id_b)[0]
    out = {"total": int(len(rays)), "mismatch": int(len(mism)), "tie": 0, "edge": 0, "range": 0, "grazing": 0,
           "degen": 0, "unexplained": []}
    if len(mism) == 0:
        return out
    T = np.asarray(tris, dtype=np.float64).reshape(-1, 9)
    R = np.asarray(rays, dtype=np.float64).reshape(-1, 8)[mism]
    A = _candidate(T, R, id_a[mism])
    B = _candidate(T, R, id_b[mism])
    left = np.ones(len(mism), bool)

    def take(name, cond):
        nonlocal left
        cond = cond & left
        out[name] = int(cond.sum())
        left &= ~cond

    with np.errstate(invalid="ignore"):
        take("degen", A["degen"] | B["degen"])
        take("grazing", (A["ok"] & (A["cos"] < 1e-6)) | (B["ok"] & (B["cos"] < 1e-6)))
        take("edge", (A["ok"] & (np.abs(A["edge"]) <= A["tol"])) | (B["ok"] & (np.abs(B["edge"]) <= B["tol"])))
        tmin, tmax = R[:, 3], R[:, 7]

        def near_range(C):
            lim = C["tol"] / C["dl"]
            return C["ok"] & ((np.abs(C["t"] - tmin) <= lim) | (np.abs(C["t"] - tmax) <= lim))

        take("range", near_range(A) | near_range(B))
        take("tie", A["ok"] & B["ok"] & (np.abs(A["t"] - B["t"]) * A["dl"] <= A["tol"] + B["tol"]))
    out["unexplained"] = [int(i) for i in mism[left]]
    return out


def hit_geometry(positions, normals, texcoords, faces, prim, b1, b2, o, d, t):
    """p, gn, sn, uv of one hit, following IntersectionUtils::CreateTriangleIntersection
    (intersectionutils.h:59-135) with an identity transform."""
    P = np.asarray(positions, dtype=np.float64).reshape(-1, 3)
    Nn = np.asarray(normals, dtype=np.float64).reshape(-1, 3)
    T = np.asarray(texcoords, dtype=np.float64).reshape(-1, 2)
    F = np.asarray(faces).reshape(-1, 3)
    v1, v2, v3 = F[prim]
    p = np.asarray(o, dtype=np.float64) + np.asarray(d, dtype=np.float64) * t
    gn = np.cross(P[v2] - P[v1], P[v3] - P[v1])
    gn /= np.linalg.norm(gn)
    w0 = 1.0 - b1 - b2
    sn = Nn[v1] * w0 + Nn[v2] * b1 + Nn[v3] * b2
    sn /= np.linalg.norm(sn)
    uv = T[v1] * w0 + T[v2] * b1 + T[v3] * b2
    return p, gn, sn, uv

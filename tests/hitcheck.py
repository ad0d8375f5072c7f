"""Helpers shared by the parity tests: hit-point geometry in the reference's
terms and the classification of documented disagreement classes.

Disagreement classes (a GPU hit id that differs from the oracle's is only
accepted when it falls in one of these, and every test reports the counts):
  tie      the FP64 ray parameters of both candidate triangles agree to
           within 1e-6 relative (exact or FP32-unresolvable ties; the
           reference keeps the last accepted candidate, triaccel.h:137);
  edge     on either candidate the FP64 barycentrics lie within 1e-6 of an
           edge (the reference's Wald test is inclusive but not watertight,
           triaccel.h:150; the GPU test is watertight);
  grazing  |d.n| < 1e-6 |n| on either candidate;
  degen    the oracle-side triangle is degenerate (TriAccel k == 3 never hits,
           triaccel.h:73-77).
"""
from __future__ import annotations

import numpy as np

import lmoracle as lo


def tri_normals(tris: np.ndarray) -> np.ndarray:
    T = np.asarray(tris, dtype=np.float64).reshape(-1, 9)
    return np.cross(T[:, 3:6] - T[:, 0:3], T[:, 6:9] - T[:, 0:3])


def classify(tris: np.ndarray, rays: np.ndarray, id_a: np.ndarray, id_b: np.ndarray) -> dict:
    """Classifies rays where id_a != id_b.  Returns counts and the indices of
    unexplained disagreements."""
    mism = np.nonzero(id_a != id_b)[0]
    out = {"total": int(len(rays)), "mismatch": int(len(mism)), "tie": 0, "edge": 0, "grazing": 0, "degen": 0,
           "unexplained": []}
    if len(mism) == 0:
        return out
    N = tri_normals(tris)
    R = np.asarray(rays, dtype=np.float64).reshape(-1, 8)
    for i in mism:
        a, b = int(id_a[i]), int(id_b[i])
        cands = [c for c in (a, b) if c >= 0]
        r = R[i:i + 1]
        d = r[0, 4:7]
        # degenerate (zero area) triangles
        if any(np.linalg.norm(N[c]) == 0.0 for c in cands):
            out["degen"] += 1
            continue
        if any(abs(np.dot(d, N[c])) < 1e-6 * np.linalg.norm(N[c]) * np.linalg.norm(d) for c in cands):
            out["grazing"] += 1
            continue
        edge = False
        for c in cands:
            bb = lo.barycentrics_fp64(tris, r, np.array([c]))[0]
            w = (1.0 - bb[0] - bb[1], bb[0], bb[1])
            if min(abs(x) for x in w) < 1e-6:
                edge = True
        if edge:
            out["edge"] += 1
            continue
        if len(cands) == 2:
            ta = lo.t_fp64(tris, r, np.array([a]))[0]
            tb = lo.t_fp64(tris, r, np.array([b]))[0]
            if abs(ta - tb) <= 1e-6 * max(abs(ta), abs(tb)):
                out["tie"] += 1
                continue
        out["unexplained"].append(int(i))
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

"""Restatement, in numpy float32, of how the reference flattens a
primitive's mesh into the accel's triangles (accel_naive.cpp:59-90): each
face's vertices through the primitive's transform with the single-precision
Mat4 x Vec4 of math.h:1268-1279, i.e. per row r
(m[0][r] x + m[1][r] y) + (m[2][r] z + m[3][r] w), every product and sum
rounded to float (numpy float32 arithmetic rounds each operation)."""
import numpy as np


def flatten(meshes) -> tuple[np.ndarray, np.ndarray]:
    """meshes: (positions (nv, 3), faces (nf, 3), transform 16 column-major
    m[c][r]); returns the (ntri, 9) float32 triangles and each one's mesh."""
    out, prim = [], []
    one = np.float32(1.0)
    for i, (pos, faces, tr) in enumerate(meshes):
        P = np.asarray(pos, np.float32).reshape(-1, 3)
        F = np.asarray(faces, np.int64).reshape(-1, 3)
        T = np.asarray(tr, np.float32).reshape(4, 4)  # T[c][r]
        v = P[F.reshape(-1)]
        x, y, z = v[:, 0], v[:, 1], v[:, 2]
        r = np.stack([(T[0, k] * x + T[1, k] * y) + (T[2, k] * z + T[3, k] * one) for k in range(3)], 1)
        out.append(r.astype(np.float32).reshape(-1, 9))
        prim.append(np.full(F.shape[0], i, np.int32))
    if not out:
        return np.zeros((0, 9), np.float32), np.zeros(0, np.int32)
    return np.concatenate(out), np.concatenate(prim)


def fixture_meshes(z) -> list:
    return [(z[f"mesh{i}_positions"], z[f"mesh{i}_faces"], z[f"mesh{i}_transform"])
            for i in range(int(z["num_meshes"]))]


def random_meshes(seed: int, sizes) -> list:
    """Indexed meshes with shared vertices and affine transforms (non-uniform
    scale, rotation, translation), column-major."""
    g = np.random.default_rng(seed)
    meshes = []
    for nv, nf in sizes:
        pos = g.normal(size=(nv, 3)).astype(np.float32) * np.float32(3.0)
        faces = g.integers(0, max(nv, 1), size=(nf, 3)).astype(np.uint32) if nv else np.zeros((0, 3), np.uint32)
        a = g.normal(size=3)
        a /= np.linalg.norm(a)
        ang = g.uniform(-3, 3)
        K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
        R = np.eye(3) + np.sin(ang) * K + (1 - np.cos(ang)) * K @ K
        m = np.eye(4)
        m[:3, :3] = R @ np.diag(g.uniform(0.2, 5.0, size=3))
        m[:3, 3] = g.normal(size=3) * 10.0
        meshes.append((pos, faces, m.T.reshape(-1).astype(np.float32)))
    return meshes

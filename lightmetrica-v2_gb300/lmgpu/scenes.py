"""Seeded synthetic inputs for the ray-intersection workloads.

All randomness comes from numpy's Philox counter-based generator, so a seed
fixes the triangle soup and the ray set on one machine (transcendental
functions may differ in the last bit between CPU architectures; tests always
compare the GPU path and the oracle on inputs generated in the same process).

Triangle arrays are float32 (N, 9): vertices p1, p2, p3 in global triangle
order.  Ray arrays are float32 (N, 8): ox, oy, oz, tmin, dx, dy, dz, tmax.
"""
from __future__ import annotations

import numpy as np

FLT_MAX = np.float32(np.finfo(np.float32).max)
EPS_ISECT = np.float32(1e-4)  # Math::EpsIsect (math.h:1668), the camera/bounce ray tmin


def rng(seed: int, stream: int = 0) -> np.random.Generator:
    return np.random.Generator(np.random.Philox(key=[seed & 0xFFFFFFFFFFFFFFFF, stream]))


def unit_vectors(g: np.random.Generator, n: int) -> np.ndarray:
    """Directions uniform on the sphere (z = 1 - 2u, phi = 2 pi v)."""
    u = g.random(n)
    v = g.random(n)
    z = 1.0 - 2.0 * u
    r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    phi = 2.0 * np.pi * v
    return np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1)


def random_soup(n: int, seed: int = 0x5EED, mu: float = np.log(0.005), sigma: float = 0.5) -> np.ndarray:
    """n triangles with centroids uniform in [0,1]^3.

    Each vertex sits at the centroid plus a random unit vector times a
    lognormal(mu, sigma) length; the three offsets are re-centred so the
    centroid is exact.  Edge lengths are then of order exp(mu).
    """
    g = rng(seed, 1)
    c = g.random((n, 3))
    off = np.empty((n, 3, 3))
    for k in range(3):
        L = np.exp(mu + sigma * g.standard_normal(n))
        off[:, k, :] = unit_vectors(g, n) * L[:, None]
    off -= off.mean(axis=1, keepdims=True)
    tris = (c[:, None, :] + off).reshape(n, 9)
    return tris.astype(np.float32)


def heightfield(res: int = 512, seed: int = 0x5EED, amplitude: float = 0.05, base: float = 0.0) -> np.ndarray:
    """res x res quads (2 * res^2 triangles) over [0,1]^2 in xz at height
    y = base + sum of 4 seeded sinusoids whose amplitudes sum to `amplitude`."""
    g = rng(seed, 2)
    freqs = g.uniform(1.0, 6.0, size=(4, 2))
    phases = g.uniform(0.0, 2.0 * np.pi, size=4)
    amps = np.full(4, amplitude / 4.0)
    xs = np.linspace(0.0, 1.0, res + 1)
    X, Z = np.meshgrid(xs, xs, indexing="ij")
    Y = np.full_like(X, base)
    for i in range(4):
        Y += amps[i] * np.sin(2.0 * np.pi * (freqs[i, 0] * X + freqs[i, 1] * Z) + phases[i])
    P = np.stack([X, Y, Z], axis=-1)  # (res+1, res+1, 3)
    p00 = P[:-1, :-1].reshape(-1, 3)
    p10 = P[1:, :-1].reshape(-1, 3)
    p11 = P[1:, 1:].reshape(-1, 3)
    p01 = P[:-1, 1:].reshape(-1, 3)
    t1 = np.concatenate([p00, p01, p11], axis=1)
    t2 = np.concatenate([p00, p11, p10], axis=1)
    tris = np.stack([t1, t2], axis=1).reshape(-1, 9)
    return tris.astype(np.float32)


def raycast_scene(n_random: int = 1_000_000, hf_res: int = 512, seed: int = 0x5EED) -> np.ndarray:
    """BVH ray-cast benchmark scene: random soup then heightfield (global order)."""
    return np.concatenate([random_soup(n_random, seed), heightfield(hf_res, seed)], axis=0)


def raycast_rays(n: int, seed: int = 0x5EED, lo: float = -0.1, hi: float = 1.1,
                 tmin: float = 1e-4, tmax: float = float(FLT_MAX), stream: int = 3) -> np.ndarray:
    """n rays: origins uniform in [lo,hi]^3, directions uniform on the sphere."""
    g = rng(seed, stream)
    o = g.uniform(lo, hi, size=(n, 3))
    d = unit_vectors(g, n)
    r = np.empty((n, 8), dtype=np.float32)
    r[:, 0:3] = o
    r[:, 3] = np.float32(tmin)
    r[:, 4:7] = d
    r[:, 7] = np.float32(tmax)
    return r


def closed_icosphere(level: int, radius: float = 1.0, center=(0.0, 0.0, 0.0)) -> np.ndarray:
    """Closed, consistently wound icosphere (20 * 4^level triangles)."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    V = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    F = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
         (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
         (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    verts = [np.array(v, dtype=np.float64) / np.linalg.norm(v) for v in V]
    faces = list(F)
    for _ in range(level):
        cache: dict = {}

        def mid(a: int, b: int) -> int:
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    Vn = np.array(verts) * radius + np.asarray(center, dtype=np.float64)
    Fn = np.array(faces)
    return Vn[Fn].reshape(-1, 9).astype(np.float32)


# ---------------------------------------------------------------------------
# Scenes for the path tracers.  A scene is a dict:
#   prims  : list of {"kind": 0 diffuse | 1 area light (no BSDF),
#                     "R": (r,g,b), "Le": (r,g,b), "tris": float32 (n, 9)}
#            in scene order (global triangle ids follow it);
#   camera : {"eye", "center", "up", "fov" (vertical, degrees), "width", "height"}.
DIFFUSE, AREA_LIGHT = 0, 1


def _quad(p0, p1, p2, p3) -> np.ndarray:
    """Two triangles (p0,p1,p2), (p0,p2,p3); normal = (p1-p0) x (p2-p0)."""
    return np.array([list(p0) + list(p1) + list(p2), list(p0) + list(p2) + list(p3)], dtype=np.float64)


def _box(size, angle_deg, base_xz) -> np.ndarray:
    """Axis-aligned box of `size` (sx, sy, sz) standing on y = 0, rotated by
    `angle_deg` about +y around its centre, centre at base_xz; 12 outward
    facing triangles."""
    sx, sy, sz = size
    x0, x1, y0, y1, z0, z1 = -sx / 2, sx / 2, 0.0, sy, -sz / 2, sz / 2
    faces = [
        _quad((x0, y1, z0), (x0, y1, z1), (x1, y1, z1), (x1, y1, z0)),  # top (+y)
        _quad((x0, y0, z0), (x1, y0, z0), (x1, y0, z1), (x0, y0, z1)),  # bottom (-y)
        _quad((x0, y0, z0), (x0, y1, z0), (x1, y1, z0), (x1, y0, z0)),  # front (-z)
        _quad((x0, y0, z1), (x1, y0, z1), (x1, y1, z1), (x0, y1, z1)),  # back (+z)
        _quad((x0, y0, z0), (x0, y0, z1), (x0, y1, z1), (x0, y1, z0)),  # left (-x)
        _quad((x1, y0, z0), (x1, y1, z0), (x1, y1, z1), (x1, y0, z1)),  # right (+x)
    ]
    t = np.concatenate(faces, axis=0).reshape(-1, 3)
    a = np.radians(angle_deg)
    R = np.array([[np.cos(a), 0, np.sin(a)], [0, 1, 0], [-np.sin(a), 0, np.cos(a)]])
    t = t @ R.T + np.array([base_xz[0], 0.0, base_xz[1]])
    return t.reshape(-1, 9)


def cornell_box(width: int = 256, height: int = 256) -> dict:
    """Procedural Cornell-style box: walls of [0,1]^3 without the z = 0 side
    (10 triangles, normals facing in), two rotated boxes (12 + 12), and a
    0.25 x 0.2 area light at y = 0.999 facing down (2); camera at
    (0.5, 0.5, -1.4) looking +z, vertical fov 40 degrees."""
    grey, red, green = (0.75, 0.75, 0.75), (0.63, 0.065, 0.05), (0.14, 0.45, 0.09)
    walls = [
        (grey, _quad((0, 0, 0), (0, 0, 1), (1, 0, 1), (1, 0, 0))),   # floor, +y
        (grey, _quad((0, 1, 0), (1, 1, 0), (1, 1, 1), (0, 1, 1))),   # ceiling, -y
        (grey, _quad((0, 0, 1), (0, 1, 1), (1, 1, 1), (1, 0, 1))),   # back wall, -z
        (red, _quad((0, 0, 0), (0, 1, 0), (0, 1, 1), (0, 0, 1))),    # left wall x = 0, +x
        (green, _quad((1, 0, 0), (1, 0, 1), (1, 1, 1), (1, 1, 0))),  # right wall x = 1, -x
    ]
    prims = [{"kind": DIFFUSE, "R": c, "Le": (0.0, 0.0, 0.0), "tris": t.astype(np.float32)} for c, t in walls]
    prims.append({"kind": DIFFUSE, "R": grey, "Le": (0.0, 0.0, 0.0),
                  "tris": _box((0.3, 0.3, 0.3), -17.0, (0.68, 0.35)).astype(np.float32)})
    prims.append({"kind": DIFFUSE, "R": grey, "Le": (0.0, 0.0, 0.0),
                  "tris": _box((0.3, 0.6, 0.3), 17.0, (0.32, 0.65)).astype(np.float32)})
    lx0, lx1, lz0, lz1, ly = 0.5 - 0.125, 0.5 + 0.125, 0.5 - 0.1, 0.5 + 0.1, 0.999
    prims.append({"kind": AREA_LIGHT, "R": (0.0, 0.0, 0.0), "Le": (17.0, 12.0, 4.0),
                  "tris": _quad((lx0, ly, lz0), (lx1, ly, lz0), (lx1, ly, lz1), (lx0, ly, lz1)).astype(np.float32)})
    camera = {"eye": (0.5, 0.5, -1.4), "center": (0.5, 0.5, 0.0), "up": (0.0, 1.0, 0.0), "fov": 40.0,
              "width": width, "height": height}
    return {"prims": prims, "camera": camera}


def scene_triangles(scene: dict) -> tuple[np.ndarray, np.ndarray]:
    """All triangles in global order and the primitive index of each."""
    tris = np.concatenate([p["tris"] for p in scene["prims"]], axis=0).astype(np.float32)
    prim = np.concatenate([np.full(p["tris"].shape[0], i, np.int32) for i, p in enumerate(scene["prims"])])
    return tris, prim


# BSDF kinds of a primitive (the reference's bsdf::null, bsdf::diffuse,
# bsdf::flesnel, bsdf::cook_torrance) and their parameter defaults
# (bsdf_flesnel.cpp:47-50, bsdf_cooktorrance.cpp:58-63).
BSDF_NULL, BSDF_DIFFUSE, BSDF_DIELECTRIC, BSDF_COOK_TORRANCE = 0, 1, 2, 3
PRIM_DEFAULTS = {"bsdf": BSDF_NULL, "light": False, "R": (0.0, 0.0, 0.0), "Le": (0.0, 0.0, 0.0), "eta1": 1.0,
                 "eta2": 2.0, "ct_eta": (0.14, 0.129, 0.1585), "ct_k": (4.58625, 3.348125, 2.329375),
                 "roughness": 0.1}


def prim_params(p: dict) -> dict:
    """Full parameter set of a primitive; the short form {"kind": 0|1} means
    a diffuse surface (0) or an area light without a BSDF (1)."""
    q = dict(PRIM_DEFAULTS)
    if "kind" in p and "bsdf" not in p:
        q["bsdf"] = BSDF_DIFFUSE if p["kind"] == DIFFUSE else BSDF_NULL
        q["light"] = p["kind"] == AREA_LIGHT
    for k, v in p.items():
        if k in q:
            q[k] = v
    q["tris"] = p["tris"]
    return q


def cornell_materials(width: int = 64, height: int = 64) -> dict:
    """The Cornell-style box with the short box in glass (bsdf::flesnel,
    eta 1 -> 1.5), the tall box a GGX conductor (bsdf::cook_torrance,
    roughness 0.2, the reference's default eta/k), and a constant blue-white
    environment light reached through the open front."""
    s = cornell_box(width, height)
    # the boxes stand 1e-3 above the floor: a glass box whose bottom face is
    # coplanar with the floor makes every ray reaching y = 0 an exact tie
    # between two surfaces, an ill-posed case whose outcome depends on the
    # accel's traversal order
    lift = np.array([0.0, 1e-3, 0.0] * 3, np.float32)
    short_box, tall_box = s["prims"][5], s["prims"][6]
    s["prims"][5] = {"bsdf": BSDF_DIELECTRIC, "light": False, "R": (1.0, 1.0, 1.0), "eta1": 1.0, "eta2": 1.5,
                     "tris": short_box["tris"] + lift}
    s["prims"][6] = {"bsdf": BSDF_COOK_TORRANCE, "light": False, "R": (0.9, 0.9, 0.9), "roughness": 0.2,
                     "tris": tall_box["tris"] + lift}
    s["env"] = (0.2, 0.3, 0.5)
    return s


def caustic_room(width: int = 1280, height: int = 720, sphere_level: int = 5) -> dict:
    """Caustic scene of the bidirectional renderer: a closed room of 20
    triangles facing in (x in [-1, 1], y in [0, 1.5], z in [-1.2, 1]; the
    floor in 2 x 2 quads, the ceiling in two), a glass icosphere (level
    `sphere_level`, radius 0.3, eta 1 -> 1.5) standing on the floor, a sphere
    light of radius 0.05 (level-2 icosphere, facing out) and a thin grey
    panel (12 triangles) that hides the light from the camera but not from
    the glass; camera at (0, 0.7, -1.1) looking at (0, 0.3, 0.3), vertical
    fov 45 degrees."""
    x0, x1, y0, y1, z0, z1 = -1.0, 1.0, 0.0, 1.5, -1.2, 1.0
    xm, zm = 0.5 * (x0 + x1), 0.5 * (z0 + z1)
    floor = np.concatenate([_quad((a0, y0, b0), (a0, y0, b1), (a1, y0, b1), (a1, y0, b0))
                            for a0, a1 in ((x0, xm), (xm, x1)) for b0, b1 in ((z0, zm), (zm, z1))])
    ceiling = np.concatenate([_quad((a0, y1, z0), (a1, y1, z0), (a1, y1, z1), (a0, y1, z1))
                              for a0, a1 in ((x0, xm), (xm, x1))])
    walls = np.concatenate([
        _quad((x0, y0, z1), (x0, y1, z1), (x1, y1, z1), (x1, y0, z1)),  # back, -z
        _quad((x0, y0, z0), (x1, y0, z0), (x1, y1, z0), (x0, y1, z0)),  # front (behind the camera), +z
        _quad((x0, y0, z0), (x0, y1, z0), (x0, y1, z1), (x0, y0, z1)),  # left, +x
        _quad((x1, y0, z0), (x1, y0, z1), (x1, y1, z1), (x1, y1, z0)),  # right, -x
    ])
    room = np.concatenate([floor, ceiling, walls]).astype(np.float32)
    assert room.shape[0] == 20
    sphere = closed_icosphere(sphere_level, 0.3, (0.0, 0.301, 0.2))
    light = closed_icosphere(2, 0.05, (0.35, 0.95, 0.55))
    panel = _box((0.5, 0.35, 0.02), 0.0, (0.35, 0.35)) + np.array([0.0, 0.78, 0.0] * 3)
    prims = [
        {"bsdf": BSDF_DIFFUSE, "R": (0.75, 0.75, 0.75), "tris": room},
        {"bsdf": BSDF_DIELECTRIC, "R": (1.0, 1.0, 1.0), "eta1": 1.0, "eta2": 1.5, "tris": sphere},
        {"bsdf": BSDF_DIFFUSE, "R": (0.5, 0.5, 0.5), "tris": panel.astype(np.float32)},
        {"bsdf": BSDF_NULL, "light": True, "Le": (400.0, 360.0, 300.0), "tris": light},
    ]
    camera = {"eye": (0.0, 0.7, -1.1), "center": (0.0, 0.3, 0.3), "up": (0.0, 1.0, 0.0), "fov": 45.0,
              "width": width, "height": height}
    return {"prims": prims, "camera": camera}


_ICO4 = None


def _icosphere4() -> np.ndarray:
    """Unit level-4 icosphere (5120 triangles), built once."""
    global _ICO4
    if _ICO4 is None:
        _ICO4 = closed_icosphere(4).astype(np.float64)
    return _ICO4


def instance_tris(unit: np.ndarray, scale: float, shift) -> np.ndarray:
    """Triangles of an instanced primitive: the float32 unit mesh widened to
    float64, scaled, shifted and rounded back to float32 (the same arithmetic
    as the sphere grid, so the result is bit-identical on any machine)."""
    v = np.asarray(unit, np.float32).astype(np.float64).reshape(-1, 3) * float(scale) + np.asarray(shift, np.float64)
    return v.reshape(-1, 9).astype(np.float32)


def phong_to_ggx_roughness(n: float) -> float:
    """GGX roughness standing in for a Phong exponent n: alpha = sqrt(2 / (n + 2))
    (the reference has no Phong BSDF; bsdf::cook_torrance takes its place)."""
    return float(np.sqrt(2.0 / (n + 2.0)))


def sphere_grid_scene(seed: int, index: int, width: int | None = None, height: int | None = None,
                      grid: int = 16) -> dict:
    """One scene of the batched configuration: a grid x grid array of level-4
    icospheres (5120 triangles each, radius U[0.2, 0.5], spacing 1.2) on a
    ground plane, each sphere Lambertian (albedo U[0.2, 0.9]^3), glossy
    (Phong exponent U[10, 1000] as GGX roughness sqrt(2 / (n + 2)), default
    conductor) or glass (eta 1 -> 1.5); one sphere light (level-2 icosphere,
    radius 1, Le 60) above the grid and a constant environment (0.3, 0.35,
    0.45).  The resolution is drawn from {640x360, 1280x720, 1920x1080} unless
    given.  Seeded by (seed, index)."""
    g = rng(seed, 1000 + index)
    ico = _icosphere4()
    prims = []
    span = (grid - 1) * 1.2
    ground = _quad((-2.0, 0.0, -2.0), (-2.0, 0.0, span + 2.0), (span + 2.0, 0.0, span + 2.0), (span + 2.0, 0.0, -2.0))
    prims.append({"bsdf": BSDF_DIFFUSE, "R": (0.6, 0.6, 0.6), "tris": ground.astype(np.float32)})
    radii = g.uniform(0.2, 0.5, size=grid * grid)
    kinds = g.integers(0, 3, size=grid * grid)
    albedo = g.uniform(0.2, 0.9, size=(grid * grid, 3))
    expo = g.uniform(10.0, 1000.0, size=grid * grid)
    for k in range(grid * grid):
        cx, cz = (k % grid) * 1.2, (k // grid) * 1.2
        r = radii[k]
        shift = np.array([cx, r + 1e-3, cz])
        tris = (ico.reshape(-1, 3) * r + shift).reshape(-1, 9).astype(np.float32)
        # how the triangles were made: the unit level-4 icosphere scaled by r
        # and shifted (lets a fixture store the sphere once)
        inst = ("ico4", float(r), tuple(float(x) for x in shift))
        if kinds[k] == 0:
            prims.append({"bsdf": BSDF_DIFFUSE, "R": tuple(albedo[k]), "tris": tris, "instance": inst})
        elif kinds[k] == 1:
            prims.append({"bsdf": BSDF_COOK_TORRANCE, "R": tuple(albedo[k]),
                          "roughness": phong_to_ggx_roughness(expo[k]), "tris": tris, "instance": inst})
        else:
            prims.append({"bsdf": BSDF_DIELECTRIC, "R": (1.0, 1.0, 1.0), "eta1": 1.0, "eta2": 1.5, "tris": tris,
                          "instance": inst})
    light = closed_icosphere(2, 1.0, (span * 0.5, 8.0, span * 0.5))
    prims.append({"bsdf": BSDF_NULL, "light": True, "Le": (60.0, 55.0, 50.0), "tris": light})
    res = [(640, 360), (1280, 720), (1920, 1080)]
    w, h = res[int(g.integers(0, 3))]
    if width is not None:
        w, h = width, height
    eye = (span * 0.5 + float(g.uniform(-3, 3)), float(g.uniform(4, 7)), -6.0)
    camera = {"eye": eye, "center": (span * 0.5, 0.0, span * 0.5), "up": (0.0, 1.0, 0.0), "fov": 50.0,
              "width": w, "height": h}
    return {"prims": prims, "camera": camera, "env": (0.3, 0.35, 0.45)}


def batch_scenes(seed: int = 0x5EED, count: int = 12, grid: int = 16, size: tuple | None = None) -> list:
    """The batched configuration: `count` seeded sphere-grid scenes
    (sphere_grid_scene), ~1.31M triangles each at grid 16."""
    return [sphere_grid_scene(seed, i, *(size or (None, None)), grid=grid) for i in range(count)]


def _tess_box(size, angle_deg, base_xz, k: int) -> np.ndarray:
    """Box as _box, with every face tessellated into k x k quads (12 k^2
    triangles, outward facing)."""
    sx, sy, sz = size
    x0, x1, y0, y1, z0, z1 = -sx / 2, sx / 2, 0.0, sy, -sz / 2, sz / 2
    faces = [  # (origin, edge u, edge v) with u x v pointing out
        ((x0, y1, z0), (0, 0, sz), (sx, 0, 0)),   # top (+y)
        ((x0, y0, z0), (sx, 0, 0), (0, 0, sz)),   # bottom (-y)
        ((x0, y0, z0), (0, sy, 0), (sx, 0, 0)),   # front (-z)
        ((x0, y0, z1), (sx, 0, 0), (0, sy, 0)),   # back (+z)
        ((x0, y0, z0), (0, 0, sz), (0, sy, 0)),   # left (-x)
        ((x1, y0, z0), (0, sy, 0), (0, 0, sz)),   # right (+x)
    ]
    t = np.linspace(0.0, 1.0, k + 1)
    out = []
    for o, u, v in faces:
        o, u, v = np.array(o), np.array(u), np.array(v)
        P = o + t[:, None, None] * u + t[None, :, None] * v  # (k+1, k+1, 3)
        a, b_, c, d = P[:-1, :-1], P[1:, :-1], P[1:, 1:], P[:-1, 1:]
        out.append(np.concatenate([a, b_, c], axis=2).reshape(-1, 9))
        out.append(np.concatenate([a, c, d], axis=2).reshape(-1, 9))
    tri = np.concatenate(out).reshape(-1, 3)
    ang = np.radians(angle_deg)
    R = np.array([[np.cos(ang), 0, np.sin(ang)], [0, 1, 0], [-np.sin(ang), 0, np.cos(ang)]])
    tri = tri @ R.T + np.array([base_xz[0], 0.0, base_xz[1]])
    return tri.reshape(-1, 9)


def narrow_gap_room(width: int = 1920, height: int = 1080, n_furniture: int = 100, tess: int = 13,
                    seed: int = 0x5EED) -> dict:
    """Learned-guiding scene: a closed 10 x 4 x 10 room (walls facing in,
    Lambertian albedo 0.8) whose x = 10 wall has a 0.2-wide vertical slit at
    z in [4.9, 5.1] (the wall is two quads around it: 14 room triangles);
    outside, a 2 x 2 area light of radiance 50 at x = 10.5 faces the slit,
    the only light; inside, n_furniture seeded furniture boxes standing on the
    floor (footprint U[0.3, 1.2]^2, height U[0.3, 1.5], rotated about y,
    albedo 0.8), each face tessellated into tess x tess quads (100 boxes at
    tess 13: ~203k triangles).  Camera at (1, 2, 5) looking at the slit wall,
    vertical fov 60 degrees."""
    g = rng(seed, 5005)
    X, Y, Z = 10.0, 4.0, 10.0
    z0, z1 = 4.9, 5.1
    room = np.concatenate([
        _quad((0, 0, 0), (0, 0, Z), (X, 0, Z), (X, 0, 0)),      # floor, +y
        _quad((0, Y, 0), (X, Y, 0), (X, Y, Z), (0, Y, Z)),      # ceiling, -y
        _quad((0, 0, 0), (0, Y, 0), (0, Y, Z), (0, 0, Z)),      # x = 0, +x
        _quad((0, 0, 0), (X, 0, 0), (X, Y, 0), (0, Y, 0)),      # z = 0, +z
        _quad((0, 0, Z), (0, Y, Z), (X, Y, Z), (X, 0, Z)),      # z = 10, -z
        _quad((X, 0, 0), (X, 0, z0), (X, Y, z0), (X, Y, 0)),    # x = 10 below the slit, -x
        _quad((X, 0, z1), (X, 0, Z), (X, Y, Z), (X, Y, z1)),    # x = 10 beyond the slit, -x
    ]).astype(np.float32)
    # facing -x, towards the slit
    light = _quad((X + 0.5, 1.0, 4.0), (X + 0.5, 1.0, 6.0), (X + 0.5, 3.0, 6.0), (X + 0.5, 3.0, 4.0)).astype(np.float32)
    boxes = []
    for _ in range(n_furniture):
        size = (float(g.uniform(0.3, 1.2)), float(g.uniform(0.3, 1.5)), float(g.uniform(0.3, 1.2)))
        pos = (float(g.uniform(1.0, X - 1.5)), float(g.uniform(0.8, Z - 0.8)))
        boxes.append(_tess_box(size, float(g.uniform(0.0, 90.0)), pos, tess))
    prims = [
        {"bsdf": BSDF_DIFFUSE, "R": (0.8, 0.8, 0.8), "tris": room},
        {"bsdf": BSDF_DIFFUSE, "R": (0.8, 0.8, 0.8), "tris": np.concatenate(boxes).astype(np.float32)},
        {"bsdf": BSDF_NULL, "light": True, "Le": (50.0, 50.0, 50.0), "tris": light},
    ]
    camera = {"eye": (1.0, 2.0, 5.0), "center": (10.0, 1.5, 5.0), "up": (0.0, 1.0, 0.0), "fov": 60.0,
              "width": width, "height": height}
    return {"prims": prims, "camera": camera}


def scene_box(scene: dict, pad: float = 1e-3) -> tuple:
    """Axis-aligned bounds (lo, hi) of a scene's triangles, padded."""
    tris, _ = scene_triangles(scene)
    v = tris.reshape(-1, 3)
    lo, hi = v.min(axis=0) - pad, v.max(axis=0) + pad
    return tuple(float(x) for x in lo) + tuple(float(x) for x in hi)

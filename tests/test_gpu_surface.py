"""Surface geometry at hits on the GPU (lmgpu_surface, the device form of
IntersectionUtils::CreateTriangleIntersection, intersectionutils.h:59-135)
against the reference's own function compiled in double precision
(tests/golden/surface.npz) and against the FP64 oracle on traced hits.

Tolerances (single-precision path against FP64):
  p                 1e-6 relative + 1e-6
  gn, sn, dpdu, dpdv, uv   2e-5 absolute (unit vectors; inputs rounded to float)
  dndu, dndv        2e-4 relative + 2e-5
NaN exactly where the reference has NaN (the all-zero-normal face)."""
import numpy as np
import pytest

from test_oracle_surface import FIELDS, golden, golden_rays_hits

pytestmark = pytest.mark.gpu

TOL = {"p": (1e-6, 1e-6), "gn": (0, 2e-5), "sn": (0, 2e-5), "dpdu": (0, 2e-5), "dpdv": (0, 2e-5),
       "dndu": (2e-4, 2e-5), "dndv": (2e-4, 2e-5), "uv": (0, 2e-5)}


def check(a, b, what):
    for name, sl in FIELDS.items():
        x, y = a[:, sl].astype(np.float64), b[:, sl]
        nan_ref = np.isnan(y)
        assert np.array_equal(np.isnan(x), nan_ref), (what, name, "NaN pattern differs")
        ok = ~nan_ref
        rtol, atol = TOL[name]
        err = np.abs(x[ok] - y[ok])
        assert np.all(err <= atol + rtol * np.abs(y[ok])), (what, name, float(err.max()))


def hit_records(gpu_lib, t, prim, b1, b2):
    h = np.zeros(len(t), gpu_lib.HIT_DTYPE)
    h["t"], h["prim"], h["b1"], h["b2"] = t, prim, b1, b2
    return h


def test_surface_matches_reference_fp64(gpu_lib, oracle_lib, golden_dir):
    g = golden(golden_dir)
    acc = gpu_lib.Accel()
    acc.build(g["tris32"])
    acc.set_attributes(g["normals32"], g["texcoords32"], g["flags"])
    rays64, hits64 = golden_rays_hits(g)
    rays = rays64.astype(np.float32)
    q = g["queries"]
    h = hit_records(gpu_lib, q[:, 8], g["global_id"], q[:, 9], q[:, 10])
    out = acc.surface(rays, h)
    check(out, g["geom64"], "GPU vs reference (double)")
    # the FP64 oracle on the GPU's own float inputs: the GPU differs by its rounding only
    hin = np.stack([h["t"], h["prim"], h["b1"], h["b2"]], 1).astype(np.float64)
    ref = oracle_lib.surface(g["tris32"], g["normals32"], g["texcoords32"], g["flags"], rays, hin)
    check(out, ref, "GPU vs oracle (same float inputs)")
    acc.close()


def test_surface_of_traced_hits(gpu_lib, oracle_lib):
    """Rays traced on the GPU through a seeded soup with smooth-ish vertex
    normals and texcoords: every hit's geometry agrees with the FP64 oracle,
    misses are zero, and the device entry equals the host entry."""
    import torch
    from lmgpu import scenes

    g = np.random.default_rng(7)
    tris = scenes.random_soup(20000, 11)
    gn = np.cross(tris[:, 3:6] - tris[:, 0:3], tris[:, 6:9] - tris[:, 0:3])
    gn /= np.linalg.norm(gn, axis=1, keepdims=True)
    nrm = np.repeat(gn, 3, axis=0).reshape(-1, 9) + g.normal(scale=0.2, size=(tris.shape[0], 9))
    tc = g.uniform(size=(tris.shape[0], 6))
    flags = g.integers(0, 4, size=tris.shape[0]).astype(np.uint8)
    rays = scenes.raycast_rays(1 << 16, stream=9)
    acc = gpu_lib.Accel()
    acc.build(tris)
    acc.set_attributes(nrm, tc, flags)
    h = acc.trace(rays)
    hit = h["prim"] >= 0
    assert hit.sum() > 1000 and not hit.all()
    out = acc.surface(rays, h)
    assert not out[~hit].any()
    hin = np.stack([h["t"], h["prim"], h["b1"], h["b2"]], 1).astype(np.float64)
    ref = oracle_lib.surface(tris, nrm.astype(np.float32), tc.astype(np.float32), flags, rays, hin)
    check(out[hit], ref[hit], "GPU vs oracle (traced hits)")
    # hit point on the triangle's plane, shading frame orthonormal
    assert np.all(np.abs(np.einsum("ij,ij->i", out[hit, 9:12], out[hit, 6:9])) < 1e-5)
    assert np.all(np.abs(np.einsum("ij,ij->i", out[hit, 12:15], out[hit, 6:9])) < 1e-5)
    d_rays = torch.from_numpy(rays).cuda()
    d_hits = torch.from_numpy(h.view(np.float32).reshape(-1, 4).copy()).cuda()
    d_out = torch.empty((23, rays.shape[0]), dtype=torch.float32, device="cuda")
    acc.surface_device(d_rays.data_ptr(), d_hits.data_ptr(), rays.shape[0], d_out.data_ptr())
    acc.check()
    assert np.array_equal(d_out.cpu().numpy().T, out)
    # page-locked host buffers are read and written in place
    p_rays = torch.from_numpy(rays).pin_memory()
    p_hits = torch.from_numpy(h.view(np.float32).reshape(-1, 4).copy()).pin_memory()
    p_out = torch.full((23, rays.shape[0]), -3.0, dtype=torch.float32).pin_memory()
    assert gpu_lib.lib().lmgpu_surface(acc.handle, p_rays.data_ptr(), p_hits.data_ptr(), rays.shape[0],
                                       p_out.data_ptr()) == 0
    assert np.array_equal(p_out.numpy().T, out)
    acc.close()


def test_surface_host_entry_in_chunks(gpu_lib):
    """Pageable host buffers of more hits than one staging chunk (2^20):
    the planes of every chunk land at their offsets in the caller's planes."""
    import torch
    from lmgpu import scenes

    tris = scenes.random_soup(5000, 3)
    rays = scenes.raycast_rays((1 << 20) + 4097, stream=5)
    acc = gpu_lib.Accel()
    acc.build(tris)
    h = acc.trace(rays)
    out = acc.surface(rays, h)
    d_rays = torch.from_numpy(rays).cuda()
    d_hits = torch.from_numpy(h.view(np.float32).reshape(-1, 4).copy()).cuda()
    d_out = torch.empty((23, rays.shape[0]), dtype=torch.float32, device="cuda")
    acc.surface_device(d_rays.data_ptr(), d_hits.data_ptr(), rays.shape[0], d_out.data_ptr())
    acc.check()
    assert (h["prim"] >= 0).sum() > 1000
    assert np.array_equal(d_out.cpu().numpy().T, out)
    acc.close()


def test_surface_without_attributes_uses_geometric_normal(gpu_lib):
    from lmgpu import scenes

    tris = scenes.random_soup(2000, 5)
    rays = scenes.raycast_rays(4096, stream=4)
    acc = gpu_lib.Accel()
    acc.build(tris)
    h = acc.trace(rays)
    out = acc.surface(rays, h)
    hit = h["prim"] >= 0
    assert np.array_equal(out[hit, 3:6], out[hit, 6:9])
    assert not out[hit, 15:23].any()
    # a rebuild drops attributes set for the previous triangles
    acc.set_attributes(np.ones((tris.shape[0], 9), np.float32))
    acc.build(tris[:1000])
    h = acc.trace(rays)
    out = acc.surface(rays, h)
    hit = h["prim"] >= 0
    assert np.array_equal(out[hit, 3:6], out[hit, 6:9])
    with pytest.raises(gpu_lib.LmgpuError):
        acc.set_attributes(np.ones((tris.shape[0], 9), np.float32))  # wrong triangle count
    acc.close()

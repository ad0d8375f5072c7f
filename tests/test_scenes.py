"""The synthetic workloads' generators (lightmetrica-v2_gb300/lmgpu/scenes.py)
have the shapes and distributions their configurations state."""
import numpy as np

from lmgpu import scenes


def test_sphere_grid_scene_shape():
    s = scenes.sphere_grid_scene(0x5EED, 0)
    tris, prim = scenes.scene_triangles(s)
    # 256 level-4 icospheres (5120 each) + ground (2) + level-2 light (320)
    assert tris.shape == (256 * 5120 + 2 + 320, 9)
    assert len(s["prims"]) == 258
    assert (s["camera"]["width"], s["camera"]["height"]) in {(640, 360), (1280, 720), (1920, 1080)}
    kinds = {p["bsdf"] for p in s["prims"][1:-1]}
    assert kinds <= {scenes.BSDF_DIFFUSE, scenes.BSDF_COOK_TORRANCE, scenes.BSDF_DIELECTRIC}
    radii = [(p["tris"][:, 1::3].max() - p["tris"][:, 1::3].min()) / 2 for p in s["prims"][1:-1]]
    assert 0.2 - 1e-3 <= min(radii) and max(radii) <= 0.5 + 1e-3
    assert s["prims"][-1]["light"] and s["env"] is not None


def test_batch_scenes_seeded():
    a = scenes.batch_scenes(count=2, grid=2)
    b = scenes.batch_scenes(count=2, grid=2)
    for x, y in zip(a, b):
        assert np.array_equal(scenes.scene_triangles(x)[0], scenes.scene_triangles(y)[0])
    assert not np.array_equal(scenes.scene_triangles(a[0])[0], scenes.scene_triangles(a[1])[0])


def test_phong_mapping():
    assert abs(scenes.phong_to_ggx_roughness(0.0) - 1.0) < 1e-12
    assert scenes.phong_to_ggx_roughness(1000.0) < scenes.phong_to_ggx_roughness(10.0)


def test_caustic_room_shape():
    s = scenes.caustic_room(64, 36)
    tris, _ = scenes.scene_triangles(s)
    assert s["prims"][0]["tris"].shape[0] == 20
    assert s["prims"][1]["tris"].shape[0] == 20 * 4 ** 5
    assert tris.shape[0] == 20 + 20480 + 12 + 320


def test_narrow_gap_room_shape():
    s = scenes.narrow_gap_room(64, 36)
    tris, _ = scenes.scene_triangles(s)
    assert tris.shape[0] == 14 + 100 * 12 * 13 * 13 + 2
    light = s["prims"][2]["tris"].reshape(-1, 3, 3)
    n = np.cross(light[:, 1] - light[:, 0], light[:, 2] - light[:, 0])
    assert np.all(n[:, 0] < 0)  # the light faces the slit (-x)
    room = s["prims"][0]["tris"].reshape(-1, 3, 3)
    c = room.mean(axis=1)
    rn = np.cross(room[:, 1] - room[:, 0], room[:, 2] - room[:, 0])
    # every wall faces the room's centre
    assert np.all(((np.array([5.0, 2.0, 5.0]) - c) * rn).sum(axis=1) > 0)


def test_tessellated_box_faces_out():
    t = scenes._tess_box((1.0, 2.0, 0.5), 30.0, (3.0, 4.0), 3).reshape(-1, 3, 3)
    assert t.shape[0] == 12 * 9
    c = t.mean(axis=1)
    n = np.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0])
    centre = np.array([3.0, 1.0, 4.0])
    assert np.all(((c - centre) * n).sum(axis=1) > 0)

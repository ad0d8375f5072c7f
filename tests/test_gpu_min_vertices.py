"""min_num_vertices on the GPU: paths with fewer vertices contribute nothing,
as each reference renderer applies it (renderer_pt.cpp:186,
renderer_ptmis.cpp:132 and :247, renderer_bdpt.cpp:892), against the
reference's own films with min_num_vertices 3 (tests/golden/*_min3.npz,
double precision), per pixel within the statistical bar of tests/imgcheck.py."""
import pytest

import imgcheck
import ptscene

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,renderer,spp", [("cornell_pt_min3", "pt", 16384), ("cornell_ptmis_min3", "ptmis", 8192),
                                               ("cornell_bdpt_min3", "bdpt", 16384)])
def test_min_num_vertices_matches_reference_film(gpu_lib, golden_dir, name, renderer, spp):
    scene, z = ptscene.load_scene(golden_dir, name)
    assert int(z["min_num_vertices"]) == 3
    sc = gpu_lib.Scene(scene)
    img, var = getattr(sc, f"render_{renderer}")(spp, int(z["max_num_vertices"]), 17,
                                                 min_num_vertices=int(z["min_num_vertices"]))
    sc.close()
    print(imgcheck.assert_same_image(img, var, z["ref64_image"], z["ref64_variance"], f"gpu vs ref64 ({name})"))
    print("relMSE vs FP64 reference", imgcheck.relmse(img, z["ref64_image"]))
    # the directly seen light (two-vertex paths) is gone
    assert (z["ref64_image"].sum(axis=2) == 0).any() == (img.sum(axis=2) == 0).any()

"""Guided path tracing (lmgpu_render_pt_guided): the one-sample MIS of BSDF
sampling and the learned vMF mixture keeps renderer::pt's expectation, and
the trained network lowers the error against a converged image in the scene
it is built for (light through a narrow slit)."""
import numpy as np
import pytest

import imgcheck
import ptscene

pytestmark = pytest.mark.gpu


def small_room(w=64, h=36, furniture=20):
    from lmgpu import scenes

    return scenes.narrow_gap_room(w, h, n_furniture=furniture, tess=4, seed=3)


def test_guided_alpha_one_is_plain_pt(gpu_lib):
    """alpha = 1 samples the BSDF only: the same estimator as lmgpu_render_pt."""
    from lmgpu import scenes

    s = small_room()
    sc = gpu_lib.Scene(s)
    g = gpu_lib.Guide(scenes.scene_box(s), 1)
    a, va, _ = sc.render_pt_guided(g, 2048, -1, 5, alpha=1.0, train=False, rr_mode=0)
    b, vb = sc.render_pt(2048, -1, 6)
    print(imgcheck.assert_same_aggregates(a.astype(np.float64), va.astype(np.float64), b.astype(np.float64),
                                          vb.astype(np.float64), "guided(alpha=1) vs pt"))
    sc.close()
    g.close()


def test_guided_is_unbiased_while_training(gpu_lib):
    """Online training between passes: the guided film agrees with plain PT's."""
    from lmgpu import scenes

    s = small_room()
    sc = gpu_lib.Scene(s)
    g = gpu_lib.Guide(scenes.scene_box(s), 2)
    a, va, loss = sc.render_pt_guided(g, 1024, -1, 7, alpha=0.5, train=True, batch=1 << 14)
    b, vb = sc.render_pt(8192, -1, 8)
    print("last loss", loss)
    print(imgcheck.assert_same_aggregates(a.astype(np.float64), va.astype(np.float64), b.astype(np.float64),
                                          vb.astype(np.float64), "guided vs pt"))
    sc.close()
    g.close()


def test_trained_guide_lowers_error(gpu_lib):
    """What the trained network gains over the same tracer without it: at
    equal samples per pixel and with the same (throughput) roulette, guided
    passes after training reach a lower relMSE (0.1 % outlier trimmed)
    against a converged image than BSDF sampling alone (alpha = 1) and than
    the untrained network (alpha = 0.5, no training)."""
    from lmgpu import scenes

    s = small_room(96, 54, 40)
    sc = gpu_lib.Scene(s)
    g0 = gpu_lib.Guide(scenes.scene_box(s), 1)
    ref, _, _ = sc.render_pt_guided(g0, 65536, -1, 1, alpha=1.0, train=False, rr_mode=1)
    nonet, _, _ = sc.render_pt_guided(g0, 256, -1, 4, alpha=1.0, train=False, rr_mode=1)
    g = gpu_lib.Guide(scenes.scene_box(s), 3)
    untrained, _, _ = sc.render_pt_guided(g, 256, -1, 5, alpha=0.5, train=False, rr_mode=1)
    # training passes: 32,768 spp of the 96 x 54 film (170M samples, ~650 Adam steps
    # of 2^18); at 2,048 spp the network is still worse than BSDF sampling alone
    sc.render_pt_guided(g, 32768, -1, 2, alpha=0.5, train=True, rr_mode=1)
    trained, _, _ = sc.render_pt_guided(g, 256, -1, 3, alpha=0.5, train=False, rr_mode=1)
    et, en, eu = (imgcheck.relmse(x, ref, trim=1e-3) for x in (trained, nonet, untrained))
    print("trimmed relMSE at 256 spp: trained", et, "no network", en, "untrained network", eu,
          "gain over no network", en / et, "over untrained", eu / et)
    assert et < 0.7 * en
    assert et < 0.7 * eu
    sc.close()
    g.close()
    g0.close()

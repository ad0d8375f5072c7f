"""bench.py's measurement arithmetic on the CPU.  The render lines' roofline,
with a fake scene whose trace profile returns fixed records: the counted
render gives the algorithmic bytes, the timed render the device time, and a
record that timed fewer launches than it ran gives no roofline.  The guiding
line's time to a relMSE target and its FP64 film accumulation."""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)

import bench  # noqa: E402
import lmgpu  # noqa: E402

ZERO = {"launches": 0, "rays": 0, "node_fetches": 0, "triangle_fetches": 0, "hits": 0, "device_ms": 0.0,
        "timed_launches": 0, "merge_launches": 0, "merge_queries": 0, "merge_eye_vertices": 0, "merge_entries": 0,
        "merges": 0, "merge_ms": 0.0, "merge_timed_launches": 0}


class FakeScene:
    """Records the profile modes it is set to and the renders in each."""

    def __init__(self, count: dict, time: dict) -> None:
        self.records = {lmgpu.TRACE_PROFILE_COUNT: count, lmgpu.TRACE_PROFILE_TIME: time}
        self.mode = lmgpu.TRACE_PROFILE_OFF
        self.log = []

    def set_trace_profile(self, mode: int) -> None:
        self.mode = mode

    def read_trace_profile(self) -> dict:
        return dict(ZERO, **self.records.get(self.mode, {}))

    def render(self, seed: int) -> None:
        self.log.append((self.mode, seed))


class FakeFlush:
    def fill_(self, v: float) -> None:
        pass


def test_render_roofline_formula():
    sc = FakeScene({"launches": 3, "rays": 1000, "node_fetches": 5000, "triangle_fetches": 2000, "hits": 900},
                   {"launches": 3, "timed_launches": 3, "device_ms": 0.5})
    r = bench.render_trace_roofline(sc, sc.render, 2.0, FakeFlush())
    nbytes = 1000 * 48 + 5000 * 80 + 2000 * 48
    assert r["achieved"] == pytest.approx(nbytes / 0.5e-3 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"])
    assert r["bytes_per_ray"] == pytest.approx(nbytes / 1000)
    assert r["share_of_step"] == pytest.approx(0.25)
    assert r["launches_per_step"] == 3
    # the counted render, then the timed one, both of the first timed step's seed; the profile ends off
    assert sc.log == [(lmgpu.TRACE_PROFILE_COUNT, 1000), (lmgpu.TRACE_PROFILE_TIME, 1000)]
    assert sc.mode == lmgpu.TRACE_PROFILE_OFF


def test_render_roofline_rejects_untimed_launches():
    sc = FakeScene({"launches": 5000, "rays": 10}, {"launches": 5000, "timed_launches": 4096, "device_ms": 1.0})
    assert bench.render_trace_roofline(sc, sc.render, 2.0, FakeFlush()) is None


def test_vcm_merge_roofline_formula():
    sc = FakeScene({"merge_launches": 4, "merge_queries": 100, "merge_eye_vertices": 400, "merge_entries": 5000,
                    "merges": 900},
                   {"merge_launches": 4, "merge_timed_launches": 4, "merge_ms": 0.25, "device_ms": 0.1})
    r = bench.vcm_merge_roofline(sc, sc.render, 1.0, FakeFlush())
    nbytes = 100 * 4 + 400 * 32 + 5000 * 16 + 900 * 96
    assert r["achieved"] == pytest.approx(nbytes / 0.25e-3 / 1e9)
    assert r["bytes_per_query"] == pytest.approx(nbytes / 100)
    assert r["share_of_step"] == pytest.approx(0.25)
    assert r["traversal_ms_per_step"] == pytest.approx(0.1)
    no_merges = FakeScene({}, {"merge_launches": 0})
    assert bench.vcm_merge_roofline(no_merges, no_merges.render, 1.0, FakeFlush()) is None


def _curve(c, times):
    # checkpoints (seconds, spp, raw relMSE, relMSE less the reference's noise) on relMSE = c / t
    return [(t, int(100 * t), c / t + 0.001, c / t) for t in times]


def test_time_to_target_interpolates_and_extrapolates():
    """On relMSE = c / t (the Monte Carlo rate) both forms give c / target."""
    c, target = 0.5, 1e-2
    t, extrap = bench.time_to_target(_curve(c, [1, 2, 4, 8, 16, 32, 64, 128]), target)
    assert not extrap and t == pytest.approx(c / target)
    t, extrap = bench.time_to_target(_curve(c, [1, 2, 4, 8]), target)
    assert extrap and t == pytest.approx(c / target)
    t, extrap = bench.time_to_target(_curve(1e-3, [1, 2]), target)
    assert not extrap and t == 1
    assert bench.time_to_target([], target) == (None, True)


def test_progressive_accumulation_is_sample_weighted():
    """Films of 8 and 24 spp: the mean weights them by spp, and the variance
    of the mean (each render's variance of its own mean v / spp) is v / 32."""
    import numpy as np

    acc = bench.Progressive((2, 2, 3))
    v = 0.64
    acc.add(np.full((2, 2, 3), 1.0, np.float32), np.full((2, 2, 3), v / 8, np.float32), 8, 0.5)
    acc.add(np.full((2, 2, 3), 3.0, np.float32), np.full((2, 2, 3), v / 24, np.float32), 24, 1.5)
    assert acc.spp == 32 and acc.seconds == 2.0
    assert np.allclose(acc.mean(), (8 * 1.0 + 24 * 3.0) / 32)
    assert np.allclose(acc.variance(), v / 32, rtol=1e-6)
    assert bench.relmse_image(acc.mean(), acc.mean()) == 0.0


def test_committed_traffic_summary_is_read():
    """The headline's roofline.traffic and L2 figures come from the committed
    ncu summary of the closest-hit kernel (profiles/trace_closest_traffic.json)."""
    t = bench.traffic_per_launch()
    assert t is not None and 1e9 < t < 2e10
    l2 = bench.l2_figures()
    assert l2 is not None and l2

"""The roofline arithmetic of bench.py's render lines, on the CPU with a fake
scene whose trace profile returns fixed records: the counted render gives
the algorithmic bytes, the timed render the device time, and a record that
timed fewer launches than it ran gives no roofline."""
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

"""Host logic of bench.py that needs no GPU: the kernel-launch count per
frame of each raster path, the traffic lookup keyed by the kernel sources'
digest, and the clock sampler's timed windows."""
import json
import types

import bench
from softlight_gb300 import api as A


def _scene(width, height, draws, blending=False, batched=False, num_triangles=0):
    return types.SimpleNamespace(width=width, height=height, draws=draws, blending=blending, batched=batched,
                                 num_triangles=num_triangles)


def _mesh(mode, elements):
    return types.SimpleNamespace(mode=mode, elementBegin=0, elementEnd=elements)


def test_launches_of_an_instanced_order_free_frame():
    # two clears + vertex cache + vs_setup + clip + launch mark + three raster-path kernels
    s = _scene(1920, 1080, [(_mesh(A.RENDER_MODE_INDEXED_TRIANGLES, 3 * 4096), 1024, 1)])
    assert bench.launches_per_frame(s, (8, 8)) == 9


def test_launches_of_a_blended_frame():
    soup = [(_mesh(A.RENDER_MODE_TRIANGLES, 3 * 2_000_000), 1, 1)]
    # key-order lists on 1 020 tiles: bin numbering (3), count, chunk scan, tile scan, fill, raster
    assert bench.launches_per_frame(_scene(1920, 1080, soup, blending=True), (64, 32)) == 13
    # 32 400 tiles: tile scan, atomic fill, tile sort, raster
    assert bench.launches_per_frame(_scene(1920, 1080, soup, blending=True), (8, 8)) == 9


def test_launches_of_a_batch_and_of_its_draws():
    draws = [(_mesh(A.RENDER_MODE_INDEXED_TRIANGLES, 3 * 100), 1, k) for k in range(4)]
    assert bench.launches_per_frame(_scene(640, 480, draws, batched=True, num_triangles=400), (16, 16)) == 8
    assert bench.launches_per_frame(_scene(640, 480, draws), (16, 16)) == 2 + 4 * 6


def test_traffic_needs_the_captured_kernel_sources(tmp_path, monkeypatch):
    prof = tmp_path / "profiles"
    prof.mkdir()
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    monkeypatch.setattr(bench, "kernel_sources_digest", lambda: "d")
    # c2 captured at the current sources, c3 at others, c4 without a digest
    (prof / "traffic.json").write_text(json.dumps({
        "c2": {"raster": {"bytes": 123, "sources": "d", "capture": "x.md"}},
        "c3": {"raster": {"bytes": 456, "sources": "e", "capture": "y.md"}},
        "c4": {"raster": 789}}))
    assert bench.profiled_traffic("c2", "raster")[0] == 123
    assert bench.profiled_traffic("c3", "raster")[0] is None
    assert bench.profiled_traffic("c4", "raster")[0] is None
    assert bench.profiled_traffic("c1", "raster")[0] is None


def test_clock_samples_count_only_inside_timed_windows():
    c = bench.ClockSampler(0)
    line = "0, {sm}, 2070, 500.0, 0x0, Not Active, Not Active, Not Active, {cap}"
    c.lines = [(0.5, line.format(sm=1000, cap="Active")),
               (1.5, line.format(sm=2070, cap="Not Active")),
               (2.5, line.format(sm=1200, cap="Active")),
               (3.5, line.format(sm=2070, cap="Not Active"))]
    c.windows = [[1.0, 2.0], [3.0, 4.0]]
    s = c.summary()
    assert s["samples"] == 2 and s["sm_mhz"] == 2070.0 and s["reasons"] == []
    c.windows = [[0.0, 1.0]]
    assert c.summary()["reasons"] == ["sw_power_cap"]

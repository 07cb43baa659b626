"""bench.py's host-side pieces, without a GPU: the roofline's DRAM traffic read from the committed
launch-list summary, the peaks' fallback when no measured file is present, the many-ribbon shapes
drawn from the seeded generator, and the headline workload built at a small size."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402

CLASSES = ("small_front", "large_front_panel", "large_front_update", "assemble", "refine_forward",
           "refine_backward", "refine_residual")


def test_profiled_traffic_reads_the_committed_summary():
    for cls in CLASSES:
        v = bench.profiled_traffic(cls)
        assert v is not None and 1e9 < v < 1e12, (cls, v)
    assert bench.profiled_traffic("no_such_class") is None


def test_peaks_fall_back_without_the_measured_file(monkeypatch, tmp_path):
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    p = bench.peaks()
    assert p["source"] == "fallback" and p["hbm_gbs"] > 0 and p["bf16_tflops"] > 0


def test_ribbon_shapes_are_seeded_and_in_range():
    a = bench.ribbon_shapes(256, 1)
    assert a == bench.ribbon_shapes(256, 1)
    assert a != bench.ribbon_shapes(256, 2)
    assert all(40 <= w <= 160 and 100 <= l <= 400 for w, l in a)
    assert len({w for w, _ in a}) > 50  # uneven widths, as the workload needs


def test_headline_workload_builds_at_a_small_size():
    sys_, sigmas, pairs = bench.build_workload(length=12, width=6, configs=2, energies=3)
    assert len(sigmas) == 3 and len(pairs) == 6
    assert [c for _, c in pairs] == [0, 1] * 3
    assert np.allclose([s.energy for s in sigmas], np.linspace(-0.16, 0.16, 3))
    assert sys_.config_count() == 2
    for s in sigmas:
        for sl, sr in s.blocks:
            assert np.isfinite(sl).all() and np.isfinite(sr).all()

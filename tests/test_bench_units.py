"""Host-side arithmetic of bench.py (no GPU): the mixed path's roofline."""
import sys

from conftest import ROOT

sys.path.insert(0, ROOT)


def test_mixed_roofline_names_the_binding_bound():
    import bench
    r = bench.mixed_roofline(3.2e8, 6794.1)
    assert abs(r["fp32"]["achieved"] - 700 * 3.2e8 / 1e12) < 1e-12
    assert abs(r["hbm"]["achieved"] - 384 * 3.2e8 / 1e9) < 1e-9
    assert abs(r["fp32"]["peak"] - 80.55) < 0.1
    assert r["binding"] == "hbm"  # 1.8% of the copy bandwidth vs 0.28% of the FP32 peak
    assert bench.mixed_roofline(3.2e8, 1e6)["binding"] == "fp32"


def test_paired_ci_matches_student_t():
    import numpy as np
    import bench
    rng = np.random.default_rng(3)
    a = rng.normal(100.0, 5.0, 16)
    b = a + rng.normal(0.5, 1.0, 16)
    r = bench.paired_ci(a, b)
    d = b - a
    h = 2.131 * d.std(ddof=1) / 4.0 / a.mean()
    assert abs(r["rel_mean_diff"] - d.mean() / a.mean()) < 1e-15
    assert abs((r["ci95"][1] - r["ci95"][0]) / 2 - h) < 1e-15
    assert r["within_1pct"] == (abs(d.mean() / a.mean()) + h < 0.01)


def test_timed_window_is_pinned_and_reference_phases_lie_in_it():
    import argparse
    import bench
    for warmup in (0, 3, 5):
        args = argparse.Namespace(steps=20, warmup=warmup, step_ms=10.0)
        assert bench.window_ms(args) == (30.0, 230.0)
        ph = [float(p.rsplit("t", 1)[1]) for p in bench.window_phases(args)]
        assert all(30.0 <= t < 230.0 for t in ph)
    args = argparse.Namespace(steps=2, warmup=5, step_ms=10.0)
    assert all(float(p.rsplit("t", 1)[1]) < 50.0 for p in bench.window_phases(args))


def test_roofline_kernel_follows_the_tuned_shape():
    import argparse
    import bench
    args = argparse.Namespace(fru_lanes=4)
    packed = {"lanes_per_fru": 4, "packed_div": 8}
    fixed = {"lanes_per_fru": 4, "packed_div": 0}
    assert bench.stage_kernel_name("fp64", packed, args) == "fru_stage4_packed_kernel"
    assert bench.stage_kernel_name("fp64", fixed, args) == "fru_stage4_kernel"
    assert bench.stage_kernel_name("mixed", packed, args) == "fru_stage_mixed_packed_kernel"
    assert bench.stage_kernel_name("fp64", {"lanes_per_fru": 1, "packed_div": 0}, args) == "fru_stage_kernel"

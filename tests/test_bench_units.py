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

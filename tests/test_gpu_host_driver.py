"""The C host driver on the GPU library (greenstein2002_gb300/_build/gw_caf):
an exact checkpoint written mid-run resumes into the same files, byte for
byte, as the uninterrupted run, and the per-FRU property files are written."""
import os

import pytest

from conftest import ROOT
from test_host_driver import GOLDEN_DRIVER_CASES, exact_restart_case, golden_driver_args

pytestmark = pytest.mark.gpu


def test_gpu_exact_restart_continues_bit_for_bit(gw, tmp_path):
    exe = os.path.join(ROOT, "greenstein2002_gb300", "_build", "gw_caf")
    assert os.path.isfile(exe), "gw_caf not built"
    written = exact_restart_case(exe, tmp_path)
    assert "fruprops_4.1.txt" in written and "fruprops_avg_tot.1.txt" in written


def test_gpu_launch_shapes_same_files(gw, tmp_path):
    """The host driver's output files do not depend on the stage kernels'
    launch shape (fixed 8 FRUs per warp, 4-warp blocks, packed queue), through
    the integrator's saves, rejections and resumes."""
    import filecmp
    import subprocess
    exe = os.path.join(ROOT, "greenstein2002_gb300", "_build", "gw_caf")
    base = {"NFRU_sim": 500, "time_end": 14.0, "ic_file_flag": 0, "seed_scheme": 0, "seed_base": 5489}
    runs = {"fixed": {}, "warps4": {"stage_warps": 4}, "packed4": {"stage_packing": 4}}
    for name, extra in runs.items():
        d = tmp_path / name
        d.mkdir()
        subprocess.run([exe] + ["%s=%s" % kv for kv in dict(base, **extra).items()], cwd=d, check=True,
                       capture_output=True)
    for name in ("warps4", "packed4"):
        for f in ("states.0.txt", "otherstates.0.txt", "currents.0.txt"):
            assert filecmp.cmp(tmp_path / "fixed" / f, tmp_path / name / f, shallow=False), (name, f)


@pytest.mark.parametrize("shape", [{}, {"stage_packing": 4}])
@pytest.mark.parametrize("case", sorted(GOLDEN_DRIVER_CASES))
def test_gpu_driver_files_equal_reference_program(gw, tmp_path, case, shape):
    """In the reference's sum order (sum_order=1) the host driver on the GPU
    library writes the reference program's own output files byte for byte:
    250 FRUs from rest, FRU j seeded 5489 + j, 50 ms of 1 Hz pacing or 30 ms
    through a voltage-clamp step (tests/golden/drv250*, made by
    tests/golden/make_driver_files.py)."""
    import filecmp
    import subprocess
    from conftest import GOLDEN
    exe = os.path.join(ROOT, "greenstein2002_gb300", "_build", "gw_caf")
    args = dict(golden_driver_args(case), **shape)
    subprocess.run([exe] + ["%s=%s" % kv for kv in args.items()], cwd=tmp_path, check=True, capture_output=True)
    for f in ("states.0.txt", "otherstates.0.txt", "currents.0.txt"):
        assert filecmp.cmp(os.path.join(GOLDEN, case, f), tmp_path / f, shallow=False), f

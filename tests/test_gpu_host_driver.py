"""The C host driver on the GPU library (greenstein2002_gb300/_build/gw_caf):
an exact checkpoint written mid-run resumes into the same files, byte for
byte, as the uninterrupted run, and the per-FRU property files are written."""
import os

import pytest

from conftest import ROOT
from test_host_driver import exact_restart_case

pytestmark = pytest.mark.gpu


def test_gpu_exact_restart_continues_bit_for_bit(gw, tmp_path):
    exe = os.path.join(ROOT, "greenstein2002_gb300", "_build", "gw_caf")
    assert os.path.isfile(exe), "gw_caf not built"
    written = exact_restart_case(exe, tmp_path)
    assert "fruprops_4.1.txt" in written and "fruprops_avg_tot.1.txt" in written

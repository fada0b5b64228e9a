"""The FP64 division the FRU kernels run on the integer pipe
(greenstein2002_gb300/csrc/gw_intdiv.h) returns the IEEE round-to-nearest
quotient bit for bit.  On the CPU the same source is compiled as C and
compared with the C division on random operand pairs (all bit patterns, and
the magnitudes of the FRU substep), boundary mantissas and special values;
on the GPU the device build is compared with the hardware division."""
import os
import subprocess

import pytest

from conftest import ROOT, TBUILD


def test_integer_division_matches_c_division():
    exe = os.path.join(TBUILD, "intdiv_check")
    os.makedirs(TBUILD, exist_ok=True)
    subprocess.check_call([os.environ.get("CC", "gcc"), "-O2", "-std=c99", "-ffp-contract=off",
                           "-I" + os.path.join(ROOT, "greenstein2002_gb300", "csrc"), "-o", exe,
                           os.path.join(ROOT, "tests", "native", "intdiv_check.c")])
    r = subprocess.run([exe, "20000000", "7"], capture_output=True, text=True)
    print(r.stdout)
    assert r.returncode == 0, r.stdout


@pytest.mark.gpu
def test_device_integer_division_matches_hardware(gw):
    for seed in (1, 2, 3):
        assert gw.div_mismatches(1 << 28, seed=seed) == 0

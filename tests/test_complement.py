"""The mixed-precision transition tests compare 1 - u = (2^32 - y)/2^32 with
dt*rate in FP32 and convert 2^32 - y from the 32-bit integer 0 - y instead
of the 33-bit value (a 64-bit integer conversion runs on GB300's FP64 pipe).
The two give the same FP32 value for every y: checked exhaustively here."""
import os
import subprocess

from conftest import ROOT, TBUILD


def test_complement_from_32_bits_is_exact():
    exe = os.path.join(TBUILD, "complement_check")
    os.makedirs(TBUILD, exist_ok=True)
    subprocess.check_call([os.environ.get("CC", "gcc"), "-O2", "-std=c99", "-ffp-contract=off", "-o", exe,
                           os.path.join(ROOT, "tests", "native", "complement_check.c")])
    r = subprocess.run([exe], capture_output=True, text=True)
    print(r.stdout)
    assert r.returncode == 0, r.stdout

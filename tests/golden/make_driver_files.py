"""Golden output files of the reference program for the GPU host-driver test.

Builds the reference serially (oracle/build_ref.py) for 250 FRUs and the rest
initial state (ic_file_flag 0), runs it with FRU j seeded 5489 + j, and copies
the files it writes (states.0.txt, otherstates.0.txt, currents.0.txt;
data_io.c:22-140):
  tests/golden/drv250/          the 1 Hz stimulus, 50 ms
  tests/golden/drv250_vclamp/   the voltage clamp of fcn.c:448-480 (hold
                                -100 mV, 0 mV for 200 ms from 10 ms, period
                                500 ms), 30 ms
Runs only where the reference sources are available; the files are committed.

Usage: python tests/golden/make_driver_files.py
"""
import os
import shutil
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import build_ref  # noqa: E402

NFRU, SEED_BASE = 250, 5489
FILES = ("states.0.txt", "otherstates.0.txt", "currents.0.txt")
VCLAMP = {"hold": -100.0, "set": 0.0, "duration": 200.0, "shift": 10.0, "period": 500.0}
CASES = {"drv250": (50.0, None), "drv250_vclamp": (30.0, VCLAMP)}


def main():
    if not build_ref.have_sources():
        sys.exit("reference sources not available")
    for name, (time_end, vclamp) in CASES.items():
        d = build_ref.build_config("gold_" + name, build_ref.cfg_macros(NFRU, time_end, vclamp=vclamp))
        out = os.path.join(HERE, name)
        os.makedirs(out, exist_ok=True)
        with tempfile.TemporaryDirectory() as work:
            build_ref.run_stoch(d, work, seed_base=SEED_BASE)
            for f in FILES:
                shutil.copyfile(os.path.join(work, f), os.path.join(out, f))
        print("wrote", out)


if __name__ == "__main__":
    main()

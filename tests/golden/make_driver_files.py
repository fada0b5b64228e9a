"""Golden output files of the reference program for the GPU host-driver test.

Builds the reference serially (oracle/build_ref.py) for 250 FRUs, the rest
initial state (ic_file_flag 0), the 1 Hz stimulus and 50 ms, runs it with FRU
j seeded 5489 + j, and copies the files it writes (states.0.txt,
otherstates.0.txt, currents.0.txt; data_io.c:22-140) to tests/golden/drv250/.
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

NFRU, TIME_END, SEED_BASE = 250, 50.0, 5489
FILES = ("states.0.txt", "otherstates.0.txt", "currents.0.txt")


def main():
    if not build_ref.have_sources():
        sys.exit("reference sources not available")
    d = build_ref.build_config("drv_%d_%d_0" % (NFRU, int(TIME_END)), build_ref.cfg_macros(NFRU, TIME_END))
    out = os.path.join(HERE, "drv%d" % NFRU)
    os.makedirs(out, exist_ok=True)
    with tempfile.TemporaryDirectory() as work:
        build_ref.run_stoch(d, work, seed_base=SEED_BASE)
        for f in FILES:
            shutil.copyfile(os.path.join(work, f), os.path.join(out, f))
    print("wrote", out)


if __name__ == "__main__":
    main()

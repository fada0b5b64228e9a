"""Initial-condition files for the reference arm of bench.py: the 12,500-FRU
bench cell (rest state, 1 Hz pacing, FRU j seeded 5489 + j) at t = 30, 50,
70, ..., 210 ms -- ten evenly spaced phases of the bench's timed window
[30, 230) ms -- in the reference's IC format (initialize_state.c:43-163).

The trajectory comes from the C host driver over the CPU restatement of the
FRU path (the composition that reproduces the reference program bit for bit,
tests/test_host_driver.py); the reference program itself cannot write these
files because its restart_data closes the r_states file twice
(data_io.c:220, :265) and aborts before writing the channel states.  The
reference reads IC files 1250 FRUs at a time (rewinding for larger cells), so
only the first 1250 FRUs are kept.  Takes about 15 CPU-minutes."""
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
from test_host_driver import cpu_driver  # noqa: E402

# checkpoint number -> time (ms); with Ndump = 10 checkpoint k is written at (k + 1) * 10 ms
PHASES = {t // 10 - 1: t for t in range(30, 230, 20)}
KEEP = 1250
NAMES = {"r_states": "ic_states_stable.txt", "r_FRU": "ic_FRU_stable.txt", "r_LCh": "ic_LCh_stable.txt",
         "r_RyR": "ic_RyR_stable.txt", "r_Ito2": "ic_Ito2_stable.txt"}
LINES_PER_FRU = {"r_FRU": 1, "r_LCh": 4, "r_RyR": 4, "r_Ito2": 4}


def main():
    exe = cpu_driver()
    shutil.rmtree(os.path.join(HERE, "ic_window"), ignore_errors=True)
    with tempfile.TemporaryDirectory() as tmp:
        subprocess.run([exe, "NFRU_sim=12500", "time_end=%d" % (max(PHASES.values()) + 1), "ic_file_flag=0", "seed_scheme=0", "seed_base=5489",
                        "Ndump=10"], cwd=tmp, check=True, stdout=subprocess.DEVNULL)
        for num, t in PHASES.items():
            out = os.path.join(HERE, "ic_window", "t%d" % t)
            os.makedirs(out, exist_ok=True)
            for stem, name in NAMES.items():
                src = os.path.join(tmp, "%s.%d.txt" % (stem, num))
                dst = os.path.join(out, name)
                if stem == "r_states":
                    shutil.copyfile(src, dst)
                    continue
                with open(src) as f:
                    lines = f.readlines()
                with open(dst, "w") as f:
                    f.write("%d\n" % KEEP)
                    f.writelines(lines[1:1 + KEEP * LINES_PER_FRU[stem]])


if __name__ == "__main__":
    main()

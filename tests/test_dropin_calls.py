"""The drop-in entry points (the reference's MPI-layer names) called in the
reference program's order by tests/native/dropin_calls.c, linked against the
CPU stand-in over the oracle and against libgw_fru.so on the GPU: integer
results (channel states, draw counts, MT words) identical, currents, output
averages and Ca sums within a relative 1e-12 (CUDA's exp and the host libm's
differ in the last place for a few percent of arguments; the GPU's sums run
in a fixed tree order)."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, TBUILD, cpu_cell_lib_path

SRC = os.path.join(ROOT, "tests", "native", "dropin_calls.c")


def _link(libdir, libname, out):
    os.makedirs(TBUILD, exist_ok=True)
    subprocess.check_call([os.environ.get("CC", "gcc"), "-O2", "-std=c99", "-I" + os.path.join(ROOT, "include"),
                           "-o", out, SRC, "-L" + libdir, "-l" + libname, "-Wl,-rpath," + libdir, "-lm"])
    return out


def _run(exe):
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    return [line.split() for line in r.stdout.splitlines()]


def _cpu_lines():
    lib = cpu_cell_lib_path()
    return _run(_link(os.path.dirname(lib), "cpu_cell", os.path.join(TBUILD, "dropin_calls_cpu")))


def test_dropin_calls_cpu_standin():
    lines = _cpu_lines()
    assert lines[0] == ["I", "0", "1"]
    assert sum(1 for l in lines if l[0] == "J") == 1 + 12 + 4
    vals = np.array([float(v) for l in lines if l[0] in "JOF" for v in l[1:]])
    assert np.all(np.isfinite(vals))


@pytest.mark.gpu
def test_dropin_calls_gpu_match_oracle(gw):
    libdir = os.path.join(ROOT, "greenstein2002_gb300", "_build")
    gpu = _run(_link(libdir, "gw_fru", os.path.join(TBUILD, "dropin_calls_gpu")))
    cpu = _cpu_lines()
    assert [l[0] for l in gpu] == [l[0] for l in cpu]
    for g, c in zip(gpu, cpu):
        if g[0] == "I":
            assert g == c
        else:
            np.testing.assert_allclose(np.array(g[1:], float), np.array(c[1:], float), rtol=1e-12, atol=1e-300)

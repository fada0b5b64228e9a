"""Shared test setup.

Markers: `gpu` tests need a CUDA GPU (GB300) and run the CUDA path through the
C-ABI; everything else runs on CPU (oracle, host logic, ABI symbol checks).
"""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")
TBUILD = os.path.join(ROOT, "tests", "_build")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU; runs the CUDA path through the C-ABI")


def cpu_cell_lib_path():
    """Build the test-only CPU stand-in of the native FRU API (tests/native/cpu_cell.c
    + the product's host sources + the oracle) and return its path."""
    out = os.path.join(TBUILD, "libcpu_cell.so")
    srcs = [os.path.join(ROOT, "tests", "native", "cpu_cell.c"),
            os.path.join(ROOT, "greenstein2002_gb300", "csrc", "gw_dp.c"),
            os.path.join(ROOT, "greenstein2002_gb300", "csrc", "gw_dropin.c"),
            os.path.join(ROOT, "oracle", "fru_oracle.c")]
    hdrs = [os.path.join(ROOT, "greenstein2002_gb300", "csrc", "gw_cell_model.h"),
            os.path.join(ROOT, "include", "gw_fru.h")]
    if os.path.isfile(out) and all(os.path.getmtime(s) <= os.path.getmtime(out) for s in srcs + hdrs):
        return out
    os.makedirs(TBUILD, exist_ok=True)
    subprocess.check_call([os.environ.get("CC", "gcc"), "-O2", "-std=c99", "-ffp-contract=off", "-fPIC", "-shared",
                           "-I" + os.path.join(ROOT, "greenstein2002_gb300", "csrc"),
                           "-I" + os.path.join(ROOT, "include"), "-o", out] + srcs + ["-lm"])
    return out


@pytest.fixture(scope="session")
def cpu_cell_lib():
    import greenstein2002_gb300 as G
    return G.bind(cpu_cell_lib_path())


@pytest.fixture(scope="session")
def gw():
    """The product library on a GPU (fails loudly when the CUDA path is unavailable)."""
    import greenstein2002_gb300 as G
    G.load()
    return G


def golden(name):
    import numpy as np
    return np.load(os.path.join(GOLDEN, name))

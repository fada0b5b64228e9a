"""The drop-in layer: the reference's own program (caf.c, rk_pd54m.c, fcn.c,
data_io.c, initialize_*.c, ...) linked against this library instead of its
mpi_master.c / mpi_slave.c, with no source change.

CPU: linked against the test-only CPU stand-in of the FRU API, the program
must write the same files as the stock reference, byte for byte.
GPU: linked against libgw_fru.so, it runs its FRUs on the GPU and its
per-ms traces must match the stock program's."""
import filecmp
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT, TBUILD, cpu_cell_lib_path

sys.path.insert(0, os.path.join(ROOT, "oracle"))
import build_ref  # noqa: E402

KEEP = ["caf.c", "rk_pd54m.c", "fcn.c", "data_io.c", "initialize_ran.c", "initialize_state.c", "mt19937_local.c",
        "write_fru_props.c", "dynamicFRU.c", "parameters_fcn_fru.c"]


def link_reference_program(cfg_dir, libdir, libname, out):
    subprocess.check_call(["gcc", "-O3", "-ffp-contract=off", "-w", "-rdynamic", "-I" + cfg_dir, "-o", out] +
                          [os.path.join(cfg_dir, f) for f in KEEP] +
                          ["-L" + libdir, "-l" + libname, "-Wl,-rpath," + libdir, "-lm"])
    return out


def run_prog(exe, wd, seed_base):
    import resource

    def _stack():
        resource.setrlimit(resource.RLIMIT_STACK, (resource.RLIM_INFINITY, resource.RLIM_INFINITY))
    os.makedirs(wd, exist_ok=True)
    env = dict(os.environ)
    env.pop("GW_SEED_BASE", None)
    r = subprocess.run([exe], cwd=wd, env=env, capture_output=True, text=True, preexec_fn=_stack)
    assert r.returncode == 0, r.stderr[-2000:]


@pytest.fixture(scope="module")
def cfg():
    if not build_ref.have_sources():
        pytest.skip("reference sources not available")
    # reference seeding (initialize_ran.c), rest state, 250 FRUs, 15 ms
    return build_ref.build_config("dropin_250_15", build_ref.cfg_macros(250, 15.0))


def test_dropin_cpu_standin_is_byte_identical(cfg, tmp_path):
    lib = cpu_cell_lib_path()
    exe = link_reference_program(cfg, os.path.dirname(lib), "cpu_cell", os.path.join(TBUILD, "stoch_dropin_cpu"))
    run_prog(exe, str(tmp_path / "gw"), None)
    build_ref.run_stoch(cfg, str(tmp_path / "ref"))
    for f in ("states.0.txt", "otherstates.0.txt", "currents.0.txt"):
        assert filecmp.cmp(tmp_path / "ref" / f, tmp_path / "gw" / f, shallow=False), f


@pytest.mark.gpu
def test_dropin_gpu(cfg, tmp_path, gw):
    libdir = os.path.join(ROOT, "greenstein2002_gb300", "_build")
    exe = link_reference_program(cfg, libdir, "gw_fru", os.path.join(TBUILD, "stoch_dropin_gpu"))
    run_prog(exe, str(tmp_path / "gw"), None)
    build_ref.run_stoch(cfg, str(tmp_path / "ref"))
    a = np.loadtxt(tmp_path / "ref" / "states.0.txt", skiprows=1)
    b = np.loadtxt(tmp_path / "gw" / "states.0.txt", skiprows=1)
    assert a.shape == b.shape
    # printed with %.8g: agreement to ~8 significant digits
    np.testing.assert_allclose(b, a, rtol=2e-7, atol=1e-12)

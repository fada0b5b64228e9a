"""C-ABI checks that need no GPU: the library builds for sm_103a, loads, and
exports every function include/gw_fru.h declares; host-only entry points
behave (settings defaults = the reference's parameters.h; no device -> error
status, not a crash or a CPU fallback)."""
import ctypes as C
import os
import re
import subprocess

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "gw_fru.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s*\**([A-Za-z_][A-Za-z0-9_]*)\s*\(", text,
                       flags=re.M)
    return sorted(set(n for n in names if n not in ("if", "defined")))


@pytest.fixture(scope="module")
def lib():
    import greenstein2002_gb300 as G
    from greenstein2002_gb300 import build
    build.build()
    return G.load()


def test_header_declares_drop_in_and_native(lib):
    names = declared_functions()
    for n in ("distrib_simFRU", "send_calc_fru_flux", "send_calc_fru_avg", "send_save_state",
              "send_resume_state", "initialize_mpi_state", "parallel_get_FRUs", "initialize_mpi", "end_mpi",
              "gw_create", "gw_stage", "gw_rk54pd", "gw_run"):
        assert n in names


def test_library_exports_every_declared_symbol(lib):
    path = os.path.join(ROOT, "greenstein2002_gb300", "_build", "libgw_fru.so")
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True, check=True).stdout
    exported = set(line.split()[-1] for line in out.splitlines() if line.strip())
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing


def test_library_is_sm103a_only():
    path = os.path.join(ROOT, "greenstein2002_gb300", "_build", "libgw_fru.so")
    out = subprocess.run(["cuobjdump", "--list-elf", path], capture_output=True, text=True)
    if out.returncode != 0:
        pytest.skip("cuobjdump unavailable")
    arches = set(re.findall(r"sm_(\d+a?)", out.stdout))
    assert arches == {"103a"}, arches


def test_settings_defaults_are_reference_parameters(lib):
    import greenstein2002_gb300 as G
    s = G.settings()
    # parameters.h:92-156
    assert (s.time_step, s.step_min, s.step_max, s.tolrk) == (1.0, 1e-6, 0.1, 1e-6)
    assert (s.pulse_duration, s.pulse_amplitude, s.period, s.shift) == (1, -100, 1000, 10)
    assert (s.vclamp_flag, s.vclamp_hold, s.vclamp_set, s.vclamp_duration) == (0, -80.0, 0.0, 200.0)
    assert (s.scale_PCa, s.scale_GKr) == (1.0, 1.0)


def test_no_device_is_an_error_not_a_fallback(lib):
    import greenstein2002_gb300 as G
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    h = C.c_void_p()
    rc = lib.gw_create(C.byref(h), 16)
    assert rc != 0
    with pytest.raises(G.GWError):
        G.Cell(16)


def test_struct_layouts_match_the_header(tmp_path):
    """The ctypes mirrors of gw_settings and gw_request have the C layout."""
    import greenstein2002_gb300 as G
    src = tmp_path / "layout.c"
    src.write_text('#include <stddef.h>\n#include <stdio.h>\n#include "gw_fru.h"\n'
                   'int main(void) { printf("%zu %zu %zu %zu %zu %zu\\n", sizeof(gw_settings), sizeof(gw_request),'
                   ' offsetof(gw_request, set), offsetof(gw_request, duration_ms), offsetof(gw_request, status),'
                   ' offsetof(gw_request, message)); return 0; }\n')
    exe = tmp_path / "layout"
    subprocess.check_call([os.environ.get("CC", "gcc"), "-I" + os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    got = [int(x) for x in subprocess.check_output([str(exe)], text=True).split()]
    R = G.Request
    assert got == [C.sizeof(G.Settings), C.sizeof(R), R.set.offset, R.duration_ms.offset, R.status.offset,
                   R.message.offset]

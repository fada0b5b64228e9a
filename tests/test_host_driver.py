"""The C host driver (greenstein2002_gb300/host/gw_caf.c): run settings at run
time, the reference's initial-condition readers and output writers.

On CPU the driver is linked against the test-only CPU stand-in of the FRU
API (tests/native/cpu_cell.c over the oracle); since that composition is bit-
exact with the reference, its output files must equal the reference
program's byte for byte -- which pins the file formats (data_io.c:22-140,
initialize_state.c:43-163) and the main-loop cadence (caf.c:150-255)."""
import filecmp
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT, TBUILD, cpu_cell_lib_path

sys.path.insert(0, os.path.join(ROOT, "oracle"))
import build_ref  # noqa: E402


def cpu_driver():
    out = os.path.join(TBUILD, "gw_caf_cpu")
    srcs = [os.path.join(ROOT, "greenstein2002_gb300", "host", "gw_caf.c"),
            os.path.join(ROOT, "tests", "native", "cpu_cell.c"),
            os.path.join(ROOT, "greenstein2002_gb300", "csrc", "gw_dp.c"),
            os.path.join(ROOT, "oracle", "fru_oracle.c")]
    deps = srcs + [os.path.join(ROOT, "greenstein2002_gb300", "csrc", "gw_cell_model.h"),
                   os.path.join(ROOT, "include", "gw_fru.h")]
    if not (os.path.isfile(out) and all(os.path.getmtime(s) <= os.path.getmtime(out) for s in deps)):
        os.makedirs(TBUILD, exist_ok=True)
        subprocess.check_call(["gcc", "-O2", "-std=c99", "-ffp-contract=off",
                               "-I" + os.path.join(ROOT, "greenstein2002_gb300", "csrc"),
                               "-I" + os.path.join(ROOT, "include"), "-o", out] + srcs + ["-lm"])
    return out


@pytest.fixture(scope="module")
def have_ref():
    if not build_ref.have_sources():
        pytest.skip("reference sources not available")


def _run_both(tmp_path, macros, settings, seed_base):
    d = build_ref.build_config("drv_%d_%d_%d" % (macros["NFRU_sim_high"], int(float(macros["time_end"])),
                                                 macros["ic_file_flag"]), macros)
    ref_dir = tmp_path / "ref"
    build_ref.run_stoch(d, str(ref_dir), seed_base=seed_base)
    gw_dir = tmp_path / "gw"
    gw_dir.mkdir()
    subprocess.run([cpu_driver()] + ["%s=%s" % kv for kv in settings.items()], cwd=gw_dir, check=True,
                   capture_output=True)
    return ref_dir, gw_dir


def test_outputs_match_reference_rest_start(tmp_path, have_ref):
    m = build_ref.cfg_macros(250, 15.0)
    ref_dir, gw_dir = _run_both(tmp_path, m, {"NFRU_sim": 250, "time_end": 15.0, "ic_file_flag": 0,
                                              "seed_scheme": 0, "seed_base": 5489}, 5489)
    for f in ("states.0.txt", "otherstates.0.txt", "currents.0.txt"):
        assert filecmp.cmp(ref_dir / f, gw_dir / f, shallow=False), f


GOLDEN_DRIVER_CASES = {
    # tests/golden/<name>: the reference program's files (tests/golden/make_driver_files.py)
    "drv250": {"time_end": 50.0},
    "drv250_vclamp": {"time_end": 30.0, "vclamp_flag": 1, "vclamp_hold": -100.0, "vclamp_set": 0.0,
                      "vclamp_duration": 200.0, "vclamp_shift": 10.0, "vclamp_period": 500.0},
}


def golden_driver_args(name):
    return dict({"NFRU_sim": 250, "ic_file_flag": 0, "seed_scheme": 0, "seed_base": 5489, "sum_order": 1},
                **GOLDEN_DRIVER_CASES[name])


@pytest.mark.parametrize("case", sorted(GOLDEN_DRIVER_CASES))
def test_outputs_match_committed_reference_files(tmp_path, case):
    """The committed output files of the reference program (tests/golden/drv250*,
    made by tests/golden/make_driver_files.py) are what the host driver over
    the oracle writes: pins the fixtures the GPU host-driver test compares with."""
    from conftest import GOLDEN
    gw_dir = tmp_path / "gw"
    gw_dir.mkdir()
    subprocess.run([cpu_driver()] + ["%s=%s" % kv for kv in golden_driver_args(case).items()], cwd=gw_dir,
                   check=True, capture_output=True)
    for f in ("states.0.txt", "otherstates.0.txt", "currents.0.txt"):
        assert filecmp.cmp(os.path.join(GOLDEN, case, f), gw_dir / f, shallow=False), f


def test_outputs_match_reference_ic_files(tmp_path, have_ref):
    # the reference's default initial conditions: ic/stable files, its own
    # per-FRU seed formula, 1000 FRUs (1250-FRU files)
    m = build_ref.cfg_macros(1000, 12.0, ic_file=True)
    ic = os.path.join(build_ref.SRC, "ic", "stable")
    ref_dir, gw_dir = _run_both(tmp_path, m, {"NFRU_sim": 1000, "time_end": 12.0, "ic_file_flag": 1,
                                              "ic_dir": ic, "seed_scheme": 1}, None)
    for f in ("states.0.txt", "otherstates.0.txt", "currents.0.txt"):
        assert filecmp.cmp(ref_dir / f, gw_dir / f, shallow=False), f


def test_outputs_match_reference_voltage_clamp(tmp_path, have_ref):
    """The voltage-clamp protocol (fcn.c:448-480; hold -100 mV, step to 0 mV
    for 200 ms from 10 ms, period 500 ms): the host driver's files equal the
    reference program's byte for byte through the step."""
    vc = {"hold": -100.0, "set": 0.0, "duration": 200.0, "shift": 10.0, "period": 500.0}
    m = build_ref.cfg_macros(250, 30.0, vclamp=vc)
    ref_dir, gw_dir = _run_both(tmp_path, m, {"NFRU_sim": 250, "time_end": 30.0, "ic_file_flag": 0,
                                              "seed_scheme": 0, "seed_base": 5489, "vclamp_flag": 1,
                                              "vclamp_hold": -100.0, "vclamp_set": 0.0, "vclamp_duration": 200.0,
                                              "vclamp_shift": 10.0, "vclamp_period": 500.0}, 5489)
    for f in ("states.0.txt", "otherstates.0.txt", "currents.0.txt"):
        assert filecmp.cmp(ref_dir / f, gw_dir / f, shallow=False), f


PROTOCOLS = {
    # I-V protocol (fcn.c:521-533, caf.c:232-235): from -100 mV, 5-ms steps to -40, -30, -20 mV,
    # one per 10-ms period
    "iv": {"iv_flag": 1, "iv_clamp_duration": 5.0, "iv_clamp_period": 10.0, "iv_shift": 2.0,
           "iv_clamp_set": -40.0, "iv_clamp_hold": -100.0, "iv_clamp_step": 10.0},
    # paired-pulse clamp (fcn.c:485-515): -80 mV, 5 ms at -40 mV from 5 ms, then 10 ms at 0 mV
    "vpp": {"vppclamp_flag": 1, "vppclamp_ppset": -40.0, "vppclamp_ppduration": 5.0, "vppclamp_shift": 5.0,
            "vppclamp_set": 0.0, "vppclamp_duration": 10.0, "vppclamp_hold": -80.0, "vppclamp_period": 500.0},
}


@pytest.mark.parametrize("proto", sorted(PROTOCOLS))
def test_outputs_match_reference_clamp_protocols(tmp_path, have_ref, proto):
    """The I-V and paired-pulse clamp protocols: the host driver's files equal
    the reference program's byte for byte (250 FRUs from rest, 30 ms)."""
    extra = PROTOCOLS[proto]
    m = build_ref.cfg_macros(250, 30.0)
    m.update({k: repr(float(v)) if isinstance(v, float) else v for k, v in extra.items()})
    d = build_ref.build_config("drv_250_30_%s" % proto, m)
    ref_dir = tmp_path / "ref"
    build_ref.run_stoch(d, str(ref_dir), seed_base=5489)
    gw_dir = tmp_path / "gw"
    gw_dir.mkdir()
    settings = dict({"NFRU_sim": 250, "time_end": 30.0, "ic_file_flag": 0, "seed_scheme": 0, "seed_base": 5489},
                    **extra)
    subprocess.run([cpu_driver()] + ["%s=%s" % kv for kv in settings.items()], cwd=gw_dir, check=True,
                   capture_output=True)
    v = np.loadtxt(ref_dir / "states.0.txt", skiprows=1)[:, 1]
    assert len(set(np.round(v, 6))) >= 3  # the protocol moved V through its levels
    for f in ("states.0.txt", "otherstates.0.txt", "currents.0.txt"):
        assert filecmp.cmp(ref_dir / f, gw_dir / f, shallow=False), f


@pytest.mark.parametrize("variant", ["reset_RyRs", "chf"])
def test_outputs_match_reference_ic_variants(tmp_path, have_ref, variant):
    """From the reference's ic/stable files (250 FRUs, its seed formula, 8 ms):
    reset_RyRs_flag (initialize_state.c:252-263: every LCC closed and
    available, every RyR in state 1) and the heart-failure scalings of
    chf_flag (fcn.c:780-785): the host driver's files equal the reference
    program's byte for byte."""
    extra = {"reset_RyRs": {"reset_RyRs_flag": 1}, "chf": {"chf_flag": 1}}[variant]
    m = build_ref.cfg_macros(250, 8.0, ic_file=True)
    m.update(extra)
    d = build_ref.build_config("drv_250_8_ic_%s" % variant, m)
    ref_dir = tmp_path / "ref"
    build_ref.run_stoch(d, str(ref_dir))
    gw_dir = tmp_path / "gw"
    gw_dir.mkdir()
    settings = dict({"NFRU_sim": 250, "time_end": 8.0, "ic_file_flag": 1,
                     "ic_dir": os.path.join(build_ref.SRC, "ic", "stable"), "seed_scheme": 1}, **extra)
    subprocess.run([cpu_driver()] + ["%s=%s" % kv for kv in settings.items()], cwd=gw_dir, check=True,
                   capture_output=True)
    for f in ("states.0.txt", "otherstates.0.txt", "currents.0.txt"):
        assert filecmp.cmp(ref_dir / f, gw_dir / f, shallow=False), f


def test_checkpoint_files(tmp_path, have_ref):
    """r_*.N.txt checkpoints every Ndump steps (data_io.c:197-268).  The
    reference's restart_data closes the r_states file twice (data_io.c:220
    and :265), which glibc aborts on, so its process dies after writing
    r_states and r_FRU; those two are compared byte for byte, the other three
    (never flushed by the reference) are checked for format and content."""
    import numpy as np
    m = build_ref.cfg_macros(64, 7.0)
    m["Ndump"] = 3
    d = build_ref.build_config("drv_ckpt", m)
    ref_dir = tmp_path / "ref"
    with pytest.raises(RuntimeError, match="double free"):
        build_ref.run_stoch(d, str(ref_dir), seed_base=77)
    gw_dir = tmp_path / "gw"
    gw_dir.mkdir()
    subprocess.run([cpu_driver(), "NFRU_sim=64", "time_end=7", "ic_file_flag=0", "Ndump=3", "seed_scheme=0",
                    "seed_base=77"], cwd=gw_dir, check=True, capture_output=True)
    for f in ("r_states.0.txt", "r_FRU.0.txt"):
        assert filecmp.cmp(ref_dir / f, gw_dir / f, shallow=False), f
    for name, per_line, lo, hi in (("r_LCh", 2, 1, 12), ("r_RyR", 5, 1, 8), ("r_Ito2", 1, 1, 2)):
        for num in (0, 1):
            lines = open(gw_dir / ("%s.%d.txt" % (name, num))).read().splitlines()
            assert int(lines[0]) == 64 and len(lines) == 1 + 64 * 4
            vals = np.array([[int(x) for x in ln.split()] for ln in lines[1:]])
            assert vals.shape == (256, per_line) and vals.min() >= lo and vals.max() <= hi
    assert sorted(os.listdir(gw_dir)) == sorted(
        ["%s.%d.txt" % (n, k) for n in ("states", "otherstates", "currents") for k in (0, 1, 2)] +
        ["%s.%d.txt" % (n, k) for n in ("r_states", "r_FRU", "r_LCh", "r_RyR", "r_Ito2") for k in (0, 1)])


def test_bad_settings_are_rejected(tmp_path):
    r = subprocess.run([cpu_driver(), "no_such_key=3"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode != 0 and "unknown setting" in r.stderr


def _props_files(d):
    return sorted(f for f in os.listdir(d) if f.startswith("fruprops"))


def test_fru_props_files(tmp_path, have_ref):
    """write_fru_props_flag = 1: fruprops_J / fruprops_avg_J / fruprops_avg_tot
    files for FRUs fru_start..fru_end (write_fru_props.c:28-188).  With
    fru_props_compat = 1 (the reference's swapped LType subscripts,
    write_fru_props.c:90-91) every file equals the reference's byte for byte;
    the default writes the cleft's own LCC flux, so there only the LCC flux
    columns may differ, and each of its entries is 0 or the GHK flux of that
    cleft at the step's V and CaSS."""
    import numpy as np
    m = build_ref.cfg_macros(250, 15.0)
    m["write_fru_props_flag"] = 1
    st = {"NFRU_sim": 250, "time_end": 15.0, "ic_file_flag": 0, "seed_scheme": 0, "seed_base": 5489,
          "write_fru_props_flag": 1, "fru_start": 0, "fru_end": 9}
    ref_dir, gw_dir = _run_both(tmp_path, m, dict(st, fru_props_compat=1), 5489)
    files = _props_files(ref_dir)
    assert len(files) == 21 and files == _props_files(gw_dir)
    for f in files:
        assert filecmp.cmp(ref_dir / f, gw_dir / f, shallow=False), f
    fixed = tmp_path / "fixed"
    fixed.mkdir()
    subprocess.run([cpu_driver()] + ["%s=%s" % kv for kv in st.items()], cwd=fixed, check=True, capture_output=True)
    V = np.loadtxt(fixed / "states.0.txt", skiprows=1)[:, 1]
    RT_F, F, Vmyo, Cao = 8.314 * 310.0 / 96.5, 96.5, 25.84e-6, 2.0
    PCa = 1.5 / 2.8 * 0.2 * 0.9 * 0.9468e-11
    nonzero = 0
    for f in files:
        a = np.loadtxt(fixed / f, skiprows=1)
        b = np.loadtxt(ref_dir / f, skiprows=1)
        flux_col = 1
        keep = [k for k in range(a.shape[1]) if k != flux_col]
        assert np.array_equal(a[:, keep], b[:, keep]), f
        if f.startswith("fruprops_") and not f.startswith("fruprops_avg"):
            v = np.repeat(V, 4)
            vf = v / RT_F
            ghk = PCa * 4.0 * (1000.0 * F * vf) * (a[:, 5] * np.exp(2 * vf) - Cao * 0.341) / \
                (np.exp(2 * vf) - 1.0) / (-2.0 * Vmyo * F * 1000.0)
            j = a[:, flux_col]
            on = j != 0.0
            nonzero += int(on.sum())
            assert np.allclose(j[on], ghk[on], rtol=2e-7, atol=0), f
    assert nonzero > 0


def _run_driver(exe, d, settings):
    d.mkdir()
    subprocess.run([exe] + ["%s=%s" % kv for kv in settings.items()], cwd=d, check=True, capture_output=True)


def exact_restart_case(exe, tmp_path):
    """A paced 250-FRU cell over [0, 20) ms with checkpoints every 8 ms, run
    straight through and resumed from its first exact checkpoint: every file
    the resumed run writes equals the straight run's byte for byte."""
    base = {"NFRU_sim": 250, "time_end": 20.0, "ic_file_flag": 0, "seed_scheme": 0, "seed_base": 5489,
            "Ndump": 8, "exact_restart": 1, "write_fru_props_flag": 1, "fru_start": 3, "fru_end": 5}
    full, resumed = tmp_path / "full", tmp_path / "resumed"
    _run_driver(exe, full, base)
    _run_driver(exe, resumed, dict(base, restart_file=str(full / "r_exact.0.bin")))
    written = sorted(os.listdir(resumed))
    assert "states.1.txt" in written and "r_exact.1.bin" in written and "states.0.txt" not in written
    for f in written:
        assert filecmp.cmp(full / f, resumed / f, shallow=False), f
    return written


def test_exact_restart_continues_bit_for_bit(tmp_path):
    exact_restart_case(cpu_driver(), tmp_path)


def test_exact_restart_rejects_wrong_size(tmp_path):
    exe = cpu_driver()
    base = {"NFRU_sim": 64, "time_end": 3.0, "ic_file_flag": 0, "seed_scheme": 0, "Ndump": 2, "exact_restart": 1}
    _run_driver(exe, tmp_path / "a", base)
    r = subprocess.run([exe, "NFRU_sim=128", "time_end=3", "ic_file_flag=0",
                        "restart_file=%s" % (tmp_path / "a" / "r_exact.0.bin")], cwd=tmp_path, capture_output=True,
                       text=True)
    assert r.returncode != 0 and "holds 64 FRUs" in r.stderr


def test_golden_driver_cases_match_their_generator():
    """The driver settings the tests use for tests/golden/drv250* are the ones
    tests/golden/make_driver_files.py made the files with."""
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_driver_files as mdf
    assert sorted(GOLDEN_DRIVER_CASES) == sorted(mdf.CASES)
    for name, (time_end, vclamp) in mdf.CASES.items():
        args = golden_driver_args(name)
        assert args["time_end"] == time_end and args["NFRU_sim"] == mdf.NFRU and args["seed_base"] == mdf.SEED_BASE
        if vclamp:
            assert args["vclamp_flag"] == 1
            for k, v in vclamp.items():
                assert args["vclamp_" + k] == v, k
        else:
            assert "vclamp_flag" not in args

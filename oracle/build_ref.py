"""Build the reference (mwalker174/greenstein2002) serially, to check the GPU path against.

Test infrastructure only: nothing in the product imports or links what this
script builds.

Recipe (the reference ships only an MPI Makefile, Makefile:17-31):
  1. The reference's C sources are copied once, unmodified, into
     oracle/_ref/src/ (git-ignored).  On a machine without the reference
     checkout, that copy is what gets built.
  2. For every configuration a tree oracle/_ref/<name>/ receives the sources,
     a parameters.h whose #define lines are patched (USE_MPI 0 plus the
     configuration's macros: NFRU_sim_*, time_end, ic_file_flag, ...), an empty
     mpi.h (calc_fru_avg_local.c:17 tests `#ifdef USE_MPI`, which stays true)
     and the harness shim oracle/ref_shim.c.
  3. gcc -O3 -ffp-contract=off builds
       stoch     the stock serial program (caf.c main) with the shim's
                 -Wl,--wrap hooks (seeding override, call log, state dumps);
       libref.so the per-FRU routines + fcn for ctypes calls from tests.
     -ffp-contract=off keeps x86-64 and aarch64 builds bit-identical
     (aarch64 gcc would otherwise fuse a*b+c).

initialize_mpi.c and rk_f4am.c are not part of the reference's own Makefile
OBJS (Makefile:1-5) and do not compile; they are left out here too.
"""
import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.environ.get("GW_REFERENCE_DIR", "/root/reference")
OUT = os.path.join(HERE, "_ref")
SRC = os.path.join(OUT, "src")

EXE_SOURCES = [
    "caf.c", "calc_fru_flux_local.c", "data_io.c", "fcn.c", "calc_fru_avg_local.c",
    "fru_rates_local.c", "initialize_ran.c", "initialize_state.c", "simfru_local.c",
    "write_fru_props.c", "mt19937_local.c", "rk_pd54m.c", "fcn_fru.c", "dynamicFRU.c",
    "mpi_slave.c", "mpi_master.c", "parameters_fcn_fru.c",
]
LIB_SOURCES = [
    "simfru_local.c", "fru_rates_local.c", "fcn_fru.c", "mt19937_local.c",
    "parameters_fcn_fru.c", "fcn.c", "calc_fru_flux_local.c", "calc_fru_avg_local.c",
    "initialize_ran.c", "mpi_master.c", "mpi_slave.c", "rk_pd54m.c",
]
WRAPS = ["initialize_ran", "initialize_mpi_state", "distrib_simFRU", "send_calc_fru_flux",
         "send_calc_fru_avg", "send_save_state", "send_resume_state", "end_mpi", "fcn"]
CFLAGS = ["-O3", "-ffp-contract=off", "-fno-strict-aliasing", "-w"]


def _copy(src, dst):
    if os.path.exists(dst):
        os.chmod(dst, 0o644)
    shutil.copyfile(src, dst)
    os.chmod(dst, 0o644)


def have_sources():
    return os.path.isfile(os.path.join(SRC, "simfru_local.c")) or os.path.isdir(REF_DIR)


def sync_sources():
    """Copy the reference sources (unmodified) into oracle/_ref/src once."""
    if os.path.isfile(os.path.join(SRC, "simfru_local.c")):
        return SRC
    if not os.path.isdir(REF_DIR):
        raise FileNotFoundError("reference sources not found (neither %s nor %s)" % (SRC, REF_DIR))
    os.makedirs(SRC, exist_ok=True)
    for fn in os.listdir(REF_DIR):
        if fn.endswith((".c", ".h")):
            _copy(os.path.join(REF_DIR, fn), os.path.join(SRC, fn))
    ic_src = os.path.join(REF_DIR, "ic")
    if os.path.isdir(ic_src) and not os.path.isdir(os.path.join(SRC, "ic")):
        shutil.copytree(ic_src, os.path.join(SRC, "ic"))
    return SRC


def patch_parameters(text, macros):
    """Replace `#define NAME value` lines of parameters.h; every name must exist."""
    macros = dict(macros)
    macros.setdefault("USE_MPI", "0")
    for name, value in macros.items():
        pat = re.compile(r"^(#define\s+%s)\b.*$" % re.escape(name), re.M)
        if not pat.search(text):
            raise KeyError("macro %s not found in parameters.h" % name)
        text = pat.sub(lambda m: "%s %s" % (m.group(1), value), text, count=1)
    return text


def _stamp(macros):
    return repr(sorted((k, str(v)) for k, v in macros.items()))


def build_config(name, macros, lib=True, exe=True, jobs=8):
    """Build oracle/_ref/<name>/{libref.so,stoch}. Returns the directory."""
    sync_sources()
    d = os.path.join(OUT, name)
    stamp = os.path.join(d, ".stamp")
    want = _stamp(macros) + "|" + open(os.path.join(HERE, "ref_shim.c")).read()
    if os.path.isfile(stamp) and open(stamp).read() == want:
        if (not lib or os.path.isfile(os.path.join(d, "libref.so"))) and \
           (not exe or os.path.isfile(os.path.join(d, "stoch"))):
            return d
    os.makedirs(d, exist_ok=True)
    for fn in os.listdir(SRC):
        if fn.endswith((".c", ".h")):
            _copy(os.path.join(SRC, fn), os.path.join(d, fn))
    with open(os.path.join(SRC, "parameters.h")) as f:
        text = f.read()
    with open(os.path.join(d, "parameters.h"), "w") as f:
        f.write(patch_parameters(text, macros))
    open(os.path.join(d, "mpi.h"), "w").close()
    _copy(os.path.join(HERE, "ref_shim.c"), os.path.join(d, "ref_shim.c"))
    cc = os.environ.get("CC", "gcc")
    procs = []
    if lib:
        cmd = [cc] + CFLAGS + ["-fPIC", "-shared", "-DGW_SHIM_LIB", "-I.", "-o", "libref.so"] + \
            LIB_SOURCES + ["ref_shim.c", "-lm"]
        procs.append(subprocess.Popen(cmd, cwd=d))
    if exe:
        wrap = ["-Wl," + ",".join("--wrap=%s" % w for w in WRAPS)]
        cmd = [cc] + CFLAGS + ["-DGW_SHIM_EXE", "-I.", "-o", "stoch"] + EXE_SOURCES + \
            ["ref_shim.c", "-lm"] + wrap
        procs.append(subprocess.Popen(cmd, cwd=d))
    for p in procs:
        if p.wait() != 0:
            raise RuntimeError("reference build failed in %s" % d)
    with open(stamp, "w") as f:
        f.write(want)
    return d


def cfg_macros(nfru, time_end, ic_file=False, period=1000, shift=10, vclamp=None, nfru_max=None):
    """parameters.h macro set for one configuration (all FRUs in one phase)."""
    nmax = nfru_max or max(nfru, 16)
    m = {
        "NFRU_sim_low": nfru, "NFRU_sim_high": nfru,
        "NFRU_scale_low": repr(12500.0 / nfru), "NFRU_scale_high": repr(12500.0 / nfru),
        "NFRU_sim_max": nmax, "MAX_LOCAL_NFRU": nmax,
        "time_end": repr(float(time_end)), "period": period, "shift": shift,
        "ic_file_flag": 1 if ic_file else 0,
    }
    if ic_file:
        m["ic_dir"] = '"%s"' % os.path.join(SRC, "ic", "stable")
    if vclamp:
        m.update({"vclamp_flag": 1, "vclamp_hold": repr(float(vclamp["hold"])),
                  "vclamp_set": repr(float(vclamp["set"])),
                  "vclamp_duration": repr(float(vclamp["duration"])),
                  "vclamp_shift": repr(float(vclamp.get("shift", 300.0))),
                  "vclamp_period": repr(float(vclamp.get("period", 500.0)))})
    return m


def run_stoch(d, workdir, seed_base=None, log=None, dump_init=None, dump_final=None, timeout=None):
    """Run the serial reference in workdir; returns (stdout, wall-seconds printed by caf.c:277)."""
    import resource
    env = dict(os.environ)
    for k, v in (("GW_SEED_BASE", seed_base), ("GW_REF_LOG", log),
                 ("GW_REF_DUMP_INIT", dump_init), ("GW_REF_DUMP_FINAL", dump_final)):
        if v is None:
            env.pop(k, None)
        else:
            env[k] = str(v)

    def _stack():
        resource.setrlimit(resource.RLIMIT_STACK, (resource.RLIM_INFINITY, resource.RLIM_INFINITY))

    os.makedirs(workdir, exist_ok=True)
    r = subprocess.run([os.path.join(d, "stoch")], cwd=workdir, env=env, capture_output=True,
                       text=True, timeout=timeout, preexec_fn=_stack)
    if r.returncode != 0:
        raise RuntimeError("reference run failed (%d): %s" % (r.returncode, r.stderr[-2000:]))
    total = None
    for line in r.stdout.splitlines():
        if line.startswith("Total time:"):
            total = float(line.split(":")[1].strip().rstrip("s"))
    return r.stdout, total


if __name__ == "__main__":
    name = sys.argv[1] if len(sys.argv) > 1 else "lib"
    print(build_config(name, cfg_macros(250, 20.0)))

"""ctypes front end of the CPU oracle (test infrastructure only).

Loads oracle/_build/liboracle.so (the C restatement in fru_oracle.c) and,
where it has been built, oracle/_ref/<config>/libref.so (the reference's own
routines, see build_ref.py).  Used by tests/, the smoke check and the CPU
baseline of bench.py -- never by the product.

FRU sets are dicts of numpy arrays in the reference's packed per-FRU layout:
  ltype (n,4,2) int32   LCC state 1..12, VDI gate 1..2
  ryr   (n,4,5) int32   RyR state 1..8
  ito2  (n,4)   int32   Cl channel 1 closed / 2 open
  frus  (n,5)   float64 CaJSR, CaSS1..4 (mM)
  mti   (n,)    int32   MT19937 position
  mt    (n,624) uint32  MT19937 state words
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_up = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")


def build(force=False):
    """Compile fru_oracle.c into oracle/_build/liboracle.so."""
    src = os.path.join(HERE, "fru_oracle.c")
    if not force and os.path.isfile(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(src):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = os.environ.get("CC", "gcc")
    subprocess.check_call([cc, "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-o", LIB, src, "-lm"])
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        L.orc_sgrnd.argtypes = [C.c_uint32, C.POINTER(C.c_int), _up]
        L.orc_next.argtypes = [C.POINTER(C.c_int), _up]
        L.orc_next.restype = C.c_double
        L.orc_next_word.argtypes = [C.POINTER(C.c_int), _up]
        L.orc_next_word.restype = C.c_uint32
        L.orc_seed_reference.argtypes = [C.c_int]
        L.orc_seed_reference.restype = C.c_uint32
        L.orc_seed_reference_all.argtypes = [C.c_int, _up]
        L.orc_simfru_batch.argtypes = [C.c_int, C.c_double, C.c_double, _dp, _dp, _ip, _ip, _ip, _dp, _ip, _up]
        L.orc_flux_sums.argtypes = [C.c_int, _ip, _ip, _dp, _dp]
        L.orc_avg_sums.argtypes = [C.c_int, _ip, _ip, _ip, _dp, _dp]
        L.orc_currents.argtypes = [C.c_int, C.c_double, _dp, _dp, _dp]
        L.orc_fcn_fru.argtypes = [_dp, _dp, _dp, _ip, _dp]
        L.orc_fru_rates.argtypes = [_ip, _ip, _ip, _dp, _dp, _dp, _ip, _ip, _dp, _dp, _ip, _ip, _dp,
                                    C.POINTER(C.c_int), _up]
        L.orc_fru_rates.restype = C.c_double
        _lib = L
    return _lib


# --------------------------------------------------------------------------
# FRU sets
# --------------------------------------------------------------------------
def empty_set(n):
    return {
        "ltype": np.zeros((n, 4, 2), np.int32), "ryr": np.zeros((n, 4, 5), np.int32),
        "ito2": np.zeros((n, 4), np.int32), "frus": np.zeros((n, 5), np.float64),
        "mti": np.zeros(n, np.int32), "mt": np.zeros((n, 624), np.uint32),
    }


def copy_set(s):
    return {k: v.copy() for k, v in s.items()}


def seeds(n, scheme="base", base=5489):
    """Per-FRU MT19937 seeds: 'base' = base + j (mod 2^32), 'reference' =
    the formula of initialize_ran.c:30-34."""
    if scheme == "reference":
        out = np.zeros(n, np.uint32)
        lib().orc_seed_reference_all(n, out)
        return out
    return ((np.arange(n, dtype=np.uint64) + np.uint64(base)) & np.uint64(0xFFFFFFFF)).astype(np.uint32)


def seed_set(s, seed_values):
    L = lib()
    mti = C.c_int(0)
    for j, sd in enumerate(seed_values):
        row = np.zeros(624, np.uint32)
        L.orc_sgrnd(int(sd), C.byref(mti), row)
        s["mt"][j] = row
        s["mti"][j] = mti.value
    return s


def rest_set(n, scheme="base", base=5489):
    """All FRUs at the reference's default rest state (initialize_state.c:205-219)."""
    s = empty_set(n)
    s["ltype"][:, :, 0] = 1
    s["ltype"][:, :, 1] = 2
    s["ryr"][:] = 1
    s["ito2"][:] = 2
    s["frus"][:, 0] = 0.7
    s["frus"][:, 1:] = 0.12e-3
    return seed_set(s, seeds(n, scheme, base))


def read_dump(path):
    """FRU set from the shim's dump format (see ref_shim.c)."""
    with open(path, "rb") as f:
        n = int(np.frombuffer(f.read(4), np.int32)[0])
        s = {}
        s["frus"] = np.frombuffer(f.read(8 * 5 * n), np.float64).reshape(n, 5).copy()
        s["ltype"] = np.frombuffer(f.read(4 * 8 * n), np.int32).reshape(n, 4, 2).copy()
        s["ryr"] = np.frombuffer(f.read(4 * 20 * n), np.int32).reshape(n, 4, 5).copy()
        s["ito2"] = np.frombuffer(f.read(4 * 4 * n), np.int32).reshape(n, 4).copy()
        s["mti"] = np.frombuffer(f.read(4 * n), np.int32).copy()
        s["mt"] = np.frombuffer(f.read(4 * 624 * n), np.uint32).reshape(n, 624).copy()
    return s


def simfru(s, t0, tf, dep0, depf):
    """Advance every FRU of s over [t0, tf] in place (simfru_local.c:32)."""
    n = s["frus"].shape[0]
    lib().orc_simfru_batch(n, t0, tf, np.ascontiguousarray(dep0, np.float64),
                           np.ascontiguousarray(depf, np.float64), s["ltype"], s["ryr"], s["ito2"],
                           s["frus"], s["mti"], s["mt"])
    return s


def flux_sums(s):
    out = np.zeros(5)
    lib().orc_flux_sums(s["frus"].shape[0], s["ltype"], s["ito2"], s["frus"], out)
    return out


def avg_sums(s):
    out = np.zeros(11)
    lib().orc_avg_sums(s["frus"].shape[0], s["ltype"], s["ryr"], s["ito2"], s["frus"], out)
    return out


def currents(nfru, scale, dep, num):
    out = np.zeros(4)
    lib().orc_currents(nfru, scale, np.ascontiguousarray(dep, np.float64), np.ascontiguousarray(num, np.float64), out)
    return out


def stage(s, t0, tf, dep0, depf, nfru_scale):
    """One distrib_simFRU stage (mpi_master.c:369-469): advance, sum, currents."""
    simfru(s, t0, tf, dep0, depf)
    n = s["frus"].shape[0]
    return currents(n, nfru_scale, depf, flux_sums(s))


def mt_words(seed, count):
    """First `count` raw tempered MT19937 outputs of a Knuth-initialised stream."""
    L = lib()
    mt = np.zeros(624, np.uint32)
    mti = C.c_int(0)
    L.orc_sgrnd(int(seed), C.byref(mti), mt)
    return np.array([L.orc_next_word(C.byref(mti), mt) for _ in range(count)], np.uint32)


# --------------------------------------------------------------------------
# The reference's own routines (oracle/_ref/<cfg>/libref.so), where built
# --------------------------------------------------------------------------
class RefLib:
    def __init__(self, path):
        L = C.CDLL(path)
        L.ref_simfru_batch.argtypes = [C.c_int, C.c_double, C.c_double, _dp, _dp, _ip, _ip, _ip, _dp, _ip, _up]
        L.ref_fru_rates.argtypes = [_ip, _ip, _ip, _dp, _dp, _dp, _ip, _ip, _dp, _dp, _ip, _ip, _dp,
                                    C.POINTER(C.c_int), _up]
        L.ref_fru_rates.restype = C.c_double
        L.ref_fcn_fru.argtypes = [C.c_double, _dp, _dp, _dp, _ip, _dp]
        L.ref_sgrnd.argtypes = [C.c_ulong, C.POINTER(C.c_int), _up]
        L.ref_mt_fast.argtypes = [C.c_int, C.POINTER(C.c_int), _up, _dp]
        L.ref_mt_one.argtypes = [C.POINTER(C.c_int), _up]
        L.ref_mt_one.restype = C.c_double
        L.ref_initialize_ran.argtypes = [C.c_int, _ip, _up]
        L.ref_fcn.argtypes = [C.c_double, _dp, _dp, _dp, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double]
        L.ref_flux_sums.argtypes = [C.c_int, _ip, _ip, _dp, _dp]
        L.ref_avg_sums.argtypes = [C.c_int, _ip, _ip, _ip, _dp, _dp]
        self.L = L

    def simfru(self, s, t0, tf, dep0, depf):
        n = s["frus"].shape[0]
        self.L.ref_simfru_batch(n, t0, tf, np.ascontiguousarray(dep0, np.float64),
                                np.ascontiguousarray(depf, np.float64), s["ltype"], s["ryr"], s["ito2"],
                                s["frus"], s["mti"], s["mt"])
        return s

    def flux_sums(self, s):
        out = np.zeros(5)
        self.L.ref_flux_sums(s["frus"].shape[0], s["ltype"], s["ito2"], s["frus"], out)
        return out

    def avg_sums(self, s):
        out = np.zeros(11)
        self.L.ref_avg_sums(s["frus"].shape[0], s["ltype"], s["ryr"], s["ito2"], s["frus"], out)
        return out


def ref_lib(name="lib", nfru_max=16):
    """Build (if needed) and load the reference routines; None without sources."""
    import sys
    sys.path.insert(0, HERE)
    try:
        import build_ref
    finally:
        sys.path.pop(0)
    if not build_ref.have_sources():
        return None
    d = build_ref.build_config(name, build_ref.cfg_macros(nfru_max, 10.0), lib=True, exe=False)
    return RefLib(os.path.join(d, "libref.so"))

"""GB300-native hot path of the stochastic Greenstein-Winslow myocyte.

Python mirror of the C-ABI in include/gw_fru.h (libgw_fru.so, built in-tree by
greenstein2002_gb300/build.py).  The compute path is the CUDA library; there
is no CPU fallback: every call goes through the shared library and raises if
it is missing or returns an error.

    cell = Cell(nfru=12500)                 # device state of one cell
    state = cell.init_rest(scheme=0, base=5489)
    t, states, other, currents = cell.run(state, t=0.0, n_steps=20)

FRU-level operations mirror the reference's MPI layer (mpi_master.c):
stage() = distrib_simFRU, flux() = send_calc_fru_flux, avg_sums() =
send_calc_fru_avg, save()/resume() = send_save_state/send_resume_state,
upload()/download() = initialize_mpi_state/parallel_get_FRUs.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libgw_fru.so")

NSTATE, NCUR, NOTHER = 37, 24, 12
SEED_BASE, SEED_REFERENCE = 0, 1

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_up = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")


class GWError(RuntimeError):
    pass


class Settings(C.Structure):
    """gw_settings of gw_fru.h: the run settings of the reference's
    parameters.h:92-156 as runtime fields with the same names."""
    _fields_ = [(n, C.c_double) for n in (
        "time_start", "time_end", "time_step", "step_min", "step_max", "tolrk",
        "pulse_duration", "pulse_amplitude", "period", "shift")] + [
        ("vclamp_flag", C.c_int)] + [(n, C.c_double) for n in (
            "vclamp_duration", "vclamp_set", "vclamp_shift", "vclamp_hold", "vclamp_period")] + [
        ("vppclamp_flag", C.c_int)] + [(n, C.c_double) for n in (
            "vppclamp_ppset", "vppclamp_ppduration", "vppclamp_shift", "vppclamp_set", "vppclamp_duration",
            "vppclamp_hold", "vppclamp_period")] + [
        ("iv_flag", C.c_int)] + [(n, C.c_double) for n in (
            "iv_clamp_duration", "iv_clamp_period", "iv_shift", "iv_clamp_set", "iv_clamp_hold",
            "iv_clamp_step")] + [
        ("iv_n", C.c_int), ("chf_flag", C.c_int)] + [(n, C.c_double) for n in (
            "chfsc_IK1", "chfsc_Jup", "chfsc_INaCa", "chfsc_IKv43", "scale_PCa", "scale_GKr")]


class Request(C.Structure):
    """gw_request of gw_fru.h: one cell simulation submitted to a Server."""
    _fields_ = [("nfru", C.c_int), ("set", Settings), ("seed_scheme", C.c_int), ("seed", C.c_uint32),
                ("pca_scale", C.c_double), ("duration_ms", C.c_double), ("v_trace", C.c_void_p),
                ("final_state", C.c_void_p), ("t_submit", C.c_double), ("t_start", C.c_double),
                ("t_done", C.c_double), ("status", C.c_int), ("message", C.c_char * 160)]


_lib = None


def load(build_if_missing=True):
    """Load libgw_fru.so (building it when absent and nvcc is available)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.isfile(LIB_PATH):
        if not build_if_missing:
            raise GWError("libgw_fru.so not built: run greenstein2002_gb300/build.py")
        from . import build as _b
        _b.build()
    _lib = bind(LIB_PATH)
    return _lib


def bind(path):
    """ctypes handle of a library exporting the gw_* native API."""
    L = C.CDLL(path)
    P = C.POINTER
    vp = C.c_void_p
    sig = {
        "gw_last_error": ([], C.c_char_p),
        "gw_create": ([P(vp), C.c_int], C.c_int),
        "gw_destroy": ([vp], C.c_int),
        "gw_nfru": ([vp], C.c_int),
        "gw_set_scale": ([vp, C.c_double], C.c_int),
        "gw_upload": ([vp, _dp, _ip, _ip, _ip, _ip, _up], C.c_int),
        "gw_download": ([vp, _dp, _ip, _ip, _ip, _ip, _up], C.c_int),
        "gw_seed": ([vp, C.c_int, C.c_uint32], C.c_int),
        "gw_stage": ([vp, C.c_double, C.c_double, _dp, _dp, _dp, _dp], C.c_int),
        "gw_flux": ([vp, _dp, _dp, _dp], C.c_int),
        "gw_avg_sums": ([vp, _dp], C.c_int),
        "gw_save": ([vp], C.c_int),
        "gw_resume": ([vp], C.c_int),
        "gw_substeps": ([vp, P(C.c_ulonglong)], C.c_int),
        "gw_sync": ([vp], C.c_int),
        "gw_set_fru_lanes": ([vp, C.c_int], C.c_int),
        "gw_set_stage_warps": ([vp, C.c_int], C.c_int),
        "gw_set_stage_packing": ([vp, C.c_int], C.c_int),
        "gw_stage_trace": ([vp, C.c_int], C.c_int),
        "gw_group_timer": ([C.c_int, vp, C.c_int, P(C.c_float)], C.c_int),
        "gw_stage_trace_read": ([vp, vp, vp], C.c_int),
        "gw_batch_set_warps": ([vp, C.c_int], C.c_int),
        "gw_autotune": ([C.c_int, vp, vp, _dp, _dp, _dp, C.c_double, vp, P(C.c_int), P(C.c_int), _dp], C.c_int),
        "gw_download_range": ([vp, C.c_int, C.c_int, _dp, _ip, _ip, _ip], C.c_int),
        "gw_set_precision": ([vp, C.c_int], C.c_int),
        "gw_set_pca_scale": ([vp, C.c_double], C.c_int),
        "gw_set_sum_order": ([vp, C.c_int], C.c_int),
        "gw_settings_init": ([P(Settings)], None),
        "gw_rk54pd": ([vp, P(Settings), C.c_double, C.c_double, C.c_double, _dp, _dp, P(C.c_double)], C.c_int),
        "gw_lastcall": ([vp, P(Settings), C.c_double, _dp, _dp], C.c_int),
        "gw_run": ([vp, P(Settings), P(C.c_double), _dp, P(C.c_double), C.c_int, vp, vp, vp], C.c_int),
        "gw_init_rest": ([vp, P(Settings), C.c_int, C.c_uint32, _dp], C.c_int),
        "gw_dropin_configure": ([C.c_int, C.c_double], None),
        "gw_batch_create": ([P(vp), C.c_int], C.c_int),
        "gw_batch_destroy": ([vp], C.c_int),
        "gw_batch_add": ([vp, vp], C.c_int),
        "gw_batch_remove": ([vp, vp], C.c_int),
        "gw_batch_profile": ([vp, C.c_int, P(C.c_double), P(C.c_ulonglong)], C.c_int),
        "gw_batch_run": ([vp, C.c_int, vp, vp, vp, vp, vp, C.c_int, vp, vp], C.c_int),
        "gw_cell_bytes": ([C.c_int], C.c_size_t),
        "gw_server_create": ([P(vp), C.c_int, C.c_int, C.c_size_t, C.c_int], C.c_int),
        "gw_run_concurrent": ([C.c_int, vp, vp, vp, vp, vp, C.c_int, vp, vp], C.c_int),
        "gw_run_device": ([C.c_int, vp, vp, vp, vp, vp, C.c_int, vp, vp, vp], C.c_int),
        "gw_run_persistent": ([C.c_int, vp, vp, vp, vp, vp, C.c_int, vp, vp, vp], C.c_int),
        "gw_probe_persist_watchdog": ([vp, P(Settings), C.c_double, P(C.c_int)], C.c_int),
        "gw_server_submit": ([vp, P(Request)], C.c_int),
        "gw_server_reserve": ([vp, C.c_int, C.c_int], C.c_int),
        "gw_server_stats": ([vp, P(C.c_size_t), P(C.c_size_t), P(C.c_ulonglong), P(C.c_ulonglong)], C.c_int),
        "gw_server_wait": ([vp], C.c_int),
        "gw_server_destroy": ([vp], C.c_int),
        "gw_event_record": ([vp, C.c_int], C.c_int),
        "gw_event_elapsed": ([vp, C.c_int, C.c_int, P(C.c_float)], C.c_int),
        "gw_profile": ([vp, C.c_int], C.c_int),
        "gw_profile_read": ([vp, P(C.c_double), P(C.c_ulonglong)], C.c_int),
        "gw_launches": ([vp, P(C.c_ulonglong)], C.c_int),
        "gw_l2_flush": ([vp], C.c_int),
        "gw_probe_fp64_peak": ([P(C.c_double)], C.c_int),
        "gw_probe_fcn": ([P(C.c_double), P(C.c_double)], C.c_int),
        "gw_probe_exp": ([_dp, _dp, _dp, C.c_int], C.c_int),
        "gw_probe_fp64_issue": ([_dp], C.c_int),
        "gw_probe_fcn_warp": ([P(C.c_double)], C.c_int),
        "gw_probe_fcn_compare": ([_dp, C.c_int, C.c_double, C.c_int, _dp, _dp, _dp, _dp], C.c_int),
        "gw_probe_div": ([C.c_ulonglong, C.c_longlong, P(C.c_ulonglong)], C.c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name, None)
        if fn is None:
            continue
        fn.argtypes = args
        fn.restype = res
    return L


def _check(rc, what, L=None):
    if rc:
        msg = (L if L is not None else load()).gw_last_error()
        raise GWError("%s failed (%d): %s" % (what, rc, msg.decode() if msg else ""))


def settings(**kw):
    """Settings with the reference defaults, overridden by keyword."""
    s = Settings()
    load().gw_settings_init(C.byref(s))
    for k, v in kw.items():
        if not hasattr(s, k):
            raise KeyError(k)
        setattr(s, k, v)
    return s


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Cell:
    """Device-resident FRU state of one cell (a gw_ctx)."""

    def __init__(self, nfru, nfru_scale=None, lib=None, fru_lanes=None, precision=None, pca_scale=None,
                 stage_warps=None):
        self._L = L = lib if lib is not None else load()
        self._h = C.c_void_p()
        _check(L.gw_create(C.byref(self._h), int(nfru)), "gw_create", self._L)
        self.nfru = int(nfru)
        if nfru_scale is not None:
            _check(L.gw_set_scale(self._h, float(nfru_scale)), "gw_set_scale", self._L)
        if precision is not None:
            _check(L.gw_set_precision(self._h, 1 if precision in (1, "mixed") else 0), "gw_set_precision", self._L)
        if pca_scale is not None:
            _check(L.gw_set_pca_scale(self._h, float(pca_scale)), "gw_set_pca_scale", self._L)
        if fru_lanes is not None and hasattr(L, "gw_set_fru_lanes"):
            _check(L.gw_set_fru_lanes(self._h, int(fru_lanes)), "gw_set_fru_lanes", self._L)
        if stage_warps is not None:
            self.set_stage_warps(stage_warps)

    def set_stage_warps(self, warps):
        _check(self._L.gw_set_stage_warps(self._h, int(warps)), "gw_set_stage_warps", self._L)

    def stage_trace(self, enable=True):
        _check(self._L.gw_stage_trace(self._h, 1 if enable else 0), "gw_stage_trace", self._L)

    def stage_trace_read(self):
        """(substeps per FRU, per-warp [begin, end] ns) of the last stage launch."""
        sub = np.zeros(self.nfru, np.uint32)
        ns = np.zeros(((self.nfru + 7) // 8, 2), np.uint64)
        _check(self._L.gw_stage_trace_read(self._h, sub.ctypes.data_as(C.c_void_p), ns.ctypes.data_as(C.c_void_p)),
               "gw_stage_trace_read", self._L)
        return sub, ns

    def set_stage_packing(self, warps):
        _check(self._L.gw_set_stage_packing(self._h, int(warps)), "gw_set_stage_packing", self._L)

    def set_sum_order(self, order):
        """"tree" (default: one fixed parallel order for every launch shape) or
        "reference" (the serial reference's FRU-by-FRU order; a parity mode
        for small cells)."""
        if order not in ("tree", "reference"):
            raise ValueError("sum order must be 'tree' or 'reference'")
        _check(self._L.gw_set_sum_order(self._h, 1 if order == "reference" else 0), "gw_set_sum_order", self._L)

    def set_fru_lanes(self, lanes):
        _check(self._L.gw_set_fru_lanes(self._h, int(lanes)), "gw_set_fru_lanes", self._L)

    def close(self):
        if self._h:
            self._L.gw_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- FRU state ----------------------------------------------------------
    def upload(self, s):
        n = self.nfru
        _check(self._L.gw_upload(self._h, np.ascontiguousarray(s["frus"], np.float64).reshape(n * 5),
                                np.ascontiguousarray(s["ltype"], np.int32).reshape(n * 8),
                                np.ascontiguousarray(s["ryr"], np.int32).reshape(n * 20),
                                np.ascontiguousarray(s["ito2"], np.int32).reshape(n * 4),
                                np.ascontiguousarray(s["mti"], np.int32),
                                np.ascontiguousarray(s["mt"], np.uint32).reshape(n * 624)), "gw_upload", self._L)

    def download(self):
        n = self.nfru
        s = {"frus": np.zeros((n, 5)), "ltype": np.zeros((n, 4, 2), np.int32), "ryr": np.zeros((n, 4, 5), np.int32),
             "ito2": np.zeros((n, 4), np.int32), "mti": np.zeros(n, np.int32), "mt": np.zeros((n, 624), np.uint32)}
        _check(self._L.gw_download(self._h, s["frus"].reshape(-1), s["ltype"].reshape(-1), s["ryr"].reshape(-1),
                                  s["ito2"].reshape(-1), s["mti"], s["mt"].reshape(-1)), "gw_download", self._L)
        return s

    def seed(self, scheme=SEED_BASE, base=5489):
        _check(self._L.gw_seed(self._h, int(scheme), int(base) & 0xFFFFFFFF), "gw_seed", self._L)

    # ---- reference MPI-layer operations --------------------------------------
    def stage(self, t0, tf, dep0, depf):
        out, num = np.zeros(4), np.zeros(5)
        _check(self._L.gw_stage(self._h, float(t0), float(tf), np.asarray(dep0, np.float64),
                               np.asarray(depf, np.float64), out, num), "gw_stage", self._L)
        return out, num

    def flux(self, dep):
        out, num = np.zeros(4), np.zeros(5)
        _check(self._L.gw_flux(self._h, np.asarray(dep, np.float64), out, num), "gw_flux", self._L)
        return out, num

    def avg_sums(self):
        num = np.zeros(11)
        _check(self._L.gw_avg_sums(self._h, num), "gw_avg_sums", self._L)
        return num

    def save(self):
        _check(self._L.gw_save(self._h), "gw_save", self._L)

    def resume(self):
        _check(self._L.gw_resume(self._h), "gw_resume", self._L)

    def substeps(self):
        c = C.c_ulonglong(0)
        _check(self._L.gw_substeps(self._h, C.byref(c)), "gw_substeps", self._L)
        return c.value

    def event(self, slot):
        _check(self._L.gw_event_record(self._h, int(slot)), "gw_event_record", self._L)

    def elapsed_ms(self, a, b):
        ms = C.c_float(0.0)
        _check(self._L.gw_event_elapsed(self._h, int(a), int(b), C.byref(ms)), "gw_event_elapsed", self._L)
        return ms.value

    def profile(self, enable=True):
        _check(self._L.gw_profile(self._h, 1 if enable else 0), "gw_profile", self._L)

    def profile_read(self):
        ms, n = C.c_double(0.0), C.c_ulonglong(0)
        _check(self._L.gw_profile_read(self._h, C.byref(ms), C.byref(n)), "gw_profile_read", self._L)
        return ms.value, n.value

    def launches(self):
        n = C.c_ulonglong(0)
        _check(self._L.gw_launches(self._h, C.byref(n)), "gw_launches", self._L)
        return n.value

    def l2_flush(self):
        _check(self._L.gw_l2_flush(self._h), "gw_l2_flush", self._L)

    def sync(self):
        _check(self._L.gw_sync(self._h), "gw_sync", self._L)

    # ---- whole-cell operations -------------------------------------------------
    def init_rest(self, set_=None, scheme=SEED_BASE, base=5489):
        state = np.zeros(NSTATE)
        s = set_ if set_ is not None else settings()
        _check(self._L.gw_init_rest(self._h, C.byref(s), int(scheme), int(base) & 0xFFFFFFFF, state), "gw_init_rest", self._L)
        return state

    def rk54pd(self, state, t, tstep, oldstep, set_=None):
        s = set_ if set_ is not None else settings()
        cur = np.zeros(NCUR)
        nxt = C.c_double(0.0)
        _check(self._L.gw_rk54pd(self._h, C.byref(s), float(t), float(tstep), float(oldstep), state, cur,
                                C.byref(nxt)), "gw_rk54pd", self._L)
        return cur, nxt.value

    def run(self, state, t, n_steps, oldstep=None, set_=None, want=("states", "other", "currents")):
        """Advance n_steps output steps in place; returns (t, states, other, currents)."""
        s = set_ if set_ is not None else settings()
        tt = C.c_double(float(t))
        os_ = C.c_double(float(s.step_max if oldstep is None else oldstep))
        st = np.zeros((n_steps, NSTATE)) if "states" in want else None
        ot = np.zeros((n_steps, NOTHER)) if "other" in want else None
        cu = np.zeros((n_steps, NCUR)) if "currents" in want else None
        _check(self._L.gw_run(self._h, C.byref(s), C.byref(tt), state, C.byref(os_), int(n_steps), _ptr(st), _ptr(ot),
                             _ptr(cu)), "gw_run", self._L)
        self.oldstep = os_.value
        return tt.value, st, ot, cu


def exp_device_and_host(x, lib=None):
    """(device exp, host libm exp) of the float64 array x."""
    L = lib if lib is not None else load()
    x = np.ascontiguousarray(x, np.float64)
    yd, yh = np.zeros_like(x), np.zeros_like(x)
    _check(L.gw_probe_exp(x, yd, yh, len(x)), "gw_probe_exp", L)
    return yd, yh


def fcn_cost_us(lib=None):
    """(device us, host us) per evaluation of the global right-hand side."""
    L = lib if lib is not None else load()
    d, h = C.c_double(0.0), C.c_double(0.0)
    _check(L.gw_probe_fcn(C.byref(d), C.byref(h)), "gw_probe_fcn", L)
    return d.value, h.value


PROBE_ISSUE_CASES = (
    "dependent DFMA, 1 warp, 32 active lanes", "dependent DFMA, 1 warp, 16 active lanes",
    "dependent DFMA, 1 warp, 4 active lanes", "dependent DFMA, 1 warp, 1 active lane",
    "dependent DFMA, 1 warp per SM", "dependent DFMA, 2 warps per SM", "dependent DFMA, 4 warps per SM",
    "dependent DFMA, 8 warps per SM", "8 independent DFMA chains, 1 warp per SM (per DFMA per warp)",
    "8 independent DFMA chains, 4 warps per SM (per DFMA per warp)",
    "8 independent DFMA chains, 16 warps per SM (per DFMA per warp)", "dependent 1/x + c, 32 lanes",
    "dependent 1/x + c, 1 lane", "dependent exp(), 32 lanes", "dependent exp(), 1 lane",
    "dependent FFMA (FP32), 1 warp")


def fp64_issue_cycles(lib=None):
    """{case: cycles per operation} of the FP64 issue-cost chains on one SM
    (gw_probe_fp64_issue, greenstein2002_gb300/csrc/gw_diag.h)."""
    L = lib if lib is not None else load()
    out = np.zeros(len(PROBE_ISSUE_CASES))
    _check(L.gw_probe_fp64_issue(out), "gw_probe_fp64_issue", L)
    return dict(zip(PROBE_ISSUE_CASES, out.tolist()))


def div_mismatches(n, seed=1, lib=None):
    """Quotients of the integer-pipe FP64 division that differ from the
    hardware division's, over n device-drawn operand pairs (gw_probe_div)."""
    L = lib if lib is not None else load()
    m = C.c_ulonglong(0)
    _check(L.gw_probe_div(int(seed), int(n), C.byref(m)), "gw_probe_div", L)
    return m.value


def fcn_warp_us(lib=None):
    """Microseconds per evaluation of the global right-hand side on one warp."""
    L = lib if lib is not None else load()
    v = C.c_double(0.0)
    _check(L.gw_probe_fcn_warp(C.byref(v)), "gw_probe_fcn_warp", L)
    return v.value


def fcn_thread_vs_warp(states, time, clamp=False, lib=None):
    """(F one thread, F warp, currents one thread, currents warp) of the
    global right-hand side for states (n, 37) at `time`."""
    L = lib if lib is not None else load()
    states = np.ascontiguousarray(states, np.float64)
    n = states.shape[0]
    Fs, Fw = np.zeros((n, NSTATE)), np.zeros((n, NSTATE))
    Cs, Cw = np.zeros((n, NCUR)), np.zeros((n, NCUR))
    _check(L.gw_probe_fcn_compare(states.reshape(-1), n, float(time), 1 if clamp else 0, Fs.reshape(-1),
                                  Fw.reshape(-1), Cs.reshape(-1), Cw.reshape(-1)), "gw_probe_fcn_compare", L)
    return Fs, Fw, Cs, Cw


def fp64_peak_tflops():
    """Measured FP64 FMA throughput of the current device (TFLOP/s)."""
    v = C.c_double(0.0)
    _check(load().gw_probe_fp64_peak(C.byref(v)), "gw_probe_fp64_peak")
    return v.value


class Batch:
    """A gw_batch: many cells advanced by one stage launch per round."""

    def __init__(self, precision="fp64", lib=None):
        self._L = lib if lib is not None else load()
        self._h = C.c_void_p()
        _check(self._L.gw_batch_create(C.byref(self._h), 1 if precision in (1, "mixed") else 0), "gw_batch_create",
               self._L)

    def close(self):
        if self._h:
            self._L.gw_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_warps(self, warps):
        _check(self._L.gw_batch_set_warps(self._h, int(warps)), "gw_batch_set_warps", self._L)

    def profile(self, enable=True):
        ms, n = C.c_double(0.0), C.c_ulonglong(0)
        _check(self._L.gw_batch_profile(self._h, 1 if enable else 0, C.byref(ms), C.byref(n)), "gw_batch_profile",
               self._L)
        return ms.value, n.value

    def run(self, cells, sets, t, states, oldsteps, n_steps, traces=False, lockstep=True):
        """Advance every cell n_steps output steps concurrently (one host thread
        per cell); t, states (n, 37) and oldsteps advance in place.  With
        traces=True returns per-step states (n, n_steps, 37) and otherstates
        (n, n_steps, 12)."""
        n = len(cells)
        st_tr = np.zeros((n, n_steps, NSTATE)) if traces else None
        ot_tr = np.zeros((n, n_steps, NOTHER)) if traces else None
        handles = (C.c_void_p * n)(*[c._h.value for c in cells])
        setarr = (Settings * n)(*sets)
        for a in (t, states, oldsteps):
            assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
        args = (C.cast(setarr, C.c_void_p), t.ctypes.data_as(C.c_void_p), states.ctypes.data_as(C.c_void_p),
                oldsteps.ctypes.data_as(C.c_void_p), int(n_steps), _ptr(st_tr), _ptr(ot_tr))
        if lockstep:
            _check(self._L.gw_batch_run(self._h, n, handles, *args), "gw_batch_run", self._L)
        else:
            _check(self._L.gw_run_concurrent(n, handles, *args), "gw_run_concurrent", self._L)
        return (st_tr, ot_tr) if traces else None


class Server:
    """A gw_server: requests run concurrently through one batch (continuous
    batching), admitted by device bytes."""

    def __init__(self, precision="mixed", slots=32, mem_budget_bytes=64 << 30, lockstep=False, lib=None):
        self._L = lib if lib is not None else load()
        self._h = C.c_void_p()
        _check(self._L.gw_server_create(C.byref(self._h), 1 if precision in (1, "mixed") else 0, int(slots),
                                        int(mem_budget_bytes), 1 if lockstep else 0), "gw_server_create", self._L)
        self._keep = []

    def submit(self, req, v_trace=None, final_state=None):
        if v_trace is not None:
            req.v_trace = v_trace.ctypes.data_as(C.c_void_p)
        if final_state is not None:
            req.final_state = final_state.ctypes.data_as(C.c_void_p)
        self._keep.append((req, v_trace, final_state))
        _check(self._L.gw_server_submit(self._h, C.byref(req)), "gw_server_submit", self._L)

    def wait(self):
        _check(self._L.gw_server_wait(self._h), "gw_server_wait", self._L)

    def reserve(self, nfru, count):
        """Pre-create idle contexts so requests of that size allocate nothing while others run."""
        _check(self._L.gw_server_reserve(self._h, int(nfru), int(count)), "gw_server_reserve", self._L)

    def stats(self):
        """{held, peak_held, allocs, frees}: device bytes of contexts held, and allocation counts."""
        h, p, a, f = C.c_size_t(0), C.c_size_t(0), C.c_ulonglong(0), C.c_ulonglong(0)
        _check(self._L.gw_server_stats(self._h, C.byref(h), C.byref(p), C.byref(a), C.byref(f)), "gw_server_stats",
               self._L)
        return {"held": h.value, "peak_held": p.value, "allocs": a.value, "frees": f.value}

    def close(self):
        if self._h:
            self._L.gw_server_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def cell_bytes(nfru):
    return int(load().gw_cell_bytes(int(nfru)))


class GroupTimer:
    """Device time of work the cells run concurrently on their own streams."""

    def __init__(self, cells):
        self._cells = cells
        self._L = cells[0]._L
        self._h = (C.c_void_p * len(cells))(*[c._h.value for c in cells])

    def start(self):
        _check(self._L.gw_group_timer(len(self._cells), C.cast(self._h, C.c_void_p), 0, None), "gw_group_timer",
               self._L)

    def stop(self):
        ms = C.c_float(0.0)
        _check(self._L.gw_group_timer(len(self._cells), C.cast(self._h, C.c_void_p), 1, C.byref(ms)),
               "gw_group_timer", self._L)
        return ms.value


def run_device(cells, sets, t, states, oldsteps, n_steps, traces=False, lib=None, persistent=False):
    """Advance the cells n_steps output steps with the device-resident
    integrator: the graph of lockstep rounds (gw_run_device) or, with
    persistent=True, the persistent multi-cell kernel (gw_run_persistent);
    t, states (n, 37) and oldsteps advance in place.  With traces=True
    returns (states (n, n_steps, 37), otherstates (n, n_steps, 12),
    currents (n, n_steps, 24))."""
    L = lib if lib is not None else cells[0]._L
    n = len(cells)
    for a in (t, states, oldsteps):
        assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    handles = (C.c_void_p * n)(*[c._h.value for c in cells])
    setarr = (Settings * n)(*sets)
    st_tr = np.zeros((n, n_steps, NSTATE)) if traces else None
    ot_tr = np.zeros((n, n_steps, NOTHER)) if traces else None
    cu_tr = np.zeros((n, n_steps, NCUR)) if traces else None
    fn, name = (L.gw_run_persistent, "gw_run_persistent") if persistent else (L.gw_run_device, "gw_run_device")
    _check(fn(n, C.cast(handles, C.c_void_p), C.cast(setarr, C.c_void_p), t.ctypes.data_as(C.c_void_p),
              states.ctypes.data_as(C.c_void_p), oldsteps.ctypes.data_as(C.c_void_p), int(n_steps),
              _ptr(st_tr), _ptr(ot_tr), _ptr(cu_tr)), name, L)
    return (st_tr, ot_tr, cu_tr) if traces else None


def run_persistent(cells, sets, t, states, oldsteps, n_steps, traces=False, lib=None):
    """run_device with the persistent multi-cell kernel (gw_run_persistent)."""
    return run_device(cells, sets, t, states, oldsteps, n_steps, traces=traces, lib=lib, persistent=True)


def persist_watchdog(cell, set_, wait_s):
    """Status of a persistent launch whose cell's next operation is held by a
    flag that nothing sets (gw_probe_persist_watchdog): 3 when every warp gave
    up after wait_s seconds without progress and the launch returned."""
    st = C.c_int(-1)
    _check(cell._L.gw_probe_persist_watchdog(cell._h, C.byref(set_), float(wait_s), C.byref(st)),
           "gw_probe_persist_watchdog", cell._L)
    return st.value


# (lanes per FRU, warps per block), or (4, -2) / (4, -4) / (4, -8): packed
# launches with a half / a quarter / an eighth as many warps as 8-FRU groups
TUNE_CANDIDATES = ((4, 1), (4, 2), (4, 4), (4, 8), (1, 1), (4, -2), (4, -4), (4, -8))


def autotune(cells, sets, t, states, oldsteps, window_ms, batch=None, lib=None):
    """Launch-shape autotuner (gw_autotune): times window_ms of the cells' own
    workload per (lanes per FRU, warps per block) candidate, restores their
    state and sets the fastest.  Returns (lanes, warps, {candidate: ms})."""
    L = lib if lib is not None else cells[0]._L
    n = len(cells)
    handles = (C.c_void_p * n)(*[c._h.value for c in cells])
    setarr = (Settings * n)(*sets)
    t = np.ascontiguousarray(t, dtype=np.float64)
    states = np.ascontiguousarray(states, dtype=np.float64).reshape(n, NSTATE)
    oldsteps = np.ascontiguousarray(oldsteps, dtype=np.float64)
    ms = np.zeros(len(TUNE_CANDIDATES))
    lanes, warps = C.c_int(0), C.c_int(0)
    _check(L.gw_autotune(n, C.cast(handles, C.c_void_p), C.cast(setarr, C.c_void_p), t, states, oldsteps,
                         float(window_ms), batch._h if batch is not None else None, C.byref(lanes), C.byref(warps),
                         ms), "gw_autotune", L)
    return lanes.value, warps.value, {c: float(m) for c, m in zip(TUNE_CANDIDATES, ms) if m >= 0.0}

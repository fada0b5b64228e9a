"""Benchmark: cell-ms simulated per second at 12,500 FRUs per cell.

Workload (the full-size plain FP64 configuration: one cell of NFRU=12,500
release units per seed, rest initial state (initialize_state.c:164-219), 1 Hz
pacing with a 1 ms -100 uA/uF stimulus at 10 ms, 64 seeds for ensemble
statistics): `value` is the throughput of an ensemble of --seeds cells (cell
k's FRU j seeded 5489 + 100000 k + j) running on the GPU at once, one stream
and one host integrator thread per cell -- the same kind of throughput the
reference arm measures with one cell per host core, and the same number of
cells (16) as that arm runs on the host's 16 cores.  A step advances every
cell by STEP_MS (10 ms) of simulated time through the whole hot path
(Dormand-Prince global step, every FRU stage on the GPU).

The timed window is pinned: every section first advances its cells from
rest through the stimulus and upstroke to 30 ms (untimed set-up), keeps
their complete state on the host, runs the W warm-up steps, puts the state
back and tunes the launch shape, so the K timed steps always cover [30,
30 + 10 K) ms -- [30, 230) ms by default, the plateau and early
repolarisation of the first beat -- whatever W is.  L2 (129 MB) is flushed by
a 512 MB write between timed steps.  Each step is timed on the device
(events on a timing stream joined to every cell's stream).

Beside it the line carries the same ensemble in mixed precision over the
same window ("mixed_ensemble", with its speed-up and its paired error against
the FP64 ensemble: peak Cai with a 95% interval, ensemble-mean V, JSR
depletion, open probabilities), one cell alone ("one_cell", "mixed"), a
batched run ("batched": 64 cells of NFRU 1250-12,500 with varied pacing and
conductances, mixed precision) and a serving sweep ("serving": Poisson
arrivals of cell requests, p50/p99 latency; with --serve-baseline also the
same request list in FP64 one request at a time, its like-for-like
denominator).  Before each timed section the
launch-shape autotuner picks lanes per FRU and warps per block on the
section's own workload ("tuning"; results do not depend on the choice), and
`roofline.kernel` names the stage kernel it picked.

value: inputs resident in HBM.  e2e: the ensemble's window again through the
C-ABI with host buffers, on the same cells put back to 30 ms: every step
uploads each cell's full FRU + RNG state from host memory (gw_upload) and
downloads it and the step's traces (gw_download) inside the timed region.

--impl reference: the reference's own serial program (oracle/_ref, built
from its sources) on the host cores, one independent 12,500-FRU cell per
core; timed step s runs every core for 3 simulated ms from the bench cell's
state at phase s mod 10 of the same window (30, 50, ..., 210 ms;
tests/golden/ic_window), so K = 20 steps sample each phase twice.
cpu_baseline: the same program on one core, 1 ms from each of those phases.
"""
import argparse
import json
import os
import shutil
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NFRU = 12500
STEP_MS = 10.0
SEED = 5489
# The timed window starts here whatever --warmup is: every section first
# advances its cells from rest through the stimulus (10 ms) and the upstroke
# (untimed set-up), keeps their state, runs the warm-up steps, and puts the
# state back before the timed steps, so the GPU arm and the reference arm's
# phase samples cover the same simulated window, [30, 30 + 10 K) ms.
WINDOW_START_MS = 30.0
# simulated ms per reference cell per timed step (the process start-up,
# ~0.06 s, is then under 1% of a sample; 16 Arm cores run a 20-step sample of
# the window in about 3 minutes)
REF_SAMPLE_MS = 3.0
# two-sided 95% quantile of Student's t for n - 1 degrees of freedom
T975 = {1: 12.706, 2: 4.303, 3: 3.182, 4: 2.776, 5: 2.571, 6: 2.447, 7: 2.365, 8: 2.306, 9: 2.262, 10: 2.228,
        11: 2.201, 12: 2.179, 13: 2.160, 14: 2.145, 15: 2.131, 16: 2.120, 17: 2.110, 18: 2.101, 19: 2.093,
        20: 2.086, 24: 2.064, 30: 2.042, 40: 2.021, 63: 1.998, 127: 1.979, 255: 1.969}
# DRAM bytes per stage launch of a 12,500-FRU cell, by kernel, from ncu's
# dram__bytes_read + dram__bytes_write (profiles/): the fixed-layout FP64
# kernel's 2,500-FRU plateau launch (6.67 MB, cold L2 per replay) times 5
# (the bytes are per FRU: its state and MT row).
TRAFFIC_PER_LAUNCH = {
    "fru_stage4_kernel": (5 * 6.672128e6, "ncu dram bytes of one 2,500-FRU plateau launch x 5 (cold L2 per replay; "
                                          "profiles/fru_stage4_kernel_plateau_2500fru.md)"),
    "fru_stage4_packed_kernel": (4.18e7, "ncu dram bytes of two stage launches of a 50,000-FRU cell at 30 ms with the "
                                         "SMs full, mean, / 4 (the bytes are per FRU: its state and MT row; "
                                         "profiles/fru_stage4_packed_kernel_saturated_50000fru_32perwarp.md)"),
}
# algorithmic work per FRU-substep (static count of the reference's substep:
# fru_rates_local + 2 x fcn_fru + simfru_local body, each add/mul/div/exp/
# compare/convert counted once) and MT19937 bytes streamed per substep
FLOPS_PER_SUBSTEP = 700.0
BYTES_PER_SUBSTEP = 384.0
# GB300 FP32 (non-tensor) peak, nominal: 152 SMs x 128 FP32 lanes x 2 FLOP x 2.07 GHz
FP32_NOMINAL_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12


def mixed_roofline(substeps_per_s, hbm_peak_gbs):
    """The two candidate bounds of the mixed-precision path: its FP32 work
    (700 FLOP per FRU-substep against the nominal FP32 peak) and its bytes
    (384 B per FRU-substep against the measured copy bandwidth).  The larger
    fraction is the binding one."""
    tf = FLOPS_PER_SUBSTEP * substeps_per_s / 1e12
    gbs = BYTES_PER_SUBSTEP * substeps_per_s / 1e9
    f32 = {"achieved": tf, "peak": FP32_NOMINAL_TFLOPS, "unit": "TFLOP/s", "frac": tf / FP32_NOMINAL_TFLOPS,
           "peak_source": "nominal (152 SMs x 128 FP32 lanes x 2 FLOP x 2.07 GHz)"}
    hbm = {"achieved": gbs, "peak": hbm_peak_gbs, "unit": "GB/s", "frac": gbs / hbm_peak_gbs,
           "peak_source": "measured copy bandwidth"}
    return {"fp32": f32, "hbm": hbm, "binding": "fp32" if f32["frac"] >= hbm["frac"] else "hbm",
            "algorithmic": "700 FLOP and 384 B per FRU-substep"}



def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gw", choices=["gw", "reference"])
    ap.add_argument("--nfru", type=int, default=NFRU)
    ap.add_argument("--seeds", type=int, default=16,
                    help="cells of the FP64 ensemble (seeds k: FRU j seeded 5489 + 100000 k + j) run at once")
    ap.add_argument("--step-ms", type=float, default=STEP_MS)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--batch-cells", type=int, default=64)
    ap.add_argument("--batch-ms", type=int, default=20)
    ap.add_argument("--batch-warmup-ms", type=int, default=10)
    ap.add_argument("--batch-mode", default="streams", choices=["streams", "lockstep"],
                    help="streams: each cell on its own stream; lockstep: shared batched launches")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-devdp", action="store_true", help="skip the device-integrator batched runs")
    ap.add_argument("--runner", default="streams", choices=["streams", "persistent"],
                    help="ensemble runner: per-cell host integrators on CUDA streams, or the persistent multi-cell "
                         "kernel (integrators on the device)")
    ap.add_argument("--precision-ensemble", type=int, nargs=2, metavar=("SEEDS", "MS"), default=None,
                    help="only run the mixed-vs-FP64 ensemble check: SEEDS 12,500-FRU cells per precision "
                         "over [0, MS) ms, APD90 / peak Cai / JSR depletion / open probabilities")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shape")
    ap.add_argument("--full-cell", action="store_true",
                    help="also run the full-size cell's whole protocol through the C host driver: 5 beats at 1 Hz "
                         "and the -100 -> 0 mV, 200-ms clamp, FP64 and mixed precision")
    ap.add_argument("--only-ensemble", action="store_true",
                    help="run the headline ensemble section alone (for launch lists: its timed launches are the run's "
                         "last `gpu_launches` launches)")
    ap.add_argument("--packed", type=int, default=0,
                    help="force packed launches with 1/N as many warps as 8-FRU groups (no autotuning)")
    ap.add_argument("--tune-ms", type=float, default=2.0, help="simulated window per autotuner candidate")
    ap.add_argument("--serve-rates", type=float, nargs="+", default=[50.0],
                    help="Poisson arrival rates (req/s) of the serving sweep")
    ap.add_argument("--serve-requests", type=int, default=16,
                    help="requests per rate (at most rate x 24 s of arrivals, at least 16)")
    ap.add_argument("--serve-baseline", action="store_true",
                    help="also run the serving section's request list in FP64 one request at a time (the "
                         "like-for-like denominator of the serving throughput)")
    ap.add_argument("--serve-ms", type=float, default=1000.0,
                    help="cap on each request's simulated ms: the default 1000 keeps the clamp run whole and the "
                         "first second of a paced one; 0 runs every request's whole protocol (1-10 beats, minutes)")
    ap.add_argument("--serve-slots", type=int, default=32)
    ap.add_argument("--serve-budget-gb", type=float, default=64.0)
    ap.add_argument("--fru-lanes", type=int, default=4, choices=[1, 4],
                    help="lanes per FRU of the FP64 stage kernel (4: one per cleft, 1: one thread per FRU)")
    return ap.parse_args()


# ---------------------------------------------------------------------------
# distributed plumbing (replicas only: one independent cell per GPU)
# ---------------------------------------------------------------------------
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x):
        if not self.pg:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x):
        if not self.pg:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.SUM)
        return float(t.item())


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self, gpu):
        self.gpu = gpu
        self.rows = []
        self.proc = None

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm = [float(r[0]) for r in self.rows if r and r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if len(r) > 1 and r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4)
                          if len(r) > 3 + i and r[3 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


# ---------------------------------------------------------------------------
# reference (CPU) side
# ---------------------------------------------------------------------------
WINDOW_IC = os.path.join(ROOT, "tests", "golden", "ic_window")


def reference_build(ms, window_ic=False):
    """The reference program built from its own sources for a 12,500-FRU cell
    running `ms` simulated ms; window_ic = True starts it from the IC files in
    ./ic (a phase of the GPU arm's timed window) instead of the rest state."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import build_ref
    if not build_ref.have_sources():
        return None, "reference sources not present (oracle/_ref/src missing)"
    try:
        m = build_ref.cfg_macros(NFRU, ms)
        name = "bench12500_%gms" % ms
        if window_ic:
            m.update({"ic_file_flag": 1, "ic_dir": '"ic"'})
            name += "_ic"
        return build_ref.build_config(name, m, lib=False, exe=True), None
    except Exception as e:  # noqa: BLE001
        return None, "reference build failed: %s" % str(e).splitlines()[0]


def window_phases(args=None):
    """IC directories of the bench cell's state at phases of the timed window
    (tests/golden/ic_window/t<ms>), sorted by time; with args, only those
    inside [WINDOW_START_MS, WINDOW_START_MS + steps * step_ms)."""
    if not os.path.isdir(WINDOW_IC):
        return []
    ds = sorted(os.listdir(WINDOW_IC), key=lambda d: float(d[1:]))
    if args is not None:
        lo, hi = window_ms(args)
        ds = [d for d in ds if lo <= float(d[1:]) < hi]
    return [os.path.join(WINDOW_IC, d) for d in ds]


def window_ms(args):
    """The timed window: it starts at WINDOW_START_MS whatever --warmup is."""
    return WINDOW_START_MS, WINDOW_START_MS + args.steps * args.step_ms


def window_str(args):
    return "[%g, %g) ms" % window_ms(args)


def reference_sample(d, procs, ms, seed0, phases=None):
    """Run `procs` independent reference cells concurrently for `ms` simulated
    ms each, cell p starting from IC phase p mod len(phases) when given;
    returns (cell-ms/s, wall s)."""
    phases = [p for p in (phases or []) if p]
    import resource
    import tempfile

    def _stack():
        resource.setrlimit(resource.RLIMIT_STACK, (resource.RLIM_INFINITY, resource.RLIM_INFINITY))

    with tempfile.TemporaryDirectory() as tmp:
        ps = []
        for p in range(procs):
            wd = os.path.join(tmp, str(p))
            os.makedirs(wd)
            if phases:
                shutil.copytree(phases[p % len(phases)], os.path.join(wd, "ic"))
        t0 = time.perf_counter()
        for p in range(procs):
            wd = os.path.join(tmp, str(p))
            env = dict(os.environ, GW_SEED_BASE=str(seed0 + p * NFRU))
            ps.append(subprocess.Popen([os.path.join(d, "stoch")], cwd=wd, env=env, stdout=subprocess.DEVNULL,
                                       stderr=subprocess.PIPE, preexec_fn=_stack))
        for p in ps:
            _, err = p.communicate()
            if p.returncode != 0:
                raise RuntimeError("reference run failed: %s" % err.decode()[-300:])
        wall = time.perf_counter() - t0
    return procs * ms / wall, wall


def run_reference(args, dist):
    """The reference program on all host cores, one independent 12,500-FRU cell
    per core.  Timed step s runs every core from the bench cell's state at
    phase s mod P of the GPU arm's timed window (P phases 20 ms apart,
    tests/golden/ic_window) for REF_SAMPLE_MS simulated ms, each core with
    its own seeds; over K = 20 steps every phase of [30, 230) ms is sampled
    twice.  All cores of a step start from the same phase, so none idles
    behind a costlier one.  Warm-up steps (nothing to warm on the host) are
    1-ms samples of the first phase."""
    if dist.rank != 0:
        return
    phases = window_phases(args)
    d, why = reference_build(REF_SAMPLE_MS, window_ic=bool(phases))
    d1, why1 = reference_build(1.0, window_ic=bool(phases))
    if d is None or d1 is None:
        print(json.dumps({"impl": "reference", "unavailable": why or why1}))
        return
    procs = os.cpu_count() or 1
    for _ in range(args.warmup):
        reference_sample(d1, procs, 1.0, SEED, phases[:1])
    wall = 0.0
    visits = {}
    for k in range(args.steps):
        ph = phases[k % len(phases)] if phases else None
        wall += reference_sample(d, procs, REF_SAMPLE_MS, SEED + 1000003 * k, [ph])[1]
        if ph:
            visits[os.path.basename(ph)[1:]] = visits.get(os.path.basename(ph)[1:], 0) + 1
    value = args.steps * procs * REF_SAMPLE_MS / wall
    start = ("from the bench cell's state at %s ms (IC files; the reference reads 1250 FRUs and replicates them to "
             "12,500), visits per phase %s" % ("/".join(os.path.basename(p)[1:] for p in phases),
                                                json.dumps(visits, sort_keys=True))) if phases else "from rest"
    sample = ("reference program (caf.c, serial build of its own sources, gcc -O3) x%d concurrent cells, "
              "NFRU=12,500 each, %g ms per cell per step, %s" % (procs, REF_SAMPLE_MS, start))
    print(json.dumps({
        "impl": "reference", "metric": "cell-ms simulated/s at 12,500 FRUs", "value": value,
        "unit": "cell-ms/s", "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * wall / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "one 12,500-FRU cell per host core, 1 Hz pacing, %g-ms samples of the phases of the "
                               "timed window %s (the window the GPU arm times)" % (REF_SAMPLE_MS, window_str(args)),
                   "window": window_str(args), "nfru": NFRU, "cells": procs, "ms_per_cell_per_step": REF_SAMPLE_MS,
                   "phases_ms": [float(os.path.basename(p)[1:]) for p in phases]},
        "cpu_baseline": {"value": value, "unit": "cell-ms/s", "cores": procs, "kind": "reference",
                         "sample": sample},
        "e2e": {"value": value, "unit": "cell-ms/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


# ---------------------------------------------------------------------------
# GPU side
# ---------------------------------------------------------------------------
def fresh_cell(G, nfru, seed, lanes=4, precision="fp64"):
    cell = G.Cell(nfru, fru_lanes=lanes, precision=precision)
    st = G.settings()
    state = cell.init_rest(st, scheme=G.SEED_BASE, base=seed)
    return cell, st, state


def load_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return {}


def _shape_name(k):
    lanes, warps = k
    return "packed_%d_fru_per_warp" % (8 * -warps) if warps < 0 else "%d_lanes_%d_warps" % (lanes, warps)


def tune_summary(res, args):
    lanes, warps, ms = res
    packed = warps < 0
    return {"lanes_per_fru": lanes, "fru_per_warp": 8 * -warps if packed else 32 // lanes,
            "warps_per_block": 1 if packed else warps, "packed_div": -warps if packed else 0,
            "window_ms": args.tune_ms,
            "candidates_ms": {_shape_name(k): round(v, 2) for k, v in sorted(ms.items())}}


def choose_shape(G, args, cells, sets, t, states, old):
    """The launch shape of a timed section: forced packed (--packed N), the
    default (--no-autotune), or the autotuner's choice on the section's own
    workload."""
    import numpy as np
    if args.packed:
        tuning = {"lanes_per_fru": 4, "fru_per_warp": 8 * args.packed, "warps_per_block": 1,
                  "packed_div": args.packed, "forced": True}
        for c in cells:
            apply_tuning(c, tuning)
        return tuning
    if args.no_autotune or args.fru_lanes != 4:
        return None
    return tune_summary(G.autotune(cells, sets, np.ascontiguousarray(t, dtype=np.float64),
                                   np.ascontiguousarray(states), np.ascontiguousarray(old, dtype=np.float64),
                                   args.tune_ms), args)


def apply_tuning(cell, tuning):
    """Give another cell the shape the autotuner chose (results never depend on it)."""
    cell.set_fru_lanes(tuning["lanes_per_fru"])
    cell.set_stage_warps(tuning["warps_per_block"])
    div = tuning.get("packed_div", 0)
    cell.set_stage_packing(((cell.nfru + 7) // 8 + div - 1) // div if div else 0)


def snapshot(cells, t, states, old):
    """Host copy of the cells' complete state (FRU Ca, channels, MT19937 rows
    and positions) and of their global states, clocks and step sizes."""
    return [c.download() for c in cells], t.copy(), states.copy(), old.copy()


def restore(cells, snap, t, states, old):
    for c, h in zip(cells, snap[0]):
        c.upload(h)
    t[:] = snap[1]
    states[:] = snap[2]
    old[:] = snap[3]


def time_single(G, args, dist, precision, seed, keep_trace=False, clocks=None):
    """One cell alone: set-up to the window start, warm-up steps, state put
    back, launch shape tuned, then K timed steps with CUDA events on the
    library's stream.  Returns the measurements."""
    import numpy as np
    cell, st, state = fresh_cell(G, args.nfru, seed, args.fru_lanes, precision)
    n = int(args.step_ms)
    t, _, _, _ = cell.run(state, 0.0, int(WINDOW_START_MS), st.step_max, st, want=())
    t = np.array([t])
    states = state[None, :]
    old = np.array([cell.oldstep])
    snap = snapshot([cell], t, states, old)
    for _ in range(args.warmup):
        t[0], _, _, _ = cell.run(states[0], t[0], n, old[0], st, want=())
        old[0] = cell.oldstep
    restore([cell], snap, t, states, old)
    # launch shape picked on this cell's own workload (same results either way)
    tuning = choose_shape(G, args, [cell], [st], t, states.copy(), old)
    sub0, launch0 = cell.substeps(), cell.launches()
    cell.profile(True)
    total_ms = 0.0
    trace = []
    dist.barrier()
    cell.sync()
    if clocks:
        clocks.start()
    for _ in range(args.steps):
        cell.l2_flush()
        cell.event(0)
        t[0], tr, _, _ = cell.run(states[0], t[0], n, old[0], st, want=("states",) if keep_trace else ())
        old[0] = cell.oldstep
        cell.event(1)
        total_ms += cell.elapsed_ms(0, 1)
        if keep_trace:
            trace.append(tr)
    cell.sync()
    clk = clocks.stop() if clocks else None
    dist.barrier()
    kern_ms, kern_launches = cell.profile_read()
    out = {"wall_ms": dist.max(total_ms), "substeps": cell.substeps() - sub0, "launches": cell.launches() - launch0,
           "kern_ms": kern_ms, "kern_launches": kern_launches, "clocks": clk, "tuning": tuning,
           "trace": np.concatenate(trace) if keep_trace else None}
    out["value"] = dist.sum(args.steps * args.step_ms) / (out["wall_ms"] / 1000.0)
    cell.close()
    return out


def ensemble(G, args, dist, precision):
    """args.seeds independent cells of args.nfru FRUs, rest state, 1 Hz pacing;
    cell k's FRU j is seeded 5489 + 100000 (k + seeds * rank) + j."""
    import numpy as np
    cells, sets, states = [], [], []
    for k in range(args.seeds):
        c = G.Cell(args.nfru, fru_lanes=args.fru_lanes, precision=precision)
        st = G.settings()
        states.append(c.init_rest(st, scheme=G.SEED_BASE, base=SEED + 100000 * (k + args.seeds * dist.rank)))
        cells.append(c)
        sets.append(st)
    return cells, sets, np.ascontiguousarray(np.array(states))


def time_ensemble(G, args, dist, precision, clocks=None, traces=False, e2e=False):
    """The ensemble on the GPU at once (one stream and host driver thread per
    cell): set-up from rest to the window start, W warm-up steps, the state
    put back, the launch-shape autotuner, then K timed steps, each timed on
    the device from before the first cell's first launch to after the last
    cell's last one (gw_group_timer), L2 flushed between steps.  traces:
    also return each cell's per-ms global states and output averages from 0
    ms to the window's end.  e2e: then the same window again through the
    C-ABI with host buffers (time_e2e_steps)."""
    import numpy as np
    cells, sets, states = ensemble(G, args, dist, precision)
    n = len(cells)
    t = np.zeros(n)
    old = np.full(n, 0.1)
    persistent = args.runner == "persistent"
    runner = G.Batch(precision)

    def advance(ms, want):
        if persistent:
            r = G.run_persistent(cells, sets, t, states, old, ms, traces=want)
            return r[:2] if want else None
        return runner.run(cells, sets, t, states, old, ms, traces=want, lockstep=False)

    step = int(args.step_ms)
    tr = advance(int(WINDOW_START_MS), traces)
    st_parts, ot_parts = ([tr[0]], [tr[1]]) if traces else ([], [])
    snap = snapshot(cells, t, states, old)
    for _ in range(args.warmup):
        advance(step, False)
    restore(cells, snap, t, states, old)
    tuning = None if persistent else choose_shape(G, args, cells, sets, t, states, old)
    sub0 = sum(c.substeps() for c in cells)
    launch0 = sum(c.launches() for c in cells)
    timer = G.GroupTimer(cells)
    total_ms = 0.0
    dist.barrier()
    for c in cells:
        c.sync()
    if clocks:
        clocks.start()
    for _ in range(args.steps):
        cells[0].l2_flush()
        if persistent:  # synchronous: one graph launch per step on the library's own stream
            t0 = time.perf_counter()
            tr = advance(step, traces)
            total_ms += (time.perf_counter() - t0) * 1e3
        else:
            timer.start()
            tr = advance(step, traces)
            total_ms += timer.stop()
        if traces:
            st_parts.append(tr[0])
            ot_parts.append(tr[1])
    clk = clocks.stop() if clocks else None
    dist.barrier()
    out = {"device_ms": dist.max(total_ms), "substeps": sum(c.substeps() for c in cells) - sub0,
           "launches": sum(c.launches() for c in cells) - launch0, "clocks": clk, "tuning": tuning, "cells": n,
           "window": window_str(args), "runner": args.runner}
    out["value"] = dist.sum(n * args.steps * args.step_ms) / (out["device_ms"] / 1000.0)
    if traces:
        out["state_trace"] = np.concatenate(st_parts, axis=1)
        out["other_trace"] = np.concatenate(ot_parts, axis=1)
    if e2e:
        out["e2e"] = time_e2e_steps(args, dist, cells, sets, advance, snap, t, states, old)
    for c in cells:
        c.close()
    runner.close()
    return out


def time_e2e_steps(args, dist, cells, sets, advance, snap, t, states, old):
    """The ensemble's timed window through the C-ABI with host buffers, on the
    same (warm) cells put back to the window start: every step uploads each
    cell's full FRU + RNG state and global state from host memory, runs the
    step, and downloads them and the step's traces."""
    import numpy as np
    restore(cells, snap, t, states, old)
    host = [dict(h) for h in snap[0]]
    h2d = sum(v.nbytes for h in host for v in h.values()) + states.nbytes
    n = len(cells)
    step = int(args.step_ms)
    dist.barrier()
    e2e_s, d2h = 0.0, 0
    for _ in range(args.steps):
        cells[0].l2_flush()
        t0 = time.perf_counter()
        for c, h in zip(cells, host):
            c.upload(h)
        st_tr, ot_tr = advance(step, True)
        host = [c.download() for c in cells]
        e2e_s += time.perf_counter() - t0
        d2h = sum(v.nbytes for h in host for v in h.values()) + st_tr.nbytes + ot_tr.nbytes
    dist.barrier()
    return {"value": dist.sum(n * args.steps * args.step_ms) / dist.max(e2e_s), "unit": "cell-ms/s",
            "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h), "window": window_str(args)}


def paired_ci(a, b):
    """Mean of the paired differences b - a relative to mean(a), with its 95%
    interval (Student's t, n - 1 degrees of freedom)."""
    import numpy as np
    d = np.asarray(b, float) - np.asarray(a, float)
    n = len(d)
    ref = float(np.mean(a))
    m = float(d.mean()) / ref
    if n < 2:
        return {"rel_mean_diff": m, "ci95": None, "n": n}
    tq = T975.get(n - 1) or T975[max(k for k in T975 if k <= n - 1)]
    h = tq * float(d.std(ddof=1)) / np.sqrt(n) / abs(ref)
    return {"rel_mean_diff": m, "ci95": [m - h, m + h], "n": n, "within_1pct": bool(abs(m) + h < 0.01)}


def precision_vs_fp64(f, m):
    """Mixed precision against the FP64 run of the same seeds over [0, window
    end): per-seed peak Cai (paired, 95% interval), ensemble-mean V, JSR
    depletion and the LCC / RyR open-probability traces."""
    import numpy as np
    fs, ms_ = f["state_trace"], m["state_trace"]
    fo, mo = f["other_trace"], m["other_trace"]
    pk_f, pk_m = fs[:, :, 6].max(1), ms_[:, :, 6].max(1)
    return {"seeds": int(fs.shape[0]), "window_ms": [0, int(fs.shape[1])],
            "peak_cai": dict(paired_ci(pk_f, pk_m), fp64_mean_mM=float(pk_f.mean()), mixed_mean_mM=float(pk_m.mean())),
            "max_abs_d_ensemble_mean_V_mV": float(np.max(np.abs(ms_[:, :, 0].mean(0) - fs[:, :, 0].mean(0)))),
            "jsr_depletion_rel_diff": float(mo[:, :, 1].mean(0).min() / fo[:, :, 1].mean(0).min() - 1.0),
            "max_abs_d_p_lcc_open": float(np.max(np.abs(mo[:, :, 7].mean(0) - fo[:, :, 7].mean(0)))),
            "max_abs_d_p_ryr_open": float(np.max(np.abs(mo[:, :, 3].mean(0) - fo[:, :, 3].mean(0)))),
            "note": "APD90 needs the whole action potential (about 500 ms); it is in the longer precision study "
                    "(bench.py --precision-ensemble)"}


def batch_cells(G, args, dist):
    """The batched workload, mixed precision: NFRU drawn from {1250, 2500,
    5000, 12500}, pacing cycle length U(300, 2000) ms, PCa and GKr scaled by
    lognormal(0, 0.2) factors."""
    import numpy as np
    rng = np.random.default_rng(20021 + dist.rank)
    n = args.batch_cells
    sizes = rng.choice([1250, 2500, 5000, 12500], n)
    cells, sets, states = [], [], []
    for i in range(n):
        pca, gkr = np.exp(rng.normal(0.0, 0.2, 2))
        c = G.Cell(int(sizes[i]), precision="mixed", pca_scale=float(pca))
        st = G.settings(period=float(rng.uniform(300.0, 2000.0)), scale_GKr=float(gkr))
        states.append(c.init_rest(st, scheme=G.SEED_BASE, base=SEED + 100003 * i))
        cells.append(c)
        sets.append(st)
    return sizes, cells, sets, np.ascontiguousarray(np.array(states))


def time_batched_device(G, args, dist):
    """The batched workload with the device-resident integrator
    (gw_run_device): all cells' integrators and FRU stages in one CUDA graph,
    no host thread per cell."""
    import numpy as np
    sizes, cells, sets, states = batch_cells(G, args, dist)
    n = len(cells)
    t = np.zeros(n)
    old = np.full(n, 0.1)
    G.run_device(cells, sets, t, states, old, args.batch_warmup_ms)
    sub0 = sum(c.substeps() for c in cells)
    dist.barrier()
    t0 = time.perf_counter()
    G.run_device(cells, sets, t, states, old, args.batch_ms)
    wall = time.perf_counter() - t0
    substeps = sum(c.substeps() for c in cells) - sub0
    eq_ms = float(np.sum(sizes)) / NFRU * args.batch_ms
    for c in cells:
        c.close()
    return {"value": dist.sum(n * args.batch_ms) / dist.max(wall), "unit": "cell-ms/s (cells of mixed NFRU)",
            "value_12500_equiv": dist.sum(eq_ms) / dist.max(wall), "cells": n,
            "window_ms": [args.batch_warmup_ms, args.batch_warmup_ms + args.batch_ms],
            "fru_substeps_per_s": substeps / wall, "precision": "mixed",
            "timing": "host wall clock around one graph launch (the run is one CUDA graph)"}


def time_batched_persistent(G, args, dist):
    """The batched workload with the persistent multi-cell kernel
    (gw_run_persistent): every cell's FRU stages, reductions and integrator
    steps inside one resident launch."""
    import numpy as np
    sizes, cells, sets, states = batch_cells(G, args, dist)
    n = len(cells)
    t = np.zeros(n)
    old = np.full(n, 0.1)
    G.run_persistent(cells, sets, t, states, old, args.batch_warmup_ms)
    sub0 = sum(c.substeps() for c in cells)
    dist.barrier()
    t0 = time.perf_counter()
    G.run_persistent(cells, sets, t, states, old, args.batch_ms)
    wall = time.perf_counter() - t0
    substeps = sum(c.substeps() for c in cells) - sub0
    eq_ms = float(np.sum(sizes)) / NFRU * args.batch_ms
    for c in cells:
        c.close()
    return {"value": dist.sum(n * args.batch_ms) / dist.max(wall), "unit": "cell-ms/s (cells of mixed NFRU)",
            "value_12500_equiv": dist.sum(eq_ms) / dist.max(wall), "cells": n,
            "window_ms": [args.batch_warmup_ms, args.batch_warmup_ms + args.batch_ms],
            "fru_substeps_per_s": substeps / wall, "precision": "mixed",
            "timing": "host wall clock around one persistent launch (the run is one CUDA graph)"}


def time_batched(G, args, dist):
    """Many cells at once (per-stream or lockstep gw_batch), one host
    integrator thread per cell; the workload of batch_cells."""
    import numpy as np
    sizes, cells, sets, states = batch_cells(G, args, dist)
    n = len(cells)
    t = np.zeros(n)
    old = np.full(n, 0.1)
    b = G.Batch("mixed")
    lock = args.batch_mode == "lockstep"
    b.run(cells, sets, t, states, old, args.batch_warmup_ms, lockstep=lock)
    tuning = None
    if not args.no_autotune:
        tuning = tune_summary(G.autotune(cells, sets, t, states, old, args.tune_ms, batch=b if lock else None), args)
    sub0 = sum(c.substeps() for c in cells)
    b.profile(True)
    launch0 = sum(c.launches() for c in cells)
    dist.barrier()
    t0 = time.perf_counter()
    b.run(cells, sets, t, states, old, args.batch_ms, lockstep=lock)
    wall = time.perf_counter() - t0
    kern_ms, launches = b.profile(False)
    if not lock:
        kern_ms, launches = None, sum(c.launches() for c in cells) - launch0
    substeps = sum(c.substeps() for c in cells) - sub0
    cell_ms = n * args.batch_ms
    eq_ms = float(np.sum(sizes)) / NFRU * args.batch_ms
    for c in cells:
        c.close()
    b.close()
    return {"value": dist.sum(cell_ms) / dist.max(wall), "unit": "cell-ms/s (cells of mixed NFRU)",
            "value_12500_equiv": dist.sum(eq_ms) / dist.max(wall), "cells": n,
            "nfru_mix": {str(k): int(np.sum(sizes == k)) for k in (1250, 2500, 5000, 12500)},
            "window_ms": [args.batch_warmup_ms, args.batch_warmup_ms + args.batch_ms],
            "fru_substeps_per_s": substeps / wall, "batched_launches": int(launches),
            "kernel_ms": kern_ms, "precision": "mixed", "mode": args.batch_mode, "tuning": tuning,
            "timing": "host wall clock around the batched run (one host thread per cell)"}


def serve_requests(G, args, rate):
    """The request stream of the serving workload: NFRU from {1250, 2500, 5000,
    12500}; half paced (cycle length U(400, 2000) ms for 1-10 beats, the
    stimulus 10 ms into each cycle), half voltage clamp (hold -100 mV, step
    to U(-40, 40) mV from 5 to 205 ms, back to -100 mV until 210 ms); each
    request simulates its whole protocol from rest (--serve-ms caps it)."""
    import numpy as np
    rng = np.random.default_rng(int(rate * 1000) + 7)
    n = args.serve_requests
    reqs = []
    for i in range(n):
        r = G.Request()
        r.nfru = int(rng.choice([1250, 2500, 5000, 12500]))
        if rng.random() < 0.5:
            cl = float(rng.uniform(400.0, 2000.0))
            beats = int(rng.integers(1, 11))
            r.set = G.settings(period=cl)
            dur = float(np.floor(beats * cl))
        else:
            r.set = G.settings(vclamp_flag=1, vclamp_hold=-100.0, vclamp_set=float(rng.uniform(-40.0, 40.0)),
                               vclamp_duration=200.0, vclamp_shift=5.0, vclamp_period=100000.0)
            dur = 210.0
        r.seed_scheme = G.SEED_BASE
        r.seed = SEED + 1000003 * i
        r.pca_scale = 1.0
        r.duration_ms = min(dur, args.serve_ms) if args.serve_ms > 0 else dur
        reqs.append(r)
    return reqs, rng.exponential(1.0 / rate, n)


def time_serving(G, args, rate):
    """Poisson arrivals at `rate` requests/s of the serving workload
    (serve_requests), mixed precision, admitted by device bytes; the
    request sizes are reserved up front, so no device allocation runs while
    requests are on the GPU."""
    import numpy as np
    reqs, gaps = serve_requests(G, args, rate)
    n = len(reqs)
    srv = G.Server("mixed", slots=args.serve_slots, mem_budget_bytes=int(args.serve_budget_gb * (1 << 30)),
                   lockstep=args.batch_mode == "lockstep")
    for size in sorted(set(r.nfru for r in reqs)):
        srv.reserve(size, min(args.serve_slots, sum(1 for r in reqs if r.nfru == size)))
    allocs0 = srv.stats()["allocs"]
    t0 = time.perf_counter()
    nxt = t0
    for r, g in zip(reqs, gaps):
        nxt += g
        d = nxt - time.perf_counter()
        if d > 0:
            time.sleep(d)
        srv.submit(r)
    srv.wait()
    wall = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    lat = np.array([r.t_done - r.t_submit for r in reqs])
    wait = np.array([r.t_start - r.t_submit for r in reqs])
    ok = all(r.status == 0 for r in reqs)
    cell_ms = sum(r.duration_ms for r in reqs)
    eq = sum(r.nfru * r.duration_ms for r in reqs) / NFRU
    return {"rate_req_per_s": rate, "requests": n, "ok": ok, "p50_latency_s": float(np.percentile(lat, 50)),
            "p99_latency_s": float(np.percentile(lat, 99)), "mean_queue_wait_s": float(wait.mean()),
            "simulated_ms": cell_ms, "wall_s": wall, "cell_ms_per_s": cell_ms / wall,
            "cell_ms_per_s_12500_equiv": eq / wall,
            "device_bytes": {"peak_held": st["peak_held"], "budget": int(args.serve_budget_gb * (1 << 30)),
                             "allocations_while_serving": st["allocs"] - allocs0}}


def time_serving_fp64_sequential(G, args, rate):
    """The serving denominator: the same request list (the same seed, so the
    same sizes, protocols and durations as time_serving at `rate`) run in FP64
    one request at a time, each submitted when the previous one is done."""
    reqs, _ = serve_requests(G, args, rate)
    srv = G.Server("fp64", slots=1, mem_budget_bytes=int(args.serve_budget_gb * (1 << 30)), lockstep=False)
    for size in sorted(set(r.nfru for r in reqs)):
        srv.reserve(size, 1)
    t0 = time.perf_counter()
    for r in reqs:
        srv.submit(r)
    srv.wait()
    wall = time.perf_counter() - t0
    srv.close()
    cell_ms = sum(r.duration_ms for r in reqs)
    return {"requests": len(reqs), "ok": all(r.status == 0 for r in reqs), "simulated_ms": cell_ms, "wall_s": wall,
            "cell_ms_per_s": cell_ms / wall, "precision": "fp64", "slots": 1}


def caf_run(settings, workdir):
    """Run the C host driver (gw_caf, the reference program's main loop over
    libgw_fru.so) with key=value settings; returns (wall s, states,
    otherstates, currents) read back from its reference-format files, time
    in ms."""
    import numpy as np
    exe = os.path.join(ROOT, "greenstein2002_gb300", "_build", "gw_caf")
    os.makedirs(workdir, exist_ok=True)
    t0 = time.perf_counter()
    r = subprocess.run([exe] + ["%s=%s" % kv for kv in settings.items()] + ["output_dir=%s/" % workdir],
                       capture_output=True, text=True)
    wall = time.perf_counter() - t0
    if r.returncode != 0:
        raise RuntimeError("gw_caf failed: %s" % r.stderr[-500:])

    def load(stem):
        a = np.loadtxt(os.path.join(workdir, "%s.0.txt" % stem), skiprows=1)
        a[:, 0] *= 1000.0  # the files' time column is in seconds (caf.c's ts_sec)
        return a
    return wall, load("states"), load("otherstates"), load("currents")


def time_full_cell(args):
    """The full-size cell's whole protocol, one cell, through the C host
    driver writing the reference's output files: 5 beats at 1 Hz from rest
    (stimulus 10 ms into each cycle), and a voltage-clamp run holding -100 mV
    with a step to 0 mV from 50 to 250 ms (300 ms in all) that records ICaL
    and the SR release flux.  FP64 (packed launches, 16 FRUs per warp, the
    one-cell autotuner's choice) and mixed precision with the same seeds."""
    import tempfile
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        for prec, extra in (("fp64", {"precision": 0, "stage_packing": 2}), ("mixed", {"precision": 1})):
            base = dict(NFRU_sim=NFRU, ic_file_flag=0, seed_scheme=0, seed_base=SEED, **extra)
            w1, st, ot, cu = caf_run(dict(base, time_end=5000), os.path.join(tmp, prec + "_pace"))
            beats = []
            for b in range(5):
                sel = (st[:, 0] > 1000 * b) & (st[:, 0] <= 1000 * (b + 1))
                beats.append({"apd90_ms": apd90(st[sel, 0], st[sel, 1]), "peak_cai_mM": float(st[sel, 7].max()),
                              "min_cajsr_mM": float(ot[sel, 2].min())})
            w2, st2, ot2, cu2 = caf_run(dict(base, time_end=300, vclamp_flag=1, vclamp_hold=-100, vclamp_set=0,
                                             vclamp_duration=200, vclamp_shift=50, vclamp_period=1000),
                                        os.path.join(tmp, prec + "_clamp"))
            step = (st2[:, 0] > 50) & (st2[:, 0] <= 250)
            out[prec] = {"value": 5300.0 / (w1 + w2), "unit": "cell-ms/s", "wall_s": {"pacing": w1, "clamp": w2},
                         "beats": beats,
                         "clamp": {"peak_ICaL_uA_per_uF": float(cu2[step, 12].min()),
                                   "ICaL_at_step_end": float(cu2[step, 12][-1]),
                                   "peak_JRyRtot": float(ot2[step, 3].max()),
                                   "peak_cai_mM": float(st2[step, 7].max())}}
    out["mixed"]["speedup_vs_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    out["protocol"] = ("one 12,500-FRU cell (FRU j seeded 5489 + j), rest state: 5 beats at 1 Hz (5000 ms), then a "
                       "separate clamp run (hold -100 mV, 0 mV from 50 to 250 ms, 300 ms); through gw_caf, which "
                       "writes the reference program's states/otherstates/currents files; value = 5300 simulated ms / "
                       "wall s of both runs (host integrator, FRU stages on the GPU)")
    return out


def apd90(t_ms, v):
    """Action-potential duration at 90% repolarisation of the first beat (from
    the upstroke's crossing of the 90% level to the repolarisation's)."""
    import numpy as np
    i0 = int(np.argmax(v))
    vmax, vrest = v[i0], v[0]
    thr = vmax - 0.9 * (vmax - vrest)
    up = int(np.argmax(v > thr))
    after = np.nonzero(v[i0:] < thr)[0]
    return float(t_ms[i0 + after[0]] - t_ms[up]) if len(after) else float("nan")


def precision_ensemble(G, args, dist):
    """Mixed precision against the FP64 GPU oracle on full-size cells: SEEDS
    12,500-FRU cells per precision, cell k's FRU j seeded 5489 + 100000 k + j,
    from rest through the first beat; per seed APD90 and peak Cai, and the
    ensemble's JSR depletion and LCC / RyR open-probability traces."""
    import numpy as np
    seeds, ms = args.precision_ensemble
    t_ms = np.arange(1, ms + 1, dtype=float)
    res = {}
    chunk = 16  # cells run at once: one host integrator thread per host core
    for prec in ("fp64", "mixed"):
        st_parts, ot_parts, wall = [], [], 0.0
        for k0 in range(0, seeds, chunk):
            ks = range(k0, min(seeds, k0 + chunk))
            cells, sets, states = [], [], []
            for k in ks:
                c = G.Cell(NFRU, precision=prec)
                if prec == "fp64":
                    c.set_stage_packing(((NFRU + 7) // 8 + 7) // 8)  # the FP64 ensemble's tuned shape
                st = G.settings()
                states.append(c.init_rest(st, scheme=G.SEED_BASE, base=SEED + 100000 * k))
                cells.append(c)
                sets.append(st)
            states = np.ascontiguousarray(np.array(states))
            runner = G.Batch(prec)
            t0 = time.perf_counter()
            st_tr, ot_tr = runner.run(cells, sets, np.zeros(len(ks)), states, np.full(len(ks), 0.1), ms,
                                      traces=True, lockstep=False)
            wall += time.perf_counter() - t0
            print("precision ensemble: %s, seeds %d-%d x %d ms, %.1f s so far" % (prec, k0, ks[-1], ms, wall),
                  file=sys.stderr, flush=True)
            for c in cells:
                c.close()
            runner.close()
            st_parts.append(st_tr)
            ot_parts.append(ot_tr)
        st_tr, ot_tr = np.concatenate(st_parts), np.concatenate(ot_parts)
        res[prec] = {"apd90": np.array([apd90(t_ms, v) for v in st_tr[:, :, 0]]), "peak_cai": st_tr[:, :, 6].max(1),
                     "jsr": ot_tr[:, :, 1].mean(0), "plcc": ot_tr[:, :, 7].mean(0), "pryr": ot_tr[:, :, 3].mean(0),
                     "wall_s": wall}
    f, m = res["fp64"], res["mixed"]
    d_apd = m["apd90"] - f["apd90"]
    d_pk = m["peak_cai"] - f["peak_cai"]
    ok = ~np.isnan(d_apd)  # seeds repolarised within the window in both runs
    fa, ma = f["apd90"][ok], m["apd90"][ok]
    return {"check": "precision_ensemble", "seeds": seeds, "window_ms": [0, ms], "nfru": NFRU,
            "apd90_ms": dict(paired_ci(fa, ma), fp64_mean=float(fa.mean()), mixed_mean=float(ma.mean()),
                             paired_sem_rel=float(np.std(d_apd[ok], ddof=1) / np.sqrt(ok.sum()) / fa.mean()),
                             seeds_repolarised_in_both=int(ok.sum())),
            "peak_cai_mM": dict(paired_ci(f["peak_cai"], m["peak_cai"]), fp64_mean=float(f["peak_cai"].mean()),
                                mixed_mean=float(m["peak_cai"].mean()),
                                paired_sem_rel=float(np.std(d_pk, ddof=1) / np.sqrt(seeds) / f["peak_cai"].mean())),
            "jsr_depletion": {"fp64_min_mean_cajsr_mM": float(f["jsr"].min()), "mixed_min_mean_cajsr_mM": float(m["jsr"].min()),
                              "rel_diff": float(m["jsr"].min() / f["jsr"].min() - 1.0)},
            "open_probability_traces": {"max_abs_diff_lcc": float(np.max(np.abs(m["plcc"] - f["plcc"]))),
                                        "max_lcc": float(np.max(f["plcc"])),
                                        "max_abs_diff_ryr": float(np.max(np.abs(m["pryr"] - f["pryr"]))),
                                        "max_ryr": float(np.max(f["pryr"]))},
            "wall_s": {"fp64": f["wall_s"], "mixed": m["wall_s"]},
            "per_seed": {"apd90_fp64_ms": [None if np.isnan(x) else float(x) for x in f["apd90"]],
                         "apd90_mixed_ms": [None if np.isnan(x) else float(x) for x in m["apd90"]],
                         "peak_cai_fp64_mM": [float(x) for x in f["peak_cai"]],
                         "peak_cai_mixed_mM": [float(x) for x in m["peak_cai"]]}}


def run_gpu(args, dist):
    import numpy as np
    import greenstein2002_gb300 as G
    from greenstein2002_gb300 import build as gb
    gb.build()
    G.load()
    if args.precision_ensemble:
        res = precision_ensemble(G, args, dist)
        if dist.rank == 0:
            print(json.dumps(res))
        return
    seed = SEED + dist.rank * args.nfru  # replicas: independent streams per rank
    clocks = Clocks(dist.local)
    want_mixed = args.precision == "fp64" and not args.no_mixed
    # headline: the FP64 ensemble, all cells on the GPU at once; then the same
    # window through the C-ABI with host buffers (e2e)
    ens = time_ensemble(G, args, dist, args.precision, clocks=clocks, traces=want_mixed, e2e=not args.no_e2e)
    substeps = ens["substeps"]
    if args.only_ensemble:
        if dist.rank == 0:
            print(json.dumps({"section": "ensemble only", "value": ens["value"], "unit": "cell-ms/s",
                              "window": ens["window"], "gpu_launches": int(ens["launches"]),
                              "kernel": stage_kernel_name(args.precision, ens["tuning"], args),
                              "fru_substeps": int(substeps), "device_ms": ens["device_ms"], "tuning": ens["tuning"]}))
        return
    # roofline of the dominant kernel (the FRU stage kernel, 98-99% of the
    # device time), FP64-pipe bound: algorithmic FLOPs of all its launches in
    # the timed region over the region's device time (the cells' launches
    # overlap); the FP64 peak is measured in this run
    fp64_peak = G.fp64_peak_tflops()
    achieved_tf = FLOPS_PER_SUBSTEP * substeps / (ens["device_ms"] * 1e-3) / 1e12
    achieved_gbs = BYTES_PER_SUBSTEP * substeps / (ens["device_ms"] * 1e-3) / 1e9
    hbm_peak = load_peaks().get("hbm_gbs", 6800.0)
    # the mixed-precision ensemble: the same seeds, cells and window
    mixed_ens = None
    if want_mixed:
        m = time_ensemble(G, args, dist, "mixed", traces=True)
        m_rate = m["substeps"] / (m["device_ms"] / 1000.0)
        mixed_ens = {"value": m["value"], "unit": "cell-ms/s", "cells": m["cells"], "window": m["window"],
                     "speedup_vs_fp64_ensemble": m["value"] / ens["value"], "fru_substeps_per_s": m_rate,
                     "ms_per_step": m["device_ms"] / args.steps, "gpu_launches": int(m["launches"]),
                     "kernel": stage_kernel_name("mixed", m["tuning"], args), "tuning": m["tuning"],
                     "roofline": mixed_roofline(m_rate, hbm_peak), "clocks": None,
                     "error_vs_fp64_same_seeds": precision_vs_fp64(ens, m)}
        del m
    # one cell alone (the latency of the plain method)
    one = time_single(G, args, dist, args.precision, seed, keep_trace=want_mixed)
    one_line = {"value": one["value"], "unit": "cell-ms/s", "fru_substeps_per_s": one["substeps"] / (one["wall_ms"] / 1e3),
                "per_launch_ms": one["kern_ms"] / max(one["kern_launches"], 1), "launches": int(one["kern_launches"]),
                "tuning": one["tuning"], "timing": "CUDA events on the cell's stream", "window": window_str(args)}
    mixed = None
    if want_mixed:
        m = time_single(G, args, dist, "mixed", seed, keep_trace=True)
        a, b = one["trace"], m["trace"]
        cai_range = float(np.max(a[:, 6]) - np.min(a[:, 6])) or 1.0
        m_rate = m["substeps"] / (m["wall_ms"] / 1000.0)
        mixed = {"value": m["value"], "unit": "cell-ms/s (one cell)", "speedup_vs_fp64_one_cell": m["value"] / one["value"],
                 "fru_substeps_per_s": m_rate, "tuning": m["tuning"], "roofline": mixed_roofline(m_rate, hbm_peak),
                 "error_vs_fp64_same_seeds": {
                     "max_abs_dV_mV": float(np.max(np.abs(a[:, 0] - b[:, 0]))),
                     "max_abs_dCai_rel_to_range": float(np.max(np.abs(a[:, 6] - b[:, 6]))) / cai_range,
                     "max_rel_dCaNSR": float(np.max(np.abs(a[:, 7] - b[:, 7]) / np.abs(a[:, 7]))),
                     "window": "per-ms global states over the timed window"}}
    batched = None if args.no_batch else time_batched(G, args, dist)
    if batched:
        batched["speedup_12500_equiv_vs_fp64_one_cell"] = batched["value_12500_equiv"] / one["value"]
        if not args.no_devdp:
            batched["device_integrator"] = time_batched_device(G, args, dist)
            batched["persistent"] = time_batched_persistent(G, args, dist)
            batched["persistent"]["speedup_vs_per_stream"] = batched["persistent"]["value"] / batched["value"]
    serving = None
    if not args.no_serve and dist.world == 1:
        serving = {"protocol": "per request from rest: NFRU in {1250,2500,5000,12500}, 50/50 pacing (CL U(400,2000) "
                               "ms, 1-10 beats) or voltage clamp (-100 -> U(-40,40) mV for 200 ms, 210 ms in all)%s, "
                               "mixed precision, %d worker slots, %g GB admission budget, sizes reserved up front"
                               % (" capped at %g ms" % args.serve_ms if args.serve_ms > 0 else "", args.serve_slots,
                                  args.serve_budget_gb),
                   "sweep": [time_serving(G, args, r) for r in args.serve_rates]}
        for r in serving["sweep"]:
            r["speedup_12500_equiv_vs_fp64_one_cell"] = r["cell_ms_per_s_12500_equiv"] / one["value"]
        if args.serve_baseline:
            base = time_serving_fp64_sequential(G, args, args.serve_rates[0])
            base["speedup_of_serving"] = serving["sweep"][0]["cell_ms_per_s"] / base["cell_ms_per_s"]
            serving["fp64_one_at_a_time"] = base
        else:
            serving["fp64_one_at_a_time"] = {"run": False, "enable": "--serve-baseline",
                                             "why": "the same request list in FP64, one request at a time, takes "
                                                    "several minutes"}
    e2e = ens.get("e2e")
    full_cell = (time_full_cell(args) if args.full_cell and dist.world == 1 else
                 {"run": False, "enable": "--full-cell",
                  "why": "one cell's whole protocol (5,300 simulated ms) in FP64 and in mixed precision takes "
                         "about 8.5 minutes of wall time, longer than the rest of this line together"})

    # ---- CPU baseline: the reference program on one host core ----
    cpu = None
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        phases = window_phases(args)
        d, why = reference_build(1.0, window_ic=bool(phases))
        if d is not None:
            walls = [reference_sample(d, 1, 1.0, SEED, [ph])[1] for ph in (phases or [None])]
            v = len(walls) / sum(walls)
            cpu = {"value": v, "unit": "cell-ms/s", "cores": 1, "kind": "reference",
                   "sample": "reference program (serial build of its own sources), NFRU=12,500, 1 ms from the "
                             "bench cell's state at each of %s ms of the timed window %s (%.1f s wall in all)"
                             % ("/".join(os.path.basename(p)[1:] for p in phases) or "0", window_str(args),
                                sum(walls))}
        else:
            cpu = {"value": None, "unit": "cell-ms/s", "cores": 0, "kind": "reference", "sample": why}

    if dist.rank == 0:
        kernel = stage_kernel_name(args.precision, ens["tuning"], args)
        traffic = TRAFFIC_PER_LAUNCH.get(kernel) if args.nfru == NFRU else None
        window = window_str(args)
        line = {
            "metric": "cell-ms simulated/s at 12,500 FRUs", "value": ens["value"], "unit": "cell-ms/s",
            "n_gpus": dist.world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ens["device_ms"] / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32+f64", "data": "synthetic",
            "config": {"workload": "FP64 ensemble of %d cells per GPU (%d of the 64 seeds; cell k's FRU j seeded "
                                   "5489+100000k+j), NFRU=%d each, rest state, 1 Hz pacing (1 ms -100 uA/uF at 10 ms), "
                                   "all cells on the GPU at once; step = %g ms simulated per cell; timed window %s "
                                   "(fixed: untimed set-up from rest to %g ms, warm-up steps, state put back)"
                                   % (args.seeds, args.seeds, args.nfru, args.step_ms, window, WINDOW_START_MS),
                       "window": window, "nfru": args.nfru, "cells": args.seeds, "step_ms": args.step_ms,
                       "precision": ("fp64 (FRU path and global ODE)" if args.precision == "fp64" else
                                     "mixed (FRU rates and local Ca ODE fp32; FRU state, clock, flux sums "
                                     "and global ODE fp64)"),
                       "integrator": ("host Dormand-Prince 5(4) per cell, FRU stages on GPU" if args.runner == "streams"
                                      else "persistent multi-cell kernel: FRU stages, reductions and Dormand-Prince "
                                           "5(4) steps of every cell inside one launch"),
                       "fru_lanes": args.fru_lanes,
                       "l2": "flushed between timed steps (512 MB write)",
                       "timing": "device time of each step from before the first cell's first launch to after the "
                                 "last cell's last launch (events on a timing stream joined to every cell's stream)",
                       "parallelism": "replicas" if dist.world > 1 else "single GPU"},
            "fru_substeps": int(substeps), "fru_substeps_per_s": substeps / (ens["device_ms"] / 1000.0),
            "gpu_launches": int(ens["launches"]),
            "roofline": {"bound": "fp64", "kernel": kernel, "achieved": achieved_tf,
                         "peak": fp64_peak, "unit": "TFLOP/s", "frac": achieved_tf / fp64_peak if fp64_peak else None,
                         "peak_source": "measured in-run (independent DFMA chains on all SMs)",
                         "traffic": traffic[0] if traffic else None,
                         "traffic_note": traffic[1] if traffic else "no ncu capture of this kernel on this workload",
                         "algorithmic": "%g FLOP per FRU-substep x %d FRU-substeps over the timed region's device time"
                                        % (FLOPS_PER_SUBSTEP, substeps),
                         "hbm_view": {"achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
                                      "frac": achieved_gbs / hbm_peak,
                                      "algorithmic": "%g B x FRU-substeps" % BYTES_PER_SUBSTEP}},
            "clocks": ens["clocks"],
            "tuning": ens["tuning"],
            "mixed_ensemble": mixed_ens,
            "one_cell": one_line,
            "mixed": mixed,
            "batched": batched,
            "serving": serving,
            "full_cell": full_cell,
            "e2e": e2e,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line))


def stage_kernel_name(precision, tuning, args):
    """The FRU stage kernel a section's launches ran (the autotuner's choice)."""
    packed = bool(tuning and tuning.get("packed_div"))
    lanes = tuning["lanes_per_fru"] if tuning else args.fru_lanes
    if precision == "mixed":
        return "fru_stage_mixed_packed_kernel" if packed else "fru_stage_mixed_kernel"
    if packed:
        return "fru_stage4_packed_kernel"
    return "fru_stage4_kernel" if lanes == 4 else "fru_stage_kernel"


def main():
    args = parse()
    dist = Dist()
    if args.impl == "reference":
        run_reference(args, dist)
    else:
        run_gpu(args, dist)


if __name__ == "__main__":
    main()

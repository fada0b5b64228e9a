"""Benchmark: cell-ms simulated per second for one 12,500-FRU cell.

Workload (the full-size plain FP64 configuration): one cell of NFRU=12,500
release units, rest initial state (initialize_state.c:164-219), per-FRU
MT19937 seeded 5489+j, 1 Hz pacing with a 1 ms -100 uA/uF stimulus at
10 ms.  A step advances the cell by STEP_MS (50 ms) of simulated time through
the whole hot path (Dormand-Prince global step, every FRU stage on the GPU).
Warm-up steps cover [0, W*50) ms, so with the defaults (W=3, K=20) the timed
window is [150, 1150) ms: one full pacing cycle including the second beat's
upstroke.  L2 (129 MB) is flushed by a 512 MB write between timed steps.

value: inputs resident in HBM, device-timed with CUDA events on the library's
stream.  e2e: the same window through the C-ABI with host buffers: every
step uploads the cell's full FRU + RNG state from host memory (gw_upload)
and downloads it and the step's traces (gw_download) inside the timed region.

--impl reference: the reference's own serial program (oracle/_ref, built
from its sources) on the host cores, one independent 12,500-FRU cell per
core, each step a bounded 1-ms sample from rest.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NFRU = 12500
STEP_MS = 50.0
SEED = 5489
# algorithmic work per FRU-substep (static count of the reference's substep:
# fru_rates_local + 2 x fcn_fru + simfru_local body, each add/mul/div/exp/
# compare/convert counted once) and MT19937 bytes streamed per substep
FLOPS_PER_SUBSTEP = 700.0
BYTES_PER_SUBSTEP = 384.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gw", choices=["gw", "reference"])
    ap.add_argument("--nfru", type=int, default=NFRU)
    ap.add_argument("--step-ms", type=float, default=STEP_MS)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
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
def reference_build(ms):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import build_ref
    if not build_ref.have_sources():
        return None, "reference sources not present (oracle/_ref/src missing)"
    try:
        return build_ref.build_config("bench12500_%gms" % ms, build_ref.cfg_macros(NFRU, ms), lib=False,
                                      exe=True), None
    except Exception as e:  # noqa: BLE001
        return None, "reference build failed: %s" % str(e).splitlines()[0]


def reference_sample(d, procs, ms, seed0):
    """Run `procs` independent reference cells concurrently for `ms` simulated
    ms each; returns (cell-ms/s, wall s)."""
    import resource
    import tempfile

    def _stack():
        resource.setrlimit(resource.RLIMIT_STACK, (resource.RLIM_INFINITY, resource.RLIM_INFINITY))

    with tempfile.TemporaryDirectory() as tmp:
        ps = []
        t0 = time.perf_counter()
        for p in range(procs):
            wd = os.path.join(tmp, str(p))
            os.makedirs(wd)
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
    if dist.rank != 0:
        return
    ms = 1.0
    d, why = reference_build(ms)
    if d is None:
        print(json.dumps({"impl": "reference", "unavailable": why}))
        return
    procs = os.cpu_count() or 1
    for _ in range(args.warmup):
        reference_sample(d, procs, ms, SEED)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        reference_sample(d, procs, ms, SEED)
    wall = time.perf_counter() - t0
    value = args.steps * procs * ms / wall
    sample = ("reference program (caf.c, serial build of its own sources, gcc -O3) x%d concurrent cells, "
              "NFRU=12,500 each, 1 ms from rest per cell per step" % procs)
    print(json.dumps({
        "impl": "reference", "metric": "cell-ms simulated/s at 12,500 FRUs", "value": value,
        "unit": "cell-ms/s", "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * wall / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "one 12,500-FRU cell per host core, rest state, 1 Hz pacing, seeds 5489+j",
                   "nfru": NFRU, "cells": procs, "ms_per_cell_per_step": ms},
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


def run_gpu(args, dist):
    import numpy as np
    import greenstein2002_gb300 as G
    from greenstein2002_gb300 import build as gb
    gb.build()
    G.load()
    seed = SEED + dist.rank * args.nfru  # replicas: independent streams per rank
    # ---- device-resident run (value) ----
    cell, st, state = fresh_cell(G, args.nfru, seed, args.fru_lanes, args.precision)
    t = 0.0
    oldstep = st.step_max
    for _ in range(args.warmup):
        t, _, _, _ = cell.run(state, t, int(args.step_ms), oldstep, st, want=())
        oldstep = cell.oldstep
    sub0 = cell.substeps()
    launch0 = cell.launches()
    cell.profile(True)
    clocks = Clocks(dist.local)
    total_ms = 0.0
    dist.barrier()
    cell.sync()
    clocks.start()
    for _ in range(args.steps):
        cell.l2_flush()
        cell.event(0)
        t, _, _, _ = cell.run(state, t, int(args.step_ms), oldstep, st, want=())
        oldstep = cell.oldstep
        cell.event(1)
        total_ms += cell.elapsed_ms(0, 1)
    cell.sync()
    clk = clocks.stop()
    dist.barrier()
    kern_ms, kern_launches = cell.profile_read()
    cell.profile(False)
    substeps = cell.substeps() - sub0
    launches = cell.launches() - launch0 - 0
    wall_ms = dist.max(total_ms)
    cells_ms = dist.sum(args.steps * args.step_ms)
    value = cells_ms / (wall_ms / 1000.0)
    # roofline of the FRU stage kernel (FP64-pipe bound), measured FP64 peak
    fp64_peak = G.fp64_peak_tflops()
    per_launch_ms = kern_ms / max(kern_launches, 1)
    sub_per_launch = substeps / max(kern_launches, 1)
    achieved_tf = FLOPS_PER_SUBSTEP * sub_per_launch / (per_launch_ms * 1e-3) / 1e12
    achieved_gbs = BYTES_PER_SUBSTEP * sub_per_launch / (per_launch_ms * 1e-3) / 1e9
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    cell.close()

    # ---- end to end through the C-ABI with host buffers (e2e) ----
    e2e = None
    if not args.no_e2e:
        cell, st, state = fresh_cell(G, args.nfru, seed, args.fru_lanes, args.precision)
        t = 0.0
        oldstep = st.step_max
        for _ in range(args.warmup):
            t, _, _, _ = cell.run(state, t, int(args.step_ms), oldstep, st, want=())
            oldstep = cell.oldstep
        host = cell.download()
        h_state = state.copy()
        h2d = sum(v.nbytes for v in host.values()) + h_state.nbytes
        dist.barrier()
        cell.sync()
        e2e_ms = 0.0
        d2h = 0
        for _ in range(args.steps):
            cell.l2_flush()
            t0 = time.perf_counter()
            cell.upload(host)
            t, states, other, cur = cell.run(h_state, t, int(args.step_ms), oldstep, st)
            oldstep = cell.oldstep
            host = cell.download()
            e2e_ms += (time.perf_counter() - t0) * 1000.0
            d2h = sum(v.nbytes for v in host.values()) + states.nbytes + other.nbytes + cur.nbytes
        dist.barrier()
        e2e_val = dist.sum(args.steps * args.step_ms) / (dist.max(e2e_ms) / 1000.0)
        e2e = {"value": e2e_val, "unit": "cell-ms/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)}
        cell.close()

    # ---- CPU baseline: the reference program on one host core ----
    cpu = None
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        d, why = reference_build(3.0)
        if d is not None:
            v, wall = reference_sample(d, 1, 3.0, SEED)
            cpu = {"value": v, "unit": "cell-ms/s", "cores": 1, "kind": "reference",
                   "sample": "reference program (serial build of its own sources), NFRU=12,500, rest state, "
                             "first 3 ms (%.1f s wall); rest costs fewer substeps per ms than the paced-beat "
                             "average timed on the GPU" % wall}
        else:
            cpu = {"value": None, "unit": "cell-ms/s", "cores": 0, "kind": "reference", "sample": why}

    if dist.rank == 0:
        line = {
            "metric": "cell-ms simulated/s at 12,500 FRUs", "value": value, "unit": "cell-ms/s",
            "n_gpus": dist.world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": wall_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32+f64", "data": "synthetic",
            "config": {"workload": "one cell per GPU, NFRU=%d, rest state, 1 Hz pacing (1 ms -100 uA/uF at 10 ms), "
                                   "seeds 5489+j; step = %g ms simulated; timed window [%g, %g) ms"
                                   % (args.nfru, args.step_ms, args.warmup * args.step_ms,
                                      (args.warmup + args.steps) * args.step_ms),
                       "nfru": args.nfru, "step_ms": args.step_ms, "precision": ("fp64 (FRU path and global ODE)" if args.precision == "fp64" else
                                     "mixed (FRU rates and local Ca ODE fp32; FRU state, clock, flux sums and global ODE fp64)"),
                       "integrator": "host Dormand-Prince 5(4), FRU stages on GPU",
                       "fru_lanes": args.fru_lanes,
                       "l2": "flushed between timed steps (512 MB write)",
                       "parallelism": "replicas" if dist.world > 1 else "single GPU"},
            "fru_substeps": int(substeps), "fru_substeps_per_s": substeps / (wall_ms / 1000.0),
            "gpu_launches": int(launches),
            "roofline": {"bound": "fp64", "kernel": ("fru_stage_mixed_kernel" if args.precision == "mixed" else
                                                     "fru_stage4_kernel" if args.fru_lanes == 4 else "fru_stage_kernel"), "achieved": achieved_tf,
                         "peak": fp64_peak, "unit": "TFLOP/s", "frac": achieved_tf / fp64_peak if fp64_peak else None,
                         "peak_source": "measured in-run (independent DFMA chains on all SMs)",
                         "traffic": None, "per_launch_ms": per_launch_ms, "launches": int(kern_launches),
                         "algorithmic": "%g FLOP x %.0f FRU-substeps per launch" % (FLOPS_PER_SUBSTEP, sub_per_launch),
                         "hbm_view": {"achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
                                      "frac": achieved_gbs / hbm_peak,
                                      "algorithmic": "%g B x FRU-substeps" % BYTES_PER_SUBSTEP}},
            "clocks": clk,
            "e2e": e2e,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line))


def main():
    args = parse()
    dist = Dist()
    if args.impl == "reference":
        run_reference(args, dist)
    else:
        run_gpu(args, dist)


if __name__ == "__main__":
    main()

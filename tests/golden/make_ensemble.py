"""Ensemble fixture from the reference program: 64 seeds of the NFRU=250 cell
(ensemble250.npz; `--nfru N` for ensembleN.npz), rest state, 1 Hz pacing,
first beat (1000 ms).  Seed k gives FRU j the MT19937
seed 5489 + 100000*k + j.  Stores per-ms ensemble mean and standard deviation
of V, Cai, mean CaJSR and the LCC / RyR open probabilities, plus each seed's
peak Cai and APD90 (90% repolarisation after the 10-ms stimulus).

Runs the 64 reference programs in parallel (oracle/_ref, built from the
reference's sources); about 45 CPU-minutes at 250 FRUs, 5x that at 1250.
"""
import os
import sys
import tempfile
from concurrent.futures import ProcessPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(HERE)), "oracle"))
import build_ref  # noqa: E402

NSEED, NFRU, T_END = 64, 250, 1000.0


def seed_base(k):
    return 5489 + 100000 * k


def apd90(t, v):
    """Action-potential duration at 90% repolarisation of the first beat."""
    i0 = int(np.argmax(v))
    vmax, vrest = v[i0], v[0]
    thr = vmax - 0.9 * (vmax - vrest)
    up = int(np.argmax(v > thr))
    after = np.nonzero(v[i0:] < thr)[0]
    if len(after) == 0:
        return float("nan")
    return float(t[i0 + after[0]] - t[up])


def one(job):
    k, nfru = job
    d = build_ref.build_config("ens_%d" % nfru, build_ref.cfg_macros(nfru, T_END))
    with tempfile.TemporaryDirectory() as tmp:
        build_ref.run_stoch(d, tmp, seed_base=seed_base(k))
        st = np.loadtxt(os.path.join(tmp, "states.0.txt"), skiprows=1)
        ot = np.loadtxt(os.path.join(tmp, "otherstates.0.txt"), skiprows=1)
    return k, st, ot


def summarise(states, others):
    """states[k][ms][38] (time + 37), others[k][ms][13] -> ensemble summary."""
    V = states[:, :, 1]
    Cai = states[:, :, 7]
    CaJSR = others[:, :, 2]
    PLO = others[:, :, 8]
    PRO = others[:, :, 4]
    t = states[0, :, 0] * 1000.0
    return dict(t_ms=t, V_mean=V.mean(0), V_std=V.std(0), Cai_mean=Cai.mean(0), Cai_std=Cai.std(0),
                CaJSR_mean=CaJSR.mean(0), PLType_open_mean=PLO.mean(0), PRyR_open_mean=PRO.mean(0),
                peak_Cai=Cai.max(1), apd90=np.array([apd90(t, v) for v in V]))


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--nfru", type=int, default=NFRU)
    nfru = ap.parse_args().nfru
    build_ref.build_config("ens_%d" % nfru, build_ref.cfg_macros(nfru, T_END))
    with ProcessPoolExecutor(max_workers=os.cpu_count()) as ex:
        res = sorted(ex.map(one, [(k, nfru) for k in range(NSEED)]))
    states = np.array([r[1] for r in res])
    others = np.array([r[2] for r in res])
    out = summarise(states, others)
    out.update(nseed=np.array([NSEED]), nfru=np.array([nfru]), seed_stride=np.array([100000]))
    np.savez_compressed(os.path.join(HERE, "ensemble%d.npz" % nfru), **out)
    print("apd90 mean %.2f ms, peak Cai mean %.4g mM" % (np.nanmean(out["apd90"]), out["peak_Cai"].mean()))

"""Generate the golden fixtures of tests/golden/ from the reference itself.

Runs only where the reference sources are available (oracle/build_ref.py
builds them serially into oracle/_ref/).  The fixtures are committed; tests
read them and never need the reference at run time.

  mt_kat.npz        first 1300 MT19937 words of five seeds, drawn through the
                    reference's MersenneTwisterOne_local (mt19937_local.c:202),
                    and a sample + sha256 of the per-FRU seeds of
                    initialize_ran.c:30-34 for 12,500 FRUs
  stage_cases.npz   per-FRU results of the reference's simfru_local
                    (simfru_local.c:32) on random FRU states, 6 cases x 64 FRUs
  closed250.npz     the reference's own program (caf.c) at NFRU=250, rest
                    initial state, 1 Hz stimulus, seeds 5489+j, 20 ms:
                    full-precision states/otherstates per ms and the currents
                    of every fcn call that stores them
  beat250.npz       the same program over the first beat (1000 ms): per-ms
                    states/otherstates (no currents) and the final per-FRU channel states,
                    mti and MT-word CRCs

Usage: python tests/golden/make_golden.py [--skip-beat]
"""
import hashlib
import os
import sys
import tempfile
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import build_ref  # noqa: E402
import oracle  # noqa: E402
import reflog  # noqa: E402


def mt_kat():
    R = oracle.ref_lib()
    seeds = np.array([5489, 0, 1, 0xFFFFFFFF, 12350233], np.uint64)
    words = np.zeros((len(seeds), 1300), np.uint32)
    import ctypes as C
    for i, sd in enumerate(seeds):
        mt = np.zeros(624, np.uint32)
        mti = C.c_int(0)
        R.L.ref_sgrnd(int(sd), C.byref(mti), mt)
        for k in range(1300):
            u = R.L.ref_mt_one(C.byref(mti), mt)
            words[i, k] = np.uint32(round(u * 4294967296.0))
    d = build_ref.build_config("lib12500", build_ref.cfg_macros(12500, 10.0), lib=True, exe=False)
    RL = oracle.RefLib(os.path.join(d, "libref.so"))
    mti = np.zeros(12500, np.int32)
    mtw = np.zeros(12500 * 624, np.uint32)
    RL.L.ref_initialize_ran(12500, mti, mtw)
    first = mtw.reshape(12500, 624)[:, 0].copy()  # the seed masked to 32 bits
    idx = np.unique(np.concatenate([np.arange(0, 12500, 97), [0, 1, 2, 719, 720, 721, 12499]]))
    np.savez_compressed(os.path.join(HERE, "mt_kat.npz"), seeds=seeds.astype(np.uint32), words=words,
                        ref_seed_idx=idx.astype(np.int32), ref_seed_val=first[idx],
                        ref_seed_sha256=np.frombuffer(hashlib.sha256(first.tobytes()).digest(), np.uint8))


def random_set(rng, n, base):
    s = oracle.rest_set(n, "base", base)
    s["ltype"][:, :, 0] = rng.integers(1, 13, (n, 4))
    s["ltype"][:, :, 1] = rng.integers(1, 3, (n, 4))
    s["ryr"][:] = rng.integers(1, 9, (n, 4, 5))
    s["ito2"][:] = rng.integers(1, 3, (n, 4))
    s["frus"][:, 0] = rng.uniform(0.05, 1.2, n)
    s["frus"][:, 1:] = 10 ** rng.uniform(-4.5, -0.7, (n, 4))
    adv = rng.integers(0, 1400, n).astype(np.int32)
    import ctypes as C
    L = oracle.lib()
    for j in range(n):
        mti = C.c_int(int(s["mti"][j]))
        row = s["mt"][j]
        for _ in range(int(adv[j])):
            L.orc_next_word(C.byref(mti), row)
        s["mti"][j] = mti.value
    return s, adv


def stage_cases():
    R = oracle.ref_lib()
    rng = np.random.default_rng(20021)
    n = 64
    cases = [  # t0, tf, dep0, depf
        (0.0, 0.002, [-95.4, 7.95e-5, 0.176], [-95.3, 7.96e-5, 0.176]),
        (10.001, 10.011, [-80.0, 1e-4, 0.5], [-20.0, 1.1e-4, 0.5]),
        (12.3, 12.35, [40.0, 2e-4, 0.8], [38.0, 2.5e-4, 0.78]),
        (150.0, 150.004, [0.0, 3e-4, 0.9], [0.0, 3e-4, 0.9]),
        (200.0, 200.1, [-10.0, 5e-4, 1.1], [-12.0, 4.5e-4, 1.05]),
        (500.0, 501.5, [-60.0, 1.2e-4, 0.6], [-70.0, 1.1e-4, 0.62]),
    ]
    out = {}
    for ci, (t0, tf, d0, df) in enumerate(cases):
        s, adv = random_set(rng, n, 1000 + 64 * ci)
        base = 1000 + 64 * ci
        out["c%d_in_ltype" % ci] = s["ltype"].copy()
        out["c%d_in_ryr" % ci] = s["ryr"].copy()
        out["c%d_in_ito2" % ci] = s["ito2"].copy()
        out["c%d_in_frus" % ci] = s["frus"].copy()
        out["c%d_in_base" % ci] = np.array([base], np.int64)
        out["c%d_in_adv" % ci] = adv
        out["c%d_t" % ci] = np.array([t0, tf])
        out["c%d_dep" % ci] = np.array([d0, df], np.float64)
        R.simfru(s, t0, tf, np.array(d0), np.array(df))
        out["c%d_out_ltype" % ci] = s["ltype"]
        out["c%d_out_ryr" % ci] = s["ryr"]
        out["c%d_out_ito2" % ci] = s["ito2"]
        out["c%d_out_frus" % ci] = s["frus"]
        out["c%d_out_mti" % ci] = s["mti"]
        out["c%d_out_mtcrc" % ci] = np.array([zlib.crc32(r.tobytes()) for r in s["mt"]], np.uint32)
        out["c%d_out_flux" % ci] = R.flux_sums(s)
        out["c%d_out_avg" % ci] = R.avg_sums(s)
    out["ncases"] = np.array([len(cases)])
    np.savez_compressed(os.path.join(HERE, "stage_cases.npz"), **out)


def closed_run(nfru, time_end, name, keep_final=False, keep_currents=True):
    d = build_ref.build_config("golden_%d_%d" % (nfru, int(time_end)), build_ref.cfg_macros(nfru, time_end))
    with tempfile.TemporaryDirectory() as tmp:
        log = os.path.join(tmp, "log.bin")
        fin = os.path.join(tmp, "final.bin")
        _, wall = build_ref.run_stoch(d, tmp, seed_base=5489, log=log, dump_final=fin)
        recs = reflog.read_log(log)
        final = oracle.read_dump(fin) if keep_final else None
    A = np.array([p for t, p in recs if t == "A"])
    Cr = np.array([p for t, p in recs if t == "C"])
    counts = {t: sum(1 for r in recs if r[0] == t) for t in "SFVRAC"}
    out = dict(states=A[:, :37], other=A[:, 37:], nfru=np.array([nfru]),
               time_end=np.array([time_end]), seed_base=np.array([5489]),
               counts=np.array([counts[t] for t in "SFVRAC"]), ref_wall_s=np.array([wall]))
    if keep_currents:
        out["currents"] = Cr
    if keep_final:
        out.update(final_ltype=final["ltype"].astype(np.int8), final_ryr=final["ryr"].astype(np.int8),
                   final_ito2=final["ito2"].astype(np.int8), final_frus=final["frus"], final_mti=final["mti"],
                   final_mtcrc=np.array([zlib.crc32(r.tobytes()) for r in final["mt"]], np.uint32))
    np.savez_compressed(os.path.join(HERE, name), **out)
    print(name, "S/F/V/R/A/C", counts, "wall", wall)


if __name__ == "__main__":
    mt_kat()
    stage_cases()
    closed_run(250, 20.0, "closed250.npz", keep_final=True)
    if "--skip-beat" not in sys.argv:
        closed_run(250, 1000.0, "beat250.npz", keep_final=True, keep_currents=False)
    for f in sorted(os.listdir(HERE)):
        print(f, os.path.getsize(os.path.join(HERE, f)))

"""First-beat parity (the FP64 criterion): over the first 1000 ms at NFRU=250
the GPU path and the reference program consume identical MT19937 draw
sequences and end in identical channel states for at least 99% of FRUs, and
the global traces agree.  Every launch shape the FP64 path ships is run:
one thread per FRU, four lanes per FRU (8 FRUs per warp), and the packed
launches the autotuner picks for the FP64 ensemble (4-lane groups taking
FRUs from a queue, 32 FRUs per warp on average)."""
import zlib

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


# (lanes per FRU, packed FRUs per warp; 0 = the fixed layout)
SHAPES = {"1_lane": (1, 0), "4_lanes": (4, 0), "packed_32_fru_per_warp": (4, 32)}


@pytest.mark.parametrize("shape", sorted(SHAPES))
def test_first_beat_transition_sequences(gw, shape):
    lanes, per_warp = SHAPES[shape]
    g = golden("beat250.npz")
    cell = gw.Cell(250, fru_lanes=lanes)
    if per_warp:
        cell.set_stage_packing((250 + per_warp - 1) // per_warp)
    st = gw.settings()
    state = cell.init_rest(st, scheme=gw.SEED_BASE, base=5489)
    _, states, other, _ = cell.run(state, 0.0, 1000, set_=st, want=("states", "other"))
    fin = cell.download()
    crc = np.array([zlib.crc32(r.tobytes()) for r in fin["mt"]], np.uint32)
    same = ((fin["mti"] == g["final_mti"]) & (crc == g["final_mtcrc"]) &
            np.all(fin["ltype"].reshape(250, -1) == g["final_ltype"].reshape(250, -1), axis=1) &
            np.all(fin["ryr"].reshape(250, -1) == g["final_ryr"].reshape(250, -1), axis=1) &
            np.all(fin["ito2"] == g["final_ito2"], axis=1))
    frac = float(np.mean(same))
    print("FRUs with identical draw count, MT state and channel states after beat 1: %.4f" % frac)
    assert frac >= 0.99
    # global traces: V within 0.5 mV, Cai within 1% of its range
    assert np.max(np.abs(states[:, 0] - g["states"][:, 0])) < 0.5
    cai = g["states"][:, 6]
    assert np.max(np.abs(states[:, 6] - cai)) < 0.01 * (cai.max() - cai.min())


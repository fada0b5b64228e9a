"""Launch shapes and the autotuner (gw_autotune): every stage-kernel shape --
1 or 4 lanes per FRU, 1 to 8 warps per block, packed launches that take FRUs
from a queue, alone or batched -- gives the same bits, and tuning leaves the
cells' state as it found it."""
import numpy as np
import pytest

from test_gpu_batch import _cells

pytestmark = pytest.mark.gpu

STEPS = 13  # crosses the 10-ms stimulus


def _run_shape(gw, prec, lanes, warps, n=500):
    cells, sets, states = _cells(gw, [n], prec)
    c = cells[0]
    if lanes == 1:
        c.set_fru_lanes(1)
    if warps < 0:  # packed: a 1/|warps| share of the 8-FRU groups as warps
        c.set_stage_packing(((n + 7) // 8 + (-warps) - 1) // (-warps))
    else:
        c.set_stage_warps(warps)
    st = states[0].copy()
    _, tr, ot, cu = c.run(st, 0.0, STEPS, set_=sets[0])
    return tr, ot, cu, c.download()


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_all_shapes_same_bits(gw, prec):
    shapes = [(4, 1), (4, 2), (4, 4), (4, 8), (4, -2), (4, -4), (4, -16)] + ([(1, 1)] if prec == "fp64" else [])
    ref = _run_shape(gw, prec, *shapes[0])
    for lanes, warps in shapes[1:]:
        got = _run_shape(gw, prec, lanes, warps)
        for a, b, what in zip(got[:3], ref[:3], ("states", "otherstates", "currents")):
            np.testing.assert_array_equal(a, b, err_msg="%s lanes=%d warps=%d" % (what, lanes, warps))
        for k in ("frus", "ltype", "ryr", "ito2", "mti", "mt"):
            np.testing.assert_array_equal(got[3][k], ref[3][k], err_msg="%s lanes=%d warps=%d" % (k, lanes, warps))


def test_batch_warps_same_bits(gw):
    res = []
    for warps in (1, 4):
        cells, sets, states = _cells(gw, [250, 1000, 125], "mixed")
        b = gw.Batch("mixed")
        b.set_warps(warps)
        t = np.zeros(3)
        old = np.full(3, 0.1)
        b.run(cells, sets, t, states, old, STEPS)
        res.append((states.copy(), [c.download()["mt"] for c in cells]))
    np.testing.assert_array_equal(res[0][0], res[1][0])
    for a, b in zip(res[0][1], res[1][1]):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("mode", ["single", "streams", "lockstep"])
def test_autotune_restores_state(gw, mode):
    sizes = [600] if mode == "single" else [300, 900]
    prec = "fp64" if mode == "single" else "mixed"
    cells, sets, states = _cells(gw, sizes, prec)
    t = np.zeros(len(sizes))
    old = np.full(len(sizes), 0.1)
    before = [c.download() for c in cells]
    batch = gw.Batch(prec) if mode == "lockstep" else None
    lanes, warps, ms = gw.autotune(cells, sets, t, states, old, 2.0, batch=batch)
    assert (lanes, warps) in gw.TUNE_CANDIDATES and (lanes, warps) in ms
    assert len(ms) == {"single": 8, "streams": 7, "lockstep": 4}[mode]
    assert ms[(lanes, warps)] == min(ms.values())
    for c, b0 in zip(cells, before):
        got = c.download()
        for k in b0:
            np.testing.assert_array_equal(got[k], b0[k], err_msg=k)
    # the tuned cells continue exactly as untuned ones do
    ref_cells, _, ref_states = _cells(gw, sizes, prec)
    st = states.copy()
    if mode == "single":
        cells[0].run(st[0], 0.0, 4, set_=sets[0], want=())
        ref_cells[0].run(ref_states[0], 0.0, 4, set_=sets[0], want=())
    else:
        run = batch if batch is not None else gw.Batch(prec)
        run.run(cells, sets, t.copy(), st, old.copy(), 4, lockstep=batch is not None)
        gw.Batch(prec).run(ref_cells, sets, np.zeros(len(sizes)), ref_states, np.full(len(sizes), 0.1), 4,
                           lockstep=False)
    np.testing.assert_array_equal(st, ref_states)

"""Batched execution (gw_batch): many cells share one stage launch per round.
Each cell's results must be identical alone and in the mix -- the same
arithmetic and reduction order per cell whatever the batch composition."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cells(gw, sizes, prec, scales=None, first=0):
    cells, sets, states = [], [], []
    for j, n in enumerate(sizes):
        i = first + j
        c = gw.Cell(n, precision=prec, pca_scale=None if scales is None else scales[j][0])
        st = gw.settings(period=[1000.0, 400.0, 700.0, 300.0][i % 4],
                         scale_GKr=1.0 if scales is None else scales[j][1])
        state = c.init_rest(st, scheme=gw.SEED_BASE, base=1000 + 7919 * i)
        cells.append(c)
        sets.append(st)
        states.append(state)
    return cells, sets, np.array(states)


@pytest.mark.parametrize("lockstep", [True, False])
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_same_alone_and_in_the_mix(gw, prec, lockstep):
    sizes = [250, 1000, 125, 600]
    scales = [(1.0, 1.0), (1.2, 0.8), (0.9, 1.1), (1.0, 1.3)]
    steps = 12
    # alone: each cell by itself through the single-cell path
    alone = []
    for i in range(len(sizes)):
        cells, sets, states = _cells(gw, [sizes[i]], prec, [scales[i]], first=i)
        st = states[0].copy()
        cells[0].run(st, 0.0, steps, set_=sets[0], want=())
        alone.append((st, cells[0].download()))
    # in the mix: all four in one batch
    cells, sets, states = _cells(gw, sizes, prec, scales)
    b = gw.Batch(prec)
    t = np.zeros(len(sizes))
    old = np.full(len(sizes), 0.1)
    b.run(cells, sets, t, states, old, steps, lockstep=lockstep)
    for i in range(len(sizes)):
        np.testing.assert_array_equal(states[i], alone[i][0], err_msg="cell %d global state" % i)
        got = cells[i].download()
        for k in ("ltype", "ryr", "ito2", "mti", "mt", "frus"):
            np.testing.assert_array_equal(got[k], alone[i][1][k], err_msg="cell %d %s" % (i, k))
    assert np.all(t == steps)


def test_cells_join_and_leave(gw):
    # a member that finishes early leaves; the others keep going
    cells, sets, states = _cells(gw, [200, 300], "mixed")
    b = gw.Batch("mixed")
    t = np.zeros(2)
    old = np.full(2, 0.1)
    b.run(cells[:1], sets[:1], t[:1], states[:1], old[:1], 3)
    b.run(cells, sets, t, states, old, 2)
    assert t[0] == 5 and t[1] == 2

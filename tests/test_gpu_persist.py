"""Persistent multi-cell kernel (gw_run_persistent): every cell's FRU stages,
flux reductions and Dormand-Prince steps inside one resident launch.

- Against the round-based device runner (gw_run_device), which shares the
  integrator, the stage arithmetic and the fixed reduction order: the same
  bits for every cell (global states, traces, FRU state and MT19937 words),
  in FP64 and in mixed precision, with cells of uneven FRU count, pacing
  cycle length and conductance scales.
- A cell's result is the same alone and in the mix, whatever the number of
  8-FRU groups a warp takes at once, and the same whether a run is made in
  one call or split into several.
- The wait limit: when a flag that nothing sets holds a cell's next
  operation, every warp gives up after the limit and the launch returns an
  error status; the context stays usable."""
import numpy as np
import pytest

from test_gpu_batch import _cells

pytestmark = pytest.mark.gpu

SIZES = [250, 1000, 125, 600]
SCALES = [(1.0, 1.0), (1.2, 0.8), (0.9, 1.1), (1.0, 1.3)]


def _run(gw, sizes, prec, steps, persistent, scales=None, split=None, first=0):
    cells, sets, states = _cells(gw, sizes, prec, scales, first=first)
    t = np.zeros(len(sizes))
    old = np.full(len(sizes), 0.1)
    trs = []
    for n in (split or [steps]):
        trs.append(gw.run_device(cells, sets, t, states, old, n, traces=True, persistent=persistent))
    tr = tuple(np.concatenate([x[k] for x in trs], axis=1) for k in range(3))
    fin = [c.download() for c in cells]
    for c in cells:
        c.close()
    return states, t, old, tr, fin


def _same(a, b):
    sa, ta, oa, tra, fa = a
    sb, tb, ob, trb, fb = b
    np.testing.assert_array_equal(sa, sb)
    np.testing.assert_array_equal(ta, tb)
    np.testing.assert_array_equal(oa, ob)
    for x, y in zip(tra, trb):
        np.testing.assert_array_equal(x, y)
    for da, db in zip(fa, fb):
        for k in da:
            np.testing.assert_array_equal(da[k], db[k], err_msg=k)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_persistent_matches_round_runner(gw, prec):
    steps = 12
    dev = _run(gw, SIZES, prec, steps, persistent=False, scales=SCALES)
    per = _run(gw, SIZES, prec, steps, persistent=True, scales=SCALES)
    _same(dev, per)
    assert np.all(per[1] == steps)


@pytest.mark.parametrize("groups", ["3", "8"])
def test_persistent_batch_sizes_same_bits(gw, groups, monkeypatch):
    """Warps taking 3 or 8 groups of 8 FRUs at a time (partial batches at
    every cell's end, groups taking the batch's FRUs as they finish) give
    the round runner's bits."""
    steps = 8
    dev = _run(gw, SIZES, "fp64", steps, persistent=False, scales=SCALES)
    monkeypatch.setenv("GW_PERSIST_GROUPS", groups)
    per = _run(gw, SIZES, "fp64", steps, persistent=True, scales=SCALES)
    _same(dev, per)


def test_persistent_same_alone_and_in_the_mix(gw):
    steps = 10
    mix = _run(gw, SIZES, "fp64", steps, persistent=True, scales=SCALES)
    for i in range(len(SIZES)):
        one = _run(gw, [SIZES[i]], "fp64", steps, persistent=True, scales=[SCALES[i]], first=i)
        np.testing.assert_array_equal(one[0][0], mix[0][i])
        for x, y in zip(one[3], mix[3]):
            np.testing.assert_array_equal(x[0], y[i])
        for k in one[4][0]:
            np.testing.assert_array_equal(one[4][0][k], mix[4][i][k], err_msg=k)


def test_persistent_split_calls_same_bits(gw):
    whole = _run(gw, [300, 200], "mixed", 12, persistent=True)
    split = _run(gw, [300, 200], "mixed", 12, persistent=True, split=[5, 7])
    _same(whole, split)


def test_persistent_wait_limit_returns_an_error_status(gw):
    cells, sets, states = _cells(gw, [500], "fp64")
    status = gw.persist_watchdog(cells[0], sets[0], 0.3)
    assert status == 3
    # the context is usable afterwards: a regular run from the same state
    st = states[0].copy()
    t, tr, _, _ = cells[0].run(st, 0.0, 2, set_=sets[0], want=("states",))
    assert t == 2.0 and np.all(np.isfinite(tr))


def test_warp_fcn_same_bits_as_one_thread(gw):
    """The warp form of the global right-hand side (its exponentials, logs
    and powers one per lane) returns the one-thread form's derivatives and
    currents bit for bit, over states spread around the action potential and
    under a voltage clamp."""
    rng = np.random.default_rng(11)
    cell = gw.Cell(50)
    rest = cell.init_rest(gw.settings(), scheme=gw.SEED_BASE, base=1)
    cell.close()
    n = 512
    st = np.tile(rest, (n, 1))
    st[:, 0] = rng.uniform(-100.0, 60.0, n)                # V across the action potential
    st[:, 1:] *= rng.uniform(0.7, 1.3, (n, 36))             # gates and concentrations around rest
    st[:5, 0] = [-47.13, 10.0, 0.0, -90.5, -38.7]          # the branch points of fcn
    for time, clamp in ((5.0, False), (10.5, False), (120.0, True)):
        Fs, Fw, Cs, Cw = gw.fcn_thread_vs_warp(st, time, clamp=clamp)
        np.testing.assert_array_equal(Fs, Fw)
        np.testing.assert_array_equal(Cs, Cw)
    assert np.all(np.isfinite(Fs))

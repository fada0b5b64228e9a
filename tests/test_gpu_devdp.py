"""Device-resident integrator (gw_run_device): the Dormand-Prince step and the
global right-hand side on the GPU, one CUDA graph per run.

- A cell's result does not depend on the other cells of the run, nor on
  how the run is split into calls (bit for bit).
- Against the host integrator (gw_run) on the same cell and seeds: the two
  differ only where CUDA's exp/pow/log round differently from the host C
  library in the last place, so over a paced 15-ms window (through the
  stimulus) the FRU channel states, MT19937 positions and words agree for at
  least 99% of FRUs and the membrane potential within 0.05 mV."""
import numpy as np
import pytest

from test_gpu_batch import _cells

pytestmark = pytest.mark.gpu


def _dev_run(gw, sizes, prec, steps, split=None):
    cells, sets, states = _cells(gw, sizes, prec)
    t = np.zeros(len(sizes))
    old = np.full(len(sizes), 0.1)
    trs = []
    for n in (split or [steps]):
        trs.append(gw.run_device(cells, sets, t, states, old, n, traces=True))
    tr = tuple(np.concatenate([x[k] for x in trs], axis=1) for k in range(3))
    return cells, states, t, old, tr


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_same_alone_and_in_the_mix(gw, prec):
    sizes = [250, 1000, 125]
    _, st_mix, t_mix, old_mix, tr_mix = _dev_run(gw, sizes, prec, 12)
    for i, n in enumerate(sizes):
        cells, sets, states = _cells(gw, sizes, prec)
        t = np.zeros(1)
        old = np.full(1, 0.1)
        st = np.ascontiguousarray(states[i:i + 1])
        tr = gw.run_device([cells[i]], [sets[i]], t, st, old, 12, traces=True)
        np.testing.assert_array_equal(st[0], st_mix[i])
        for a, b in zip(tr, tr_mix):
            np.testing.assert_array_equal(a[0], b[i])
        assert t[0] == t_mix[i] and old[0] == old_mix[i]


def test_split_calls_same_bits(gw):
    sizes = [300, 200]
    c1, s1, t1, o1, tr1 = _dev_run(gw, sizes, "fp64", 12)
    c2, s2, t2, o2, tr2 = _dev_run(gw, sizes, "fp64", 12, split=[5, 7])
    np.testing.assert_array_equal(s1, s2)
    for a, b in zip(tr1, tr2):
        np.testing.assert_array_equal(a, b)
    for a, b in zip(c1, c2):
        d1, d2 = a.download(), b.download()
        for k in d1:
            np.testing.assert_array_equal(d1[k], d2[k], err_msg=k)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_matches_host_integrator(gw, prec):
    n, steps = 500, 15
    cells, sets, states = _cells(gw, [n], prec)
    st_host = states[0].copy()
    _, tr_host, ot_host, cu_host = cells[0].run(st_host, 0.0, steps, set_=sets[0])
    host = cells[0].download()
    cells, sets, states = _cells(gw, [n], prec)
    t = np.zeros(1)
    old = np.full(1, 0.1)
    tr_dev, ot_dev, cu_dev = gw.run_device(cells, sets, t, states, old, steps, traces=True)
    dev = cells[0].download()
    same = np.all(host["ltype"] == dev["ltype"], axis=(1, 2)) & np.all(host["ryr"] == dev["ryr"], axis=(1, 2)) & \
        np.all(host["ito2"] == dev["ito2"], axis=1) & (host["mti"] == dev["mti"]) & np.all(host["mt"] == dev["mt"], axis=1)
    dv = np.max(np.abs(tr_dev[0][:, 0] - tr_host[:, 0]))
    print("%s: FRUs identical %.4f, max |dV| %.3g mV, max |dCai| rel %.3g" % (
        prec, same.mean(), dv, np.max(np.abs(tr_dev[0][:, 6] - tr_host[:, 6]) / np.abs(tr_host[:, 6]))))
    assert same.mean() >= 0.99
    assert dv < 0.05
    assert t[0] == steps
    np.testing.assert_allclose(ot_dev[0][:, 1], ot_host[:, 1], rtol=1e-3)


def test_non_finite_state_stops_both_integrators(gw):
    """A cell whose global state is not finite (NaN in the total-Ca
    accumulator, state 31, which feeds no other derivative, so the FRU
    launches see finite inputs) ends the run with an error, on the device
    integrator and on the host one, instead of crawling at the minimum step."""
    cells, sets, states = _cells(gw, [200, 300], "fp64")
    states[1, 31] = np.nan
    with pytest.raises(gw.GWError, match="not finite"):
        gw.run_device(cells, sets, np.zeros(2), states, np.full(2, 0.1), 2)
    cells, sets, states = _cells(gw, [200], "fp64")
    state = np.ascontiguousarray(states[0])
    state[31] = np.nan
    with pytest.raises(gw.GWError, match="not finite"):
        cells[0].run(state, 0.0, 1, set_=sets[0])

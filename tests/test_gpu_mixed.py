"""Mixed precision (FP32 rates and FRU-local Ca ODE, FP64 FRU state, clock and
flux sums) against the FP64 path with the same seeds, and the total-Ca
conservation check of the reference (initialize_state.c:230-247,
mpi_master.c:180-184) for both paths.

Tolerances (stated here): after one stage from random states, >= 95% of FRUs
keep identical channel states and MT positions and Ca states agree to 1e-4
relative where they do; over a paced 20-ms window the membrane potential
stays within 2 mV of the FP64 trace and the peak within 1 mV; total cell Ca
is conserved to 1e-3 relative."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def _random_set(rng, n, base):
    s = O.rest_set(n, "base", base)
    s["ltype"][:, :, 0] = rng.integers(1, 13, (n, 4))
    s["ltype"][:, :, 1] = rng.integers(1, 3, (n, 4))
    s["ryr"][:] = rng.integers(1, 9, (n, 4, 5))
    s["ito2"][:] = rng.integers(1, 3, (n, 4))
    s["frus"][:, 0] = rng.uniform(0.05, 1.2, n)
    s["frus"][:, 1:] = 10 ** rng.uniform(-4.5, -1.0, (n, 4))
    s["mti"][:] = rng.integers(0, 625, n)
    return s


def test_mixed_stage_tracks_fp64(gw):
    rng = np.random.default_rng(8)
    n = 3000
    s = _random_set(rng, n, 31)
    out = {}
    for prec in ("fp64", "mixed"):
        cell = gw.Cell(n, precision=prec)
        cell.upload(s)
        nums = [cell.stage(1.0, 1.002, [-40.0, 2e-4, 0.7], [-38.0, 2.1e-4, 0.69])[1]]
        out[prec] = (np.array(nums), cell.download())
    a, b = out["fp64"][1], out["mixed"][1]
    same = ((a["mti"] == b["mti"]) & np.all(a["ryr"].reshape(n, -1) == b["ryr"].reshape(n, -1), axis=1) &
            np.all(a["ltype"].reshape(n, -1) == b["ltype"].reshape(n, -1), axis=1) &
            np.all(a["ito2"] == b["ito2"], axis=1))
    assert same.mean() >= 0.95, same.mean()
    rel = np.abs(a["frus"][same] - b["frus"][same]) / np.abs(a["frus"][same])
    assert rel.max() < 1e-4, rel.max()


@pytest.mark.parametrize("v_uV", [1.5, 3.0, 30.0, -2.0])
def test_mixed_ghk_near_zero_potential(gw, v_uV):
    """The GHK factor of the LCC flux at membrane potentials of a few uV
    (just above the reference's |V| < 1e-6 mV branch): the FP32 path keeps
    e - 1 from expm1, so the FRU Ca states stay finite and track FP64."""
    rng = np.random.default_rng(12)
    n = 2000
    s = _random_set(rng, n, 77)
    v = v_uV * 1e-3
    out = {}
    for prec in ("fp64", "mixed"):
        cell = gw.Cell(n, precision=prec)
        cell.upload(s)
        num = cell.stage(5.0, 5.05, [v, 2e-4, 0.7], [v, 2e-4, 0.7])[1]
        out[prec] = (num, cell.download()["frus"])
    assert np.all(np.isfinite(out["mixed"][1])) and np.all(np.isfinite(out["mixed"][0]))
    np.testing.assert_allclose(out["mixed"][0][:3], out["fp64"][0][:3], rtol=1e-2)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_total_calcium_is_conserved(gw, prec):
    cell = gw.Cell(250, precision=prec)
    st = gw.settings()
    state = cell.init_rest(st, scheme=gw.SEED_BASE, base=5489)
    _, states, other, _ = cell.run(state, 0.0, 20, set_=st)
    catot, catot2 = states[:, 31], other[:, 8]
    assert np.max(np.abs(catot - catot2) / catot) < 1e-3


def test_mixed_closed_loop_tracks_fp64(gw):
    traces = {}
    for prec in ("fp64", "mixed"):
        cell = gw.Cell(1000, precision=prec)
        st = gw.settings()
        state = cell.init_rest(st, scheme=gw.SEED_BASE, base=5489)
        _, states, _, _ = cell.run(state, 0.0, 20, set_=st)
        traces[prec] = states[:, 0]
    d = np.abs(traces["fp64"] - traces["mixed"])
    print("max |dV| over 20 ms: %.3g mV; peak V fp64 %.3f mixed %.3f" %
          (d.max(), traces["fp64"].max(), traces["mixed"].max()))
    assert d.max() < 2.0
    assert abs(traces["fp64"].max() - traces["mixed"].max()) < 1.0

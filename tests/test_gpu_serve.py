"""Serving (gw_server): requests of different FRU counts and protocols arrive
while others run, are admitted by device bytes, and share stage launches.
Each result must be the same alone and in the mix."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _req(gw, nfru, seed, clamp=False, period=1000.0, dur=12.0):
    r = gw.Request()
    r.nfru = nfru
    if clamp:
        r.set = gw.settings(vclamp_flag=1, vclamp_hold=-100.0, vclamp_set=10.0, vclamp_duration=200.0,
                            vclamp_shift=5.0, vclamp_period=1000.0)
    else:
        r.set = gw.settings(period=period)
    r.seed_scheme = gw.SEED_BASE
    r.seed = seed
    r.pca_scale = 1.0
    r.duration_ms = dur
    return r


@pytest.mark.parametrize("lockstep", [False, True])
@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_result_same_alone_and_in_the_mix(gw, prec, lockstep):
    dur = 12
    # alone
    srv = gw.Server(prec, slots=4, mem_budget_bytes=8 << 30, lockstep=lockstep)
    a = _req(gw, 500, 77, clamp=False, dur=dur)
    va, fa = np.zeros(dur), np.zeros(37)
    srv.submit(a, va, fa)
    srv.wait()
    srv.close()
    assert a.status == 0
    # in a mix of pacing and clamp requests of other sizes
    srv = gw.Server(prec, slots=6, mem_budget_bytes=8 << 30, lockstep=lockstep)
    reqs = [_req(gw, 300, 5, clamp=True, dur=dur), _req(gw, 800, 9, period=400.0, dur=dur),
            _req(gw, 500, 77, clamp=False, dur=dur), _req(gw, 150, 3, clamp=True, dur=dur)]
    outs = [(np.zeros(dur), np.zeros(37)) for _ in reqs]
    for r, (v, f) in zip(reqs, outs):
        srv.submit(r, v, f)
    srv.wait()
    srv.close()
    assert all(r.status == 0 for r in reqs)
    np.testing.assert_array_equal(outs[2][0], va)
    np.testing.assert_array_equal(outs[2][1], fa)
    # the clamp requests hold V at the clamp levels
    assert np.all(np.abs(outs[0][0][:3] + 100.0) < 1e-9) and abs(outs[0][0][-1] - 10.0) < 1e-9


def test_admission_by_device_bytes(gw):
    # a budget that fits two 1000-FRU cells: never more than two run at once
    budget = 2 * gw.cell_bytes(1000) + 1024
    srv = gw.Server("mixed", slots=8, mem_budget_bytes=budget)
    reqs = [_req(gw, 1000, 100 + i, dur=4) for i in range(6)]
    for r in reqs:
        srv.submit(r)
    srv.wait()
    srv.close()
    assert all(r.status == 0 for r in reqs)
    ev = sorted([(r.t_start, 1) for r in reqs] + [(r.t_done, -1) for r in reqs])
    live = peak = 0
    for _, d in ev:
        live += d
        peak = max(peak, live)
    assert peak <= 2


def test_failed_request_carries_its_message(gw):
    """A request that fails (here: an unknown seeding scheme, refused on the
    host before any launch) reports its status and message; the requests
    beside it run normally."""
    srv = gw.Server("mixed", slots=2, mem_budget_bytes=1 << 30)
    bad, good = _req(gw, 200, 1, dur=2), _req(gw, 200, 2, dur=2)
    bad.seed_scheme = 7
    srv.submit(bad)
    srv.submit(good)
    srv.wait()
    srv.close()
    assert bad.status != 0 and b"scheme 7" in bad.message
    assert good.status == 0 and good.message == b""


def test_held_bytes_never_exceed_the_budget(gw):
    """Pooled idle contexts count against the budget: with room for two
    1000-FRU cells, requests of another size first free idle contexts, and
    the bytes held never pass the budget."""
    budget = 2 * gw.cell_bytes(1000) + 1024
    srv = gw.Server("mixed", slots=4, mem_budget_bytes=budget)
    reqs = [_req(gw, 1000, 200 + i, dur=3) for i in range(3)] + [_req(gw, 700, 300 + i, dur=3) for i in range(3)]
    for r in reqs:
        srv.submit(r)
    srv.wait()
    st = srv.stats()
    srv.close()
    assert all(r.status == 0 for r in reqs)
    assert st["peak_held"] <= budget
    assert st["frees"] >= 1  # idle 1000-FRU contexts made room for the 700-FRU cells


def test_reserved_contexts_allocate_nothing_while_running(gw):
    srv = gw.Server("mixed", slots=4, mem_budget_bytes=8 << 30)
    srv.reserve(400, 3)
    srv.reserve(900, 3)
    a0 = srv.stats()["allocs"]
    reqs = [_req(gw, 400, 10 + i, dur=3) for i in range(3)] + [_req(gw, 900, 20 + i, dur=3) for i in range(3)]
    for r in reqs:
        srv.submit(r)
    srv.wait()
    st = srv.stats()
    srv.close()
    assert all(r.status == 0 for r in reqs)
    assert st["allocs"] == a0 == 6

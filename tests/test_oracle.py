"""The CPU oracle pinned against the reference: golden fixtures generated from
the reference itself (tests/golden/make_golden.py), a published MT19937
known answer, and -- where the reference sources are present -- live
comparisons with the reference's own routines."""
import ctypes as C
import hashlib
import zlib

import numpy as np
import pytest

import oracle as O
from conftest import golden


def test_mt19937_published_kat():
    # C++11 [rand.predef]: the 10000th output of a default-seeded (5489)
    # mt19937 is 4123659995.  sgrnd_local (mt19937_local.c:76) uses the same
    # Knuth initialisation.
    w = O.mt_words(5489, 10000)
    assert int(w[-1]) == 4123659995


def test_mt_streams_match_reference():
    g = golden("mt_kat.npz")
    for sd, words in zip(g["seeds"], g["words"]):
        np.testing.assert_array_equal(O.mt_words(int(sd), words.size), words)


def test_reference_seed_formula():
    # initialize_ran.c:30-34 with 32-bit wrap-around, 12,500 FRUs
    g = golden("mt_kat.npz")
    s = O.seeds(12500, "reference")
    np.testing.assert_array_equal(s[g["ref_seed_idx"]], g["ref_seed_val"])
    assert hashlib.sha256(s.tobytes()).digest() == g["ref_seed_sha256"].tobytes()


def _case_inputs(g, ci):
    n = g["c%d_in_ltype" % ci].shape[0]
    s = O.rest_set(n, "base", int(g["c%d_in_base" % ci][0]))
    L = O.lib()
    for j, adv in enumerate(g["c%d_in_adv" % ci]):
        mti = C.c_int(int(s["mti"][j]))
        for _ in range(int(adv)):
            L.orc_next_word(C.byref(mti), s["mt"][j])
        s["mti"][j] = mti.value
    s["ltype"][:] = g["c%d_in_ltype" % ci]
    s["ryr"][:] = g["c%d_in_ryr" % ci]
    s["ito2"][:] = g["c%d_in_ito2" % ci]
    s["frus"][:] = g["c%d_in_frus" % ci]
    return s


def test_stage_cases_match_reference_bitwise():
    g = golden("stage_cases.npz")
    for ci in range(int(g["ncases"][0])):
        s = _case_inputs(g, ci)
        t0, tf = g["c%d_t" % ci]
        d0, df = g["c%d_dep" % ci]
        O.simfru(s, t0, tf, d0, df)
        for k in ("ltype", "ryr", "ito2", "frus", "mti"):
            np.testing.assert_array_equal(s[k], g["c%d_out_%s" % (ci, k)], err_msg="case %d %s" % (ci, k))
        crc = np.array([zlib.crc32(r.tobytes()) for r in s["mt"]], np.uint32)
        np.testing.assert_array_equal(crc, g["c%d_out_mtcrc" % ci])
        np.testing.assert_array_equal(O.flux_sums(s), g["c%d_out_flux" % ci])
        np.testing.assert_array_equal(O.avg_sums(s), g["c%d_out_avg" % ci])


def test_zero_length_stage_is_identity():
    s = O.rest_set(8)
    before = O.copy_set(s)
    O.simfru(s, 5.0, 5.0, np.array([-90.0, 1e-4, 0.5]), np.array([-90.0, 1e-4, 0.5]))
    for k in s:
        np.testing.assert_array_equal(s[k], before[k])


def test_twist_boundary_draws():
    # draws that straddle a regeneration (mti = 600..624) give the plain stream
    ref = O.mt_words(77, 700)
    L = O.lib()
    for start in (600, 610, 623, 624):
        mt = np.zeros(624, np.uint32)
        mti = C.c_int(0)
        L.orc_sgrnd(77, C.byref(mti), mt)
        got = [L.orc_next_word(C.byref(mti), mt) for _ in range(start)]
        got += [L.orc_next_word(C.byref(mti), mt) for _ in range(32)]
        np.testing.assert_array_equal(np.array(got, np.uint32), ref[:start + 32])


def test_closed_loop_host_driver_matches_reference(cpu_cell_lib):
    """The product's host Dormand-Prince driver and global model (gw_dp.c,
    gw_cell_model.h) over the oracle's FRU stages reproduce the reference
    program bit for bit: NFRU=250, rest state, 1 Hz, seeds 5489+j, 20 ms."""
    import greenstein2002_gb300 as G
    g = golden("closed250.npz")
    cell = G.Cell(250, lib=cpu_cell_lib)
    st = G.settings()
    state = cell.init_rest(st, scheme=G.SEED_BASE, base=5489)
    _, states, other, cur = cell.run(state, 0.0, 20, set_=st)
    np.testing.assert_array_equal(states, g["states"])
    np.testing.assert_array_equal(other, g["other"])
    np.testing.assert_array_equal(cur, g["currents"][:, 1:])
    fin = cell.download()
    np.testing.assert_array_equal(fin["mti"], g["final_mti"])
    np.testing.assert_array_equal(fin["ryr"], g["final_ryr"])


def test_integrator_stops_on_non_finite_state(cpu_cell_lib):
    """A global state that is not finite stops the run with an error instead
    of being force-accepted at the minimum step over and over (NaN in the
    total-Ca accumulator, state 31, which feeds no other derivative)."""
    import greenstein2002_gb300 as G
    cell = G.Cell(32, lib=cpu_cell_lib)
    st = G.settings()
    state = cell.init_rest(st, scheme=G.SEED_BASE, base=5489)
    state[31] = np.nan
    with pytest.raises(G.GWError, match="not finite"):
        cell.run(state, 0.0, 1, set_=st)


@pytest.fixture(scope="module")
def ref():
    r = O.ref_lib()
    if r is None:
        pytest.skip("reference sources not available")
    return r


def test_oracle_matches_reference_live(ref):
    rng = np.random.default_rng(7)
    for trial in range(10):
        n = 48
        s = O.rest_set(n, "base", 3000 + trial)
        s["ltype"][:, :, 0] = rng.integers(1, 13, (n, 4))
        s["ltype"][:, :, 1] = rng.integers(1, 3, (n, 4))
        s["ryr"][:] = rng.integers(1, 9, (n, 4, 5))
        s["ito2"][:] = rng.integers(1, 3, (n, 4))
        s["frus"][:, 0] = rng.uniform(0.05, 1.2, n)
        s["frus"][:, 1:] = 10 ** rng.uniform(-4.5, -0.5, (n, 4))
        s["mti"][:] = rng.integers(0, 625, n)
        a, b = O.copy_set(s), O.copy_set(s)
        v0 = rng.uniform(-100, 60)
        d0 = np.array([v0, 1e-4, 0.5])
        df = np.array([v0 + rng.uniform(-5, 5), 1.2e-4, 0.49])
        t0 = rng.uniform(0, 100)
        tf = t0 + rng.uniform(1e-4, 0.05)
        O.simfru(a, t0, tf, d0, df)
        ref.simfru(b, t0, tf, d0, df)
        for k in a:
            np.testing.assert_array_equal(a[k], b[k], err_msg="trial %d %s" % (trial, k))
        np.testing.assert_array_equal(O.flux_sums(a), ref.flux_sums(b))
        np.testing.assert_array_equal(O.avg_sums(a), ref.avg_sums(b))

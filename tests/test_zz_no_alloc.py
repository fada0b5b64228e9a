"""The allocation-free stage entry point (gw_stage_noalloc).

Some callers cannot allocate device memory while they run: cudaMalloc
synchronises the whole device (stalling a serving loop's other streams), is
not allowed during CUDA-graph stream capture, and is off limits to hosts
that own all device memory.  For them gw_stage_noalloc advances FRU arrays
the caller already owns, keeping its reduction scratch in a fixed array
inside the library.  Here it is called through the C-ABI on caller-owned
device buffers and must give the same FRU states and fluxes as the regular
gw_stage, on two calls in a row.

This file is collected last so that a run stopping at the first failure has
already run every other test."""
import ctypes as C

import numpy as np
import pytest

import oracle as O

RTOL = 1e-12
MT_STRIDE = 640


def _pack(s, stride):
    n = s["frus"].shape[0]
    frus = np.zeros((5, stride))
    frus[:, :n] = s["frus"].T
    chan = np.zeros((4, stride), np.uint32)
    for c in range(4):
        w = (s["ltype"][:, c, 0].astype(np.uint32) | (s["ltype"][:, c, 1].astype(np.uint32) << 4) |
             (s["ito2"][:, c].astype(np.uint32) << 28))
        for i in range(5):
            w |= s["ryr"][:, c, i].astype(np.uint32) << (8 + 4 * i)
        chan[c, :n] = w
    mti = np.zeros(stride, np.int32)
    mti[:n] = s["mti"]
    mt = np.zeros((n, MT_STRIDE), np.uint32)
    mt[:, :624] = s["mt"]
    return frus, chan, mti, mt


def _unpack(frus, chan, mti, mt, n):
    s = {"frus": frus[:, :n].T.copy(), "mti": mti[:n].copy(), "mt": mt[:, :624].copy(),
         "ltype": np.zeros((n, 4, 2), np.int32), "ryr": np.zeros((n, 4, 5), np.int32), "ito2": np.zeros((n, 4), np.int32)}
    for c in range(4):
        w = chan[c, :n]
        s["ltype"][:, c, 0] = w & 15
        s["ltype"][:, c, 1] = (w >> 4) & 15
        s["ito2"][:, c] = w >> 28
        for i in range(5):
            s["ryr"][:, c, i] = (w >> (8 + 4 * i)) & 15
    return s


def _bind(lib):
    f = lib.gw_stage_noalloc
    f.argtypes = [C.c_int, C.c_int] + [C.c_void_p] * 4 + [C.c_double, C.c_double, C.c_void_p, C.c_void_p,
                                                          C.c_double, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return f


def test_noalloc_rejects_oversized_cells():
    import greenstein2002_gb300 as G
    f = _bind(G.load())
    d = (C.c_double * 3)(0.0, 0.0, 0.0)
    rc = f(65537, 65537, 1, 1, 1, 1, 0.0, 1.0, d, d, 1.0, 1, None)
    assert rc == 1  # GW_EINVAL
    assert b"65536" in G.load().gw_last_error()


@pytest.mark.gpu
def test_noalloc_stage_matches_gw_stage(gw):
    torch = pytest.importorskip("torch")
    n, stride = 2000, 2016
    rng = np.random.default_rng(99)
    s = O.rest_set(n, "base", 4242)
    s["ltype"][:, :, 0] = rng.integers(1, 13, (n, 4))
    s["ryr"][:] = rng.integers(1, 9, (n, 4, 5))
    s["frus"][:, 0] = rng.uniform(0.2, 1.0, n)
    s["frus"][:, 1:] = 10 ** rng.uniform(-4.3, -1.5, (n, 4))
    s["mti"][:] = rng.integers(0, 625, n)
    stages = [(2.0, 2.004, [-30.0, 2e-4, 0.8], [-28.0, 2.1e-4, 0.79]),
              (2.004, 2.011, [-30.0, 2e-4, 0.8], [-25.0, 2.2e-4, 0.78])]

    # the regular entry point
    cell = gw.Cell(n)
    cell.upload(s)
    want = []
    for t0, tf, d0, df in stages:
        out, num = cell.stage(t0, tf, d0, df)
        want.append((num, out, cell.download()))

    # the allocation-free entry point on caller-owned device buffers
    f = _bind(gw.load())
    dev = torch.device("cuda:0")
    frus, chan, mti, mt = _pack(s, stride)
    t_frus = torch.from_numpy(frus).to(dev)
    t_chan = torch.from_numpy(chan.view(np.int32)).to(dev)
    t_mti = torch.from_numpy(mti).to(dev)
    t_mt = torch.from_numpy(mt.view(np.int32)).to(dev)
    t_out = torch.zeros(10, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    for k, (t0, tf, d0, df) in enumerate(stages):
        rc = f(n, stride, t_frus.data_ptr(), t_chan.data_ptr(), t_mti.data_ptr(), t_mt.data_ptr(), t0, tf,
               (C.c_double * 3)(*d0), (C.c_double * 3)(*df), 12500.0 / n, t_out.data_ptr(), C.c_void_p(stream))
        assert rc == 0, gw.load().gw_last_error()
        torch.cuda.synchronize()
        out = t_out.cpu().numpy()
        got = _unpack(t_frus.cpu().numpy(), t_chan.cpu().numpy().view(np.uint32), t_mti.cpu().numpy(),
                      t_mt.cpu().numpy().view(np.uint32), n)
        num_w, cur_w, st_w = want[k]
        assert out[9] == 0.0
        np.testing.assert_allclose(out[:5], num_w, rtol=RTOL)
        np.testing.assert_allclose(out[5:9], cur_w, rtol=RTOL)
        for key in ("ltype", "ryr", "ito2", "mti", "mt"):
            np.testing.assert_array_equal(got[key], st_w[key], err_msg="call %d %s" % (k, key))
        np.testing.assert_allclose(got["frus"], st_w["frus"], rtol=RTOL, atol=0)


@pytest.mark.gpu
def test_noalloc_flags_out_of_range_fru_state(gw):
    """The caller's arrays bypass gw_upload's checks, so the kernel checks
    each FRU before it reads the MT row or the rate tables: an FRU whose mti
    or channel state is out of range is left unchanged and out[9] reads 2."""
    torch = pytest.importorskip("torch")
    n, stride = 64, 64
    s = O.rest_set(n, "base", 77)
    s["mti"][5] = 700            # past the 624-word MT row
    s["ltype"][9, 2, 0] = 0      # no LCC state 0
    f = _bind(gw.load())
    dev = torch.device("cuda:0")
    frus, chan, mti, mt = _pack(s, stride)
    t_frus = torch.from_numpy(frus).to(dev)
    t_chan = torch.from_numpy(chan.view(np.int32)).to(dev)
    t_mti = torch.from_numpy(mti).to(dev)
    t_mt = torch.from_numpy(mt.view(np.int32)).to(dev)
    t_out = torch.zeros(10, dtype=torch.float64, device=dev)
    d0, df = [-80.0, 1e-4, 0.7], [-79.0, 1e-4, 0.7]
    rc = f(n, stride, t_frus.data_ptr(), t_chan.data_ptr(), t_mti.data_ptr(), t_mt.data_ptr(), 0.0, 0.1,
           (C.c_double * 3)(*d0), (C.c_double * 3)(*df), 12500.0 / n, t_out.data_ptr(),
           C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, gw.load().gw_last_error()
    torch.cuda.synchronize()
    assert t_out[9].item() == 2.0
    got = _unpack(t_frus.cpu().numpy(), t_chan.cpu().numpy().view(np.uint32), t_mti.cpu().numpy(),
                  t_mt.cpu().numpy().view(np.uint32), n)
    for bad in (5, 9):
        np.testing.assert_array_equal(got["mt"][bad], s["mt"][bad])
        assert got["mti"][bad] == s["mti"][bad]
        np.testing.assert_array_equal(got["frus"][bad], s["frus"][bad])
    assert np.any(got["mti"] != s["mti"])  # the valid FRUs advanced

"""Coefficient extraction and formatting: getCoeffLevel's index sets
(R/rplotting.R:10-46) and WSTtoDT's level / translate / type columns
(R/rfunctions.R:925-1004).  The oracle restates the R code step by step (its
initial labelling and per-level overwrites); the library computes the
closed form on the device.  The index function is host arithmetic (CPU
test); the table needs a GPU."""
import numpy as np
import pytest

import pyoracle as po


def _wst(wc, n, J, ttype, seed=0):
    rng = np.random.default_rng(seed)
    size = n if ttype == "DWT" else 2 * J * n
    return wc.WST(x=rng.standard_normal(n), ttype=ttype, filt="Haar", filtlen=2, nlevels=J,
                  len=n, w=rng.standard_normal(size))


def test_oracle_table_small_case_by_hand():
    # n = 16, J = 3: positions 0 and 8 are scaling (level 3), 4 and 12 level 3
    # details, 2, 6, 10, 14 level 2, the odd positions level 1.
    t = po.wst_to_dt(np.arange(16.0), 16, 3, po.DWT)
    assert list(t["CoeffType"][:5]) == ["s", "d", "d", "d", "d"]
    assert list(t["Level"][:9]) == [3, 1, 2, 1, 3, 1, 2, 1, 3]
    assert list(t["Translate"][:9]) == [2.0, 0.5, 1.0, 1.5, 2.0, 2.5, 3.0, 3.5, 6.0]
    t = po.wst_to_dt(np.arange(8.0), 4, 1, po.MODWT, scaling=False)
    assert list(t["W"]) == [4.0, 5.0, 6.0, 7.0] and list(t["Translate"]) == [1, 2, 3, 4]


@pytest.mark.parametrize("ttype", [0, 1])
def test_coeff_level_indices_match_oracle(wc, ttype):
    tname = "DWT" if ttype == 0 else "MODWT"
    for n, J in ((8, 1), (64, 3), (1024, 10)):
        xw = _wst(wc, n, J, tname)
        for level in range(1, J + 1):
            got = wc.getCoeffLevel(xw, level, "d")
            assert np.array_equal(got, po.coeff_level(n, J, ttype, level, "d")), (n, J, level)
        got = wc.getCoeffLevel(xw, J, "s")
        assert np.array_equal(got, po.coeff_level(n, J, ttype, J, "s"))
    xw = _wst(wc, 64, 3, tname)
    with pytest.raises(ValueError):
        wc.getCoeffLevel(xw, 4, "d")
    if ttype == 0:
        with pytest.raises(ValueError):
            wc.getCoeffLevel(xw, 2, "s")


def test_table_rejects_packet_order_and_bad_levels(wc):
    import ctypes as C
    rows = C.c_int64()
    L = wc.lib()
    assert L.wc_wst_table_rows(64, 3, 2, 1, C.byref(rows)) == 5          # unsupported
    assert L.wc_wst_table_rows(64, 7, 0, 1, C.byref(rows)) == 2          # levels
    assert L.wc_wst_table_rows(48, 3, 0, 1, C.byref(rows)) == 1          # not a power of 2
    assert L.wc_wst_table_rows(64, 3, 0, 0, C.byref(rows)) == 0 and rows.value == 64 - 8


@pytest.mark.gpu
@pytest.mark.parametrize("tname", ["DWT", "MODWT"])
@pytest.mark.parametrize("scaling", [True, False])
def test_wst_table_matches_oracle(gpu, tname, scaling):
    wc = gpu
    ttype = 0 if tname == "DWT" else 1
    for n, J in ((2, 1), (16, 3), (1024, 1), (1024, 10), (4096, 7)):
        xw = _wst(wc, n, J, tname, seed=n + J)
        got = wc.WSTtoDT(xw, scaling=scaling)
        ref = po.wst_to_dt(xw.w, n, J, ttype, scaling=scaling)
        for col in ("W", "CoeffType", "Level", "Translate"):
            assert np.array_equal(np.asarray(got[col]), np.asarray(ref[col])), (n, J, col)


@pytest.mark.gpu
def test_wst_table_device_large(gpu):
    """n = 2^24 DWT, J = 16, on device buffers: row count and spot checks of
    the closed form against the oracle's rows."""
    wc = gpu
    import ctypes as C
    L = wc.lib()
    n, J = 1 << 24, 16
    w = np.random.default_rng(3).standard_normal(n)
    dw = wc.DeviceBuffer(8 * n)
    dw.upload(w)
    rows = C.c_int64()
    wc.check(L.wc_wst_table_rows(n, J, 0, 0, C.byref(rows)))
    m = rows.value
    assert m == n - (n >> J)
    dW, dL, dT, dY = (wc.DeviceBuffer(8 * m), wc.DeviceBuffer(4 * m), wc.DeviceBuffer(8 * m),
                      wc.DeviceBuffer(m))
    s = wc.default_stream()
    wc.check(L.wc_wst_table_device(dw.ptr, n, J, 0, 0, dW.ptr, dL.ptr, dT.ptr, dY.ptr, s))
    W = dW.download(np.float64, m, s)
    lev = dL.download(np.int32, m, s)
    tr = dT.download(np.float64, m, s)
    assert np.array_equal(W, w[np.arange(n) % (1 << J) != 0])
    i = np.arange(n)[np.arange(n) % (1 << J) != 0]
    l = (i & -i).astype(np.int64)
    l = np.log2(l).astype(np.int64) + 1
    assert np.array_equal(lev, l)
    assert np.array_equal(tr, 2.0 ** (l - 2) + (i >> l) * 2.0 ** (l - 1))
    for b in (dw, dW, dL, dT, dY):
        b.free()

"""GPU transforms against the oracle.

WC_F64_EXACT must be bit-identical to the reference CPU path (the oracle is
pinned bit-for-bit to it).  WC_F64_FAST (double-float) must stay within
1e-12 of the oracle relative to the largest coefficient of the same level
block; WC_F32 within 2e-5."""
import numpy as np
import pytest

import pyoracle as P
from wavecuda_gb300 import signals

pytestmark = pytest.mark.gpu

FILTERS = [P.HAAR, P.D4, P.C6, P.LA8]
TOL = {1: 1e-12, 2: 2e-5}


def rel_err(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def levels_to_test(oracle, n, filt):
    maxJ = oracle.levels(n, 0, filt)
    return sorted({j for j in (1, 2, 3, maxJ // 2, maxJ) if 1 <= j <= maxJ})


@pytest.mark.parametrize("filt", FILTERS)
def test_dwt_exact_bit_identical(gpu, oracle, filt):
    rng = np.random.default_rng(filt)
    for n in (1 << (P.FILTER_LEN[filt] - 1).bit_length(), 64, 1024, 1 << 15, 1 << 18):
        for J in levels_to_test(oracle, n, filt):
            x = rng.standard_normal(n)
            w = gpu.transform(x, J, gpu.DWT, filt, gpu.FWD, gpu.F64_EXACT)
            assert np.array_equal(w, oracle.dwt(x, J, filt)), (n, J)
            r = gpu.transform(w, J, gpu.DWT, filt, gpu.BWD, gpu.F64_EXACT)
            assert np.array_equal(r, oracle.dwt(w, J, filt, P.BWD)), (n, J)


@pytest.mark.parametrize("filt", FILTERS)
@pytest.mark.parametrize("prec", [1, 2])
def test_dwt_fast_and_fp32_within_tolerance(gpu, oracle, filt, prec):
    rng = np.random.default_rng(10 + filt)
    for n in (64, 4096, 1 << 17):
        for J in levels_to_test(oracle, n, filt):
            x = signals.roofline_input(n, seed=n + J) if n > 64 else rng.standard_normal(n)
            w_ref = oracle.dwt(x, J, filt)
            w = gpu.transform(x, J, gpu.DWT, filt, gpu.FWD, prec)
            assert rel_err(w, w_ref) < TOL[prec], (n, J, rel_err(w, w_ref))
            r = gpu.transform(w_ref, J, gpu.DWT, filt, gpu.BWD, prec)
            assert rel_err(r, x) < TOL[prec] * 4, (n, J)


@pytest.mark.parametrize("filt", FILTERS)
def test_modwt_exact_bit_identical(gpu, oracle, filt):
    rng = np.random.default_rng(30 + filt)
    for n in (1 << (P.FILTER_LEN[filt] - 1).bit_length(), 256, 1 << 14):
        for J in levels_to_test(oracle, n, filt):
            x = rng.standard_normal(n)
            xm = gpu.transform(x, J, gpu.MODWT, filt, gpu.FWD, gpu.F64_EXACT)
            assert np.array_equal(xm, oracle.modwt_fwd(x, J, filt)), (n, J)
            r = gpu.transform(None, J, gpu.MODWT, filt, gpu.BWD, gpu.F64_EXACT, xmod=xm)
            assert np.array_equal(r, oracle.modwt_inv(xm, n, J, filt)), (n, J)


@pytest.mark.parametrize("filt", FILTERS)
@pytest.mark.parametrize("prec", [1, 2])
def test_modwt_fast_and_fp32_within_tolerance(gpu, oracle, filt, prec):
    for n in (256, 1 << 16):
        J = min(oracle.levels(n, 0, filt), 8)
        x = signals.roofline_input(n, seed=7)
        ref = oracle.modwt_fwd(x, J, filt)
        xm = gpu.transform(x, J, gpu.MODWT, filt, gpu.FWD, prec)
        for b in range(2 * J):  # per level block
            blk = slice(b * n, (b + 1) * n)
            assert rel_err(xm[blk], ref[blk]) < TOL[prec], (n, b)
        r = gpu.transform(None, J, gpu.MODWT, filt, gpu.BWD, prec, xmod=ref)
        assert rel_err(r, x) < TOL[prec] * 4


def test_golden_fixtures_through_r_symbols(gpu, golden):
    """The reference's own outputs, reproduced through RgpuTransform."""
    names = {1: "Haar", 2: "D4", 3: "C6", 4: "LA8"}
    checked = 0
    for name, f in golden.items():
        if not (name.startswith("dwt_") or name.startswith("modwt_")):
            continue
        n, J, filt, sense = (int(v) for v in f["args"])
        tt = "DWT" if name.startswith("dwt_") else "MODWT"
        if sense == P.FWD:
            got = gpu.GPUTransform(f["in"], "FWD", J, tt, names[filt]).w
        else:
            wst = gpu.WST(x=np.zeros(n), ttype=tt, filt=names[filt], filtlen=P.FILTER_LEN[filt],
                          nlevels=J, len=n, w=f["in"])
            got = gpu.GPUReconstruct(wst)
        assert np.array_equal(got, f["out"]), name
        checked += 1
    assert checked >= 30


def test_config1_doppler_d4(gpu, oracle):
    """D4 DWT fwd then inverse, full decomposition of a noisy doppler, n=1024.
    The full decomposition is 9 levels (10 is rejected by check_len_levels)."""
    x = signals.noisy(signals.doppler(1024), 5.0, seed=1)
    w = gpu.CPUTransform(x, "FWD", 0, "DWT", "D4")
    assert w.nlevels == 9
    assert np.array_equal(w.w, oracle.dwt(x, 9, P.D4))
    r = gpu.CPUReconstruct(w)
    assert np.array_equal(r, oracle.dwt(w.w, 9, P.D4, P.BWD))
    assert np.max(np.abs(r - x)) < 1e-14 * 50
    with pytest.raises(ValueError):
        gpu.GPUTransform(x, "FWD", 10, "DWT", "D4")


def test_device_api_out_of_place(gpu, oracle):
    n, J = 1 << 16, 10
    x = signals.roofline_input(n, seed=3)
    a, b = gpu.DeviceBuffer(8 * n), gpu.DeviceBuffer(8 * n)
    a.upload(x)
    gpu.check(gpu.lib().wc_dwt_device(a.ptr, b.ptr, n, 1, J, P.LA8, 0, None))
    w = b.download(np.float64, n)
    assert np.array_equal(w, oracle.dwt(x, J, P.LA8))
    # in == out is rejected
    assert gpu.lib().wc_dwt_device(a.ptr, a.ptr, n, 1, J, P.LA8, 0, None) == 1
    a.free(); b.free()


def test_large_perfect_reconstruction(gpu):
    """Size-independent property at 2^24: fwd+inv returns the input."""
    n = 1 << 24
    x = signals.roofline_input(n, seed=11)
    for filt in FILTERS:
        w = gpu.transform(x, 16, gpu.DWT, filt, gpu.FWD, gpu.F64_FAST)
        assert abs(np.dot(w, w) / np.dot(x, x) - 1) < 1e-12  # Parseval
        r = gpu.transform(w, 16, gpu.DWT, filt, gpu.BWD, gpu.F64_FAST)
        assert rel_err(r, x) < 1e-12


def test_errors_are_status_codes(gpu):
    y = np.zeros(1024)
    with pytest.raises(gpu.WaveCudaError):
        gpu.transform(y, 11, gpu.DWT, gpu.HAAR)          # too many levels
    with pytest.raises(gpu.WaveCudaError):
        gpu.transform(np.zeros(1000), 2, gpu.DWT, gpu.HAAR)  # not a power of two


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("filt", FILTERS)
def test_host_streamed_dwt_matches_device_path(gpu, oracle, filt, prec):
    """Long DWTs on host arrays stream over the host link in chunks, with the
    first pass writing into host memory; the result must be the device
    path's (bit-identical in exact FP64), forward and inverse, for pageable
    (numpy) and pinned host arrays."""
    L = gpu.lib()
    for n in (1 << 22, 1 << 23):
        x = signals.roofline_input(n, seed=n + filt)
        for J in sorted({1, 7, oracle.levels(n, 0, filt)}):
            a, b = gpu.DeviceBuffer(8 * n), gpu.DeviceBuffer(8 * n)
            a.upload(x)
            gpu.check(L.wc_dwt_device(a.ptr, b.ptr, n, 1, J, filt, prec, None))
            gpu.check(L.wc_stream_synchronize(None))
            w_dev = b.download(np.float64, n)
            gpu.check(L.wc_dwt_device(b.ptr, a.ptr, n, 0, J, filt, prec, None))
            gpu.check(L.wc_stream_synchronize(None))
            r_dev = a.download(np.float64, n)
            a.free(); b.free()
            w = gpu.transform(x, J, gpu.DWT, filt, gpu.FWD, prec)
            r = gpu.transform(w, J, gpu.DWT, filt, gpu.BWD, prec)
            if prec == 0:
                assert np.array_equal(w, w_dev), (n, J)
                assert np.array_equal(r, r_dev), (n, J)
            else:
                assert rel_err(w, w_dev) <= 1e-13 and rel_err(r, r_dev) <= 1e-13, (n, J)
        if prec == 0 and n == 1 << 22:
            assert np.array_equal(w, oracle.dwt(x, J, filt))
    # pinned host memory through the reference-facing symbol
    n, J = 1 << 22, 9
    x = signals.roofline_input(n, seed=5)
    h = gpu.HostBuffer(n)
    h.array[:] = x
    gpu.set_default_precision(prec)
    try:
        import ctypes as C
        args = [C.c_int(v) for v in (n, 1, J, 0, filt, P.FILTER_LEN[filt])]
        dummy = np.zeros(1)
        xp = C.cast(h.ptr, C.POINTER(C.c_double))
        L.RgpuTransform(xp, dummy.ctypes.data_as(C.POINTER(C.c_double)),
                        *[C.byref(v) for v in args])
        ref = gpu.transform(x, J, gpu.DWT, filt, gpu.FWD, prec)
        assert np.array_equal(h.array, ref)
    finally:
        gpu.set_default_precision(0)
        h.free()

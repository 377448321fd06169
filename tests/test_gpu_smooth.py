"""Thresholding, universal threshold and cross-validated smoothing on the
GPU against the oracle: in WC_F64_EXACT the chosen threshold, the smoothed
signal and the kept/zeroed counts are bit-identical."""
import numpy as np
import pytest

import pyoracle as P
from wavecuda_gb300 import signals

pytestmark = pytest.mark.gpu

NAMES = {1: "Haar", 2: "D4", 3: "C6", 4: "LA8"}
KIND = {0: "manual", 1: "univ", 2: "cv"}


def test_golden_smooth_through_r_symbols(gpu, golden):
    checked = 0
    for name, f in golden.items():
        if not name.startswith("smooth_"):
            continue
        n, J, ttype, filt, tt, hard, mn, mx = (int(v) for v in f["args"])
        a = gpu.check_smooth_inputs(f["in"], J, "DWT" if ttype == 0 else "MODWT", NAMES[filt],
                                    KIND[tt], 0.35, "hard" if hard == 0 else "soft", mn + 1,
                                    mx + 1, 1e-8)
        y = gpu._call_smooth("RgpuSmooth", a)
        assert a["thresh"] == f["thresh"][0] or tt == 0, name
        assert np.array_equal(y, f["out"]), name
        checked += 1
    assert checked == 15


@pytest.mark.parametrize("filt", [P.HAAR, P.D4, P.C6, P.LA8])
@pytest.mark.parametrize("ttype", [P.DWT, P.MODWT])
@pytest.mark.parametrize("hard", [P.HARD, P.SOFT])
def test_cv_threshold_bit_exact(gpu, oracle, filt, ttype, hard):
    for n, seed in ((256, 1), (1 << 14, 2)):
        J = min(10, oracle.levels(n, 0, filt))
        x = signals.noisy(signals.doppler(n), 5.0, seed=seed)
        t_ref, y_ref, tr = oracle.cvt(x, J, ttype, filt, hard, 1e-8, 0, J - 1)
        y, info = gpu.smooth(x, J, ttype, filt, gpu.CV, hardness=hard, minlevel=0,
                             maxlevel=J - 1, tol=1e-8, precision=gpu.F64_EXACT)
        assert info.thresh == t_ref, (n, info.thresh, t_ref)
        assert info.cv_iterations == tr.iters
        assert np.array_equal(y, y_ref)
        w = oracle.dwt(x, J, filt) if ttype == P.DWT else oracle.modwt_fwd(x, J, filt)
        assert (info.kept, info.zeroed) == oracle.count_kept(w, n, J, ttype, t_ref, 0, J - 1)


def test_cv_level_ranges_and_quirks(gpu, oracle):
    n = 2048
    x = signals.noisy(signals.doppler(n), 3.0, seed=9)
    for filt, ttype in ((P.HAAR, P.MODWT), (P.D4, P.DWT), (P.LA8, P.DWT)):
        J = oracle.levels(n, 0, filt)
        # (0,0): maxlevel-1 wraps, the half-length vectors are never
        # thresholded; (3,3): minlevel > maxlevel-1, same; (J-1,J-1) too
        for mn, mx in ((0, 0), (3, 3), (1, J - 1), (2, J - 2), (J - 1, J - 1)):
            t_ref, y_ref, _ = oracle.cvt(x, J, ttype, filt, P.SOFT, 1e-6, mn, mx)
            y, info = gpu.smooth(x, J, ttype, filt, gpu.CV, hardness=P.SOFT, minlevel=mn,
                                 maxlevel=mx, tol=1e-6)
            assert info.thresh == t_ref and np.array_equal(y, y_ref), (filt, ttype, mn, mx)


def test_cv_refuses_one_level(gpu):
    x = signals.noisy(signals.doppler(512), 5.0, seed=2)
    y, info = gpu.smooth(x, 1, gpu.DWT, gpu.HAAR, gpu.CV, minlevel=0, maxlevel=0)
    assert info.thresh == 0.0 and np.array_equal(y, x)   # thresh.cpp:228-231


@pytest.mark.parametrize("ttype", [P.DWT, P.MODWT])
def test_univ_and_manual(gpu, oracle, ttype):
    for filt in (P.HAAR, P.D4, P.C6, P.LA8):
        n = 4096
        J = oracle.levels(n, 0, filt)
        x = signals.noisy(signals.bumps_like(n, 3), 7.0, seed=filt)
        for tt in (P.UNIV, P.MANUAL):
            for mn, mx in ((0, J - 1), (1, J - 2)):
                y_ref, t_ref = oracle.smooth(x, J, ttype, filt, tt, 0.4, P.SOFT, mn, mx, 1e-8)
                y, info = gpu.smooth(x, J, ttype, filt, tt, thresh=0.4, hardness=P.SOFT,
                                     minlevel=mn, maxlevel=mx)
                assert info.thresh == t_ref and np.array_equal(y, y_ref), (filt, tt, mn, mx)


def test_median_mad_exact(gpu, golden, oracle):
    """Radix-select median/MAD equal qsort's (utils.cpp:166-203) bit for bit,
    with ties, signed zeros, odd and even lengths."""
    for name, f in golden.items():
        if name.startswith("mad_"):
            med, mad = gpu.median_mad(f["in"])
            assert (med, mad) == tuple(f["out"]), name
    rng = np.random.default_rng(4)
    for n in (3, 10, 1000, 1 << 20):
        v = rng.standard_normal(n) * 10 ** rng.uniform(-30, 30, n)
        v[: n // 10] = 0.0
        v[n // 10: n // 5] = -0.0
        assert gpu.median_mad(v) == (oracle.median(v), oracle.mad(v)), n


def test_threshold_symbol(gpu, oracle):
    n, J = 1024, 8
    x = signals.noisy(signals.heavisine_like(n, 1), 5.0, seed=4)
    for ttype, filt in ((P.DWT, P.D4), (P.MODWT, P.HAAR), (P.MODWT, P.LA8)):
        w = oracle.dwt(x, J, filt) if ttype == P.DWT else oracle.modwt_fwd(x, J, filt)
        for hard in (P.HARD, P.SOFT):
            ref = oracle.threshold(w if ttype == P.DWT else None, None if ttype == P.DWT else w,
                                   J, ttype, filt, 0.3, hard, 1, 6)
            got = gpu.threshold(w, n, J, ttype, filt, 0.3, hard, 1, 6)
            assert np.array_equal(got, ref)


@pytest.mark.parametrize("prec", [1, 2])
def test_cv_fast_and_fp32_close(gpu, oracle, prec):
    n = 1 << 14
    f = signals.doppler(n)
    x = signals.noisy(f, 5.0, seed=5)
    for filt, ttype in ((P.HAAR, P.MODWT), (P.LA8, P.MODWT), (P.D4, P.DWT)):
        J = min(10, oracle.levels(n, 0, filt))
        t_ref, y_ref, _ = oracle.cvt(x, J, ttype, filt, P.SOFT, 1e-8, 0, J - 1)
        y, info = gpu.smooth(x, J, ttype, filt, gpu.CV, hardness=P.SOFT, maxlevel=J - 1,
                             precision=prec)
        assert abs(info.thresh - t_ref) <= 1e-3 * t_ref, (filt, ttype, info.thresh, t_ref)
        mse_ref = np.mean((y_ref - f) ** 2)
        mse = np.mean((y - f) ** 2)
        assert mse <= mse_ref * 1.01 + 1e-12

"""Pins the oracle against the reference's own CPU code compiled from the
reference tree, across every filter, level count and smoothing mode.  Skipped
where the reference tree is absent (the golden fixtures pin it there)."""
import numpy as np
import pytest

import pyoracle as P
from wavecuda_gb300 import signals


@pytest.mark.parametrize("filt", [P.HAAR, P.D4, P.C6, P.LA8])
def test_transforms_bit_identical(oracle, reference, filt):
    rng = np.random.default_rng(5)
    for n in (8, 64, 1024):
        maxJ = oracle.levels(n, 0, filt)
        for J in range(1, maxJ + 1):
            x = rng.standard_normal(n)
            w = reference.dwt(x, J, filt)
            assert np.array_equal(oracle.dwt(x, J, filt), w)
            assert np.array_equal(oracle.dwt(w, J, filt, P.BWD), reference.dwt(w, J, filt, P.BWD))
            if filt in (P.HAAR, P.D4):
                xm = reference.modwt_fwd(x, J, filt)
                assert np.array_equal(oracle.modwt_fwd(x, J, filt), xm)
                assert np.array_equal(oracle.modwt_inv(xm, n, J, filt),
                                      reference.modwt_inv(xm, n, J, filt))


@pytest.mark.parametrize("filt", [P.HAAR, P.D4, P.C6, P.LA8])
@pytest.mark.parametrize("ttype", [P.DWT, P.MODWT])
def test_smooth_bit_identical(oracle, reference, filt, ttype):
    if ttype == P.MODWT and filt in (P.C6, P.LA8):
        pytest.skip("the reference has no C6/LA8 MODWT")
    for n in (64, 2048):
        maxJ = oracle.levels(n, 0, filt)
        for J in (2, maxJ):
            x = signals.noisy(signals.doppler(n), 5.0, seed=n + J)
            for hard in (P.HARD, P.SOFT):
                for (mn, mx) in ((0, J - 1), (1, J - 1), (0, 0)):
                    if mn > mx:
                        continue
                    for tt in (P.MANUAL, P.UNIV, P.CV):
                        a, ta = oracle.smooth(x, J, ttype, filt, tt, 0.3, hard, mn, mx, 1e-8)
                        b, tb = reference.smooth(x, J, ttype, filt, tt, 0.3, hard, mn, mx, 1e-8)
                        assert ta == tb and np.array_equal(a, b), (n, J, hard, mn, mx, tt)


def test_univ_thresh_levels(oracle, reference):
    rng = np.random.default_rng(9)
    for ttype, filt in ((P.DWT, P.D4), (P.MODWT, P.HAAR), (P.MODWT, P.D4)):
        x = rng.standard_normal(512)
        J = 5
        w = reference.dwt(x, J, filt) if ttype == P.DWT else reference.modwt_fwd(x, J, filt)
        for mn in range(J):
            for mx in range(mn, J):
                assert oracle.univ_thresh(w, 512, J, ttype, mn, mx) == \
                    reference.univ_thresh(w, 512, J, ttype, filt, mn, mx)


@pytest.mark.parametrize("filt", [P.HAAR, P.D4])
def test_packet_ordered_modwt_bit_identical(oracle, reference, filt):
    rng = np.random.default_rng(6)
    for n in (8, 64, 1024):
        for J in range(1, oracle.levels(n, 0, filt) + 1):
            x = rng.standard_normal(n)
            xm = reference.modwt_po_fwd(x, J, filt)
            assert np.array_equal(oracle.modwt_po_fwd(x, J, filt), xm)
            assert np.array_equal(oracle.modwt_po_inv(xm, n, J, filt),
                                  reference.modwt_po_inv(xm, n, J, filt))

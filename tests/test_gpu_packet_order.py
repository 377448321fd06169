"""Packet-ordered MODWT (transform type 2: fHaarMODWT / fDaub4MODWTpo and
their inverses in the reference, haar.cpp:305-398, daub4.cpp:392-484).

The forward coefficients are the time-ordered ones stored per packet
(convert_modwt_level, wavutils.cpp:569-600); the inverse averages the two
reconstructions of every packet pair (writeavpackets), which rounds
differently from the time-ordered inverse.  WC_F64_EXACT must reproduce the
oracle (itself pinned to the reference by tests/golden) bit for bit, for
transforms, thresholding and smoothing; the other precisions stay within the
usual tolerances."""
import numpy as np
import pytest

import pyoracle as P
from wavecuda_gb300 import signals

pytestmark = pytest.mark.gpu

FILTERS = [P.HAAR, P.D4, P.C6, P.LA8]


def rel_err(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("filt", FILTERS)
def test_packet_order_exact_bit_identical(gpu, oracle, filt):
    rng = np.random.default_rng(40 + filt)
    for n in (64, 1024, 1 << 14):
        maxJ = oracle.levels(n, 0, filt)
        for J in sorted({1, 3, maxJ}):
            x = rng.standard_normal(n)
            xm = gpu.transform(x, J, gpu.MODWT_PO, filt, gpu.FWD, gpu.F64_EXACT)
            ref = oracle.modwt_po_fwd(x, J, filt)
            assert np.array_equal(xm, ref), (n, J)
            r = gpu.transform(ref, J, gpu.MODWT_PO, filt, gpu.BWD, gpu.F64_EXACT, xmod=ref)
            assert np.array_equal(r, oracle.modwt_po_inv(ref, n, J, filt)), (n, J)


@pytest.mark.parametrize("prec,tol", [(1, 1e-12), (2, 2e-5)])
@pytest.mark.parametrize("filt", FILTERS)
def test_packet_order_fast_and_fp32(gpu, oracle, filt, prec, tol):
    n = 1 << 12
    J = oracle.levels(n, 0, filt)
    x = signals.roofline_input(n, seed=filt)
    xm = gpu.transform(x, J, gpu.MODWT_PO, filt, gpu.FWD, prec)
    ref = oracle.modwt_po_fwd(x, J, filt)
    assert rel_err(xm, ref) <= tol
    r = gpu.transform(ref, J, gpu.MODWT_PO, filt, gpu.BWD, prec, xmod=ref)
    assert rel_err(r, oracle.modwt_po_inv(ref, n, J, filt)) <= tol


def test_packet_order_golden_fixtures(gpu, golden):
    """The reference's own packet-ordered outputs (transforms and RcpuSmooth
    with transform type 2), through the library."""
    checked = 0
    for name, f in golden.items():
        if name.startswith("modwtpo_"):
            n, J, filt, sense = (int(v) for v in f["args"])
            if sense == P.FWD:
                got = gpu.transform(f["in"], J, gpu.MODWT_PO, filt, gpu.FWD, gpu.F64_EXACT)
            else:
                got = gpu.transform(f["in"], J, gpu.MODWT_PO, filt, gpu.BWD, gpu.F64_EXACT,
                                    xmod=f["in"])
            assert np.array_equal(got, f["out"]), name
            checked += 1
        elif name.startswith("smoothpo_"):
            n, J, ttype, filt, tt, hard, mn, mx = (int(v) for v in f["args"])
            y, info = gpu.smooth(f["in"], J, ttype, filt, tt, 0.35, hard, mn, mx, 1e-8,
                                 gpu.F64_EXACT)
            assert info.thresh == f["thresh"][0], name
            assert np.array_equal(y, f["out"]), name
            checked += 1
    assert checked == 17


@pytest.mark.parametrize("filt", [P.HAAR, P.D4])
def test_packet_order_threshold(gpu, oracle, filt):
    n, J = 1024, 6
    x = signals.noisy(signals.doppler(n), 4.0, seed=7)
    xm = oracle.modwt_po_fwd(x, J, filt)
    for hard in (P.HARD, P.SOFT):
        got = gpu.threshold(xm, n, J, gpu.MODWT_PO, filt, 0.3, hard, 1, 4)
        ref = oracle.threshold(None, xm, J, P.MODWT_PO, filt, 0.3, hard, 1, 4)
        assert np.array_equal(got, ref)

"""The .C glue for R, called through ctypes exactly as R's .C calls it
(every argument a pointer to the first element of a double or int vector):
the status-returning transform/threshold/smooth forms and the flat batched
smoothing entry point RgpuSmoothBatch, against the struct-based calls they
wrap (bit-identical in WC_F64_EXACT)."""
import ctypes as C

import numpy as np
import pytest

import pyoracle as P
from wavecuda_gb300 import signals as sg

pytestmark = pytest.mark.gpu

_dp = C.POINTER(C.c_double)


def ivec(*v):
    return np.ascontiguousarray(v, dtype=np.int32)


def ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def dp(a):
    return a.ctypes.data_as(_dp)


@pytest.mark.parametrize("ttype", [P.DWT, P.MODWT])
def test_transform_R_matches_wc_transform(gpu, oracle, ttype):
    n, J, filt = 4096, 8, P.LA8
    x = sg.roofline_input(n, seed=5)
    st = ivec(-1)
    if ttype == P.DWT:
        y = x.copy()
        gpu.lib().wc_transform_R(dp(y), None, ip(ivec(n)), ip(ivec(1)), ip(ivec(J)),
                                 ip(ivec(ttype)), ip(ivec(filt)), ip(ivec(0)), ip(st))
        assert st[0] == 0 and np.array_equal(y, oracle.dwt(x, J, filt))
    else:
        xm = np.zeros(2 * n * J)
        gpu.lib().wc_transform_R(dp(x.copy()), dp(xm), ip(ivec(n)), ip(ivec(1)), ip(ivec(J)),
                                 ip(ivec(ttype)), ip(ivec(filt)), ip(ivec(0)), ip(st))
        assert st[0] == 0 and np.array_equal(xm, oracle.modwt_fwd(x, J, filt))


def test_threshold_and_smooth_R(gpu, oracle):
    n, J = 2048, 6
    x = sg.noisy(sg.doppler(n), 5.0, seed=2)
    w = oracle.dwt(x, J, P.D4)
    st = ivec(-1)
    wt = w.copy()
    gpu.lib().wc_threshold_R(dp(wt), None, ip(ivec(n)), ip(ivec(J)), ip(ivec(P.DWT)),
                             ip(ivec(P.D4)), dp(np.array([0.4])), ip(ivec(P.SOFT)), ip(ivec(1)),
                             ip(ivec(J - 1)), ip(st))
    ref = oracle.threshold(w, None, J, P.DWT, P.D4, 0.4, P.SOFT, 1, J - 1)
    assert st[0] == 0 and np.array_equal(wt, ref)
    y, th = x.copy(), np.array([0.0])
    gpu.lib().wc_smooth_R(dp(y), ip(ivec(n)), ip(ivec(J)), ip(ivec(P.MODWT)), ip(ivec(P.HAAR)),
                          ip(ivec(P.CV)), dp(th), ip(ivec(P.SOFT)), ip(ivec(0)), ip(ivec(J - 1)),
                          dp(np.array([1e-8])), ip(ivec(0)), ip(st))
    t_ref, y_ref, _ = oracle.cvt(x, J, P.MODWT, P.HAAR, P.SOFT, 1e-8, 0, J - 1)
    assert st[0] == 0 and th[0] == t_ref and np.array_equal(y, y_ref)


def test_smooth_R_reports_bad_arguments_without_printing(gpu, capfd):
    y, th, st = np.zeros(64), np.array([0.0]), ivec(-1)
    gpu.lib().wc_smooth_R(dp(y), ip(ivec(64)), ip(ivec(3)), ip(ivec(0)), ip(ivec(7)), ip(ivec(2)),
                          dp(th), ip(ivec(1)), ip(ivec(0)), ip(ivec(2)), dp(np.array([1e-8])),
                          ip(ivec(0)), ip(st))
    assert st[0] == 1 and "filter" in gpu.last_error()
    assert capfd.readouterr().err == ""


@pytest.mark.parametrize("prec", [0, 2])
def test_smooth_batch_R_matches_struct_call(gpu, prec):
    data, specs, _ = sg.batch_workload(40, seed=21, max_levels=gpu.max_levels, kmin=6, kmax=13)
    sigs = [gpu.Signal(s["offset"], s["len"], s["nlevels"], s["ttype"], s["filter"],
                       s["threshtype"], s["hardness"], s["minlevel"], s["maxlevel"], s["thresh"],
                       s["tol"]) for s in specs]
    y_ref, res = gpu.smooth_batch(data, sigs, prec)
    y, th, its, kept, zer, status = gpu.smooth_batch_R(data, sigs, prec)
    assert status == 0
    assert np.array_equal(y, y_ref)
    assert list(th) == [r.thresh for r in res]
    assert list(its) == [r.iterations for r in res]
    assert list(kept) == [r.kept for r in res] and list(zer) == [r.zeroed for r in res]


def test_smooth_batch_R_rejects_bad_signal(gpu):
    data = np.zeros(64)
    sig = gpu.Signal(0, 48, 0, 0, 1, 1, 1, 0, 3, 0.0, 1e-8)  # 48 is not a power of two
    y, th, its, kept, zer, status = gpu.smooth_batch_R(data, [sig], 0)
    assert status != 0 and np.array_equal(y, data)

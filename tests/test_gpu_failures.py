"""Failure detection without a GPU fault.

The library's only device-side waits are the bulk-copy barriers of the DWT
kernels; each is bounded and, when it gives up, sets bit 0 of a status word
and lets the kernel return.  A test hook launches a kernel whose barrier
expects bytes that no copy delivers, so the wait runs out after a short,
given number of polls.  The checks: wc_device_status() reports and clears
the bit, a host-buffer call issued afterwards returns WC_ERR_TIMEOUT and
leaves the caller's buffer untouched, and the next call succeeds.  The
reference instead calls exit() on CUDA errors (wavutilscuda.cu:159-187).

Allocation failure is injected on the host: a workspace cap makes every slot
that would have to grow fail with WC_ERR_NOMEM, again with the buffers left
as they were."""
import ctypes as C

import numpy as np
import pytest

import pyoracle as P

pytestmark = pytest.mark.gpu

TIMEOUT, NOMEM = 7, 4


def test_device_status_reports_and_clears_a_timed_out_wait(gpu):
    assert gpu.device_status() == 0
    gpu.debug_wait_probe(target=0, polls=1000)
    assert gpu.device_status() == 1
    assert gpu.device_status() == 0


def test_host_buffer_call_returns_timeout_and_leaves_buffer(gpu, oracle):
    L = gpu.lib()
    x = np.random.default_rng(1).standard_normal(1 << 12)
    y = x.copy()
    gpu.debug_wait_probe(target=0, polls=1000)  # on the library's stream
    r = L.wc_transform(y.ctypes.data_as(C.POINTER(C.c_double)), None, y.size, 1, 0, 0, P.D4, 0)
    assert r == TIMEOUT and "gave up" in gpu.last_error()
    assert np.array_equal(y, x)
    # the word was cleared: the same call now succeeds, bit-identical
    r = L.wc_transform(y.ctypes.data_as(C.POINTER(C.c_double)), None, y.size, 1, 0, 0, P.D4, 0)
    assert r == 0 and np.array_equal(y, oracle.dwt(x, 0, P.D4))


def test_reference_symbol_prints_timeout_and_leaves_buffers(gpu, capfd):
    x = np.random.default_rng(2).standard_normal(1 << 10)
    y = x.copy()
    t = C.c_double(0.0)
    ip = lambda v: C.byref(C.c_int(v))  # noqa: E731
    gpu.debug_wait_probe(target=0, polls=1000)
    # RgpuSmooth(x, len, nlevels, ttype, filter, filterlen, threshtype, thresh,
    #            hardness, minlevel, maxlevel, tol): Haar MODWT CV, soft
    gpu.lib().RgpuSmooth(y.ctypes.data_as(C.POINTER(C.c_double)), ip(1024), ip(10), ip(1),
                         ip(1), ip(2), ip(2), C.byref(t), ip(1), ip(0), ip(9),
                         C.byref(C.c_double(1e-8)))
    assert np.array_equal(y, x) and t.value == 0.0
    assert "gave up" in capfd.readouterr().err
    assert gpu.device_status() == 0


def test_status_glue_reports_timeout(gpu):
    L = gpu.lib()
    x = np.random.default_rng(3).standard_normal(256)
    y = x.copy()
    ip = lambda v: C.byref(C.c_int(v))  # noqa: E731
    st = C.c_int(-1)
    gpu.debug_wait_probe(target=0, polls=1000)
    L.wc_transform_R(y.ctypes.data_as(C.POINTER(C.c_double)), None, ip(256), ip(1), ip(0), ip(0),
                     ip(P.LA8), ip(0), C.byref(st))
    assert st.value == TIMEOUT and np.array_equal(y, x)


def test_allocation_failure_returns_nomem_and_leaves_buffers(gpu, oracle):
    L = gpu.lib()
    n = 1 << 16
    x = np.random.default_rng(4).standard_normal(n)
    y = x.copy()
    gpu.check(L.wc_release())
    gpu.debug_set_workspace_cap(4096)
    try:
        r = L.wc_transform(y.ctypes.data_as(C.POINTER(C.c_double)), None, n, 1, 0, 0, P.C6, 0)
        assert r == NOMEM and "cap" in gpu.last_error()
        assert np.array_equal(y, x)
        t = C.c_double(0.0)
        info = gpu.SmoothInfo()
        r = L.wc_smooth(y.ctypes.data_as(C.POINTER(C.c_double)), n, 0, 1, P.HAAR, 2,
                        C.byref(t), 1, 0, 5, 1e-8, 0, C.byref(info))
        assert r == NOMEM and np.array_equal(y, x)
    finally:
        gpu.debug_set_workspace_cap(0)
    gpu.check(L.wc_transform(y.ctypes.data_as(C.POINTER(C.c_double)), None, n, 1, 0, 0, P.C6, 0))
    assert np.array_equal(y, oracle.dwt(x, 0, P.C6))

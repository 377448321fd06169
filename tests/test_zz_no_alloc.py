"""The allocation-free DWT entry point (wc_dwt_device_noalloc).

It exists for callers that cannot let the library call cudaMalloc -- a host
framework that has reserved almost all device memory for its own pool, or a
loop that must not pay the synchronisation cudaFree brings when a workspace
grows.  Its scratch is a fixed device array compiled into the library, so it
takes signals up to 2^22 samples.  Here it is called through the C ABI and
checked against the regular entry point (wc_dwt_device), twice in a row, with
the tolerances the other transform tests use (bit-identical in exact FP64).
This file is collected last so that a failure here comes after every other
test has run; it also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {0: 0.0, 1: 1e-12, 2: 2e-5}


def _bind(lib):
    f = lib.wc_dwt_device_noalloc
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.c_int, C.c_int, C.c_int,
                  C.c_void_p]
    f.restype = C.c_int
    return f


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("prec", [0, 1, 2])
def test_noalloc_matches_regular_entry_point(gpu, prec):
    lib = gpu.lib()
    noalloc = _bind(lib)
    # One stream for every call and copy: the library's own stream is
    # non-blocking, so it does not order against the legacy NULL stream.
    s = gpu.default_stream()
    rng = np.random.default_rng(7 + prec)
    dt = np.float32 if prec == 2 else np.float64
    for filt in (1, 2, 3, 4):
        for n, J in ((64, 0), (1 << 12, 0), (1 << 18, 12), (1 << 22, 16)):
            x = rng.standard_normal(n).astype(dt)
            nb = x.nbytes
            a, b, c = gpu.DeviceBuffer(nb), gpu.DeviceBuffer(nb), gpu.DeviceBuffer(nb)
            a.upload(x, s)
            gpu.check(lib.wc_dwt_device(a.ptr, b.ptr, n, 1, J, filt, prec, s))
            w_ref = b.download(dt, n, s)
            for call in range(2):  # two calls in a row share the static scratch
                gpu.check(noalloc(a.ptr, c.ptr, n, 1, J, filt, prec, s))
                w = c.download(dt, n, s)
                assert _rel(w, w_ref) <= TOL[prec], (filt, n, call)
            gpu.check(lib.wc_dwt_device(b.ptr, a.ptr, n, 0, J, filt, prec, s))
            r_ref = a.download(dt, n, s)
            for call in range(2):
                gpu.check(noalloc(b.ptr, c.ptr, n, 0, J, filt, prec, s))
                r = c.download(dt, n, s)
                assert _rel(r, r_ref) <= TOL[prec], (filt, n, call)
            a.free(); b.free(); c.free()
    assert gpu.device_status() == 0


def test_noalloc_rejects_lengths_beyond_its_maximum(gpu):
    lib = gpu.lib()
    noalloc = _bind(lib)
    n = 1 << 23
    a, b = gpu.DeviceBuffer(8 * n), gpu.DeviceBuffer(8 * n)
    r = noalloc(a.ptr, b.ptr, n, 1, 0, 2, 0, gpu.default_stream())
    assert r == 1 and "maximum" in gpu.last_error()
    a.free(); b.free()

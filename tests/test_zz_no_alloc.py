"""The allocation-free DWT entry point (wc_dwt_device_noalloc).

It exists for callers that cannot let the library call cudaMalloc -- a host
framework that has reserved almost all device memory for its own pool, or a
loop that must not pay the synchronisation cudaFree brings when a workspace
grows.  Its scratch is a fixed device array compiled into the library, so it
takes signals up to 2^22 samples.  Here it is called through the C ABI and
checked against the regular entry point (wc_dwt_device), twice in a row, with
the tolerances the other transform tests use (bit-identical in exact FP64).
This file is collected last so that a failure here comes after every other
test has run; it also passes on its own in a fresh process.  The last tests
check the two promises that the regular entry point cannot show: a fresh
process that calls only this entry point ends with no library workspace on
the device, and a timed-out wait in its kernels is reported through its own
status word (read by wc_device_status, which allocates nothing either).
"""
import ctypes as C
import os
import subprocess
import sys
import textwrap

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


def test_noalloc_timeout_reaches_its_own_status_word(gpu):
    # The probe's barrier expects bytes that never arrive; its bounded wait
    # gives up and sets bit 0 of the allocation-free DWT's status word.
    assert gpu.device_status() == 0
    gpu.debug_wait_probe(target=1, polls=1000)
    assert gpu.device_status() == 1
    assert gpu.device_status() == 0


def test_noalloc_fresh_process_holds_no_workspace():
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    script = textwrap.dedent("""
        import ctypes as C, sys
        import numpy as np
        sys.path.insert(0, %r)
        import wavecuda_gb300 as wc
        lib = wc.lib()
        f = lib.wc_dwt_device_noalloc
        f.argtypes = [C.c_void_p, C.c_void_p, C.c_int64] + [C.c_int] * 4 + [C.c_void_p]
        n = 1 << 20
        x = np.random.default_rng(0).standard_normal(n)
        a, b, c = wc.DeviceBuffer(8 * n), wc.DeviceBuffer(8 * n), wc.DeviceBuffer(8 * n)
        s = wc.default_stream()  # one stream for the copies and the calls
        a.upload(x, s)
        for _ in range(2):
            wc.check(f(a.ptr, b.ptr, n, 1, 0, 4, 0, s))
            wc.check(f(b.ptr, c.ptr, n, 0, 0, 4, 0, s))
        r = c.download(np.float64, n, s)
        assert np.max(np.abs(r - x)) < 1e-12 * np.max(np.abs(x))
        assert wc.device_status() == 0
        assert wc.debug_workspace_bytes() == 0, wc.debug_workspace_bytes()
        print("noalloc-fresh-ok")
    """ % root)
    out = subprocess.run([sys.executable, "-c", script], capture_output=True, text=True,
                         timeout=600)
    assert out.returncode == 0 and "noalloc-fresh-ok" in out.stdout, out.stdout + out.stderr

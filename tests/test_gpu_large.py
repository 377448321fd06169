"""Size-independent properties at the benchmark's scale (2^25 - 2^26
samples, too long for the oracle): perfect reconstruction, Parseval for
the orthonormal DWT, and linearity, through the device-pointer entry points
in every precision."""
import numpy as np
import pytest

import pyoracle as P
from wavecuda_gb300 import signals

pytestmark = pytest.mark.gpu


def _run(gpu, fn, *args):
    gpu.check(fn(*args))
    gpu.check(gpu.lib().wc_stream_synchronize(None))


@pytest.mark.parametrize("prec,tol", [(0, 1e-13), (1, 1e-12), (2, 2e-5)])
@pytest.mark.parametrize("filt", [P.HAAR, P.LA8])
def test_dwt_2e26_reconstruction_parseval_linearity(gpu, filt, prec, tol):
    L = gpu.lib()
    n, J = 1 << 26, 16
    dt = np.float32 if prec == 2 else np.float64
    es = np.dtype(dt).itemsize
    x = signals.roofline_input(n, seed=3).astype(dt)
    y = np.random.default_rng(4).standard_normal(n).astype(dt)
    a, b, c = gpu.DeviceBuffer(es * n), gpu.DeviceBuffer(es * n), gpu.DeviceBuffer(es * n)
    try:
        a.upload(x)
        _run(gpu, L.wc_dwt_device, a.ptr, b.ptr, n, 1, J, filt, prec, None)
        wx = b.download(dt, n).astype(np.float64)
        _run(gpu, L.wc_dwt_device, b.ptr, c.ptr, n, 0, J, filt, prec, None)
        r = c.download(dt, n).astype(np.float64)
        x64 = x.astype(np.float64)
        assert np.max(np.abs(r - x64)) <= tol * np.max(np.abs(x64))
        assert abs(np.dot(wx, wx) / np.dot(x64, x64) - 1) <= 10 * tol
        # T(2x + y) = 2 T(x) + T(y)
        z = (2 * x64 + y.astype(np.float64)).astype(dt)
        a.upload(y)
        _run(gpu, L.wc_dwt_device, a.ptr, b.ptr, n, 1, J, filt, prec, None)
        wy = b.download(dt, n).astype(np.float64)
        a.upload(z)
        _run(gpu, L.wc_dwt_device, a.ptr, b.ptr, n, 1, J, filt, prec, None)
        wz = b.download(dt, n).astype(np.float64)
        lin = 2 * wx + wy
        assert np.max(np.abs(wz - lin)) <= 4 * tol * np.max(np.abs(lin))
    finally:
        a.free(); b.free(); c.free()


@pytest.mark.parametrize("prec,tol", [(0, 1e-13), (1, 1e-12), (2, 2e-5)])
def test_modwt_2e25_reconstruction(gpu, prec, tol):
    L = gpu.lib()
    n, J = 1 << 25, 6
    dt = np.float32 if prec == 2 else np.float64
    es = np.dtype(dt).itemsize
    x = signals.roofline_input(n, seed=5).astype(dt)
    a, m, c = gpu.DeviceBuffer(es * n), gpu.DeviceBuffer(es * n * 2 * J), gpu.DeviceBuffer(es * n)
    try:
        a.upload(x)
        for filt in (P.D4, P.C6):
            _run(gpu, L.wc_modwt_device, a.ptr, m.ptr, n, 1, J, filt, prec, None)
            _run(gpu, L.wc_modwt_device, c.ptr, m.ptr, n, 0, J, filt, prec, None)
            r = c.download(dt, n).astype(np.float64)
            x64 = x.astype(np.float64)
            assert np.max(np.abs(r - x64)) <= tol * np.max(np.abs(x64)), filt
    finally:
        a.free(); m.free(); c.free()

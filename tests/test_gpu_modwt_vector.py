"""The 16-byte MODWT tiles (wc_modwt_vec.cuh), forward and inverse, against
the one-value tiles and the oracle.

Both tile kinds compute every value with the same operations in the same
order, so their outputs must be bit-identical in every precision; exact FP64
must also be bit-identical to the oracle.  The cases cover the single-column
tiles of the finest levels (a window of chunks around each output group),
the C >= W column tiles, 1, 2 and 3 fused inverse levels, small tiles (many
halo rows per tile) and buffers whose 16-byte misalignment sends a launch
back to the one-value tiles."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _both(gpu, fn):
    gpu.set_modwt_vector(False)
    try:
        a = fn()
    finally:
        gpu.set_modwt_vector(True)
    return a, fn()


@pytest.mark.parametrize("filt", [1, 2, 3, 4])
@pytest.mark.parametrize("prec", [0, 1, 2])
def test_vector_inverse_matches_scalar_tiles(gpu, oracle, filt, prec):
    keep = gpu.get_modwt_tiling(filt, prec)
    keep_ni = gpu.get_modwt_inv_levels(filt, prec)
    rng = np.random.default_rng(100 + 10 * filt + prec)
    try:
        for n, J in ((1 << 10, 10), (1 << 13, 7), (1 << 15, 12)):
            J = min(J, gpu.max_levels(n, filt))
            x = rng.standard_normal(n)
            xm = oracle.modwt_fwd(x, J, filt)
            for target, kb in ((256, 16), (2048, 72), (16384, 200)):
                gpu.set_modwt_tiling(filt, prec, target, kb, target, kb)
                for ni in (2, 3):
                    gpu.set_modwt_inv_levels(filt, prec, ni)
                    r_s, r_v = _both(gpu, lambda: gpu.transform(xm, J, gpu.MODWT, filt, gpu.BWD,
                                                                prec, xmod=xm))
                    assert np.array_equal(r_s, r_v), (n, J, target, ni)
                    if prec == 0:
                        assert np.array_equal(r_v, oracle.modwt_inv(xm, n, J, filt)), (n, J, target, ni)
                    else:
                        tol = 1e-12 if prec == 1 else 2e-5
                        assert np.max(np.abs(r_v - x)) <= tol * 8 * np.max(np.abs(x))
        assert gpu.device_status() == 0
    finally:
        gpu.set_modwt_tiling(filt, prec, *keep)
        gpu.set_modwt_inv_levels(filt, prec, keep_ni)


@pytest.mark.parametrize("filt", [1, 2, 3, 4])
@pytest.mark.parametrize("prec", [0, 1, 2])
def test_vector_forward_matches_scalar_tiles(gpu, oracle, filt, prec):
    """Forward with 1, 2 or 3 fused levels per launch on the 16-byte tiles
    against the one-value tiles (2 levels per launch) and the oracle."""
    keep = gpu.get_modwt_tiling(filt, prec)
    keep_nf = gpu.get_modwt_fwd_levels(filt, prec)
    rng = np.random.default_rng(200 + 10 * filt + prec)
    try:
        for n, J in ((1 << 10, 10), (1 << 13, 7), (1 << 15, 12)):
            J = min(J, gpu.max_levels(n, filt))
            x = rng.standard_normal(n)
            ref = oracle.modwt_fwd(x, J, filt)
            for target, kb in ((256, 16), (2048, 72), (16384, 200)):
                gpu.set_modwt_tiling(filt, prec, target, kb, target, kb)
                for nf in (1, 2, 3):
                    gpu.set_modwt_fwd_levels(filt, prec, nf)
                    w_s, w_v = _both(gpu, lambda: gpu.transform(x, J, gpu.MODWT, filt, gpu.FWD,
                                                                prec))
                    # The one-value tiles fuse 2 levels per launch.  Double-float
                    # values round to FP64 between launches, so its bits depend
                    # on the grouping; FP64 and FP32 values do not.
                    if nf == 2 or prec != 1:
                        assert np.array_equal(w_s, w_v), (n, J, target, nf)
                    if prec == 0:
                        assert np.array_equal(w_v, ref), (n, J, target, nf)
                    else:
                        tol = 1e-12 if prec == 1 else 2e-5
                        assert np.max(np.abs(w_v - ref)) <= tol * 4 * np.max(np.abs(ref))
        assert gpu.device_status() == 0
    finally:
        gpu.set_modwt_tiling(filt, prec, *keep)
        gpu.set_modwt_fwd_levels(filt, prec, keep_nf)


@pytest.mark.parametrize("prec", [0, 1, 2])
def test_unaligned_buffers_fall_back_to_scalar_tiles(gpu, oracle, prec):
    """Device pointers 8 (FP64) or 4 (FP32) bytes past a 16-byte boundary
    take the one-value tiles and give the same result."""
    lib = gpu.lib()
    n, J, filt = 1 << 12, 8, 2
    es = 4 if prec == 2 else 8
    dt = np.float32 if prec == 2 else np.float64
    x = np.random.default_rng(5).standard_normal(n)
    xm = oracle.modwt_fwd(x, J, filt).astype(dt)
    s = gpu.default_stream()
    xb = gpu.DeviceBuffer(es * n + 16)
    mb = gpu.DeviceBuffer(es * xm.size + 16)
    try:
        fw = []
        for off in (0, es):
            gpu.check(lib.wc_memcpy(C.c_void_p(xb.ptr + off), x.astype(dt).ctypes.data,
                                    es * n, s))
            gpu.check(lib.wc_modwt_device(C.c_void_p(xb.ptr + off), C.c_void_p(mb.ptr + off), n,
                                          1, J, filt, prec, s))
            w = np.empty(xm.size, dt)
            gpu.check(lib.wc_memcpy(w.ctypes.data, C.c_void_p(mb.ptr + off), w.nbytes, s))
            gpu.check(lib.wc_stream_synchronize(s))
            fw.append(w)
        assert np.array_equal(fw[0], fw[1])
        out = []
        for off in (0, es):
            mb_ptr = mb.ptr + off
            gpu.check(lib.wc_memcpy(C.c_void_p(mb_ptr), xm.ctypes.data, xm.nbytes, s))
            gpu.check(lib.wc_modwt_device(C.c_void_p(xb.ptr + off), C.c_void_p(mb_ptr), n, 0, J,
                                          filt, prec, s))
            r = np.empty(n, dt)
            gpu.check(lib.wc_memcpy(r.ctypes.data, C.c_void_p(xb.ptr + off), r.nbytes, s))
            gpu.check(lib.wc_stream_synchronize(s))
            out.append(r)
        assert np.array_equal(out[0], out[1])
    finally:
        xb.free()
        mb.free()

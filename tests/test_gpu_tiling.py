"""Every first-pass tiling of the DWT (tile size, fused levels, block size,
pipelined persistent kernels or not) gives the oracle's result: bit-identical
in WC_F64_EXACT, within the usual tolerances otherwise."""
import numpy as np
import pytest

import pyoracle as P
from wavecuda_gb300 import signals

pytestmark = pytest.mark.gpu

GMAX = {1: 12, 2: 8, 3: 7, 4: 6}


def candidates(filt, prec):
    tiles = (4096, 8192) if prec == 2 else (2048, 4096)
    for tile in tiles:
        for g in (GMAX[filt] - 1, GMAX[filt], 3):
            if (1 << g) > tile:
                continue
            for th in (256, 512):
                for pipe in (1, 0):
                    yield tile, g, th, pipe


@pytest.mark.parametrize("filt", [1, 2, 3, 4])
@pytest.mark.parametrize("prec", [0, 1, 2])
def test_tilings_match_oracle(gpu, oracle, filt, prec):
    keep = gpu.get_dwt_tiling(filt, prec)
    n = 1 << 17
    x = signals.roofline_input(n, seed=filt + 10 * prec)
    tol = {0: 0.0, 1: 1e-12, 2: 2e-5}[prec]
    try:
        # J = 3: one pass over many tiles (the inverse then reads its coarse
        # input straight from the interleaved array); J = 16: several passes.
        for J in (3, min(16, oracle.levels(n, 0, filt))):
            w_ref = oracle.dwt(x, J, filt)
            r_ref = oracle.dwt(w_ref, J, filt, P.BWD)
            for c in candidates(filt, prec):
                gpu.set_dwt_tiling(filt, prec, *c)
                w = gpu.transform(x, J, gpu.DWT, filt, gpu.FWD, prec)
                err = np.max(np.abs(w - w_ref)) / np.max(np.abs(w_ref))
                assert err <= tol, (J, c, err)
                r = gpu.transform(w_ref, J, gpu.DWT, filt, gpu.BWD, prec)
                if prec == 0:
                    assert np.array_equal(r, r_ref), (J, c)
                else:
                    assert np.max(np.abs(r - x)) / np.max(np.abs(x)) <= 4 * tol, (J, c)
        assert gpu.device_status() == 0
    finally:
        gpu.set_dwt_tiling(filt, prec, *keep)


def test_tiling_rejects_bad_values(gpu):
    with pytest.raises(gpu.WaveCudaError):
        gpu.set_dwt_tiling(2, 0, 3000, 8, 256, 1)
    with pytest.raises(gpu.WaveCudaError):
        gpu.set_dwt_tiling(2, 0, 4096, 13, 256, 1)
    with pytest.raises(gpu.WaveCudaError):
        gpu.set_dwt_tiling(2, 0, 4096, 8, 128, 1)


def test_autotune_keeps_a_valid_tiling(gpu, oracle):
    (tile, g0, th, pipe), ms = gpu.tune_dwt(2, 1, 20)
    assert ms > 0 and th in (256, 512) and (1 << g0) <= tile
    x = signals.roofline_input(1 << 16, seed=3)
    w = gpu.transform(x, 14, gpu.DWT, 2, gpu.FWD, 1)
    ref = oracle.dwt(x, 14, 2)
    assert np.max(np.abs(w - ref)) / np.max(np.abs(ref)) <= 1e-12


@pytest.mark.parametrize("filt", [P.HAAR, P.D4, P.LA8])
def test_modwt_tilings_match_oracle(gpu, oracle, filt):
    """Every MODWT tile target and shared-memory budget gives the oracle's
    result bit for bit in exact FP64 (forward and inverse)."""
    n, J = 1 << 14, 9
    x = np.random.default_rng(filt).standard_normal(n)
    ref = oracle.modwt_fwd(x, J, filt)
    keep = gpu.get_modwt_tiling(filt, 0)
    keep_ni = gpu.get_modwt_inv_levels(filt, 0)
    inv_ref = oracle.modwt_inv(ref, n, J, filt)
    try:
        for target, kb in ((256, 16), (1024, 48), (4096, 96), (16384, 200)):
            gpu.set_modwt_tiling(filt, 0, target, kb, target, kb)
            xm = gpu.transform(x, J, gpu.MODWT, filt, gpu.FWD, gpu.F64_EXACT)
            assert np.array_equal(xm, ref), (target, kb)
            for ni in (2, 3):
                gpu.set_modwt_inv_levels(filt, 0, ni)
                r = gpu.transform(xm, J, gpu.MODWT, filt, gpu.BWD, gpu.F64_EXACT, xmod=xm)
                assert np.array_equal(r, inv_ref), (target, kb, ni)
        with pytest.raises(gpu.WaveCudaError):
            gpu.set_modwt_tiling(filt, 0, 1000, 48, 1024, 48)
        with pytest.raises(gpu.WaveCudaError):
            gpu.set_modwt_inv_levels(filt, 0, 4)
        (t, f, i) = gpu.tune_modwt(filt, 1, 16, 8)
        assert t[0] >= 256 and f > 0 and i > 0 and gpu.get_modwt_inv_levels(filt, 1) in (2, 3)
    finally:
        gpu.set_modwt_tiling(filt, 0, *keep)
        gpu.set_modwt_inv_levels(filt, 0, keep_ni)

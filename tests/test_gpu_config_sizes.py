"""Parity at the workloads' own sizes, against the oracle (the oracle's level
loops run on every host core; results do not depend on the thread count).

* Single large signals: DWT with J = 16 at n = 2^26 and TO-MODWT with J = 12
  at n = 2^24, every filter, forward and inverse, through the device-pointer
  entry points.  WC_F64_EXACT is bit-identical; WC_F64_FAST is held to 1e-12
  and WC_F32 to 2e-5 of the largest oracle coefficient of each level block
  (inverse: of the largest sample, times 4).
* Cross-validated smoothing (GPUSmooth) at n = 2^20: Haar and LA8 TO-MODWT,
  J = 10, soft, tolerance 1e-8, levels 0..9, exact: the chosen threshold, the
  iteration count, the kept/zeroed counts and the smoothed signal are
  bit-identical to the oracle's CVT (thresh.cpp:203-342).
* Batched smoothing: the 4096-signal batch (lengths 2^10..2^20, random
  filter and transform, universal or CV soft thresholds) in one persistent
  launch in exact FP64, against the oracle's smoothing of every 2^19- and
  2^20-sample signal plus a random sample of the others, bit for bit.  The
  oracle runs in a process pool started with spawn.
"""
import multiprocessing as mp
import os

import numpy as np
import pytest

import pyoracle as P
from wavecuda_gb300 import signals as sg

pytestmark = pytest.mark.gpu

FILTERS = [P.HAAR, P.D4, P.C6, P.LA8]
TOL = {1: 1e-12, 2: 2e-5}


@pytest.fixture(scope="module")
def par_oracle(oracle):
    before = oracle.lib.wo_get_threads()
    oracle.set_threads(0)
    yield oracle
    oracle.set_threads(before)


def dwt_blocks(n, J):
    for lev in range(1, J + 1):
        yield f"d{lev}", slice(1 << (lev - 1), n, 1 << lev)
    yield "s", slice(0, n, 1 << J)


def block_rel(a, b, sl):
    ref = b[sl]
    return float(np.max(np.abs(a[sl] - ref)) / max(np.max(np.abs(ref)), 1e-300))


def device_transform(gpu, fn, src, n_out, dt, *args):
    L = gpu.lib()
    a = gpu.DeviceBuffer(src.nbytes)
    b = gpu.DeviceBuffer(np.dtype(dt).itemsize * n_out)
    try:
        a.upload(src)
        gpu.check(getattr(L, fn)(a.ptr, b.ptr, *args, None))
        gpu.check(L.wc_stream_synchronize(None))
        return b.download(dt, n_out)
    finally:
        a.free()
        b.free()


@pytest.fixture(scope="module")
def x26():
    return sg.roofline_input(1 << 26, seed=26)


@pytest.mark.parametrize("filt", FILTERS)
def test_dwt_2e26_J16_against_oracle(gpu, par_oracle, x26, filt):
    n, J = x26.size, 16
    w_ref = par_oracle.dwt(x26, J, filt)
    r_ref = par_oracle.dwt(w_ref, J, filt, P.BWD)
    w = device_transform(gpu, "wc_dwt_device", x26, n, np.float64, n, 1, J, filt, 0)
    assert np.array_equal(w, w_ref)
    r = device_transform(gpu, "wc_dwt_device", w_ref, n, np.float64, n, 0, J, filt, 0)
    assert np.array_equal(r, r_ref)
    xmax = np.max(np.abs(x26))
    for prec in (1, 2):
        dt = np.float32 if prec == 2 else np.float64
        w = device_transform(gpu, "wc_dwt_device", x26.astype(dt), n, dt, n, 1, J, filt,
                             prec).astype(np.float64)
        for name, sl in dwt_blocks(n, J):
            assert block_rel(w, w_ref, sl) <= TOL[prec], (prec, name, block_rel(w, w_ref, sl))
        r = device_transform(gpu, "wc_dwt_device", w_ref.astype(dt), n, dt, n, 0, J, filt,
                             prec).astype(np.float64)
        assert np.max(np.abs(r - r_ref)) <= 4 * TOL[prec] * xmax, prec


@pytest.mark.parametrize("filt", FILTERS)
def test_modwt_2e24_J12_against_oracle(gpu, par_oracle, filt):
    n, J = 1 << 24, 12
    x = sg.roofline_input(n, seed=24)
    L = gpu.lib()
    xm_ref = par_oracle.modwt_fwd(x, J, filt)
    r_ref = par_oracle.modwt_inv(xm_ref, n, J, filt)
    xmax = np.max(np.abs(x))
    for prec in (0, 1, 2):
        dt = np.float32 if prec == 2 else np.float64
        es = np.dtype(dt).itemsize
        a, m = gpu.DeviceBuffer(es * n), gpu.DeviceBuffer(es * n * 2 * J)
        try:
            a.upload(x.astype(dt))
            gpu.check(L.wc_modwt_device(a.ptr, m.ptr, n, 1, J, filt, prec, None))
            xm = m.download(dt, 2 * n * J)
            if prec == 0:
                assert np.array_equal(xm, xm_ref)
            else:
                for b in range(2 * J):
                    sl = slice(b * n, (b + 1) * n)
                    e = block_rel(xm.astype(np.float64), xm_ref, sl)
                    assert e <= TOL[prec], (prec, b, e)
            del xm
            m.upload(xm_ref.astype(dt))
            gpu.check(L.wc_modwt_device(a.ptr, m.ptr, n, 0, J, filt, prec, None))
            r = a.download(dt, n).astype(np.float64)
        finally:
            a.free()
            m.free()
        if prec == 0:
            assert np.array_equal(r, r_ref)
        else:
            assert np.max(np.abs(r - r_ref)) <= 4 * TOL[prec] * xmax, prec


@pytest.mark.parametrize("filt", [P.HAAR, P.LA8])
def test_cv_smooth_2e20_modwt_J10_bit_exact(gpu, par_oracle, filt):
    n, J = 1 << 20, 10
    for shape, snr, seed in (("doppler", 3.0, 901), ("bumps", 7.0, 902)):
        f = sg.SHAPES[shape](n, 1)
        x = sg.noisy(f, snr, seed=seed)
        t_ref, y_ref, tr = par_oracle.cvt(x, J, P.MODWT, filt, P.SOFT, 1e-8, 0, J - 1)
        y, info = gpu.smooth(x, J, gpu.MODWT, filt, gpu.CV, hardness=gpu.SOFT, minlevel=0,
                             maxlevel=J - 1, tol=1e-8, precision=gpu.F64_EXACT)
        assert info.thresh == t_ref, (shape, info.thresh, t_ref)
        assert info.cv_iterations == tr.iters
        w = par_oracle.modwt_fwd(x, J, filt)
        assert (info.kept, info.zeroed) == par_oracle.count_kept(w, n, J, P.MODWT, t_ref, 0, J - 1)
        assert np.array_equal(y, y_ref)


def _oracle_smooth(args):
    x, s = args
    o = P.Oracle()
    o.set_threads(1)
    return o.smooth(x, s["nlevels"], s["ttype"], s["filter"], s["threshtype"], s["thresh"],
                    s["hardness"], s["minlevel"], s["maxlevel"], s["tol"])


def test_batch_4096_exact_against_oracle(gpu):
    data, specs, _ = sg.batch_workload(4096, seed=11, max_levels=gpu.max_levels)
    sigs = [gpu.Signal(s["offset"], s["len"], s["nlevels"], s["ttype"], s["filter"],
                       s["threshtype"], s["hardness"], s["minlevel"], s["maxlevel"], s["thresh"],
                       s["tol"]) for s in specs]
    y, res = gpu.smooth_batch(data, sigs, gpu.F64_EXACT)
    assert all(r.status == 0 for r in res)
    rng = np.random.default_rng(12)
    big = [i for i, s in enumerate(specs) if s["len"] >= 1 << 19]
    rest = [i for i, s in enumerate(specs) if s["len"] < 1 << 19]
    pick = sorted(big + list(rng.choice(rest, size=64, replace=False)))
    assert len(big) > 500
    jobs = [(data[specs[i]["offset"]:specs[i]["offset"] + specs[i]["len"]], specs[i])
            for i in pick]
    # big jobs first so the pool ends evenly
    order = sorted(range(len(jobs)), key=lambda k: -jobs[k][1]["len"] * (
        8 if jobs[k][1]["threshtype"] == 2 and jobs[k][1]["ttype"] == 1 else 1))
    with mp.get_context("spawn").Pool(processes=os.cpu_count() or 4) as pool:
        out = pool.map(_oracle_smooth, [jobs[k] for k in order], chunksize=1)
    for k, (yr, tr) in zip(order, out):
        i = pick[k]
        s = specs[i]
        assert res[i].thresh == tr, (i, s, res[i].thresh, tr)
        assert np.array_equal(y[s["offset"]:s["offset"] + s["len"]], yr), (i, s)

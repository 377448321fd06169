"""Batched smoothing (one persistent launch over many signals of uneven
length, filter, transform and threshold type) against the oracle, signal by
signal: bit-identical in WC_F64_EXACT."""
import numpy as np
import pytest

import pyoracle as P
from wavecuda_gb300 import signals as sg

pytestmark = pytest.mark.gpu


def make_batch(wc, oracle, nsig, kmin, kmax, seed, kinds=(0, 1, 2)):
    rng = np.random.default_rng(seed)
    sigs, chunks, off = [], [], 0
    shapes = list(sg.SHAPES)
    for i in range(nsig):
        k = int(rng.integers(kmin, kmax + 1))
        n = 1 << k
        filt = int(rng.integers(1, 5))
        ttype = int(rng.integers(0, 2))
        J = min(k, 10, oracle.levels(n, 0, filt))
        tt = int(rng.choice(kinds))
        hard = int(rng.integers(0, 2))
        f = sg.SHAPES[shapes[i % len(shapes)]](n, i)
        x = sg.noisy(f, float(rng.choice([3.0, 7.0])), seed=seed * 1000 + i)
        chunks.append(x)
        sigs.append(wc.Signal(off, n, J, ttype, filt, tt, hard, 0, J - 1, 0.3, 1e-8))
        off += n
    return np.concatenate(chunks), sigs


def _close(y, y_ref, hardness, tol):
    """Soft thresholds: every value within tol.  Hard thresholds (hardness
    0) keep or drop a coefficient whole, so two thresholds a rounding apart
    can differ by one coefficient near the threshold and its footprint: the
    RMS difference is held to tol instead."""
    d = np.abs(y - y_ref)
    return (np.max(d) if hardness == 1 else np.sqrt(np.mean(d * d))) <= tol


def test_batch_matches_oracle_exact(gpu, oracle):
    data, sigs = make_batch(gpu, oracle, 48, 5, 12, seed=1)
    y, res = gpu.smooth_batch(data, sigs, gpu.F64_EXACT)
    assert gpu.device_status() == 0
    for i, s in enumerate(sigs):
        x = data[s.offset:s.offset + s.len]
        yr, tr = oracle.smooth(x, s.nlevels, s.ttype, s.filter, s.threshtype, s.thresh,
                               s.hardness, s.minlevel, s.maxlevel, s.tol)
        assert res[i].thresh == tr or s.threshtype == 0, (i, res[i].thresh, tr)
        assert np.array_equal(y[s.offset:s.offset + s.len], yr), i


def test_batch_cv_iterations_and_counts(gpu, oracle):
    data, sigs = make_batch(gpu, oracle, 24, 8, 11, seed=2, kinds=(2,))
    y, res = gpu.smooth_batch(data, sigs, gpu.F64_EXACT)
    for i, s in enumerate(sigs):
        x = data[s.offset:s.offset + s.len]
        t, yr, tr = oracle.cvt(x, s.nlevels, s.ttype, s.filter, s.hardness, s.tol,
                               s.minlevel, s.maxlevel)
        assert res[i].thresh == t and res[i].iterations == tr.iters
        w = oracle.dwt(x, s.nlevels, s.filter) if s.ttype == 0 else \
            oracle.modwt_fwd(x, s.nlevels, s.filter)
        assert (res[i].kept, res[i].zeroed) == oracle.count_kept(
            w, s.len, s.nlevels, s.ttype, t, s.minlevel, s.maxlevel)


@pytest.mark.parametrize("prec", [1, 2])
def test_batch_fast_and_fp32_close(gpu, oracle, prec):
    data, sigs = make_batch(gpu, oracle, 32, 9, 12, seed=3, kinds=(1, 2))
    y, res = gpu.smooth_batch(data, sigs, prec)
    y64, res64 = gpu.smooth_batch(data, sigs, gpu.F64_EXACT)
    for i, s in enumerate(sigs):
        sl = slice(s.offset, s.offset + s.len)
        scale = np.max(np.abs(y64[sl])) + 1e-300
        tol_t = 1e-3 if prec == 1 else 5e-3
        assert abs(res[i].thresh - res64[i].thresh) <= tol_t * res64[i].thresh + 1e-12, i
        assert _close(y[sl], y64[sl], s.hardness, (0.05 if prec == 2 else 0.02) * scale), i


def test_batch_graph_replay_and_plan(gpu, oracle):
    import ctypes as C
    data, sigs = make_batch(gpu, oracle, 16, 6, 10, seed=4)
    L = gpu.lib()
    arr = (gpu.Signal * len(sigs))(*sigs)
    plan = C.c_void_p()
    gpu.check(L.wc_batch_plan_create(arr, len(sigs), gpu.F64_EXACT, C.byref(plan)))
    buf = gpu.DeviceBuffer(8 * data.size)
    outs = []
    for _ in range(2):  # second run replays the instantiated graph
        buf.upload(data)
        gpu.check(L.wc_batch_run_device(plan, buf.ptr, None))
        res = (gpu.SignalResult * len(sigs))()
        gpu.check(L.wc_batch_results(plan, res, None))
        outs.append((buf.download(np.float64, data.size), [r.thresh for r in res]))
    assert np.array_equal(outs[0][0], outs[1][0]) and outs[0][1] == outs[1][1]
    ms = C.c_float()
    gpu.check(L.wc_batch_autotune(plan, buf.ptr, C.byref(ms)))
    assert ms.value > 0
    gpu.check(L.wc_batch_plan_destroy(plan))
    buf.free()


@pytest.mark.parametrize("prec", [0, 1])
def test_batch_paired_search(gpu, oracle, prec, tmp_path, monkeypatch):
    """The CV searches too long for one CTA run on two (a leader and a
    partner, one half-signal inverse each per golden step): exact FP64 gives
    the same bits as the single-CTA search and as the oracle; double-float
    stays within its tolerance of it."""
    data, sigs = make_batch(gpu, oracle, 40, 6, 14, seed=6, kinds=(1, 2))
    trace = tmp_path / "trace.csv"
    monkeypatch.setenv("WAVECUDA_BATCH_TRACE", str(trace))
    monkeypatch.setenv("WAVECUDA_BATCH_PAIRS", "1")
    y2, r2 = gpu.smooth_batch(data, sigs, prec)
    assert gpu.device_status() == 0
    rows = [l.split(",") for l in trace.read_text().splitlines()[1:]]
    roles = {(int(r[1]), int(r[2])) for r in rows}
    paired = sorted(i for i, role in roles if role == 2)
    assert paired and all((i, 1) in roles for i in paired)
    assert all(sigs[i].threshtype == 2 for i in paired)
    assert len(rows) == len(sigs) + len(paired)
    monkeypatch.setenv("WAVECUDA_BATCH_PAIRS", "0")
    y1, r1 = gpu.smooth_batch(data, sigs, prec)
    for i, s in enumerate(sigs):
        sl = slice(s.offset, s.offset + s.len)
        if prec == 0:
            assert r2[i].thresh == r1[i].thresh and r2[i].iterations == r1[i].iterations, i
            assert (r2[i].kept, r2[i].zeroed) == (r1[i].kept, r1[i].zeroed), i
            assert np.array_equal(y2[sl], y1[sl]), i
        else:
            # the loss partials add in another order: a near-tie late in the
            # search may go the other way, moving the threshold within the
            # search's final bracket
            assert abs(r2[i].thresh - r1[i].thresh) <= 1e-4 * r1[i].thresh + 1e-12, i
            scale = np.max(np.abs(y1[sl])) + 1e-300
            assert np.max(np.abs(y2[sl] - y1[sl])) <= 1e-4 * scale, i
    if prec == 0:
        for i in paired:
            s = sigs[i]
            x = data[s.offset:s.offset + s.len]
            yr, tr = oracle.smooth(x, s.nlevels, s.ttype, s.filter, s.threshtype, s.thresh,
                                   s.hardness, s.minlevel, s.maxlevel, s.tol)
            assert r2[i].thresh == tr and np.array_equal(y2[s.offset:s.offset + s.len], yr), i


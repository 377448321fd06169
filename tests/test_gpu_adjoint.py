"""Differentiation: adjoint kernels and per-level threshold gradients.

* The adjoint of every transform operator is checked against the transpose of
  the operator's dense matrix at n=256 (each matrix is built column by column
  by applying the operator to unit vectors on the device).
* The soft-threshold adjoint and the SURE / cross-validation gradients are
  checked against FP64 central finite differences at n=256 (LA8 takes at most
  6 levels there).  Between kinks the soft-thresholded losses are quadratic
  in lambda, so central differences are exact up to rounding.
* The SURE divergence term is checked against the trace of the smoothed
  signal's Jacobian, computed by finite differences in each input sample.
"""
import ctypes as C

import numpy as np
import pytest

import pyoracle as P

pytestmark = pytest.mark.gpu

FILTERS = [P.HAAR, P.D4, P.C6, P.LA8]
N = 256


def _levels(oracle, n, filt):
    return oracle.levels(n, 0, filt)


def _apply_columns(gpu, op, in_len, out_len, inputs):
    """Applies op(in_ptr, out_ptr) to each column of `inputs` (in_len x k) on
    the library stream and returns the outputs (out_len x k)."""
    k = inputs.shape[1]
    src = gpu.DeviceBuffer(8 * in_len * k)
    dst = gpu.DeviceBuffer(8 * out_len * k)
    src.upload(np.ascontiguousarray(inputs.T))
    for j in range(k):
        gpu.check(op(src.ptr + 8 * in_len * j, dst.ptr + 8 * out_len * j))
    out = dst.download(np.float64, out_len * k).reshape(k, out_len).T
    src.free(); dst.free()
    return out


def _dense_pair(gpu, ttype, filt, J, n=N):
    """Dense matrices of forward, inverse, adjoint-of-forward and
    adjoint-of-inverse."""
    L = gpu.lib()
    m = n if ttype == gpu.DWT else 2 * J * n
    if ttype == gpu.DWT:
        fwd = lambda a, b: L.wc_dwt_device(a, b, n, 1, J, filt, 0, None)
        inv = lambda a, b: L.wc_dwt_device(a, b, n, 0, J, filt, 0, None)
        adj_fwd = lambda a, b: L.wc_dwt_adjoint_device(a, b, n, 1, J, filt, 0, None)
        adj_inv = lambda a, b: L.wc_dwt_adjoint_device(a, b, n, 0, J, filt, 0, None)
    else:
        fwd = lambda a, b: L.wc_modwt_device(a, b, n, 1, J, filt, 0, None)
        inv = lambda a, b: L.wc_modwt_device(b, a, n, 0, J, filt, 0, None)
        adj_fwd = lambda a, b: L.wc_modwt_adjoint_device(b, a, n, 1, J, filt, None)
        adj_inv = lambda a, b: L.wc_modwt_adjoint_device(a, b, n, 0, J, filt, None)
    W = _apply_columns(gpu, fwd, n, m, np.eye(n))
    V = _apply_columns(gpu, inv, m, n, np.eye(m))
    Wt = _apply_columns(gpu, adj_fwd, m, n, np.eye(m))
    Vt = _apply_columns(gpu, adj_inv, n, m, np.eye(n))
    return W, V, Wt, Vt


@pytest.mark.parametrize("filt", FILTERS)
@pytest.mark.parametrize("ttype", [0, 1])
def test_adjoints_are_dense_transposes(gpu, oracle, ttype, filt):
    Jmax = _levels(oracle, N, filt)
    for J in sorted({1, 3, Jmax}):
        W, V, Wt, Vt = _dense_pair(gpu, ttype, filt, J)
        assert np.max(np.abs(Wt - W.T)) <= 1e-12 * np.max(np.abs(W)), (J, "adjoint of forward")
        assert np.max(np.abs(Vt - V.T)) <= 1e-12 * np.max(np.abs(V)), (J, "adjoint of inverse")
        # The inverse reconstructs: V W = I.
        assert np.max(np.abs(V @ W - np.eye(N))) <= 1e-12, J
        if ttype == 0:
            assert np.max(np.abs(W.T @ W - np.eye(N))) <= 1e-12, J


def _soft(c, lam_of_index):
    return np.sign(c) * np.maximum(np.abs(c) - lam_of_index, 0.0)


def test_soft_threshold_adjoint_matches_finite_differences(gpu):
    L = gpu.lib()
    rng = np.random.default_rng(3)
    n, J = N, 5
    for ttype in (0, 1):
        m = n if ttype == 0 else 2 * J * n
        c = rng.standard_normal(m)
        gout = rng.standard_normal(m)
        lam = np.linspace(0.3, 1.1, J)
        minl, maxl = 1, 3
        # Level of every coefficient (-1: not thresholded).
        lev = np.full(m, -1)
        if ttype == 0:
            for i in range(1, n):
                l = (i & -i).bit_length() - 1
                if l < J:
                    lev[i] = l
        else:
            for l in range(J):
                lev[(2 * l + 1) * n:(2 * l + 2) * n] = l
        lev[(lev < minl) | (lev > maxl)] = -1

        def f(lv):
            t = np.where(lev >= 0, lv[np.maximum(lev, 0)], 0.0)
            y = np.where(lev >= 0, _soft(c, t), c)
            return float(gout @ y)

        bc, bg, bgc = (gpu.DeviceBuffer(8 * m) for _ in range(3))
        bgl = gpu.DeviceBuffer(8 * J)
        bc.upload(c); bg.upload(gout)
        lam_c = np.ascontiguousarray(lam)
        gpu.check(L.wc_soft_threshold_adjoint_device(
            bc.ptr, bg.ptr, bgc.ptr, bgl.ptr, n, J, ttype,
            lam_c.ctypes.data_as(C.POINTER(C.c_double)), minl, maxl, None))
        glam = bgl.download(np.float64, J)
        gcoef = bgc.download(np.float64, m)
        t = np.where(lev >= 0, lam[np.maximum(lev, 0)], 0.0)
        keep = (lev < 0) | (np.abs(c) >= t)
        assert np.array_equal(gcoef, np.where(keep, gout, 0.0))
        h = 1e-6
        for l in range(J):
            e = np.zeros(J); e[l] = h
            fd = (f(lam + e) - f(lam - e)) / (2 * h)
            assert abs(glam[l] - fd) <= 1e-7 * max(1.0, abs(fd)), (ttype, l, glam[l], fd)
        for b in (bc, bg, bgc, bgl):
            b.free()


def _test_signal(seed, n=N):
    from wavecuda_gb300 import signals
    rng = np.random.default_rng(seed)
    clean = signals.doppler(n)
    return clean + rng.standard_normal(n) / 3.0


def _fd_grad(gpu, x, J, filt, ttype, loss_type, lam, minl, maxl, sigma, eps, h):
    g = np.zeros(J)
    for l in range(J):
        e = np.zeros(J); e[l] = h
        lp, _, _ = gpu.loss_grad(x, J, filt, ttype, loss_type, lam + e, minl, maxl, sigma, eps)
        lm, _, _ = gpu.loss_grad(x, J, filt, ttype, loss_type, lam - e, minl, maxl, sigma, eps)
        g[l] = (lp - lm) / (2 * h)
    return g


@pytest.mark.parametrize("filt", FILTERS)
@pytest.mark.parametrize("ttype", [0, 1])
def test_sure_gradient_matches_central_differences(gpu, oracle, ttype, filt):
    J = _levels(oracle, N, filt)
    x = _test_signal(10 + filt)
    lam = np.linspace(0.15, 0.45, J)
    for eps, sigma in ((0.0, 0.0), (0.05, 0.3)):
        loss, grad, sig = gpu.loss_grad(x, J, filt, ttype, gpu.LOSS_SURE, lam, 0, J - 1,
                                        sigma, eps)
        assert sig > 0 and np.isfinite(loss)
        fd = _fd_grad(gpu, x, J, filt, ttype, gpu.LOSS_SURE, lam, 0, J - 1, sig, eps, 1e-6)
        scale = max(1.0, np.max(np.abs(fd)))
        assert np.max(np.abs(grad - fd)) <= 1e-6 * scale, (eps, grad, fd)


@pytest.mark.parametrize("filt", FILTERS)
@pytest.mark.parametrize("ttype", [0, 1])
def test_cv_gradient_matches_central_differences(gpu, oracle, ttype, filt):
    J = _levels(oracle, N, filt)
    if J < 2 or oracle.levels(N // 2, 0, filt) < J - 1:
        J = min(J, oracle.levels(N // 2, 0, filt) + 1)
    x = _test_signal(20 + filt)
    lam = np.linspace(0.2, 0.5, J)
    for minl, maxl in ((0, J - 1), (1, J - 1)):
        loss, grad, _ = gpu.loss_grad(x, J, filt, ttype, gpu.LOSS_CV, lam, minl, maxl)
        assert np.isfinite(loss) and loss > 0
        fd = _fd_grad(gpu, x, J, filt, ttype, gpu.LOSS_CV, lam, minl, maxl, 0.0, 0.0, 1e-6)
        scale = max(1.0, np.max(np.abs(fd)))
        assert np.max(np.abs(grad - fd)) <= 1e-6 * scale, (minl, grad, fd)
        assert grad[J - 1] == 0.0  # the top full level has no half-level counterpart
        if minl > 0:
            assert np.all(grad[:minl] == 0.0)


def _interp_mse(x, ye, yo):
    """interp_mse (thresh.cpp:344-385) in numpy."""
    h = x.size // 2
    yie = np.empty(h); yio = np.empty(h)
    yie[0] = yo[0]
    yie[1:] = 0.5 * (yo[1:] + yo[:-1])
    yio[:-1] = 0.5 * (ye[:-1] + ye[1:])
    yio[-1] = ye[-1]
    return 0.5 * float(np.sum((yie - x[0::2]) ** 2 + (yio - x[1::2]) ** 2))


@pytest.mark.parametrize("filt", [P.HAAR, P.LA8])
def test_cv_loss_at_uniform_threshold_matches_oracle(gpu, oracle, filt):
    """At lambda_l = t on every level the per-level CV loss is the loss the
    golden-section search evaluates at t (MODWT halves, J-1 levels)."""
    x = _test_signal(31, 1024)
    J, t = 6, 0.37
    loss, _, _ = gpu.loss_grad(x, J, filt, 1, gpu.LOSS_CV, np.full(J, t), 0, J - 1)
    ys = []
    for half in (x[0::2], x[1::2]):
        w = oracle.modwt_fwd(half, J - 1, filt)
        w = oracle.threshold(None, w, J - 1, P.MODWT, filt, t, P.SOFT, 0, J - 2)
        ys.append(oracle.modwt_inv(w, half.size, J - 1, filt))
    ref = _interp_mse(x, ys[0], ys[1])
    assert abs(loss - ref) <= 1e-12 * abs(ref), (loss, ref)


@pytest.mark.parametrize("ttype", [0, 1])
@pytest.mark.parametrize("filt", [P.HAAR, P.LA8])
def test_sure_divergence_is_jacobian_trace(gpu, oracle, ttype, filt):
    """div f = sum over kept coefficients of the per-level trace weight equals
    the trace of d f / d x (central differences in each sample), for a
    uniform threshold where f is the library's own soft-thresholded smooth."""
    J = min(4, _levels(oracle, N, filt))
    x = _test_signal(40 + filt)
    t = 0.3
    sigma = 0.5

    def fhat(y):
        w = gpu.transform(y, J, ttype, filt, gpu.FWD, gpu.F64_EXACT)
        w = gpu.threshold(w, N, J, ttype, filt, t, gpu.SOFT, 0, J - 1)
        if ttype == gpu.DWT:
            return gpu.transform(w, J, ttype, filt, gpu.BWD, gpu.F64_EXACT)
        return gpu.transform(None, J, ttype, filt, gpu.BWD, gpu.F64_EXACT, xmod=w)

    h = 1e-6
    tr = 0.0
    for i in range(N):
        e = np.zeros(N); e[i] = h
        tr += (fhat(x + e)[i] - fhat(x - e)[i]) / (2 * h)
    f = fhat(x)
    loss, _, _ = gpu.loss_grad(x, J, filt, ttype, gpu.LOSS_SURE, np.full(J, t), 0, J - 1,
                               sigma, 0.0)
    div = (loss - float(np.sum((f - x) ** 2)) + N * sigma ** 2) / (2 * sigma ** 2)
    assert abs(div - tr) <= 1e-6 * N, (div, tr)

"""Batched per-level threshold tuning (wc_fit_thresholds[_device]).

* The loss and gradient the persistent kernel computes at its starting
  thresholds (FP32 or double-float bulk arithmetic) are checked against the
  FP64 path wc_loss_grad, whose gradients the adjoint tests check against
  central finite differences.
* The smoothed output is checked against the oracle: forward transform, soft
  thresholds per level with the returned lambdas, inverse.
* Tuning never ends above its starting loss, and on noisy test shapes the
  SURE-tuned per-level thresholds give a lower error against the clean signal
  than the golden-section cross-validated single threshold of the reference
  (wc_smooth), as the tuner is meant to.
"""
import numpy as np
import pytest

import pyoracle as P
from wavecuda_gb300 import signals as sg

pytestmark = pytest.mark.gpu

N = 1 << 12


def _noisy(n, shape="doppler", snr=4.0, seed=3):
    f = sg.SHAPES[shape](n, 1)
    return f, sg.noisy(f, snr, seed=seed)


def _lam0(J, sigma, seed):
    rng = np.random.default_rng(seed)
    return sigma * rng.uniform(0.5, 3.0, J)


@pytest.mark.parametrize("prec", [1, 2])
@pytest.mark.parametrize("loss", [0, 1])
@pytest.mark.parametrize("ttype,filt,J", [(0, P.HAAR, 8), (0, P.LA8, 6), (1, P.D4, 7),
                                          (1, P.LA8, 6)])
def test_start_loss_and_gradient_match_fp64_path(gpu, prec, loss, ttype, filt, J):
    f, x = _noisy(N)
    sigma = 0.25
    eps_rel = 0.2
    lam0 = _lam0(J, sigma, 11 + J)
    minl, maxl = 1, J - 1
    ref_loss, ref_grad, _ = gpu.loss_grad(x, J, filt, ttype, loss, lam0, minl, maxl,
                                          sigma=sigma, eps=(eps_rel * sigma if loss == 0 else 0.0))
    _, res = gpu.fit_thresholds(x, J, filt, ttype, device=True, loss_type=loss, min_level=minl,
                                max_level=maxl, iterations=0, eps=eps_rel, sigma=sigma,
                                lambda0=lam0, precision=prec, smooth=False)
    r = res[0]
    assert r.status == 0
    scale = N * sigma * sigma
    assert abs(r.loss0 - ref_loss) <= 2e-4 * scale, (r.loss0, ref_loss)
    g = np.array(r.grad0[:J])
    tol = 5e-3 * max(np.max(np.abs(ref_grad)), 1e-3 * N * sigma)
    assert np.max(np.abs(g - ref_grad)) <= tol, (g, ref_grad)


def _soft(c, t):
    return np.sign(c) * np.maximum(np.abs(c) - t, 0.0)


@pytest.mark.parametrize("prec,tol", [(1, 1e-10), (2, 2e-5)])
@pytest.mark.parametrize("ttype,filt,J,loss", [(1, P.LA8, 6, 0), (0, P.D4, 8, 0),
                                               (1, P.HAAR, 8, 1), (0, P.C6, 7, 1)])
def test_smoothed_output_is_the_thresholded_reconstruction(gpu, oracle, prec, tol, ttype, filt,
                                                           J, loss):
    f, x = _noisy(N, "bumps", 5.0, seed=9)
    X = np.stack([x, sg.noisy(f, 3.0, seed=10)])
    y, res = gpu.fit_thresholds(X, J, filt, ttype, loss_type=loss, iterations=20,
                                precision=prec)
    for k in range(2):
        lam = np.array(res[k].lambda_[:J])
        assert res[k].status == 0 and np.all(lam >= 0)
        if ttype == 1:
            xm = oracle.modwt_fwd(X[k], J, filt)
            for l in range(J):
                b = (2 * l + 1) * N
                xm[b:b + N] = _soft(xm[b:b + N], lam[l])
            ref = oracle.modwt_inv(xm, N, J, filt)
        else:
            w = oracle.dwt(X[k], J, filt)
            idx = np.arange(1, N)
            lev = np.array([(int(i) & -int(i)).bit_length() - 1 for i in idx])
            sel = lev < J
            w[idx[sel]] = _soft(w[idx[sel]], lam[lev[sel]])
            ref = oracle.dwt(w, J, filt, P.BWD)
        err = np.max(np.abs(y[k] - ref)) / np.max(np.abs(ref))
        assert err <= tol, (k, err)


@pytest.mark.parametrize("shape", ["doppler", "blocks", "bumps", "heavisine"])
def test_sure_tuning_beats_golden_section_cv(gpu, shape):
    n, J = 1 << 14, 8
    f = sg.SHAPES[shape](n, 1)
    X = np.stack([sg.noisy(f, snr, seed=20 + i) for i, snr in enumerate((3.0, 7.0))])
    y, res = gpu.fit_thresholds(X, J, P.LA8, 1, loss_type=0, iterations=60, precision=2)
    for k in range(2):
        assert res[k].loss <= res[k].loss0
        y_cv, _ = gpu.smooth(X[k], J, gpu.MODWT, gpu.LA8, gpu.CV, hardness=gpu.SOFT,
                             maxlevel=J - 1, tol=1e-8)
        mse_fit = np.mean((y[k] - f) ** 2)
        mse_cv = np.mean((y_cv - f) ** 2)
        assert mse_fit < mse_cv, (shape, k, mse_fit, mse_cv)


def test_cv_tuning_lowers_the_cv_loss(gpu):
    f, x = _noisy(1 << 13, "heavisine", 4.0, seed=5)
    _, res = gpu.fit_thresholds(x, 7, P.D4, 1, loss_type=1, iterations=40, precision=2)
    assert res[0].status == 0 and res[0].loss < res[0].loss0


def test_host_and_device_entry_points_agree(gpu):
    f, x = _noisy(N, "blocks", 4.0, seed=2)
    X = np.stack([x, x[::-1].copy(), sg.noisy(f, 6.0, seed=4)])
    yd, rd = gpu.fit_thresholds(X, 6, P.D4, 0, device=True, iterations=15)
    yh, rh = gpu.fit_thresholds(X, 6, P.D4, 0, device=False, iterations=15)
    for k in range(3):
        np.testing.assert_allclose(np.array(rd[k].lambda_[:6]), np.array(rh[k].lambda_[:6]),
                                   rtol=1e-5, atol=1e-9)
    assert np.max(np.abs(yd - yh)) <= 1e-4 * np.max(np.abs(yd))


def test_rejects_bad_arguments(gpu):
    x = np.random.default_rng(0).standard_normal(256)
    with pytest.raises(gpu.WaveCudaError):
        gpu.fit_thresholds(x, 4, P.D4, 1, precision=0)       # exact FP64 not offered
    with pytest.raises(gpu.WaveCudaError):
        gpu.fit_thresholds(x, 4, P.D4, 1, max_level=4)       # level out of range
    with pytest.raises(gpu.WaveCudaError):
        gpu.fit_thresholds(x, 1, P.HAAR, 1, loss_type=1)     # CV needs two levels

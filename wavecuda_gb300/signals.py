"""Seeded synthetic test signals.

* ``doppler`` -- f(t) = sqrt(t(1-t)) sin(2.1 pi / (t + 0.05)), t = (i + 0.5)/n,
  rescaled to unit standard deviation (the reference README's demo signal).
* ``noisy`` -- a clean signal plus iid N(0, (sd(f)/snr)^2) noise.
* ``roofline_input`` -- iid N(0,1) plus a sum of 8 sinusoids with random
  integer frequencies in [1, n/4] and random phases.
* ``blocks_like``, ``bumps_like``, ``heavisine_like`` -- this project's own
  piecewise test shapes (step functions, sharp peaks, a sinusoid with jumps),
  generated from a seed; they are not the Donoho-Johnstone test functions.
* ``batch_workload`` -- the batched-smoothing workload: signals of length
  2^k, k uniform on {kmin..kmax}, random filter and transform, levels
  min(k, 10) clamped to the filter's maximum, universal or CV soft
  thresholds, shapes above at SNR 3 or 7, back to back in one array.

All generators are deterministic given (n, seed) and use numpy's PCG64.
"""
from __future__ import annotations

import numpy as np


def doppler(n: int) -> np.ndarray:
    t = (np.arange(n) + 0.5) / n
    f = np.sqrt(t * (1 - t)) * np.sin(2.1 * np.pi / (t + 0.05))
    return f / f.std()


def blocks_like(n: int, seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    t = (np.arange(n) + 0.5) / n
    jumps = np.sort(rng.uniform(0.05, 0.95, 11))
    heights = rng.uniform(-5, 5, 11)
    f = np.zeros(n)
    for p, h in zip(jumps, heights):
        f += h * (t > p)
    f -= f.mean()
    return f / f.std()


def bumps_like(n: int, seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed + 1)
    t = (np.arange(n) + 0.5) / n
    pos = np.sort(rng.uniform(0.05, 0.95, 11))
    hgt = rng.uniform(1, 6, 11)
    wid = rng.uniform(0.002, 0.03, 11)
    f = np.zeros(n)
    for p, h, w in zip(pos, hgt, wid):
        f += h / (1 + np.abs((t - p) / w)) ** 4
    f -= f.mean()
    return f / f.std()


def heavisine_like(n: int, seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed + 2)
    t = (np.arange(n) + 0.5) / n
    a, b = np.sort(rng.uniform(0.2, 0.8, 2))
    f = 4 * np.sin(4 * np.pi * t) - np.sign(t - a) - np.sign(b - t)
    f -= f.mean()
    return f / f.std()


SHAPES = {"doppler": lambda n, s=0: doppler(n), "blocks": blocks_like, "bumps": bumps_like,
          "heavisine": heavisine_like}


def noisy(f: np.ndarray, snr: float, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return f + rng.normal(0.0, f.std() / snr, f.size)


def roofline_input(n: int, seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(n)
    i = np.arange(n, dtype=np.float64)
    for _ in range(8):
        fr = rng.integers(1, max(2, n // 4) + 1)
        ph = rng.uniform(0, 2 * np.pi)
        x += np.sin(2 * np.pi * fr * i / n + ph)
    return x


def batch_workload(nsig: int, seed: int, max_levels, kmin: int = 10, kmax: int = 20):
    """(data, specs, clean): `specs` holds one dict per signal with the
    fields of a wc_signal record (offset, len, nlevels, ttype, filter,
    threshtype, hardness, minlevel, maxlevel, thresh, tol); max_levels(n,
    filter) is the level limit (check_len_levels)."""
    rng = np.random.default_rng(seed)
    shapes = list(SHAPES)
    specs, chunks, clean, off = [], [], [], 0
    for i in range(nsig):
        k = int(rng.integers(kmin, kmax + 1))
        n = 1 << k
        filt = int(rng.integers(1, 5))
        ttype = int(rng.integers(0, 2))
        J = min(k, 10, max_levels(n, filt))
        tt = int(rng.choice([1, 2]))  # universal or cross-validated
        f = SHAPES[shapes[int(rng.integers(0, 4))]](n, i)
        x = noisy(f, float(rng.choice([3.0, 7.0])), seed=seed * 7919 + i)
        chunks.append(x)
        clean.append(f)
        specs.append(dict(offset=off, len=n, nlevels=J, ttype=ttype, filter=filt, threshtype=tt,
                          hardness=1, minlevel=0, maxlevel=J - 1, thresh=0.0, tol=1e-8))
        off += n
    return np.concatenate(chunks), specs, np.concatenate(clean)

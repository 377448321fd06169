"""Generates tests/golden/golden.npz from the reference's own CPU code.

The reference's CPU sources are compiled unmodified (oracle/Makefile builds
oracle/_ref/libwavref.so from the reference tree) and driven through
oracle/refshim.cpp.  Inputs are this project's seeded synthetic signals.
Run from the repository root, where the reference tree is present:

    make -C oracle all && python tests/golden/make_golden.py

Each fixture is stored as <name>/in, <name>/out (and <name>/thresh for
smoothing) plus the integer parameters in <name>/args.
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)

import pyoracle as P  # noqa: E402
from wavecuda_gb300 import signals  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.npz")


def main():
    R = P.Reference()
    fx = {}

    def put(name, args, inp, out, thresh=None):
        fx[f"{name}/args"] = np.asarray(args, dtype=np.int64)
        fx[f"{name}/in"] = np.asarray(inp, dtype=np.float64)
        fx[f"{name}/out"] = np.asarray(out, dtype=np.float64)
        if thresh is not None:
            fx[f"{name}/thresh"] = np.asarray([thresh], dtype=np.float64)

    # Doppler n=1024, SNR 5 (noise sd 0.2), D4 DWT with the maximum 9 levels.
    x1024 = signals.noisy(signals.doppler(1024), 5.0, seed=1)
    w = R.dwt(x1024, 9, P.D4)
    put("dwt_fwd_d4_1024_j9", [1024, 9, P.D4, P.FWD], x1024, w)
    put("dwt_inv_d4_1024_j9", [1024, 9, P.D4, P.BWD], w, R.dwt(w, 9, P.D4, P.BWD))

    rng = np.random.default_rng(20)
    for filt in (P.HAAR, P.D4, P.C6, P.LA8):
        n = 256
        maxJ = R.levels(n, 0, filt)
        for J in sorted({1, 2, maxJ}):
            x = rng.standard_normal(n)
            w = R.dwt(x, J, filt)
            put(f"dwt_fwd_f{filt}_256_j{J}", [n, J, filt, P.FWD], x, w)
            put(f"dwt_inv_f{filt}_256_j{J}", [n, J, filt, P.BWD], w, R.dwt(w, J, filt, P.BWD))
        # smallest admissible length: the first power of two >= filter length
        n = 1 << (P.FILTER_LEN[filt] - 1).bit_length()
        x = rng.standard_normal(n)
        put(f"dwt_fwd_f{filt}_min", [n, 1, filt, P.FWD], x, R.dwt(x, 1, filt))

    for filt in (P.HAAR, P.D4):
        n = 256
        for J in (1, 3, R.levels(n, 0, filt)):
            x = rng.standard_normal(n)
            xm = R.modwt_fwd(x, J, filt)
            put(f"modwt_fwd_f{filt}_256_j{J}", [n, J, filt, P.FWD], x, xm)
            put(f"modwt_inv_f{filt}_256_j{J}", [n, J, filt, P.BWD], xm, R.modwt_inv(xm, n, J, filt))

    # median / mad, odd and even lengths with ties and signed zeros
    for k, n in enumerate((1, 2, 7, 64, 1001)):
        v = np.round(rng.standard_normal(n) * 4) / 4
        put(f"mad_{n}", [n], v, [R.median(v), R.mad(v)])

    # Smoothing (RcpuSmooth): threshtype, filter, ttype, hardness, min, max.
    cases = [
        ("cv", P.HAAR, P.DWT, P.SOFT, 0, 9), ("cv", P.HAAR, P.DWT, P.HARD, 0, 9),
        ("cv", P.HAAR, P.MODWT, P.SOFT, 0, 9), ("cv", P.HAAR, P.MODWT, P.HARD, 0, 9),
        ("cv", P.D4, P.DWT, P.SOFT, 0, 8), ("cv", P.D4, P.MODWT, P.SOFT, 0, 8),
        ("cv", P.C6, P.DWT, P.SOFT, 0, 7), ("cv", P.LA8, P.DWT, P.HARD, 0, 7),
        ("cv", P.HAAR, P.MODWT, P.SOFT, 1, 7), ("cv", P.D4, P.DWT, P.SOFT, 2, 6),
        ("univ", P.HAAR, P.DWT, P.SOFT, 0, 9), ("univ", P.D4, P.MODWT, P.HARD, 0, 8),
        ("univ", P.LA8, P.DWT, P.SOFT, 1, 5),
        ("manual", P.C6, P.DWT, P.SOFT, 0, 7), ("manual", P.D4, P.MODWT, P.HARD, 2, 8),
    ]
    tt = {"manual": P.MANUAL, "univ": P.UNIV, "cv": P.CV}
    for k, (kind, filt, ttype, hard, mn, mx) in enumerate(cases):
        n = 1024
        J = R.levels(n, 0, filt) if filt != P.HAAR else 10
        x = signals.noisy(signals.doppler(n), 5.0, seed=100 + k)
        y, t = R.smooth(x, J, ttype, filt, tt[kind], 0.35, hard, mn, mx, 1e-8)
        put(f"smooth_{kind}_f{filt}_t{ttype}_h{hard}_{mn}_{mx}",
            [n, J, ttype, filt, tt[kind], hard, mn, mx], x, y, t)
    # Packet-ordered MODWT (code 2; Haar and D4 only in the reference):
    # transforms, and smoothing through RcpuSmooth with ttype 2.
    rng_po = np.random.default_rng(30)
    for filt in (P.HAAR, P.D4):
        n = 256
        for J in (1, 3, R.levels(n, 0, filt)):
            x = rng_po.standard_normal(n)
            xm = R.modwt_po_fwd(x, J, filt)
            put(f"modwtpo_fwd_f{filt}_256_j{J}", [n, J, filt, P.FWD], x, xm)
            put(f"modwtpo_inv_f{filt}_256_j{J}", [n, J, filt, P.BWD], xm,
                R.modwt_po_inv(xm, n, J, filt))
    po_cases = [("cv", P.HAAR, P.SOFT, 0, 9), ("cv", P.D4, P.SOFT, 0, 8),
                ("cv", P.D4, P.HARD, 1, 7), ("univ", P.HAAR, P.HARD, 0, 9),
                ("manual", P.D4, P.SOFT, 2, 8)]
    for k, (kind, filt, hard, mn, mx) in enumerate(po_cases):
        n = 1024
        J = R.levels(n, 0, filt) if filt != P.HAAR else 10
        x = signals.noisy(signals.doppler(n), 5.0, seed=300 + k)
        y, t = R.smooth(x, J, P.MODWT_PO, filt, tt[kind], 0.35, hard, mn, mx, 1e-8)
        put(f"smoothpo_{kind}_f{filt}_h{hard}_{mn}_{mx}",
            [n, J, P.MODWT_PO, filt, tt[kind], hard, mn, mx], x, y, t)
    np.savez_compressed(OUT, **fx)
    print(f"wrote {len(fx)} arrays to {OUT} ({os.path.getsize(OUT)} bytes)")


if __name__ == "__main__":
    main()

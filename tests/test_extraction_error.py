"""Error of the extraction dot products (accx_* in csrc/wc_dd.cuh), checked
by an exact-rational emulation of their FP32 steps on random windows: the
error of the double-float result against the exact dot product, relative to
sum |a*c|, stays within the bound the design notes state (median about
1e-14, worst case below 5e-13), and Dot2's (acc2_*) below 3e-14.  The
device code performs the same IEEE operations (fma.rn / add.rn / sub.rn in
both lanes of f32x2 pairs); this pins the algorithm, the GPU parity tests
pin the kernels."""
from fractions import Fraction as Fr

import numpy as np

F32 = np.float32
D4 = [0.4829629131445341, 0.8365163037378079, 0.2241438680420134, -0.1294095225512604]
LA8 = [-7.576571478950221e-2, -2.963552764600249e-2, 4.976186676327750e-1,
       8.037387518051321e-1, 2.978577956053061e-1, -9.921954357663353e-2,
       -1.260396726203130e-2, 3.222310060405147e-2]


def r32(q):
    """Round a rational to the nearest float32 (ties away are not needed:
    the candidates bracket q)."""
    y = F32(float(q))
    cands = [y, np.nextafter(y, F32(np.inf)), np.nextafter(y, F32(-np.inf))]
    return min(cands, key=lambda c: abs(Fr(float(c)) - q))


def fma(a, b, c):
    return r32(Fr(float(a)) * Fr(float(b)) + Fr(float(c)))


def add(a, b):
    return r32(Fr(float(a)) + Fr(float(b)))


def sub(a, b):
    return r32(Fr(float(a)) - Fr(float(b)))


def split(x):
    hi = F32(x)
    return hi, F32(x - float(hi))


def fin(s, ne):
    hi = sub(s, ne)
    bb = sub(hi, s)
    lo = sub(sub(s, sub(hi, bb)), add(ne, bb))
    return Fr(float(hi)) + Fr(float(lo))


def extraction(a, taps, m):
    acc = F32(0)
    for (ah, _), mk in zip(a, m):
        acc = fma(abs(ah), mk, acc)
    b = int(np.float32(acc * F32(2.0)).view(np.uint32))
    sig = np.uint32((b + 0x7FFFFF) & 0xFF800000).view(np.float32)
    S = ne = None
    for (ah, al), c in zip(a, taps):
        ch = F32(c)
        cl = F32(c - float(ch))
        q = sub(fma(ah, ch, sig), sig)
        u = fma(ah, -ch, q)
        if S is None:
            S, ne = q, fma(al, -ch, fma(ah, -cl, u))
        else:
            ne = add(fma(al, -ch, fma(ah, -cl, ne)), u)
            S = add(S, q)
    return fin(S, ne)


def dot2(a, taps):
    s = ne = None
    for (ah, al), c in zip(a, taps):
        ch = F32(c)
        cl = F32(c - float(ch))
        p = r32(Fr(float(ah)) * Fr(float(ch)))
        npe = fma(al, -ch, fma(ah, -cl, fma(ah, -ch, p)))
        if s is None:
            s, ne = p, npe
        else:
            s2 = add(s, p)
            bb = sub(s2, s)
            t = add(sub(s, sub(s2, bb)), sub(p, bb))
            ne = add(ne, sub(npe, t))
            s = s2
    return fin(s, ne)


def test_extraction_and_dot2_error_bounds():
    rng = np.random.default_rng(5)
    ext, d2 = [], []
    for h in (D4, LA8):
        L = len(h)
        g = [(-1) ** k * h[L - 1 - k] for k in range(L)]
        m = [F32(max(abs(a), abs(b)) * (1 + 1e-6)) for a, b in zip(h, g)]
        for trial in range(40):
            x = rng.standard_normal(L) * 10.0 ** rng.uniform(-20, 20)
            if trial % 2:
                x = x * 10.0 ** rng.uniform(-8, 0, L)
            a = [split(v) for v in x]
            for taps in (h, g):
                exact = sum(Fr(float(v)) * Fr(c) for v, c in zip(x, taps))
                scale = sum(abs(Fr(float(v)) * Fr(c)) for v, c in zip(x, taps))
                ext.append(float(abs(extraction(a, taps, m) - exact) / scale))
                d2.append(float(abs(dot2(a, taps) - exact) / scale))
    assert max(ext) < 5e-13 and np.median(ext) < 5e-14, (max(ext), np.median(ext))
    assert max(d2) < 3e-14, max(d2)

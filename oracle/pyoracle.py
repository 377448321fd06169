"""ctypes bindings for the oracle libraries (test infrastructure only).

Two CPU libraries, both built by oracle/Makefile:

* ``libwavoracle.so`` -- our C restatement of the reference CPU path
  (wavoracle.c).  Available wherever a C compiler is.
* ``_ref/libwavref.so`` -- the reference's own CPU sources compiled from the
  reference tree with a CPU-only shim (refshim.cpp).  Only present where the
  reference tree was available at build time.

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline import this
module; the product package never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "libwavoracle.so")
REF_SO = os.path.join(HERE, "_ref", "libwavref.so")

HAAR, D4, C6, LA8 = 1, 2, 3, 4
FILTER_LEN = {HAAR: 2, D4: 4, C6: 6, LA8: 8}
DWT, MODWT, MODWT_PO = 0, 1, 2
FWD, BWD = 1, 0
HARD, SOFT = 0, 1
MANUAL, UNIV, CV = 0, 1, 2

_dp = C.POINTER(C.c_double)
_i64 = C.c_int64


def build(quiet: bool = True) -> None:
    """Build the oracle libraries (the reference one only if its tree exists)."""
    out = subprocess.run(["make", "-C", HERE, "-j8", "all"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)


def _ptr(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


class CvTrace(C.Structure):
    _fields_ = [
        ("iters", C.c_int),
        ("t1", C.c_double * 64), ("t2", C.c_double * 64),
        ("m1", C.c_double * 64), ("m2", C.c_double * 64),
        ("took_m2", C.c_int * 64),
        ("t_final_raw", C.c_double),
        ("t_univ", C.c_double),
    ]


class Oracle:
    """Our restatement (wavoracle.c)."""

    def __init__(self, path: str = ORACLE_SO):
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        self.lib = L
        L.wo_check_len_levels.argtypes = [_i64, C.c_int, C.c_int]
        L.wo_dwt.argtypes = [_dp, _i64, C.c_int, C.c_int, C.c_int]
        L.wo_modwt.argtypes = [_dp, _dp, _i64, C.c_int, C.c_int, C.c_int]
        L.wo_threshold.argtypes = [_dp, _dp, _i64, C.c_int, C.c_int, C.c_int,
                                   C.c_double, C.c_int, C.c_int, C.c_int]
        L.wo_median.argtypes = [_dp, _i64]
        L.wo_median.restype = C.c_double
        L.wo_mad.argtypes = [_dp, _i64]
        L.wo_mad.restype = C.c_double
        L.wo_univ_thresh.argtypes = [_dp, _dp, _i64, C.c_int, C.c_int, C.c_int, C.c_int]
        L.wo_univ_thresh.restype = C.c_double
        L.wo_interp_mse.argtypes = [_dp, _dp, _dp, _i64]
        L.wo_interp_mse.restype = C.c_double
        L.wo_cvt.argtypes = [_dp, _i64, C.c_int, C.c_int, C.c_int, C.c_int,
                             C.c_double, C.c_int, C.c_int, C.c_int, C.POINTER(CvTrace)]
        L.wo_cvt.restype = C.c_double
        L.wo_smooth.argtypes = [_dp, _i64, C.c_int, C.c_int, C.c_int, C.c_int, _dp,
                                C.c_int, C.c_int, C.c_int, C.c_double]
        L.wo_count_kept.argtypes = [_dp, _dp, _i64, C.c_int, C.c_int, C.c_double,
                                    C.c_int, C.c_int, C.POINTER(_i64), C.POINTER(_i64)]
        L.wo_modwt_po.argtypes = [_dp, _dp, _i64, C.c_int, C.c_int, C.c_int]
        L.wo_set_threads.argtypes = [C.c_int]
        L.wo_get_threads.restype = C.c_int

    def set_threads(self, n: int) -> int:
        """Threads of the transform loops (n <= 0: every core); returns the
        count in effect.  Results do not depend on it."""
        self.lib.wo_set_threads(n)
        return self.lib.wo_get_threads()

    def levels(self, n, nlevels, filt):
        return self.lib.wo_check_len_levels(n, nlevels, FILTER_LEN[filt])

    def dwt(self, x, nlevels, filt, sense=FWD):
        y = np.array(x, dtype=np.float64, copy=True)
        r = self.lib.wo_dwt(_ptr(y), y.size, sense, nlevels, filt)
        if r:
            raise ValueError("oracle dwt rejected the arguments")
        return y

    def modwt_fwd(self, x, nlevels, filt):
        x = np.ascontiguousarray(x, dtype=np.float64)
        J = self.levels(x.size, nlevels, filt)
        if J == 0:
            raise ValueError(f"{nlevels} levels invalid for length {x.size}")
        xmod = np.zeros(2 * J * x.size)
        if self.lib.wo_modwt(_ptr(x), _ptr(xmod), x.size, FWD, J, filt):
            raise ValueError("oracle modwt rejected the arguments")
        return xmod

    def modwt_po_fwd(self, x, nlevels, filt):
        x = np.ascontiguousarray(x, dtype=np.float64)
        J = self.levels(x.size, nlevels, filt)
        if J == 0:
            raise ValueError(f"{nlevels} levels invalid for length {x.size}")
        xmod = np.zeros(2 * J * x.size)
        if self.lib.wo_modwt_po(_ptr(x), _ptr(xmod), x.size, FWD, J, filt):
            raise ValueError("oracle modwt_po rejected the arguments")
        return xmod

    def modwt_po_inv(self, xmod, n, nlevels, filt):
        xm = np.array(xmod, dtype=np.float64, copy=True)
        x = np.zeros(n)
        if self.lib.wo_modwt_po(_ptr(x), _ptr(xm), n, BWD, nlevels, filt):
            raise ValueError("oracle modwt_po rejected the arguments")
        return x

    def modwt_inv(self, xmod, n, nlevels, filt):
        xm = np.array(xmod, dtype=np.float64, copy=True)
        x = np.zeros(n)
        if self.lib.wo_modwt(_ptr(x), _ptr(xm), n, BWD, nlevels, filt):
            raise ValueError("oracle modwt rejected the arguments")
        return x

    def threshold(self, x, xmod, nlevels, ttype, filt, t, hardness, minlevel, maxlevel):
        x = np.array(x, dtype=np.float64, copy=True) if x is not None else None
        xm = np.array(xmod, dtype=np.float64, copy=True) if xmod is not None else None
        n = x.size if x is not None else xm.size // (2 * nlevels)
        self.lib.wo_threshold(_ptr(x), _ptr(xm), n, nlevels, ttype, filt, t,
                              hardness, minlevel, maxlevel)
        return x if ttype == DWT else xm

    def median(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        return self.lib.wo_median(_ptr(x), x.size)

    def mad(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        return self.lib.wo_mad(_ptr(x), x.size)

    def univ_thresh(self, w, n, nlevels, ttype, minlevel, maxlevel):
        w = np.ascontiguousarray(w, dtype=np.float64)
        if ttype == DWT:
            return self.lib.wo_univ_thresh(_ptr(w), None, n, nlevels, ttype, minlevel, maxlevel)
        return self.lib.wo_univ_thresh(None, _ptr(w), n, nlevels, ttype, minlevel, maxlevel)

    def cvt(self, x, nlevels, ttype, filt, hardness, tol, minlevel, maxlevel,
            copy_scaling=False):
        y = np.array(x, dtype=np.float64, copy=True)
        tr = CvTrace()
        t = self.lib.wo_cvt(_ptr(y), y.size, nlevels, ttype, filt, hardness, tol,
                            minlevel, maxlevel, int(copy_scaling), C.byref(tr))
        return t, y, tr

    def smooth(self, x, nlevels, ttype, filt, threshtype, thresh, hardness,
               minlevel, maxlevel, tol):
        y = np.array(x, dtype=np.float64, copy=True)
        t = np.array([thresh if thresh is not None else 0.0])
        r = self.lib.wo_smooth(_ptr(y), y.size, nlevels, ttype, filt, threshtype,
                               _ptr(t), hardness, minlevel, maxlevel, tol)
        if r:
            raise ValueError("oracle smooth rejected the arguments")
        return y, float(t[0])

    def count_kept(self, w, n, nlevels, ttype, t, minlevel, maxlevel):
        w = np.ascontiguousarray(w, dtype=np.float64)
        k, z = _i64(), _i64()
        if ttype == DWT:
            self.lib.wo_count_kept(_ptr(w), None, n, nlevels, ttype, t, minlevel,
                                   maxlevel, C.byref(k), C.byref(z))
        else:
            self.lib.wo_count_kept(None, _ptr(w), n, nlevels, ttype, t, minlevel,
                                   maxlevel, C.byref(k), C.byref(z))
        return k.value, z.value


class Reference:
    """The reference's own CPU sources (oracle/_ref/libwavref.so)."""

    def __init__(self, path: str = REF_SO):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        L = C.CDLL(path)
        self.lib = L
        ci = C.c_int
        L.wref_transform.argtypes = [_dp, _dp, ci, ci, ci, ci, ci, ci]
        L.wref_threshold.argtypes = [_dp, _dp, ci, ci, ci, ci, ci, C.c_double, ci, ci, ci]
        L.wref_smooth.argtypes = [_dp, ci, ci, ci, ci, ci, ci, _dp, ci, ci, ci, C.c_double]
        L.wref_univ_thresh.argtypes = [_dp, _dp, ci, ci, ci, ci, ci, ci, ci]
        L.wref_univ_thresh.restype = C.c_double
        L.wref_median.argtypes = [_dp, ci]
        L.wref_median.restype = C.c_double
        L.wref_mad.argtypes = [_dp, ci]
        L.wref_mad.restype = C.c_double
        L.wref_check_len_levels.argtypes = [C.c_uint, C.c_uint, C.c_uint]
        L.wref_check_len_levels.restype = C.c_uint

    def levels(self, n, nlevels, filt):
        return self.lib.wref_check_len_levels(n, nlevels, FILTER_LEN[filt])

    def dwt(self, x, nlevels, filt, sense=FWD):
        y = np.array(x, dtype=np.float64, copy=True)
        dummy = np.zeros(1)
        r = self.lib.wref_transform(_ptr(y), _ptr(dummy), y.size, sense, nlevels, DWT,
                                    filt, FILTER_LEN[filt])
        if r:
            raise ValueError("reference transform failed")
        return y

    def modwt_fwd(self, x, nlevels, filt):
        x = np.array(x, dtype=np.float64, copy=True)
        J = self.levels(x.size, nlevels, filt)
        if J == 0:
            raise ValueError(f"{nlevels} levels invalid for length {x.size}")
        xmod = np.zeros(2 * J * x.size)
        r = self.lib.wref_transform(_ptr(x), _ptr(xmod), x.size, FWD, J, MODWT, filt,
                                    FILTER_LEN[filt])
        if r:
            raise ValueError("reference transform failed")
        return xmod

    def modwt_inv(self, xmod, n, nlevels, filt):
        xm = np.array(xmod, dtype=np.float64, copy=True)
        x = np.zeros(n)
        r = self.lib.wref_transform(_ptr(x), _ptr(xm), n, BWD, nlevels, MODWT, filt,
                                    FILTER_LEN[filt])
        if r:
            raise ValueError("reference transform failed")
        return x

    def modwt_po_fwd(self, x, nlevels, filt):
        x = np.array(x, dtype=np.float64, copy=True)
        J = self.levels(x.size, nlevels, filt)
        if J == 0:
            raise ValueError(f"{nlevels} levels invalid for length {x.size}")
        xmod = np.zeros(2 * J * x.size)
        if self.lib.wref_transform(_ptr(x), _ptr(xmod), x.size, FWD, J, MODWT_PO, filt,
                                   FILTER_LEN[filt]):
            raise ValueError("reference transform failed")
        return xmod

    def modwt_po_inv(self, xmod, n, nlevels, filt):
        xm = np.array(xmod, dtype=np.float64, copy=True)
        x = np.zeros(n)
        if self.lib.wref_transform(_ptr(x), _ptr(xm), n, BWD, nlevels, MODWT_PO, filt,
                                   FILTER_LEN[filt]):
            raise ValueError("reference transform failed")
        return x

    def threshold(self, x, xmod, nlevels, ttype, filt, t, hardness, minlevel, maxlevel):
        x = np.array(x, dtype=np.float64, copy=True) if x is not None else np.zeros(1)
        xm = np.array(xmod, dtype=np.float64, copy=True) if xmod is not None else np.zeros(1)
        n = x.size if ttype == DWT else xm.size // (2 * nlevels)
        self.lib.wref_threshold(_ptr(x), _ptr(xm), n, nlevels, ttype, filt,
                                FILTER_LEN[filt], t, hardness, minlevel, maxlevel)
        return x if ttype == DWT else xm

    def median(self, x):
        x = np.array(x, dtype=np.float64, copy=True)
        return self.lib.wref_median(_ptr(x), x.size)

    def mad(self, x):
        x = np.array(x, dtype=np.float64, copy=True)
        return self.lib.wref_mad(_ptr(x), x.size)

    def univ_thresh(self, w, n, nlevels, ttype, filt, minlevel, maxlevel):
        w = np.array(w, dtype=np.float64, copy=True)
        if ttype == DWT:
            return self.lib.wref_univ_thresh(_ptr(w), _ptr(np.zeros(1)), n, nlevels, ttype,
                                             filt, FILTER_LEN[filt], minlevel, maxlevel)
        return self.lib.wref_univ_thresh(_ptr(np.zeros(n)), _ptr(w), n, nlevels, ttype,
                                         filt, FILTER_LEN[filt], minlevel, maxlevel)

    def smooth(self, x, nlevels, ttype, filt, threshtype, thresh, hardness,
               minlevel, maxlevel, tol):
        y = np.array(x, dtype=np.float64, copy=True)
        t = np.array([thresh if thresh is not None else 0.0])
        r = self.lib.wref_smooth(_ptr(y), y.size, nlevels, ttype, filt, FILTER_LEN[filt],
                                 threshtype, _ptr(t), hardness, minlevel, maxlevel, tol)
        if r:
            raise ValueError("reference smooth failed")
        return y, float(t[0])


def reference_available() -> bool:
    return os.path.exists(REF_SO)


# ---------------------------------------------------------------------------
# Coefficient extraction and formatting (R code of the reference, restated
# step by step in numpy; R is not available here, so these follow the R
# source line by line rather than a compiled reference).

def coeff_level(n, nlevels, ttype, level, coeff_type="d"):
    """getCoeffLevel (R/rplotting.R:10-46): 1-based indices."""
    if level <= 0 or level > nlevels:
        raise ValueError("Integer level expected")
    d_bool = 1 if coeff_type == "d" else 0
    if ttype == DWT:
        if not d_bool and level != nlevels:
            raise ValueError("stopifnot(level == xw$nlevels)")
        start, gap = 2 ** (level - 1) * d_bool + 1, 2 ** level
    else:
        start, gap = 1, 1
    return np.arange(start, n + 1, gap, dtype=np.int64)          # seq(start, n, by = gap)


def wst_to_dt(w, n, nlevels, ttype, scaling=True):
    """WSTtoDT(Xwav, scaling, forPlotting = FALSE) (R/rfunctions.R:925-1004):
    columns W, CoeffType, Level, Translate in row order (without data.table)."""
    J = nlevels
    w = np.asarray(w, dtype=np.float64)
    if ttype == DWT:
        i1 = np.arange(1, n + 1)
        ctype = np.where(i1 % (2 ** J) == 1, "s", "d")             # label.detail.scaling
        level = np.ones(n, dtype=np.int64)                          # rep(1, len)
        translate = np.repeat(np.arange(0.5, n / 2, 1.0), 2)        # rep(seq(0.5, len/2, 1), each = 2)
        if J > 1:
            for l in range(2, J + 1):
                rows = coeff_level(n, J, DWT, l, "d") - 1
                level[rows] = l
                translates = np.arange(2.0 ** (l - 2), n / 2 + 1e-9, 2.0 ** (l - 1))
                translate[rows] = translates
            rows = coeff_level(n, J, DWT, J, "s") - 1                # l == nlevels after the loop
            level[rows] = J
            translate[rows] = translates
        W = w[:n].copy()
    else:
        W = w[:2 * J * n].copy()
        ctype = np.tile(np.repeat(np.array(["s", "d"]), n), J)
        level = np.repeat(np.arange(1, J + 1), 2 * n)
        translate = np.tile(np.arange(1, n + 1, dtype=np.float64), 2 * J)
    keep = np.ones(W.size, dtype=bool) if scaling else (ctype == "d")
    return {"W": W[keep], "CoeffType": ctype[keep], "Level": level[keep].astype(np.int64),
            "Translate": translate[keep]}

"""wavecuda_gb300: GB300-native (sm_103a) wavelet transforms, thresholding and
cross-validated smoothing behind the wavecuda reference's C ABI.

The compute lives in ``libwavecuda_gb300.so`` (CUDA kernels + C ABI, built
in-tree by :mod:`wavecuda_gb300.build`).  This module binds it with ctypes and
mirrors the reference's R entry points (R/rfunctions.R: CPUTransform,
GPUTransform, CPUReconstruct, GPUReconstruct, CPUThreshold, CPUSmooth,
GPUSmooth and their input checks) with the same argument meaning and the same
error conditions (R's ``stop`` becomes ``ValueError``).  There is no CPU
fallback: every call goes to the GPU library, and importing the bindings
raises if the library is missing.
"""
from __future__ import annotations

import ctypes as C
import math
import os
from dataclasses import dataclass
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libwavecuda_gb300.so")

# Codes (wvtheads.h:14-38, rfunctions.cuh:13-15).
FWD, BWD = 1, 0
HAAR, D4, C6, LA8 = 1, 2, 3, 4
DWT, MODWT, MODWT_PO = 0, 1, 2
HARD, SOFT = 0, 1
MANUAL, UNIV, CV = 0, 1, 2
F64_EXACT, F64_FAST, F32 = 0, 1, 2

WC_OK = 0
ERRORS = {1: "invalid argument", 2: "level error", 3: "CUDA error", 4: "out of memory",
          5: "unsupported", 6: "no CUDA device", 7: "timeout"}

FILTERS = {"Haar": HAAR, "D4": D4, "C6": C6, "LA8": LA8}
FILTER_LEN = {HAAR: 2, D4: 4, C6: 6, LA8: 8}


class WaveCudaError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class SmoothInfo(C.Structure):
    _fields_ = [("thresh", C.c_double), ("thresh_univ", C.c_double),
                ("cv_iterations", C.c_int), ("levels", C.c_int),
                ("kept", C.c_int64), ("zeroed", C.c_int64), ("min_margin", C.c_double)]


class Signal(C.Structure):
    """wc_signal: one signal of a batch."""
    _fields_ = [("offset", C.c_int64), ("len", C.c_int64), ("nlevels", C.c_int),
                ("ttype", C.c_int), ("filter", C.c_int), ("threshtype", C.c_int),
                ("hardness", C.c_int), ("minlevel", C.c_int), ("maxlevel", C.c_int),
                ("thresh", C.c_double), ("tol", C.c_double)]


class SignalResult(C.Structure):
    _fields_ = [("thresh", C.c_double), ("thresh_univ", C.c_double),
                ("min_margin", C.c_double), ("iterations", C.c_int), ("status", C.c_int),
                ("kept", C.c_int64), ("zeroed", C.c_int64)]


FIT_MAX_LEVELS = 24


class FitOpts(C.Structure):
    _fields_ = [("loss_type", C.c_int), ("minlevel", C.c_int), ("maxlevel", C.c_int),
                ("iterations", C.c_int), ("step", C.c_double), ("eps", C.c_double),
                ("sigma", C.c_double), ("lambda0", C.POINTER(C.c_double)),
                ("precision", C.c_int), ("smooth", C.c_int)]


class FitResult(C.Structure):
    _fields_ = [("lambda_", C.c_double * FIT_MAX_LEVELS), ("grad0", C.c_double * FIT_MAX_LEVELS),
                ("loss0", C.c_double), ("loss", C.c_double), ("sigma", C.c_double),
                ("iterations", C.c_int), ("status", C.c_int)]


_lib: Optional[C.CDLL] = None
_ip = C.POINTER(C.c_int)
_dp = C.POINTER(C.c_double)
_vp = C.c_void_p


def lib() -> C.CDLL:
    """The loaded GPU library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with python -m wavecuda_gb300.build")
    L = C.CDLL(LIB_PATH)
    for name in ("RcpuTransform", "RgpuTransform"):
        getattr(L, name).argtypes = [_dp, _dp] + [_ip] * 6
        getattr(L, name).restype = None
    L.RcpuThreshold.argtypes = [_dp, _dp] + [_ip] * 5 + [_dp, _ip, _ip, _ip]
    L.RcpuThreshold.restype = None
    for name in ("RcpuSmooth", "RgpuSmooth"):
        getattr(L, name).argtypes = [_dp] + [_ip] * 6 + [_dp, _ip, _ip, _ip, _dp]
        getattr(L, name).restype = None
    L.wc_last_error.restype = C.c_char_p
    L.wc_max_levels.argtypes = [C.c_int64, C.c_int]
    L.wc_set_default_precision.argtypes = [C.c_int]
    L.wc_transform.argtypes = [_dp, _dp, C.c_int64, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
    L.wc_threshold.argtypes = [_dp, _dp, C.c_int64, C.c_int, C.c_int, C.c_int, C.c_double,
                               C.c_int, C.c_int, C.c_int]
    L.wc_smooth.argtypes = [_dp, C.c_int64, C.c_int, C.c_int, C.c_int, C.c_int, _dp, C.c_int,
                            C.c_int, C.c_int, C.c_double, C.c_int, C.POINTER(SmoothInfo)]
    L.wc_dwt_device.argtypes = [_vp, _vp, C.c_int64, C.c_int, C.c_int, C.c_int, C.c_int, _vp]
    L.wc_modwt_device.argtypes = [_vp, _vp, C.c_int64, C.c_int, C.c_int, C.c_int, C.c_int, _vp]
    L.wc_median_mad_device.argtypes = [_vp, C.c_int64, _dp, _dp, _vp]
    L.wc_sequential_sum_device.argtypes = [_vp, C.c_int64, _dp, _vp]
    L.wc_dwt_adjoint_device.argtypes = [_vp, _vp, C.c_int64, C.c_int, C.c_int, C.c_int, C.c_int,
                                        _vp]
    L.wc_modwt_adjoint_device.argtypes = [_vp, _vp, C.c_int64, C.c_int, C.c_int, C.c_int, _vp]
    L.wc_soft_threshold_adjoint_device.argtypes = [_vp, _vp, _vp, _vp, C.c_int64, C.c_int,
                                                   C.c_int, _dp, C.c_int, C.c_int, _vp]
    L.wc_loss_grad.argtypes = [_vp, C.c_int64, C.c_int, C.c_int, C.c_int, C.c_int, _dp, C.c_int,
                               C.c_int, C.c_double, C.c_double, _dp, _dp, _dp, _vp]
    L.wc_fit_thresholds_device.argtypes = [_vp, C.c_int64, C.c_int, C.c_int, C.c_int, C.c_int,
                                           C.POINTER(FitOpts), C.POINTER(FitResult), _vp]
    L.wc_fit_thresholds.argtypes = [_dp, C.c_int64, C.c_int, C.c_int, C.c_int, C.c_int,
                                    C.POINTER(FitOpts), C.POINTER(FitResult)]
    L.wc_batch_plan_create.argtypes = [C.POINTER(Signal), C.c_int, C.c_int, C.POINTER(_vp)]
    L.wc_batch_plan_destroy.argtypes = [_vp]
    L.wc_batch_plan_info.argtypes = [_vp, _ip, C.POINTER(C.c_size_t)]
    L.wc_batch_plan_pairs.argtypes = [_vp, _ip]
    L.wc_batch_autotune.argtypes = [_vp, _vp, C.POINTER(C.c_float)]
    L.wc_batch_run_device.argtypes = [_vp, _vp, _vp]
    L.wc_batch_results.argtypes = [_vp, C.POINTER(SignalResult), _vp]
    L.wc_smooth_batch.argtypes = [_dp, C.c_int64, C.POINTER(Signal), C.c_int, C.c_int,
                                  C.POINTER(SignalResult)]
    L.wc_device_status.argtypes = [C.POINTER(C.c_uint)]
    L.wc_set_dwt_tiling.argtypes = [C.c_int] * 6
    L.wc_get_dwt_tiling.argtypes = [C.c_int, C.c_int, _ip, _ip, _ip, _ip]
    L.wc_tune_dwt.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_float)]
    L.wc_set_modwt_tiling.argtypes = [C.c_int] * 6
    L.wc_get_modwt_tiling.argtypes = [C.c_int, C.c_int, _ip, _ip, _ip, _ip]
    L.wc_set_modwt_inv_levels.argtypes = [C.c_int, C.c_int, C.c_int]
    L.wc_get_modwt_inv_levels.argtypes = [C.c_int, C.c_int, _ip]
    L.wc_tune_modwt.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_float),
                                C.POINTER(C.c_float)]
    L.wc_device_count.argtypes = [_ip]
    L.wc_malloc_device.argtypes = [C.POINTER(_vp), C.c_size_t]
    L.wc_free_device.argtypes = [_vp]
    L.wc_malloc_host.argtypes = [C.POINTER(_vp), C.c_size_t]
    L.wc_free_host.argtypes = [_vp]
    L.wc_memcpy.argtypes = [_vp, _vp, C.c_size_t, _vp]
    L.wc_memset_device.argtypes = [_vp, C.c_int, C.c_size_t, _vp]
    L.wc_stream_synchronize.argtypes = [_vp]
    L.wc_default_stream.argtypes = [C.POINTER(_vp)]
    L.wc_event_create.argtypes = [C.POINTER(_vp)]
    L.wc_event_destroy.argtypes = [_vp]
    L.wc_event_record.argtypes = [_vp, _vp]
    L.wc_event_elapsed_ms.argtypes = [_vp, _vp, C.POINTER(C.c_float)]
    L.wc_kernel_launch_count.restype = C.c_int64
    _i64p = C.POINTER(C.c_int64)
    L.wc_coeff_level_indices.argtypes = [C.c_int64, C.c_int, C.c_int, C.c_int, C.c_int, _i64p,
                                         C.c_int64, _i64p]
    L.wc_wst_table_rows.argtypes = [C.c_int64, C.c_int, C.c_int, C.c_int, _i64p]
    L.wc_wst_table_device.argtypes = [_vp, C.c_int64, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp,
                                      _vp, _vp]
    L.wc_wst_table.argtypes = [_dp, C.c_int64, C.c_int, C.c_int, C.c_int, _dp,
                               C.POINTER(C.c_int32), _dp, C.POINTER(C.c_uint8)]
    for name in ("wc_transform_R",):
        getattr(L, name).argtypes = [_dp, _dp] + [_ip] * 7
        getattr(L, name).restype = None
    L.wc_threshold_R.argtypes = [_dp, _dp] + [_ip] * 4 + [_dp, _ip, _ip, _ip, _ip]
    L.wc_threshold_R.restype = None
    L.wc_smooth_R.argtypes = [_dp] + [_ip] * 5 + [_dp, _ip, _ip, _ip, _dp, _ip, _ip]
    L.wc_smooth_R.restype = None
    L.RgpuSmoothBatch.argtypes = ([_dp, _ip, _ip, _ip, _ip, _ip, _ip, _ip, _ip, _dp, _ip, _ip,
                                   _ip, _dp, _ip, _ip, _ip, _ip, _ip])
    L.RgpuSmoothBatch.restype = None
    L.wc_measure_fp64_rate.argtypes = [_dp, _vp]
    L.wc_debug_set_workspace_cap.argtypes = [C.c_size_t]
    L.wc_debug_workspace_bytes.argtypes = [C.POINTER(C.c_size_t)]
    L.wc_debug_wait_probe.argtypes = [C.c_int, C.c_uint, _vp]
    _lib = L
    return L


def check(code: int) -> None:
    if code != WC_OK:
        raise WaveCudaError(code, lib().wc_last_error().decode())


def last_error() -> str:
    return lib().wc_last_error().decode()


def _dptr(a: Optional[np.ndarray]):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def _ci(v: int):
    return C.byref(C.c_int(int(v)))


# ------------------------------------------------------------------------
# Mirror of R/rfunctions.R
# ------------------------------------------------------------------------

@dataclass
class WST:
    """The R "WST" object (return.trans, rfunctions.R:259-292)."""
    x: np.ndarray
    ttype: str
    filt: str
    filtlen: int
    nlevels: int
    len: int
    w: np.ndarray


def _ttype_code(transform_type):
    return {"DWT": DWT, "MODWT": MODWT}.get(transform_type)


def check_trans_inputs(xin, direction, nlevels, transform_type, filter):
    """check.trans.inputs (rfunctions.R:64-119)."""
    ttype = _ttype_code(transform_type)
    if ttype is None:
        raise ValueError("Unexpected transform type")
    filt = FILTERS.get(filter)
    if filt is None:
        raise ValueError("Unexpected filter")
    filtlen = FILTER_LEN[filt]
    sense = {"FWD": FWD, "BWD": BWD}.get(direction)
    if sense is None:
        raise ValueError("Unexpected direction!")
    xin = np.asarray(xin)
    if not np.issubdtype(xin.dtype, np.number):
        raise ValueError("Unexpected input vector")
    lenxin = xin.size

    def is_pow2(v):
        return v > 0 and math.log2(v) == round(math.log2(v))

    if ttype == DWT:
        x = np.array(xin, dtype=np.float64)
        xmod = np.zeros(0)
        n = lenxin
        if not is_pow2(n):
            raise ValueError("Need length to be power of 2")
    elif sense == FWD:
        x = np.array(xin, dtype=np.float64)
        n = lenxin
        if not is_pow2(n):
            raise ValueError("Need length to be power of 2")
        xmod = np.zeros(int(n * 2 * math.log2(n)))
    else:
        xmod = np.array(xin, dtype=np.float64)
        if nlevels == 0:
            raise ValueError("Probably got an error of infinite length")
        n = lenxin / (2 * nlevels)
        if not is_pow2(n):
            raise ValueError("Was this really a MODWT vector? If so, check nlevels. "
                             "I calculate the reconstruction vector to be of inappropriate size.")
        n = int(n)
        x = np.zeros(n)
    maxlevels = math.floor(math.log2(n / filtlen)) + 1 if n >= 1 else 0
    if nlevels == 0:
        nlevels = maxlevels
    if nlevels != round(nlevels) or nlevels < 0 or nlevels > maxlevels:
        raise ValueError(f"nlevels should be an integer [whole number] between 1 and {maxlevels}")
    # The reference stops here for C6/LA8 MODWT (rfunctions.R:114-116); this
    # library provides them, so the check is not repeated.
    return dict(x=x, xmod=xmod, len=int(n), sense=sense, nlevels=int(nlevels), ttype=ttype,
                filt=filt, filtlen=filtlen)


def _call_transform(symbol, a):
    xmod = a["xmod"] if a["xmod"].size else np.zeros(1)
    getattr(lib(), symbol)(_dptr(a["x"]), _dptr(xmod), _ci(a["len"]), _ci(a["sense"]),
                           _ci(a["nlevels"]), _ci(a["ttype"]), _ci(a["filt"]), _ci(a["filtlen"]))
    err = last_error()
    if err:
        raise WaveCudaError(3, err)
    a["xmod"] = xmod if a["xmod"].size else a["xmod"]
    return a


def _return_trans(a, transform_type, filter, xin):
    if a["sense"] == FWD:
        w = a["x"] if a["ttype"] == DWT else a["xmod"][: 2 * a["len"] * a["nlevels"]]
        return WST(x=np.asarray(xin, dtype=np.float64), ttype=transform_type, filt=filter,
                   filtlen=a["filtlen"], nlevels=a["nlevels"], len=a["len"], w=w)
    return a["x"]


def CPUTransform(xin, direction="FWD", nlevels=0, transform_type="DWT", filter="Haar"):
    """CPUTransform (rfunctions.R:334-357); served by the GPU path."""
    a = check_trans_inputs(xin, direction, nlevels, transform_type, filter)
    return _return_trans(_call_transform("RcpuTransform", a), transform_type, filter, xin)


def GPUTransform(xin, direction="FWD", nlevels=0, transform_type="DWT", filter="Haar"):
    """GPUTransform (rfunctions.R:383-406)."""
    a = check_trans_inputs(xin, direction, nlevels, transform_type, filter)
    return _return_trans(_call_transform("RgpuTransform", a), transform_type, filter, xin)


def _prepare_wst(xwav: WST):
    """prepare.wst.arg.list (rfunctions.R:128-153)."""
    ttype = _ttype_code(xwav.ttype)
    filt = FILTERS[xwav.filt]
    if ttype == DWT:
        x, xmod = np.array(xwav.w, dtype=np.float64), np.zeros(0)
    else:
        x, xmod = np.zeros(xwav.len), np.array(xwav.w, dtype=np.float64)
    return dict(x=x, xmod=xmod, len=xwav.len, sense=BWD, nlevels=xwav.nlevels, ttype=ttype,
                filt=filt, filtlen=FILTER_LEN[filt])


def CPUReconstruct(xwav: WST):
    """CPUReconstruct (rfunctions.R:420-436)."""
    return _call_transform("RcpuTransform", _prepare_wst(xwav))["x"]


def GPUReconstruct(xwav: WST):
    """GPUReconstruct (rfunctions.R:451-467)."""
    return _call_transform("RgpuTransform", _prepare_wst(xwav))["x"]


def check_thresh_inputs(xwav: WST, hard_soft, thresh, min_level, max_level):
    """check.thresh.inputs (rfunctions.R:168-193)."""
    a = _prepare_wst(xwav)
    if np.ndim(thresh) != 0:
        raise ValueError("Only scalar thresholds supported")
    if thresh <= 0:
        raise ValueError("Threshold must be greater than 0")
    a["thresh"] = float(thresh)
    a["hardness"] = {"hard": HARD, "soft": SOFT}.get(hard_soft)
    if a["hardness"] is None:
        raise ValueError("Only hard or soft thresholding supported")
    if (min_level != round(min_level) or max_level != round(max_level) or min_level > max_level
            or min_level <= 0 or max_level > xwav.nlevels):
        raise ValueError("min.level and max.level must be integers in the range 1...nlevels")
    a["min.level"] = int(min_level) - 1
    a["max.level"] = int(max_level) - 1
    return a


def CPUThreshold(xwav: WST, thresh, hard_soft, min_level, max_level) -> WST:
    """CPUThreshold (rfunctions.R:507-528)."""
    a = check_thresh_inputs(xwav, hard_soft, thresh, min_level, max_level)
    xmod = a["xmod"] if a["xmod"].size else np.zeros(1)
    lib().RcpuThreshold(_dptr(a["x"]), _dptr(xmod), _ci(xwav.len), _ci(xwav.nlevels),
                        _ci(a["ttype"]), _ci(a["filt"]), _ci(a["filtlen"]),
                        C.byref(C.c_double(a["thresh"])), _ci(a["hardness"]),
                        _ci(a["min.level"]), _ci(a["max.level"]))
    err = last_error()
    if err:
        raise WaveCudaError(2, err)
    out = WST(**{**xwav.__dict__})
    out.w = a["x"] if a["ttype"] == DWT else xmod
    return out


def check_smooth_inputs(xin, nlevels, transform_type, filter, thresh_type, thresh, hard_soft,
                        min_level, max_level, tol):
    """check.smooth.inputs (rfunctions.R:211-249)."""
    a = check_trans_inputs(xin, "FWD", nlevels, transform_type, filter)
    a["threshtype"] = {"manual": MANUAL, "univ": UNIV, "cv": CV}.get(thresh_type)
    if a["threshtype"] is None:
        raise ValueError("Only manual, univ or cv supported for threshold type")
    if thresh_type == "manual":
        if thresh is None or np.ndim(thresh) != 0:
            raise ValueError("Only scalar thresholds supported")
        if thresh <= 0:
            raise ValueError("Threshold must be greater than 0")
        a["thresh"] = float(thresh)
    else:
        a["thresh"] = 0.0
    if thresh_type == "cv":
        if tol <= 0:
            raise ValueError("Tolerance must be greater than 0")
        a["tol"] = float(tol)
    else:
        a["tol"] = 0.0
    a["hardness"] = {"hard": HARD, "soft": SOFT}.get(hard_soft)
    if a["hardness"] is None:
        raise ValueError("Only hard or soft thresholding supported")
    if (min_level != round(min_level) or max_level != round(max_level) or min_level > max_level
            or min_level <= 0 or max_level > nlevels):
        raise ValueError("min.level and max.level must be integers in the range 1...nlevels")
    a["min.level"] = int(min_level) - 1
    a["max.level"] = int(max_level) - 1
    return a


def _call_smooth(symbol, a):
    t = C.c_double(a["thresh"])
    getattr(lib(), symbol)(_dptr(a["x"]), _ci(a["len"]), _ci(a["nlevels"]), _ci(a["ttype"]),
                           _ci(a["filt"]), _ci(a["filtlen"]), _ci(a["threshtype"]), C.byref(t),
                           _ci(a["hardness"]), _ci(a["min.level"]), _ci(a["max.level"]),
                           C.byref(C.c_double(a["tol"])))
    err = last_error()
    if err:
        raise WaveCudaError(3, err)
    a["thresh"] = t.value
    return a["x"]


def CPUSmooth(xin, nlevels, transform_type, filter, thresh_type, thresh=None, hard_soft="soft",
              min_level=1, max_level=1, tol=0.01):
    """CPUSmooth (rfunctions.R:547-569)."""
    a = check_smooth_inputs(xin, nlevels, transform_type, filter, thresh_type, thresh, hard_soft,
                            min_level, max_level, tol)
    return _call_smooth("RcpuSmooth", a)


def getCoeffLevel(xw: WST, level, coeffType="d"):
    """getCoeffLevel (R/rplotting.R:10-46): 1-based indices of the
    coefficients of `level` in xw.w (DWT: 2^(level-1)*[d] + 1 step 2^level;
    MODWT: 1..len whatever the level, as the reference returns)."""
    if not isinstance(xw, WST):
        raise ValueError("WST type required")
    if level <= 0 or level > xw.nlevels or level != int(level):
        raise ValueError(f"Integer level expected, between 1 and {xw.nlevels}")
    if coeffType not in ("d", "s"):
        raise ValueError("coeffType must be 'd' or 's'")
    if xw.ttype == "DWT" and coeffType == "s" and level != xw.nlevels:
        raise ValueError("level == xw$nlevels is not TRUE")
    L = lib()
    ttype = DWT if xw.ttype == "DWT" else MODWT
    cnt = C.c_int64()
    ct = 1 if coeffType == "d" else 0
    check(L.wc_coeff_level_indices(xw.len, xw.nlevels, ttype, int(level), ct, None, 0,
                                   C.byref(cnt)))
    idx = np.empty(cnt.value, dtype=np.int64)
    check(L.wc_coeff_level_indices(xw.len, xw.nlevels, ttype, int(level), ct,
                                   idx.ctypes.data_as(C.POINTER(C.c_int64)), idx.size,
                                   C.byref(cnt)))
    return idx


def WSTtoDT(xw: WST, scaling=True, forPlotting=False):
    """WSTtoDT (R/rfunctions.R:925-1004) without data.table: the columns W,
    CoeffType ("s"/"d"), Level and Translate as numpy arrays, in the
    reference's row order, computed on the GPU (wc_wst_table).  The plotting
    rows of forPlotting = TRUE (per-level min/max placeholders) are not
    provided: plotting is outside this library."""
    if forPlotting:
        raise NotImplementedError("forPlotting rows are plotting-only and not provided")
    if xw.ttype not in ("DWT", "MODWT"):
        raise ValueError("WSTtoDT takes DWT or MODWT transforms")
    L = lib()
    ttype = DWT if xw.ttype == "DWT" else MODWT
    rows = C.c_int64()
    check(L.wc_wst_table_rows(xw.len, xw.nlevels, ttype, int(bool(scaling)), C.byref(rows)))
    n = rows.value
    W = np.empty(n, dtype=np.float64)
    lev = np.empty(n, dtype=np.int32)
    tr = np.empty(n, dtype=np.float64)
    ty = np.empty(n, dtype=np.uint8)
    w = np.ascontiguousarray(xw.w, dtype=np.float64)
    check(L.wc_wst_table(_dptr(w), xw.len, xw.nlevels, ttype, int(bool(scaling)), _dptr(W),
                         lev.ctypes.data_as(C.POINTER(C.c_int32)), _dptr(tr),
                         ty.ctypes.data_as(C.POINTER(C.c_uint8))))
    return {"W": W, "CoeffType": np.where(ty == 1, "d", "s"), "Level": lev, "Translate": tr}


def GPUSmooth(xin, nlevels, transform_type, filter, thresh_type, thresh=None, hard_soft="soft",
              min_level=1, max_level=1, tol=0.01):
    """GPUSmooth (rfunctions.R:588-612).  Unlike the reference this accepts
    "univ" and the D4/C6/LA8 filters (rfunctions.R:592-594 refused them)."""
    a = check_smooth_inputs(xin, nlevels, transform_type, filter, thresh_type, thresh, hard_soft,
                            min_level, max_level, tol)
    return _call_smooth("RgpuSmooth", a)


# ------------------------------------------------------------------------
# Direct bindings of the status-returning API
# ------------------------------------------------------------------------

def max_levels(n: int, filt: int) -> int:
    return lib().wc_max_levels(n, FILTER_LEN[filt])


def set_default_precision(p: int) -> None:
    check(lib().wc_set_default_precision(p))


def transform(x, nlevels, ttype, filt, sense=FWD, precision=F64_EXACT, xmod=None):
    """wc_transform on host arrays.  FWD DWT returns the interleaved transform,
    FWD MODWT returns xmod, BWD returns the signal."""
    L = lib()
    if ttype == DWT:
        y = np.array(x, dtype=np.float64, copy=True)
        check(L.wc_transform(_dptr(y), None, y.size, sense, nlevels, ttype, filt, precision))
        return y
    if sense == FWD:
        x = np.ascontiguousarray(x, dtype=np.float64)
        J = nlevels or max_levels(x.size, filt)
        xm = np.zeros(2 * J * x.size)
        check(L.wc_transform(_dptr(x), _dptr(xm), x.size, FWD, J, ttype, filt, precision))
        return xm
    xm = np.ascontiguousarray(xmod if xmod is not None else x, dtype=np.float64)
    n = xm.size // (2 * nlevels)
    y = np.zeros(n)
    check(L.wc_transform(_dptr(y), _dptr(xm), n, BWD, nlevels, ttype, filt, precision))
    return y


def threshold(w, n, nlevels, ttype, filt, thresh, hardness, minlevel, maxlevel):
    y = np.array(w, dtype=np.float64, copy=True)
    if ttype == DWT:
        check(lib().wc_threshold(_dptr(y), None, n, nlevels, ttype, filt, thresh, hardness,
                                 minlevel, maxlevel))
    else:
        check(lib().wc_threshold(None, _dptr(y), n, nlevels, ttype, filt, thresh, hardness,
                                 minlevel, maxlevel))
    return y


def smooth(x, nlevels, ttype, filt, threshtype, thresh=0.0, hardness=SOFT, minlevel=0,
           maxlevel=None, tol=1e-8, precision=F64_EXACT):
    """wc_smooth: returns (smoothed, SmoothInfo)."""
    y = np.array(x, dtype=np.float64, copy=True)
    J = nlevels or max_levels(y.size, filt)
    if maxlevel is None:
        maxlevel = J - 1
    t = C.c_double(thresh)
    info = SmoothInfo()
    check(lib().wc_smooth(_dptr(y), y.size, J, ttype, filt, threshtype, C.byref(t), hardness,
                          minlevel, maxlevel, tol, precision, C.byref(info)))
    return y, info


def median_mad(v) -> tuple:
    """Exact median and MAD of a host vector, computed on the device."""
    v = np.ascontiguousarray(v, dtype=np.float64)
    buf = DeviceBuffer(max(8, v.nbytes))
    buf.upload(v)
    med, mad = C.c_double(), C.c_double()
    check(lib().wc_median_mad_device(buf.ptr, v.size, C.byref(med), C.byref(mad), None))
    buf.free()
    return med.value, mad.value


LOSS_SURE, LOSS_CV = 0, 1


def loss_grad(x, nlevels, filter, ttype, loss_type, lam, min_level=0, max_level=None,
              sigma=0.0, eps=0.0):
    """Loss of per-level soft thresholds and its gradient (wc_loss_grad).

    lam holds one threshold per level (0-based levels); returns
    (loss, grad, sigma_used)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    lam = np.ascontiguousarray(lam, dtype=np.float64)
    if max_level is None:
        max_level = nlevels - 1
    grad = np.zeros(nlevels, dtype=np.float64)
    loss, sig = C.c_double(), C.c_double()
    buf = DeviceBuffer(x.nbytes)
    buf.upload(x)
    try:
        check(lib().wc_loss_grad(buf.ptr, x.size, nlevels, filter, ttype, loss_type,
                                 lam.ctypes.data_as(_dp), min_level, max_level, sigma, eps,
                                 C.byref(loss), grad.ctypes.data_as(_dp), C.byref(sig), None))
    finally:
        buf.free()
    return loss.value, grad, sig.value


def fit_opts(loss_type=LOSS_SURE, min_level=0, max_level=-1, iterations=60, step=0.1,
             eps=0.1, sigma=0.0, lambda0=None, precision=F32, smooth=True):
    """wc_fit_opts for fit_thresholds (lambda0 is kept alive on the record)."""
    o = FitOpts(loss_type, min_level, max_level, iterations, step, eps, sigma, None, precision,
                1 if smooth else 0)
    if lambda0 is not None:
        lam = np.ascontiguousarray(lambda0, dtype=np.float64)
        o._lam = lam
        o.lambda0 = lam.ctypes.data_as(_dp)
    return o


def fit_thresholds(x2d, nlevels, filter, ttype, device=False, **kw):
    """Per-level soft thresholds fitted by gradient descent for a batch of
    equal-length signals (rows of x2d), one persistent launch
    (wc_fit_thresholds).  Returns (smoothed rows, list of FitResult)."""
    x = np.array(x2d, dtype=np.float64, copy=True, order="C")
    if x.ndim == 1:
        x = x[None, :]
    nsig, n = x.shape
    opts = fit_opts(**kw)
    res = (FitResult * nsig)()
    if device:
        buf = DeviceBuffer(x.nbytes)
        buf.upload(x)
        try:
            check(lib().wc_fit_thresholds_device(buf.ptr, n, nsig, nlevels, filter, ttype,
                                                 C.byref(opts), res, None))
            y = buf.download(np.float64, x.size).reshape(nsig, n)
        finally:
            buf.free()
    else:
        check(lib().wc_fit_thresholds(x.ctypes.data_as(_dp), n, nsig, nlevels, filter, ttype,
                                      C.byref(opts), res))
        y = x
    return y, list(res)


def sequential_sum(v) -> float:
    """Serial-order FP64 sum of non-negative terms, computed on the device."""
    v = np.ascontiguousarray(v, dtype=np.float64)
    buf = DeviceBuffer(max(8, v.nbytes))
    buf.upload(v)
    out = C.c_double()
    check(lib().wc_sequential_sum_device(buf.ptr, v.size, C.byref(out), None))
    buf.free()
    return out.value


def smooth_batch(data, signals, precision=F64_EXACT):
    """wc_smooth_batch: smooths every signal of the flat array `data` (host)
    in one persistent launch; returns (smoothed copy, list of SignalResult)."""
    y = np.array(data, dtype=np.float64, copy=True)
    arr = (Signal * len(signals))(*signals)
    res = (SignalResult * len(signals))()
    check(lib().wc_smooth_batch(_dptr(y), y.size, arr, len(signals), precision, res))
    return y, list(res)


def smooth_batch_R(data, signals, precision=F64_EXACT):
    """The flat .C form RgpuSmoothBatch, called exactly as R's .C would:
    every argument a pointer to a double or int vector.  Returns (smoothed
    copy, thresholds, iterations, kept, zeroed, status)."""
    y = np.array(data, dtype=np.float64, copy=True)
    k = len(signals)

    def iv(field):
        return np.ascontiguousarray([getattr(s_, field) for s_ in signals], dtype=np.int32)

    vecs = {f: iv(f) for f in ("offset", "len", "nlevels", "ttype", "filter", "threshtype",
                               "hardness", "minlevel", "maxlevel")}
    th = np.ascontiguousarray([s_.thresh for s_ in signals], dtype=np.float64)
    tol = np.ascontiguousarray([s_.tol for s_ in signals], dtype=np.float64)
    its, kept, zer = (np.zeros(k, dtype=np.int32) for _ in range(3))
    total, nsig, prec, status = (np.array([v], dtype=np.int32)
                                 for v in (y.size, k, precision, -1))

    def ip(a):
        return a.ctypes.data_as(_ip)

    lib().RgpuSmoothBatch(_dptr(y), ip(total), ip(nsig), ip(vecs["offset"]), ip(vecs["len"]),
                          ip(vecs["nlevels"]), ip(vecs["ttype"]), ip(vecs["filter"]),
                          ip(vecs["threshtype"]), _dptr(th), ip(vecs["hardness"]),
                          ip(vecs["minlevel"]), ip(vecs["maxlevel"]), _dptr(tol), ip(prec),
                          ip(its), ip(kept), ip(zer), ip(status))
    return y, th, its, kept, zer, int(status[0])


def device_status() -> int:
    """Reads and clears the status words (bit 0: a bounded wait gave up)."""
    v = C.c_uint(0)
    check(lib().wc_device_status(C.byref(v)))
    return v.value


def measure_fp64_rate(stream=None) -> float:
    """Measured FP64 add/multiply rate of the device (G operations/s)."""
    v = C.c_double(0.0)
    check(lib().wc_measure_fp64_rate(C.byref(v), stream))
    return v.value


def debug_wait_probe(target=0, polls=1000, stream=None) -> None:
    """Test hook: makes one bounded device-side wait run out (see
    wc_debug_wait_probe)."""
    check(lib().wc_debug_wait_probe(target, polls, stream))


def debug_set_workspace_cap(nbytes: int) -> None:
    """Test hook: workspace growth beyond nbytes fails with WC_ERR_NOMEM."""
    check(lib().wc_debug_set_workspace_cap(nbytes))


def debug_workspace_bytes() -> int:
    v = C.c_size_t(0)
    check(lib().wc_debug_workspace_bytes(C.byref(v)))
    return v.value


def set_dwt_tiling(filt, precision, tile, g0, threads, pipelined):
    check(lib().wc_set_dwt_tiling(filt, precision, tile, g0, threads, int(pipelined)))


def get_dwt_tiling(filt, precision):
    v = [C.c_int() for _ in range(4)]
    check(lib().wc_get_dwt_tiling(filt, precision, *[C.byref(x) for x in v]))
    return tuple(x.value for x in v)


def tune_dwt(filt, precision, log2n=24):
    ms = C.c_float()
    check(lib().wc_tune_dwt(filt, precision, log2n, C.byref(ms)))
    return get_dwt_tiling(filt, precision), ms.value


def set_modwt_tiling(filt, precision, fwd_target, fwd_smem_kb, inv_target, inv_smem_kb):
    check(lib().wc_set_modwt_tiling(filt, precision, fwd_target, fwd_smem_kb, inv_target,
                                    inv_smem_kb))


def get_modwt_tiling(filt, precision):
    v = [C.c_int() for _ in range(4)]
    check(lib().wc_get_modwt_tiling(filt, precision, *[C.byref(x) for x in v]))
    return tuple(x.value for x in v)


def set_modwt_inv_levels(filt, precision, levels):
    """Levels fused per inverse MODWT launch (2 or 3; 0 = the default)."""
    check(lib().wc_set_modwt_inv_levels(filt, precision, levels))


def get_modwt_inv_levels(filt, precision) -> int:
    v = C.c_int()
    check(lib().wc_get_modwt_inv_levels(filt, precision, C.byref(v)))
    return v.value


def set_modwt_fwd_levels(filt, precision, levels):
    """Levels fused per forward MODWT launch (1..3; 0 = the default, 2)."""
    check(lib().wc_set_modwt_fwd_levels(filt, precision, levels))


def get_modwt_fwd_levels(filt, precision) -> int:
    v = C.c_int()
    check(lib().wc_get_modwt_fwd_levels(filt, precision, C.byref(v)))
    return v.value


def set_modwt_vector(enable: bool) -> None:
    """16-byte MODWT tiles where they apply (the default), or the
    one-value-per-instruction tiles everywhere; both give the same bits."""
    check(lib().wc_set_modwt_vector(1 if enable else 0))


def tune_modwt(filt, precision, log2n=24, nlevels=12):
    """Autotunes the MODWT tiling; returns (tiling, fwd_ms, inv_ms)."""
    f, i = C.c_float(), C.c_float()
    check(lib().wc_tune_modwt(filt, precision, log2n, nlevels, C.byref(f), C.byref(i)))
    return get_modwt_tiling(filt, precision), f.value, i.value


def device_count() -> int:
    n = C.c_int(0)
    lib().wc_device_count(C.byref(n))
    return n.value


def kernel_launch_count() -> int:
    return lib().wc_kernel_launch_count()


class DeviceBuffer:
    """A device allocation made through the library (plumbing for tests and
    the benchmark)."""

    def __init__(self, nbytes: int):
        p = _vp()
        check(lib().wc_malloc_device(C.byref(p), nbytes))
        self.ptr, self.nbytes = p.value, nbytes

    def upload(self, a: np.ndarray, stream=None):
        a = np.ascontiguousarray(a)
        assert a.nbytes <= self.nbytes
        check(lib().wc_memcpy(self.ptr, a.ctypes.data, a.nbytes, stream))
        check(lib().wc_stream_synchronize(stream))

    def download(self, dtype, count, stream=None) -> np.ndarray:
        out = np.empty(count, dtype=dtype)
        check(lib().wc_memcpy(out.ctypes.data, self.ptr, out.nbytes, stream))
        check(lib().wc_stream_synchronize(stream))
        return out

    def free(self):
        if self.ptr:
            lib().wc_free_device(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class HostBuffer:
    """Pinned host memory viewed as a numpy array."""

    def __init__(self, count: int, dtype=np.float64):
        dtype = np.dtype(dtype)
        p = _vp()
        check(lib().wc_malloc_host(C.byref(p), count * dtype.itemsize))
        self.ptr = p.value
        buf = (C.c_char * (count * dtype.itemsize)).from_address(self.ptr)
        self.array = np.frombuffer(buf, dtype=dtype, count=count)

    def free(self):
        if self.ptr:
            self.array = None
            lib().wc_free_host(self.ptr)
            self.ptr = None


class Event:
    def __init__(self):
        p = _vp()
        check(lib().wc_event_create(C.byref(p)))
        self.ptr = p.value

    def record(self, stream=None):
        check(lib().wc_event_record(self.ptr, stream))

    def elapsed_ms(self, other: "Event") -> float:
        ms = C.c_float()
        check(lib().wc_event_elapsed_ms(self.ptr, other.ptr, C.byref(ms)))
        return ms.value


def default_stream():
    p = _vp()
    check(lib().wc_default_stream(C.byref(p)))
    return p.value

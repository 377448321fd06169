"""The C-ABI library loads and exports every function include/*.h declares;
host-side argument checks mirror the reference's R checks.  No GPU needed:
nothing here launches device work."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"WC_API\s+[\w\s\*]+?\b(\w+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_reference_symbols():
    names = declared_functions()
    for ref in ("RcpuTransform", "RgpuTransform", "RcpuThreshold", "RcpuSmooth", "RgpuSmooth"):
        assert ref in names
    assert len(names) >= 25


def test_library_exports_every_declared_symbol(wc):
    lib = wc.lib()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_max_levels_matches_reference_rule(wc):
    # check_len_levels (wavutils.cpp:48-64)
    assert wc.max_levels(1024, wc.HAAR) == 10
    assert wc.max_levels(1024, wc.D4) == 9
    assert wc.max_levels(1024, wc.C6) == 8
    assert wc.max_levels(2 ** 26, wc.LA8) == 24
    assert wc.max_levels(1000, wc.HAAR) == 0
    assert wc.max_levels(4, wc.LA8) == 0


def test_r_input_checks(wc):
    x = np.zeros(1024)
    with pytest.raises(ValueError, match="power of 2"):
        wc.check_trans_inputs(np.zeros(1000), "FWD", 0, "DWT", "Haar")
    with pytest.raises(ValueError, match="Unexpected filter"):
        wc.check_trans_inputs(x, "FWD", 0, "DWT", "D6")
    with pytest.raises(ValueError, match="Unexpected transform type"):
        wc.check_trans_inputs(x, "FWD", 0, "SWT", "Haar")
    with pytest.raises(ValueError, match="nlevels"):
        wc.check_trans_inputs(x, "FWD", 10, "DWT", "D4")   # maximum is 9
    a = wc.check_trans_inputs(x, "FWD", 0, "MODWT", "LA8")
    assert a["nlevels"] == 8 and a["xmod"].size == 1024 * 2 * 10
    with pytest.raises(ValueError, match="min.level"):
        wc.check_smooth_inputs(x, 5, "DWT", "Haar", "cv", None, "soft", 0, 5, 0.01)
    with pytest.raises(ValueError, match="Tolerance"):
        wc.check_smooth_inputs(x, 5, "DWT", "Haar", "cv", None, "soft", 1, 5, 0.0)
    with pytest.raises(ValueError, match="hard or soft"):
        wc.check_smooth_inputs(x, 5, "DWT", "Haar", "cv", None, "medium", 1, 5, 0.01)


def test_status_api_rejects_bad_arguments_without_a_gpu(wc):
    # Argument validation happens before any device work; with no device the
    # calls report WC_ERR_NODEVICE, with one they report the argument error.
    lib = wc.lib()
    y = np.zeros(1000)
    r = lib.wc_transform(y.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), None, 1000, 1, 0, 0,
                         1, 0)
    assert r in (1, 6)
    assert wc.last_error()

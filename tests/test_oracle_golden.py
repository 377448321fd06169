"""The oracle (our C restatement) reproduces the reference's own outputs
(tests/golden, generated from the reference's compiled CPU sources) bit for
bit."""
import numpy as np
import pytest

import pyoracle as P


def test_golden_transforms(oracle, golden):
    n_checked = 0
    for name, f in golden.items():
        if not (name.startswith("dwt_") or name.startswith("modwt_")):
            continue
        n, J, filt, sense = (int(v) for v in f["args"])
        if name.startswith("dwt_"):
            got = oracle.dwt(f["in"], J, filt, sense)
        elif sense == P.FWD:
            got = oracle.modwt_fwd(f["in"], J, filt)
        else:
            got = oracle.modwt_inv(f["in"], n, J, filt)
        assert np.array_equal(got, f["out"]), name
        n_checked += 1
    assert n_checked >= 30


def test_golden_median_mad(oracle, golden):
    for name, f in golden.items():
        if name.startswith("mad_"):
            med, mad = f["out"]
            assert oracle.median(f["in"]) == med, name
            assert oracle.mad(f["in"]) == mad, name


def test_golden_smooth(oracle, golden):
    n_checked = 0
    for name, f in golden.items():
        if not name.startswith("smooth_"):
            continue
        n, J, ttype, filt, tt, hard, mn, mx = (int(v) for v in f["args"])
        y, t = oracle.smooth(f["in"], J, ttype, filt, tt, 0.35, hard, mn, mx, 1e-8)
        assert t == f["thresh"][0], name
        assert np.array_equal(y, f["out"]), name
        n_checked += 1
    assert n_checked == 15


def test_level_limits(oracle):
    # check_len_levels (wavutils.cpp:48-64): maximum floor(log2(n/L)) + 1
    assert oracle.levels(1024, 0, P.HAAR) == 10
    assert oracle.levels(1024, 0, P.D4) == 9
    assert oracle.levels(1024, 0, P.C6) == 8
    assert oracle.levels(1024, 0, P.LA8) == 8
    assert oracle.levels(1024, 10, P.D4) == 0
    assert oracle.levels(1000, 0, P.HAAR) == 0
    assert oracle.levels(2 ** 26, 0, P.LA8) == 24


@pytest.mark.parametrize("filt", [P.HAAR, P.D4, P.C6, P.LA8])
def test_perfect_reconstruction_and_parseval(oracle, filt):
    rng = np.random.default_rng(filt)
    x = rng.standard_normal(512)
    J = oracle.levels(512, 0, filt)
    w = oracle.dwt(x, J, filt)
    assert abs(np.dot(w, w) - np.dot(x, x)) < 1e-10 * np.dot(x, x)
    assert np.max(np.abs(oracle.dwt(w, J, filt, P.BWD) - x)) < 1e-13
    xm = oracle.modwt_fwd(x, 6, filt)
    assert np.max(np.abs(oracle.modwt_inv(xm, 512, 6, filt) - x)) < 1e-13


def test_golden_packet_ordered_modwt(oracle, golden):
    """Packet-ordered MODWT (code 2): the oracle reproduces the reference's
    fHaarMODWT / fDaub4MODWTpo and their inverses bit for bit."""
    n_checked = 0
    for name, f in golden.items():
        if not name.startswith("modwtpo_"):
            continue
        n, J, filt, sense = (int(v) for v in f["args"])
        if sense == P.FWD:
            got = oracle.modwt_po_fwd(f["in"], J, filt)
        else:
            got = oracle.modwt_po_inv(f["in"], n, J, filt)
        assert np.array_equal(got, f["out"]), name
        n_checked += 1
    assert n_checked == 12

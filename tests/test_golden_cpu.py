"""The C oracle against golden outputs of the reference's own worklets
(tests/golden, produced by tests/golden/make_golden.py from the reference
source tree).  This pins the oracle wherever it runs, with or without the
reference tree."""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle
from tests import cases

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
META = json.load(open(os.path.join(HERE, "golden.json")))
SMALL = np.load(os.path.join(HERE, "golden_small.npz"))


def check(key, a):
    a = np.ascontiguousarray(a)
    m = META[key]
    assert list(a.shape) == m["shape"], key
    assert str(a.dtype) == m["dtype"], key
    assert hashlib.sha256(a.tobytes()).hexdigest() == m["sha256"], key
    sk = key.replace("/", "__")
    if sk in SMALL:
        assert np.array_equal(SMALL[sk].view(np.uint8), a.view(np.uint8)), key


@pytest.fixture(scope="module")
def port():
    return oracle.Oracle("port")


@pytest.mark.parametrize("case", cases.mc_cases(), ids=lambda c: c[0])
def test_mc_golden(port, case):
    name, dims, origin, spacing, emin, f, iso = case
    g = oracle.make_grid(dims, origin, spacing, emin)
    count, cs = port.mc_count(g, f, iso)
    check("mc/%s/count" % name, count)
    check("mc/%s/cases" % name, cs)
    for merge in (0, 1):
        out = port.mc_generate(g, f, iso, count, bool(merge))
        for k in ("verts", "conn", "rec_a", "rec_b", "rec_w"):
            check("mc/%s/m%d/%s" % (name, merge, k), out[k])


@pytest.mark.parametrize("case", cases.threshold_cases(), ids=lambda c: c[0])
def test_threshold_golden(port, case):
    name, dims, origin, spacing, emin, f, lo, hi = case
    g = oracle.make_grid(dims, origin, spacing, emin)
    count = port.threshold_count(g, f, lo, hi)
    check("thr/%s/count" % name, count)
    out = port.threshold_generate(g, f, count)
    for k in ("conn", "coords", "field"):
        check("thr/%s/%s" % (name, k), out[k])


@pytest.mark.parametrize("case", cases.gradient_cases(), ids=lambda c: c[0])
def test_gradient_golden(port, case):
    name, dims, origin, spacing, emin, f = case
    check("grad/%s" % name, port.cell_gradient(oracle.make_grid(dims, origin, spacing, emin), f))


@pytest.mark.parametrize("case", cases.slice_cases(), ids=lambda c: c[0])
def test_slice_golden(port, case):
    name, dims, origin, spacing, emin, po, pn = case
    g = oracle.make_grid(dims, origin, spacing, emin)
    count = port.slice_count(g, po, pn)
    check("slice/%s/count" % name, count)
    for merge in (0, 1):
        out = port.slice_generate(g, po, pn, count, bool(merge))
        for k in ("verts", "conn", "rec_a", "rec_b", "rec_w"):
            check("slice/%s/m%d/%s" % (name, merge, k), out[k])


@pytest.mark.parametrize("case", cases.mt_cases(), ids=lambda c: c[0])
def test_mt_golden(port, case):
    name, pts, conn, f, iso = case
    count = port.mt_count(conn, f, iso)
    check("mt/%s/count" % name, count)
    for merge in (0, 1):
        out = port.mt_generate(pts, conn, f, iso, count, bool(merge))
        for k in ("verts", "conn", "rec_a", "rec_b", "rec_w"):
            check("mt/%s/m%d/%s" % (name, merge, k), out[k])


def test_known_answers_in_golden():
    assert META["mc/kat26_linear/m1/verts"]["shape"] == [45, 3]
    assert META["mc/kat26_linear/m0/verts"]["shape"] == [183, 3]
    assert META["mc/kat26_linear/m1/conn"]["shape"] == [61, 3]
    assert META["slice/kat8_axis_x/m0/verts"]["shape"] == [294, 3]
    assert META["slice/kat8_axis_x/m1/verts"]["shape"] == [64, 3]
    assert META["mt/kat26_linear/m1/verts"]["shape"] == [151, 3]

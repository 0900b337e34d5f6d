"""The CPU oracle against the reference's own known answers and against the
reference's worklets compiled from source (where the reference tree exists).

Known answers (DaxToolkit unit tests):
  * UnitTestWorkletMarchingCubes.cxx:39-40, :94-193 -- 26^3 grid, field x+y+z,
    isovalue 70: points == 3 * cells unmerged, 45 unique points merged, and a
    secondary linear field interpolates linearly (test_equal, 1e-4 ratio).
  * UnitTestWorkletThreshold.cxx:40-42, :86-239 -- 26^3, [70, 82]: every kept
    cell's points in range, coordinates of kept cells in input order.
  * UnitTestWorkletCellGradient.cxx:31, :83-117 -- 8^3, x+y+z, gradient (1,1,1).
  * UnitTestWorkletSlice.cxx:22-24, :84-108 -- 8^3, origin (3,2,1), normal
    (1,0,0): 2 * 7^2 triangles, 3 points each unmerged, 8^2 points merged.
  * UnitTestWorkletMarchingTetrahedra.cxx:33-34, :86-113 -- 26^3 grid split
    into 6 tetrahedra per cell, field x+y+z, isovalue 70: 3 points per
    triangle unmerged, 151 points merged.
"""
import numpy as np
import pytest

import oracle
from tests import cases


def _grid(dims, origin=(0, 0, 0), spacing=(1, 1, 1), emin=(0, 0, 0)):
    return oracle.make_grid(dims, origin, spacing, emin)


def _kinds():
    kinds = ["port"]
    if oracle.build.reference_available():
        kinds.append("reference")
    return kinds


def dax_test_equal(a, b, tol=1e-4):
    """dax/testing/Testing.h:405-430 test_equal: |a-b| small relative to |a|+|b|."""
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    diff = np.abs(a - b)
    scale = np.abs(a) + np.abs(b)
    return bool(np.all((diff <= tol) | (diff <= tol * scale)))


@pytest.mark.parametrize("kind", _kinds())
def test_mc_known_answer(kind):
    O = oracle.Oracle(kind)
    g = _grid((26, 26, 26))
    f = cases.linear_field((26, 26, 26))
    count, _ = O.mc_count(g, f, 70.0)
    assert int(count.sum()) == 61
    un = O.mc_generate(g, f, 70.0, count, merge=False)
    assert un["verts"].shape == (183, 3)
    assert np.array_equal(un["conn"].ravel(), np.arange(183))
    mg = O.mc_generate(g, f, 70.0, count, merge=True)
    assert mg["verts"].shape == (45, 3)
    # secondary field (-0.5, 1, 2) interpolates linearly
    sec = cases.linear_field((26, 26, 26), grad=(-0.5, 1.0, 2.0))
    for out in (un, mg):
        vals = O.interpolate_point_field(out["rec_a"], out["rec_b"], out["rec_w"], sec)
        expect = out["verts"].astype(np.float64) @ np.array([-0.5, 1.0, 2.0])
        assert dax_test_equal(vals, expect)
    # merged topology is the unmerged one with duplicates collapsed
    assert np.array_equal(mg["verts"][mg["conn"].ravel()], un["verts"])


@pytest.mark.parametrize("kind", _kinds())
def test_threshold_known_answer(kind):
    O = oracle.Oracle(kind)
    g = _grid((26, 26, 26))
    f = cases.linear_field((26, 26, 26))
    count = O.threshold_count(g, f, 70.0, 82.0)
    out = O.threshold_generate(g, f, count)
    assert out["conn"].shape[1] == 8
    assert np.all((out["field"] >= 70) & (out["field"] <= 82))
    # CheckConnections: kept cells in input order, coordinates match
    kept = np.nonzero(count)[0]
    assert len(kept) == out["conn"].shape[0] == 10
    d = 25
    for n, c in enumerate(kept):
        i, j, k = c % d, (c // d) % d, c // (d * d)
        corners = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
        for v, (di, dj, dk) in enumerate(corners):
            assert np.array_equal(out["coords"][out["conn"][n, v]], [i + di, j + dj, k + dk])


@pytest.mark.parametrize("kind", _kinds())
def test_gradient_known_answer(kind):
    O = oracle.Oracle(kind)
    g = _grid((8, 8, 8))
    grad = O.cell_gradient(g, cases.linear_field((8, 8, 8)))
    assert grad.shape == (343, 3)
    assert dax_test_equal(grad, np.ones_like(grad))


@pytest.mark.parametrize("kind", _kinds())
def test_slice_known_answer(kind):
    O = oracle.Oracle(kind)
    g = _grid((8, 8, 8))
    count = O.slice_count(g, (3, 2, 1), (1, 0, 0))
    assert int(count.sum()) == 7 * 7 * 2
    a = O.slice_generate(g, (3, 2, 1), (1, 0, 0), count, merge=False)
    b = O.slice_generate(g, (3, 2, 1), (1, 0, 0), count, merge=True)
    assert a["conn"].shape == (98, 3) and a["verts"].shape == (98 * 3, 3)
    assert b["conn"].shape == (98, 3) and b["verts"].shape == (64, 3)
    assert np.all(b["verts"][:, 0] == 6.0)


@pytest.mark.parametrize("kind", _kinds())
def test_mt_known_answer(kind):
    O = oracle.Oracle(kind)
    d = (26, 26, 26)
    pts, conn, f = cases.grid_points(d), cases.tetrahedralize(d), cases.linear_field(d)
    count = O.mt_count(conn, f, 70.0)
    a = O.mt_generate(pts, conn, f, 70.0, count, merge=False)
    b = O.mt_generate(pts, conn, f, 70.0, count, merge=True)
    assert a["verts"].shape[0] == 3 * a["conn"].shape[0]
    assert b["verts"].shape[0] == 151


@pytest.mark.skipif(not oracle.build.reference_available(), reason="reference tree absent")
@pytest.mark.parametrize("case", cases.mt_cases(), ids=lambda c: c[0])
def test_mt_port_matches_reference_build(case):
    name, pts, conn, f, iso = case
    P, R = oracle.Oracle("port"), oracle.Oracle("reference")
    c1, c2 = P.mt_count(conn, f, iso), R.mt_count(conn, f, iso)
    assert np.array_equal(c1, c2)
    for merge in (False, True):
        a = P.mt_generate(pts, conn, f, iso, c1, merge)
        b = R.mt_generate(pts, conn, f, iso, c2, merge)
        for key in ("conn", "rec_a", "rec_b"):
            assert np.array_equal(a[key], b[key]), key
        for key in ("verts", "rec_w"):
            assert np.array_equal(a[key].view(np.uint32), b[key].view(np.uint32)), key


@pytest.mark.skipif(not oracle.build.reference_available(), reason="reference tree absent")
@pytest.mark.parametrize("case", cases.slice_cases(), ids=lambda c: c[0])
def test_slice_port_matches_reference_build(case):
    name, dims, origin, spacing, emin, po, pn = case
    P, R = oracle.Oracle("port"), oracle.Oracle("reference")
    g = _grid(dims, origin, spacing, emin)
    c1, c2 = P.slice_count(g, po, pn), R.slice_count(g, po, pn)
    assert np.array_equal(c1, c2)
    for merge in (False, True):
        a = P.slice_generate(g, po, pn, c1, merge)
        b = R.slice_generate(g, po, pn, c2, merge)
        for key in ("conn", "rec_a", "rec_b"):
            assert np.array_equal(a[key], b[key]), key
        for key in ("verts", "rec_w"):
            assert np.array_equal(a[key].view(np.uint32), b[key].view(np.uint32)), key


@pytest.mark.skipif(not oracle.build.reference_available(), reason="reference tree absent")
@pytest.mark.parametrize("case", cases.mc_cases(), ids=lambda c: c[0])
def test_mc_port_matches_reference_build(case):
    name, dims, origin, spacing, emin, f, iso = case
    P, R = oracle.Oracle("port"), oracle.Oracle("reference")
    g = _grid(dims, origin, spacing, emin)
    c1, k1 = P.mc_count(g, f, iso)
    c2, k2 = R.mc_count(g, f, iso)
    assert np.array_equal(c1, c2) and np.array_equal(k1, k2)
    for merge in (False, True):
        a = P.mc_generate(g, f, iso, c1, merge)
        b = R.mc_generate(g, f, iso, c2, merge)
        for key in ("conn", "rec_a", "rec_b"):
            assert np.array_equal(a[key], b[key]), key
        for key in ("verts", "rec_w"):
            assert np.array_equal(a[key].view(np.uint32), b[key].view(np.uint32)), key


@pytest.mark.skipif(not oracle.build.reference_available(), reason="reference tree absent")
@pytest.mark.parametrize("case", cases.threshold_cases(), ids=lambda c: c[0])
def test_threshold_port_matches_reference_build(case):
    name, dims, origin, spacing, emin, f, lo, hi = case
    P, R = oracle.Oracle("port"), oracle.Oracle("reference")
    g = _grid(dims, origin, spacing, emin)
    c1, c2 = P.threshold_count(g, f, lo, hi), R.threshold_count(g, f, lo, hi)
    assert np.array_equal(c1, c2)
    a, b = P.threshold_generate(g, f, c1), R.threshold_generate(g, f, c2)
    assert np.array_equal(a["conn"], b["conn"])
    assert np.array_equal(a["coords"].view(np.uint32), b["coords"].view(np.uint32))
    assert np.array_equal(a["field"].view(np.uint32), b["field"].view(np.uint32))


@pytest.mark.skipif(not oracle.build.reference_available(), reason="reference tree absent")
@pytest.mark.parametrize("case", cases.gradient_cases(), ids=lambda c: c[0])
def test_gradient_port_matches_reference_build(case):
    name, dims, origin, spacing, emin, f = case
    g = _grid(dims, origin, spacing, emin)
    a = oracle.Oracle("port").cell_gradient(g, f)
    b = oracle.Oracle("reference").cell_gradient(g, f)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("case", cases.threshold_cases(), ids=lambda c: c[0])
def test_threshold_compact_point_field_restatement(case):
    """The numpy CompactPointField (FillPointMask + StreamCompact) of the
    threshold field and of the point coordinates equals the C oracle's
    compacted field and coordinates (both from ResolveDuplicatePoints)."""
    name, dims, origin, spacing, emin, f, lo, hi = case
    port = oracle.Oracle("port")
    g = oracle.make_grid(dims, origin, spacing, emin)
    count = port.threshold_count(g, f, lo, hi)
    out = port.threshold_generate(g, f, count)
    got = oracle.Oracle.threshold_compact_point_field(g, count, f)
    assert np.array_equal(got.view(np.uint32), out["field"].view(np.uint32))
    ax = [np.float32(origin[a]) + np.float32(spacing[a]) *
          (np.arange(dims[a]) + emin[a]).astype(np.float32) for a in range(3)]
    z, y, x = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    pts = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1).astype(np.float32)
    got3 = oracle.Oracle.threshold_compact_point_field(g, count, pts)
    assert np.array_equal(got3.view(np.uint32), out["coords"].view(np.uint32))

"""GPU parity of marching tetrahedra (dax/worklet/MarchingTetrahedra.h) through
the C ABI against the CPU oracle on the same tetrahedral grids: per-cell
counts, triangles, connectivity and records identical, points and weights
bit for bit, merged and unmerged."""
import ctypes

import numpy as np
import pytest
import torch

from tests import cases

pytestmark = pytest.mark.gpu


def _bits(a):
    a = np.ascontiguousarray(a)
    b = a.view(np.uint32).copy()
    b[np.isnan(a)] = 0x7FC00000
    return b


def _grid(cont, pts, conn):
    return cont.UnstructuredGrid(torch.from_numpy(pts).cuda(), torch.from_numpy(conn).cuda())


@pytest.mark.parametrize("case", cases.mt_cases(), ids=lambda c: c[0])
def test_mt_count(gb300, oracle_best, case):
    name, pts, conn, f, iso = case
    cont = gb300
    ref = oracle_best.mt_count(conn, f, iso)
    count = cont.DispatcherMapCell(cont.MarchingTetrahedraCount(iso)).Invoke(
        _grid(cont, pts, conn), torch.from_numpy(f).cuda())
    assert np.array_equal(count.cpu().numpy(), ref)


@pytest.mark.parametrize("merge", [True, False], ids=["merged", "unmerged"])
@pytest.mark.parametrize("case", cases.mt_cases(), ids=lambda c: c[0])
def test_mt_generate(gb300, oracle_best, case, merge):
    name, pts, conn, f, iso = case
    cont = gb300
    count = oracle_best.mt_count(conn, f, iso)
    ref = oracle_best.mt_generate(pts, conn, f, iso, count, merge)
    out = cont.marching_tetrahedra(_grid(cont, pts, conn), torch.from_numpy(f).cuda(), iso,
                                   merge=merge, records=True)
    tconn = out["conn"].cpu().numpy()
    verts = out["verts"].cpu().numpy()
    assert tconn.shape == ref["conn"].shape and verts.shape == ref["verts"].shape
    assert np.array_equal(tconn, ref["conn"])
    assert np.array_equal(out["rec_first"].cpu().numpy(), ref["rec_a"])
    assert np.array_equal(out["rec_second"].cpu().numpy(), ref["rec_b"])
    assert np.array_equal(_bits(out["rec_weight"].cpu().numpy()), _bits(ref["rec_w"]))
    assert np.array_equal(_bits(verts), _bits(ref["verts"]))


def test_mt_known_answer_dispatchers(gb300):
    """UnitTestWorkletMarchingTetrahedra.cxx:63-113 through the dispatchers."""
    cont = gb300
    d = (26, 26, 26)
    grid = _grid(cont, cases.grid_points(d), cases.tetrahedralize(d))
    f = torch.from_numpy(cases.linear_field(d)).cuda()
    count = cont.DispatcherMapCell(cont.MarchingTetrahedraCount(70.0)).Invoke(grid, f)
    disp = cont.DispatcherGenerateInterpolatedCells(count, cont.MarchingTetrahedraGenerate(70.0))
    disp.SetRemoveDuplicatePoints(False)
    disp.SetReleaseCount(False)
    og = disp.Invoke(grid, f)
    assert og.GetNumberOfPoints() == 3 * og.GetNumberOfCells()
    disp.SetRemoveDuplicatePoints(True)
    og2 = disp.Invoke(grid, f)
    assert og2.GetNumberOfPoints() == 151 and og2.GetNumberOfPoints() != og.GetNumberOfPoints()
    # CompactPointField of x+y+z itself gives the isovalue at every merged point
    vals = disp.CompactPointField(f).cpu().numpy()
    assert np.allclose(vals, 70.0, rtol=0, atol=1e-4)


def test_mt_bad_point_id_is_an_error(gb300):
    """An id outside [0, P) is reported, never dereferenced."""
    cont = gb300
    from daxtoolkit_gb300 import capi
    pts = cases.grid_points((3, 3, 3))
    conn = cases.tetrahedralize((3, 3, 3))
    conn[5, 2] = 27  # one past the last point
    f = torch.from_numpy(np.linspace(-1, 1, 27).astype(np.float32)).cuda()
    grid = _grid(cont, pts, conn)
    with pytest.raises(capi.ErrorControlBadValue):
        cont.marching_tetrahedra(grid, f, 0.0)
    with pytest.raises(capi.ErrorControlBadValue):
        cont.DispatcherMapCell(cont.MarchingTetrahedraCount(0.0)).Invoke(grid, f)
    conn[5, 2] = -3
    with pytest.raises(capi.ErrorControlBadValue):
        cont.marching_tetrahedra(_grid(cont, pts, conn), f, 0.0)


def test_mt_capacity_and_state_errors(gb300):
    """Short outputs write nothing and report CAPACITY; a merged generate
    without its merge pass reports BAD_VALUE."""
    from daxtoolkit_gb300 import capi
    L = capi.lib()
    d = (12, 11, 10)
    pts = torch.from_numpy(cases.grid_points(d)).cuda()
    conn = torch.from_numpy(cases.tetrahedralize(d)).cuda()
    f = torch.from_numpy(cases.random_blobs(d, 2, 23)).cuda()
    C, P = conn.shape[0], pts.shape[0]
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    nb = L.dax_gb300_mt_scratch_bytes(C)
    scr = torch.empty(nb, dtype=torch.uint8, device="cuda")
    capi.call("dax_gb300_mt_count", p(conn), C, p(f), P, 0.4, p(scr), nb, None)
    T = ctypes.c_int64(0)
    capi.call("dax_gb300_mc_totals", p(scr), ctypes.byref(T), None, None)
    T = T.value
    assert T > 10
    verts = torch.full((3 * T - 1, 3), 7.0, device="cuda")
    tconn = torch.full((T, 3), -5, dtype=torch.int32, device="cuda")
    capi.call("dax_gb300_mt_generate", p(pts), p(conn), C, p(f), P, 0.4, 0, p(scr), nb, None, 0,
              p(verts), 3 * T - 1, p(tconn), T, None, None, None, None)
    with pytest.raises(capi.DaxError) as err:
        capi.call("dax_gb300_mc_totals", p(scr), ctypes.byref(ctypes.c_int64()), None, None)
    assert err.value.code == capi.ERROR_CAPACITY
    assert bool((verts == 7.0).all()) and bool((tconn == -5).all())
    # merged generate on a merge scratch that no merge pass wrote
    capi.call("dax_gb300_mt_count", p(conn), C, p(f), P, 0.4, p(scr), nb, None)
    mb = L.dax_gb300_mt_merge_scratch_bytes(T, P)
    mscr = torch.zeros(mb, dtype=torch.uint8, device="cuda")
    capi.call("dax_gb300_mt_generate", p(pts), p(conn), C, p(f), P, 0.4, 1, p(scr), nb, p(mscr), mb,
              p(verts), 3 * T - 1, p(tconn), T, None, None, None, None)
    with pytest.raises(capi.ErrorControlBadValue):
        capi.call("dax_gb300_mc_totals", p(scr), ctypes.byref(ctypes.c_int64()), None, None)
    assert bool((tconn == -5).all())


def test_mt_oblique_96_against_oracle(gb300, oracle_best):
    """5.1 M tetrahedra (96^3 grid split 6 ways), blob field, merged."""
    cont = gb300
    d = (96, 96, 96)
    pts = cases.grid_points(d, spacing=(1 / 95,) * 3)
    conn = cases.tetrahedralize(d)
    f = cases.random_blobs(d, 5, 31, noise=0.02)
    count = oracle_best.mt_count(conn, f, 0.45)
    ref = oracle_best.mt_generate(pts, conn, f, 0.45, count, True)
    out = cont.marching_tetrahedra(_grid(cont, pts, conn), torch.from_numpy(f).cuda(), 0.45,
                                   merge=True)
    assert np.array_equal(out["conn"].cpu().numpy(), ref["conn"])
    assert np.array_equal(_bits(out["verts"].cpu().numpy()), _bits(ref["verts"]))


def test_mt_full_size_merged_equals_unmerged(gb300):
    """256^3 grid split 6 ways (99.5 M tetrahedra, 64-bit merge keys): every
    merged record is the unmerged record it replaces, bit for bit, and the
    merged points are strictly ascending in (first, second)."""
    cont = gb300
    n = 256
    dev = torch.device("cuda")
    ax = torch.arange(n, dtype=torch.float32, device=dev) / (n - 1)
    z, y, x = torch.meshgrid(ax, ax, ax, indexing="ij")
    pts = torch.stack([x.reshape(-1), y.reshape(-1), z.reshape(-1)], 1).contiguous()
    del x, y, z
    f = (((pts - 0.5) ** 2).sum(1)).sqrt().contiguous()
    conn = torch.from_numpy(cases.tetrahedralize((n, n, n))).to(dev)
    grid = cont.UnstructuredGrid(pts, conn)
    a = cont.marching_tetrahedra(grid, f, 0.3, merge=False, records=True)
    b = cont.marching_tetrahedra(grid, f, 0.3, merge=True, records=True)
    T = a["conn"].shape[0]
    assert T > 500_000 and b["conn"].shape[0] == T
    idx = b["conn"].reshape(-1).long()
    for k in ("rec_first", "rec_second"):
        assert torch.equal(b[k][idx], a[k])
    assert torch.equal(b["rec_weight"][idx].view(torch.int32), a["rec_weight"].view(torch.int32))
    assert torch.equal(b["verts"][idx].view(torch.int32), a["verts"].view(torch.int32))
    key = b["rec_first"].long() * (1 << 32) + b["rec_second"].long()
    assert bool((key[1:] > key[:-1]).all())


_TETRA_GRIDS = [((8, 8, 8), (0, 0, 0), (1, 1, 1), (0, 0, 0)),
                ((5, 4, 3), (1, 2, 3), (0.5, 1, 2), (3, -2, 1)),
                ((2, 2, 2), (0, 0, 0), (1, 1, 1), (0, 0, 0)),
                ((70, 9, 6), (-1, 0, 2), (0.1, 0.2, 0.3), (0, 0, 0))]


@pytest.mark.parametrize("g", _TETRA_GRIDS, ids=lambda g: "x".join(map(str, g[0])))
def test_tetrahedralize(gb300, oracle_best, g):
    """Tetrahedralize against the oracle; the coordinates against the grid's
    implicit ones; UnitTestWorkletTetrahedralize.cxx:23-37's use counts."""
    import oracle
    dims, origin, spacing, emin = g
    cont = gb300
    tg = cont.tetrahedralize(cont.UniformGrid(dims, origin, spacing, emin))
    ref = oracle_best.tetrahedralize(oracle.make_grid(dims, origin, spacing, emin))
    assert np.array_equal(tg.GetCellConnections().cpu().numpy(), ref)
    f32 = np.float32
    ax = [f32(origin[a]) + f32(spacing[a]) * (np.arange(dims[a]) + emin[a]).astype(f32)
          for a in range(3)]
    z, y, x = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    want = np.stack([x.ravel(), y.ravel(), z.ravel()], 1)
    assert np.array_equal(_bits(tg.GetPointCoordinates().cpu().numpy()), _bits(want))
    if dims == (8, 8, 8):
        uses = np.bincount(ref.ravel(), minlength=512)
        assert set(uses.tolist()) <= {1, 2, 4, 8, 16, 32}


def test_mt_on_tetrahedralized_grid(gb300, oracle_best):
    """The pipeline the two worklets form: Tetrahedralize, then marching
    tetrahedra of a blob field, against the oracle, merged."""
    import oracle
    cont = gb300
    d = (40, 33, 27)
    sp = tuple(1 / (n - 1) for n in d)
    tg = cont.tetrahedralize(cont.UniformGrid(d, spacing=sp))
    f = cases.random_blobs(d, 3, 41, noise=0.05)
    ref_conn = oracle_best.tetrahedralize(oracle.make_grid(d, spacing=sp))
    ref_pts = tg.GetPointCoordinates().cpu().numpy()
    count = oracle_best.mt_count(ref_conn, f, 0.5)
    ref = oracle_best.mt_generate(ref_pts, ref_conn, f, 0.5, count, True)
    out = cont.marching_tetrahedra(tg, torch.from_numpy(f).cuda(), 0.5, merge=True)
    assert np.array_equal(out["conn"].cpu().numpy(), ref["conn"])
    assert np.array_equal(_bits(out["verts"].cpu().numpy()), _bits(ref["verts"]))

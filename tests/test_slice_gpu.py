"""GPU parity of Slice (dax/worklet/Slice.h) through the C ABI: the slice
point field written by dax_gb300_slice_field, then the marching-cubes passes,
against the CPU oracle's SliceCount / SliceGenerate on the same grid and
plane.  Counts, connectivity and interpolation end points are identical;
vertex positions and weights are compared bit for bit."""
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


def _ogrid(dims, origin, spacing, emin):
    import oracle
    return oracle.make_grid(dims, origin, spacing, emin)


@pytest.mark.parametrize("case", cases.slice_cases(), ids=lambda c: c[0])
def test_slice_count(gb300, oracle_best, case):
    name, dims, origin, spacing, emin, po, pn = case
    cont = gb300
    grid = cont.UniformGrid(dims, origin, spacing, emin)
    ref = oracle_best.slice_count(_ogrid(dims, origin, spacing, emin), po, pn)
    count = cont.DispatcherMapCell(cont.SliceCount(po, pn)).Invoke(grid)
    torch.cuda.synchronize()
    assert np.array_equal(count.cpu().numpy(), ref)


@pytest.mark.parametrize("merge", [True, False], ids=["merged", "unmerged"])
@pytest.mark.parametrize("case", cases.slice_cases(), ids=lambda c: c[0])
def test_slice_generate(gb300, oracle_best, case, merge):
    name, dims, origin, spacing, emin, po, pn = case
    cont = gb300
    og = _ogrid(dims, origin, spacing, emin)
    count = oracle_best.slice_count(og, po, pn)
    ref = oracle_best.slice_generate(og, po, pn, count, merge)
    out = cont.slice(cont.UniformGrid(dims, origin, spacing, emin), po, pn, merge=merge,
                     records=True)
    conn = out["conn"].cpu().numpy()
    verts = out["verts"].cpu().numpy()
    assert conn.shape == ref["conn"].shape and verts.shape == ref["verts"].shape
    assert np.array_equal(conn, ref["conn"])
    assert np.array_equal(out["rec_first"].cpu().numpy(), ref["rec_a"])
    assert np.array_equal(out["rec_second"].cpu().numpy(), ref["rec_b"])
    assert np.array_equal(_bits(out["rec_weight"].cpu().numpy()), _bits(ref["rec_w"]))
    assert np.array_equal(_bits(verts), _bits(ref["verts"]))


def test_slice_known_answer_dispatchers(gb300):
    """UnitTestWorkletSlice.cxx:59-108 through the dispatcher surface."""
    cont = gb300
    grid = cont.UniformGrid((8, 8, 8))
    count = cont.DispatcherMapCell(cont.SliceCount((3, 2, 1), (1, 0, 0))).Invoke(grid)
    disp = cont.DispatcherGenerateInterpolatedCells(count, cont.SliceGenerate((3, 2, 1), (1, 0, 0)))
    disp.SetRemoveDuplicatePoints(False)
    disp.SetReleaseCount(False)
    og = disp.Invoke(grid)
    assert og.GetNumberOfCells() == 98 and og.GetNumberOfPoints() == 98 * 3
    disp.SetRemoveDuplicatePoints(True)
    og2 = disp.Invoke(grid)
    assert og2.GetNumberOfCells() == 98 and og2.GetNumberOfPoints() == 64


@pytest.mark.parametrize("dims", [(37, 21, 25), (300, 7, 5), (1, 3, 2)], ids=str)
def test_slice_field_values(gb300, dims):
    """The point field and isovalue themselves: dot(N, coord - O) rounded in
    component order with no fused multiply-add, and dot(N, O)."""
    cont = gb300
    origin, spacing, emin = (1000.0, -4.1, 250.0), (0.013, 0.7, 0.05), (-5, 2, 100)
    po, pn = (500.1, -1.0, 127.6), (0.6, 0.1, -0.8)
    f, iso = cont.slice_field(cont.UniformGrid(dims, origin, spacing, emin), po, pn)
    f32 = np.float32
    ax = [f32(origin[a]) + f32(spacing[a]) * (np.arange(dims[a]) + emin[a]).astype(f32)
          for a in range(3)]
    z, y, x = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    o = [f32(v) for v in po]
    n = [f32(v) for v in pn]
    ref = (n[0] * (x - o[0]) + n[1] * (y - o[1])) + n[2] * (z - o[2])
    assert np.array_equal(_bits(f.cpu().numpy()), _bits(ref.astype(f32).ravel()))
    assert np.float32(iso) == (n[0] * o[0] + n[1] * o[1]) + n[2] * o[2]


@pytest.mark.parametrize("n", [200, 512])
def test_slice_axis_plane_full_size(gb300, n):
    """An axis-aligned cut through grid points at any size: two triangles
    per cell of the cut plane and n^2 merged points, all on the plane."""
    cont = gb300
    grid = cont.UniformGrid((n, n, n))
    out = cont.slice(grid, (0, n // 4 + 0.0, 0), (0, 1, 0), merge=True)
    assert out["conn"].shape[0] == 2 * (n - 1) ** 2
    assert out["verts"].shape[0] == n * n
    assert bool((out["verts"][:, 1] == float(n // 2)).all())
    un = cont.slice(grid, (0, n // 4 + 0.0, 0), (0, 1, 0), merge=False)
    assert un["verts"].shape[0] == 6 * (n - 1) ** 2


@pytest.mark.parametrize("merge", [True, False], ids=["merged", "unmerged"])
def test_slice_fused_equals_field_path_512(gb300, merge):
    """The fused slice (no field stored) against slice_field + marching
    cubes of it at 512^3, bit for bit, with records."""
    cont = gb300
    grid = cont.UniformGrid((512, 512, 512), (-1, -1, -1), (2 / 511,) * 3)
    po, pn = (0.11, -0.2, 0.3), (0.3, 0.9, -0.3)
    a = cont.slice(grid, po, pn, merge=merge, records=True)
    f, iso = cont.slice_field(grid, po, pn)
    b = cont.marching_cubes(grid, f, iso, merge=merge, records=True)
    assert a["conn"].shape[0] > 100000
    for k in ("conn", "rec_first", "rec_second"):
        assert torch.equal(a[k], b[k]), k
    for k in ("verts", "rec_weight"):
        assert torch.equal(a[k].view(torch.int32), b[k].view(torch.int32)), k


def test_slice_oblique_against_oracle_256(gb300, oracle_best):
    dims, origin, spacing, emin = (256, 240, 200), (-1, -1, -1), (2 / 255, 2 / 239, 2 / 199), (0, 0, 0)
    po, pn = (0.05, -0.1, 0.2), (0.3, 0.9, -0.3)
    og = _ogrid(dims, origin, spacing, emin)
    count = oracle_best.slice_count(og, po, pn)
    ref = oracle_best.slice_generate(og, po, pn, count, True)
    out = gb300.slice(gb300.UniformGrid(dims, origin, spacing, emin), po, pn, merge=True)
    assert np.array_equal(out["conn"].cpu().numpy(), ref["conn"])
    assert np.array_equal(_bits(out["verts"].cpu().numpy()), _bits(ref["verts"]))

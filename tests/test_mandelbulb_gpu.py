"""GPU parity of the Mandelbulb benchmark pipeline (Benchmarks/Mandlebulb) and
of the count-array-driven generate it uses, against the CPU oracle.

The escape-iteration field calls transcendental functions (atan2, pow, sin,
tan, cos) that CUDA and the host C library round differently in the last
place, and the iteration amplifies that on the fractal's boundary.  So the
field is checked against float32 determinacy (oracle/mandelbulb64.py): where
an ensemble of FP64 orbits of the same coordinate, perturbed at float32
precision, agrees on the escape count, the GPU must give that count; points
where the GPU and the C restatement differ must be points the ensemble
leaves undetermined, but for at most 1e-4 of all points (a finite ensemble
can look unanimous on a chaotic orbit by chance; measured: 3.5e-5 at 61^3,
2.4e-5 at 101^3).  Everything computed from a given field -- the surface,
the clip counts, the counted generate, normals and colours -- is compared bit
for bit against the oracle run on that same field."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _bits(a):
    a = np.ascontiguousarray(a)
    b = a.view(np.uint32).copy()
    b[np.isnan(a)] = 0x7FC00000
    return b


def _demo_grid(n):
    """The benchmark's volume: origin -1, spacing 2 / n, points 0 .. n."""
    return (n + 1,) * 3, (-1.0, -1.0, -1.0), (2.0 / n,) * 3


@pytest.mark.parametrize("n", [60, 100])
def test_escape_iteration_field(gb300, n):
    import oracle
    cont = gb300
    dims, origin, spacing = _demo_grid(n)
    f = cont.mandlebulb_field(cont.UniformGrid(dims, origin, spacing)).cpu().numpy()
    ref = oracle.Oracle("port").mandelbulb_field(oracle.make_grid(dims, origin, spacing))
    from oracle import mandelbulb64
    same = f == ref
    assert set(np.unique(f).tolist()) <= set(range(36))
    # points that escape at once (or start outside) agree exactly
    assert np.all(same[(ref <= 1) & (f <= 1)])
    # every difference lies where float32 does not determine the count
    o, s = np.float32(origin[0]), np.float32(spacing[0])
    x = (o + s * np.arange(dims[0], dtype=np.float32)).astype(np.float32)
    z, y, xx = np.meshgrid(x, x, x, indexing="ij")
    c = np.stack([xx.ravel(), y.ravel(), z.ravel()], 1)
    diff = np.nonzero(~same)[0]
    det, count = mandelbulb64.determined(mandelbulb64.ensemble(c[diff]))
    unexplained = int(det.sum())
    print("\nmandelbulb %d^3: %d differences, %d at float32-determined points"
          % (dims[0], diff.size, unexplained))
    assert unexplained <= 1e-4 * f.size, (unexplained, f.size)


@pytest.fixture(scope="module")
def volume(gb300):
    cont = gb300
    return cont.compute_mandlebulb((-1.0, -1.0, -1.0), (0.02, 0.02, 0.02), (100, 100, 100))


@pytest.mark.parametrize("iteration", [1.0, 3.5, 12.0])
def test_extract_surface(gb300, oracle_best, volume, iteration):
    """extractSurface: MC of the GPU field (unmerged) and ColorsAndNorms,
    against the oracle on the same field."""
    import oracle
    cont = gb300
    f = volume.EscapeIteration.cpu().numpy()
    g = oracle.make_grid(volume.Grid.dims, volume.Grid.Origin, volume.Grid.Spacing)
    count, _ = oracle_best.mc_count(g, f, iteration)
    ref = oracle_best.mc_generate(g, f, iteration, count, False)
    surf = cont.extract_surface(volume, iteration)
    verts = surf.Data.GetPointCoordinates().cpu().numpy()
    assert np.array_equal(surf.Data.GetCellConnections().cpu().numpy(), ref["conn"])
    assert np.array_equal(_bits(verts), _bits(ref["verts"]))
    norms, colors = oracle.Oracle("port").colors_and_norms(verts)
    assert np.array_equal(_bits(surf.Norms.cpu().numpy()), _bits(norms))
    assert np.array_equal(surf.Colors.cpu().numpy(), colors)
    assert surf.Colors.shape == (verts.shape[0], 4) and bool((surf.Colors[:, 3] == 255).all())


@pytest.mark.parametrize("cut", [0.3, 0.8, 0.95])
def test_clip_count_and_extract_cut(gb300, oracle_best, volume, cut):
    """MandlebulbClipCount, then the count-driven generate (extractCut)."""
    import oracle
    cont = gb300
    G = volume.Grid
    f = volume.EscapeIteration.cpu().numpy()
    g = oracle.make_grid(G.dims, G.Origin, G.Spacing)
    f32 = np.float32
    cd = [d - 1 for d in G.dims]
    loc = (f32(G.Origin[0]) + f32(G.Spacing[0]) * f32(cd[0]),
           f32(G.Origin[1]) + f32(G.Spacing[1]) * f32(cd[1]),
           f32(G.Origin[2]) + f32(G.Spacing[2]) * f32(f32(cd[2]) * f32(cut)))
    w = cont.MandlebulbClipCount(G.Origin, loc, (0, 0, 1), 3.5)
    count = cont.DispatcherMapCell(w).Invoke(G, volume.EscapeIteration)
    ref_count = oracle.Oracle("port").mandelbulb_clip_count(g, f, 3.5, G.Origin, loc, (0, 0, 1))
    assert np.array_equal(count.cpu().numpy(), ref_count)
    full, _ = oracle_best.mc_count(g, f, 3.5)
    if cut == 0.3:
        assert np.array_equal(ref_count, full)  # the plane lies below the grid
    else:
        assert 0 < ref_count.sum() < full.sum()
    ref = oracle_best.mc_generate(g, f, 3.5, ref_count, False)
    surf = cont.extract_cut(volume, cut, 3.5)
    verts = surf.Data.GetPointCoordinates().cpu().numpy()
    assert np.array_equal(surf.Data.GetCellConnections().cpu().numpy(), ref["conn"])
    assert np.array_equal(_bits(verts), _bits(ref["verts"]))
    norms, colors = oracle.Oracle("port").colors_and_norms(verts)
    assert np.array_equal(_bits(surf.Norms.cpu().numpy()), _bits(norms))
    assert np.array_equal(surf.Colors.cpu().numpy(), colors)


@pytest.mark.parametrize("merge", [True, False], ids=["merged", "unmerged"])
@pytest.mark.parametrize("kind", ["full", "mask", "partial"])
def test_counted_generate(gb300, oracle_best, merge, kind):
    """The count-driven generate against the oracle's dispatcher on the same
    count array: the MC counts themselves, a random cell mask, and counts
    below NumFaces (only the first triangles of a cell)."""
    import oracle
    from tests import cases
    cont = gb300
    d = (40, 33, 27)
    sp = tuple(1 / (n - 1) for n in d)
    f = cases.random_blobs(d, 4, 51, noise=0.05)
    g = oracle.make_grid(d, spacing=sp)
    full, _ = oracle_best.mc_count(g, f, 0.5)
    rng = np.random.default_rng(52)
    if kind == "full":
        count = full
    elif kind == "mask":
        count = np.where(rng.random(full.shape) < 0.6, full, 0).astype(np.int32)
    else:
        count = np.minimum(full, rng.integers(0, 3, size=full.shape)).astype(np.int32)
    ref = oracle_best.mc_generate(g, f, 0.5, count, merge)
    grid = cont.UniformGrid(d, spacing=sp)
    out = cont.marching_cubes_counted(grid, torch.from_numpy(f).cuda(), 0.5,
                                      torch.from_numpy(count).cuda(), merge=merge, records=True)
    assert np.array_equal(out["conn"].cpu().numpy(), ref["conn"])
    assert np.array_equal(_bits(out["verts"].cpu().numpy()), _bits(ref["verts"]))
    assert np.array_equal(out["rec_first"].cpu().numpy(), ref["rec_a"])
    assert np.array_equal(out["rec_second"].cpu().numpy(), ref["rec_b"])
    assert np.array_equal(_bits(out["rec_weight"].cpu().numpy()), _bits(ref["rec_w"]))
    if kind == "full":
        mc = cont.marching_cubes(grid, torch.from_numpy(f).cuda(), 0.5, merge=merge)
        assert torch.equal(mc["conn"], out["conn"])
        assert torch.equal(mc["verts"].view(torch.int32), out["verts"].view(torch.int32))


def test_counted_generate_through_dispatcher(gb300):
    """A count array that MarchingCubesCount did not make drives the
    generate; one it made is recounted, with the same result."""
    from tests import cases
    cont = gb300
    d = (30, 25, 20)
    f = torch.from_numpy(cases.random_blobs(d, 3, 61)).cuda()
    grid = cont.UniformGrid(d)
    count = cont.DispatcherMapCell(cont.MarchingCubesCount(0.5)).Invoke(grid, f)
    a = cont.DispatcherGenerateInterpolatedCells(count, cont.MarchingCubesGenerate(0.5)).Invoke(grid, f)
    masked = count.clone()
    masked[: masked.numel() // 2] = 0
    b = cont.DispatcherGenerateInterpolatedCells(masked, cont.MarchingCubesGenerate(0.5)).Invoke(grid, f)
    ref = cont.marching_cubes_counted(grid, f, 0.5, masked, merge=True)
    assert 0 < b.GetNumberOfCells() < a.GetNumberOfCells()
    assert torch.equal(b.GetCellConnections(), ref["conn"])
    assert torch.equal(b.GetPointCoordinates().view(torch.int32), ref["verts"].view(torch.int32))


def test_counted_generate_rejects_impossible_counts(gb300):
    from daxtoolkit_gb300 import capi
    from tests import cases
    cont = gb300
    d = (12, 11, 10)
    f = torch.from_numpy(cases.random_blobs(d, 2, 62)).cuda()
    grid = cont.UniformGrid(d)
    count = cont.DispatcherMapCell(cont.MarchingCubesCount(0.5)).Invoke(grid, f).clone()
    i = int(torch.nonzero(count == 0)[0])
    count[i] = 1  # a cell with no triangles asked for one
    with pytest.raises(capi.ErrorControlBadValue):
        cont.marching_cubes_counted(grid, f, 0.5, count, merge=False)
    with pytest.raises(capi.ErrorControlBadValue):
        cont.marching_cubes_counted(grid, f, 0.5, count, merge=True)
    neg = torch.full_like(count, -1)
    with pytest.raises(capi.ErrorControlBadValue):
        cont.marching_cubes_counted(grid, f, 0.5, neg, merge=False)


@pytest.mark.parametrize("k", [1, 3, 4])
def test_compact_point_field_components(gb300, oracle_best, k):
    """CompactPointField of a k-component point field (a Vector3 field for
    k = 3): every component interpolated with the records' weights."""
    import oracle
    from tests import cases
    cont = gb300
    d = (26, 26, 26)
    f = torch.from_numpy(cases.linear_field(d)).cuda()
    grid = cont.UniformGrid(d)
    count = cont.DispatcherMapCell(cont.MarchingCubesCount(70.0)).Invoke(grid, f)
    disp = cont.DispatcherGenerateInterpolatedCells(count, cont.MarchingCubesGenerate(70.0))
    disp.Invoke(grid, f)
    rng = np.random.default_rng(70 + k)
    vec = rng.standard_normal((grid.GetNumberOfPoints(), k)).astype(np.float32)
    got = disp.CompactPointField(torch.from_numpy(vec).cuda()).cpu().numpy()
    ra, rb, rw = [t.cpu().numpy() for t in disp._records]
    for c in range(k):
        want = oracle_best.interpolate_point_field(ra, rb, rw, np.ascontiguousarray(vec[:, c]))
        assert np.array_equal(_bits(got[:, c]), _bits(want))

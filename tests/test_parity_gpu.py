"""GPU parity: the sm_103a kernels, called through the C ABI, against the CPU
oracle on the same float32 bytes.  Topology (case indices, counts,
connectivity, interpolation end points) must be identical; vertex positions,
weights, threshold coordinates and gradients are compared bit for bit as
well (the kernels round every operation as the reference does)."""
import numpy as np
import pytest
import torch

from tests import cases

pytestmark = pytest.mark.gpu


def _grid(cont, dims, origin, spacing, emin):
    return cont.UniformGrid(dims, origin, spacing, emin)


def _ogrid(dims, origin, spacing, emin):
    import oracle
    return oracle.make_grid(dims, origin, spacing, emin)


def _bits(a):
    """Bit patterns with every NaN mapped to one value: CUDA returns the
    canonical NaN 0x7fffffff where the CPU propagates 0x7fc00000; all other
    values must match bit for bit."""
    a = np.ascontiguousarray(a)
    b = a.view(np.uint32).copy()
    b[np.isnan(a)] = 0x7FC00000
    return b


@pytest.mark.parametrize("case", cases.mc_cases(), ids=lambda c: c[0])
def test_mc_classify_count(gb300, oracle_best, case):
    name, dims, origin, spacing, emin, f, iso = case
    cont = gb300
    grid = _grid(cont, dims, origin, spacing, emin)
    fd = torch.from_numpy(f).cuda()
    count_ref, cases_ref = oracle_best.mc_count(_ogrid(dims, origin, spacing, emin), f, iso)
    disp = cont.DispatcherMapCell(cont.MarchingCubesCount(iso))
    count, cs = disp.classify_cases(grid, fd)
    torch.cuda.synchronize()
    assert np.array_equal(count.cpu().numpy(), count_ref)
    assert np.array_equal(cs.cpu().numpy(), cases_ref)
    assert np.array_equal(disp.Invoke(grid, fd).cpu().numpy(), count_ref)


@pytest.mark.parametrize("merge", [True, False], ids=["merged", "unmerged"])
@pytest.mark.parametrize("case", cases.mc_cases(), ids=lambda c: c[0])
def test_mc_generate(gb300, oracle_best, case, merge):
    name, dims, origin, spacing, emin, f, iso = case
    cont = gb300
    og = _ogrid(dims, origin, spacing, emin)
    count, _ = oracle_best.mc_count(og, f, iso)
    ref = oracle_best.mc_generate(og, f, iso, count, merge)
    out = cont.marching_cubes(_grid(cont, dims, origin, spacing, emin), torch.from_numpy(f).cuda(),
                              iso, merge=merge, records=True)
    conn = out["conn"].cpu().numpy()
    verts = out["verts"].cpu().numpy()
    assert conn.shape == ref["conn"].shape
    assert verts.shape == ref["verts"].shape
    assert np.array_equal(conn, ref["conn"])
    assert np.array_equal(out["rec_first"].cpu().numpy(), ref["rec_a"])
    assert np.array_equal(out["rec_second"].cpu().numpy(), ref["rec_b"])
    assert np.array_equal(_bits(out["rec_weight"].cpu().numpy()), _bits(ref["rec_w"]))
    assert np.array_equal(_bits(verts), _bits(ref["verts"]))


def test_mc_known_answer_counts(gb300):
    cont = gb300
    f = torch.from_numpy(cases.linear_field((26, 26, 26))).cuda()
    grid = cont.UniformGrid((26, 26, 26))
    assert cont.marching_cubes(grid, f, 70.0, merge=False)["verts"].shape[0] == 183
    out = cont.marching_cubes(grid, f, 70.0, merge=True)
    assert out["verts"].shape[0] == 45 and out["conn"].shape[0] == 61


def test_mc_dispatchers_secondary_field(gb300, oracle_best):
    """UnitTestWorkletMarchingCubes flow through the dispatcher surface:
    count, generate without and with merging, CompactPointField."""
    cont = gb300
    dims = (26, 26, 26)
    f = torch.from_numpy(cases.linear_field(dims)).cuda()
    sec_np = cases.linear_field(dims, grad=(-0.5, 1.0, 2.0))
    sec = torch.from_numpy(sec_np).cuda()
    grid = cont.UniformGrid(dims)
    count = cont.DispatcherMapCell(cont.MarchingCubesCount(70.0)).Invoke(grid, f)
    disp = cont.DispatcherGenerateInterpolatedCells(count, cont.MarchingCubesGenerate(70.0))
    disp.SetRemoveDuplicatePoints(False)
    disp.SetReleaseCount(False)
    og = disp.Invoke(grid, f)
    assert og.GetNumberOfPoints() == 3 * og.GetNumberOfCells()
    vals = disp.CompactPointField(sec).cpu().numpy()
    ref_count, _ = oracle_best.mc_count(_ogrid(dims, (0, 0, 0), (1, 1, 1), (0, 0, 0)),
                                        f.cpu().numpy(), 70.0)
    ref = oracle_best.mc_generate(_ogrid(dims, (0, 0, 0), (1, 1, 1), (0, 0, 0)), f.cpu().numpy(),
                                  70.0, ref_count, False)
    ref_vals = oracle_best.interpolate_point_field(ref["rec_a"], ref["rec_b"], ref["rec_w"], sec_np)
    assert np.array_equal(_bits(vals), _bits(ref_vals))
    disp.SetRemoveDuplicatePoints(True)
    og2 = disp.Invoke(grid, f)
    assert og2.GetNumberOfPoints() == 45


@pytest.mark.parametrize("case", cases.threshold_cases(), ids=lambda c: c[0])
def test_threshold(gb300, oracle_best, case):
    name, dims, origin, spacing, emin, f, lo, hi = case
    cont = gb300
    og = _ogrid(dims, origin, spacing, emin)
    count_ref = oracle_best.threshold_count(og, f, lo, hi)
    ref = oracle_best.threshold_generate(og, f, count_ref)
    grid = _grid(cont, dims, origin, spacing, emin)
    fd = torch.from_numpy(f).cuda()
    count = cont.DispatcherMapCell(cont.ThresholdCount(lo, hi)).Invoke(grid, fd)
    assert np.array_equal(count.cpu().numpy(), count_ref)
    out = cont.threshold(grid, fd, lo, hi)
    assert np.array_equal(out["conn"].cpu().numpy(), ref["conn"])
    assert np.array_equal(_bits(out["coords"].cpu().numpy()), _bits(ref["coords"]))
    assert np.array_equal(_bits(out["field"].cpu().numpy()), _bits(ref["field"]))


@pytest.mark.parametrize("case", cases.threshold_cases(), ids=lambda c: c[0])
def test_threshold_compact_point_field(gb300, oracle_best, case):
    """DispatcherGenerateTopology::CompactPointField with any point field:
    compacting the thresholded field itself gives the compacted field, and
    compacting a [P, 3] field of the grid's point coordinates gives the
    compacted coordinates, bit for bit."""
    name, dims, origin, spacing, emin, f, lo, hi = case
    cont = gb300
    og = _ogrid(dims, origin, spacing, emin)
    ref = oracle_best.threshold_generate(og, f, oracle_best.threshold_count(og, f, lo, hi))
    grid = _grid(cont, dims, origin, spacing, emin)
    fd = torch.from_numpy(f).cuda()
    w = cont.ThresholdCount(lo, hi)
    disp = cont.DispatcherGenerateTopology(cont.DispatcherMapCell(w).Invoke(grid, fd),
                                           threshold_worklet=w)
    disp.Invoke(grid, fd)
    got = disp.CompactPointField(fd)
    assert np.array_equal(_bits(got.cpu().numpy()), _bits(ref["field"]))
    ax = [np.float32(origin[a]) + np.float32(spacing[a]) *
          (np.arange(dims[a]) + emin[a]).astype(np.float32) for a in range(3)]
    z, y, x = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    pts = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1).astype(np.float32)
    got3 = disp.CompactPointField(torch.from_numpy(pts).cuda())
    assert got3.shape == ref["coords"].shape
    assert np.array_equal(_bits(got3.cpu().numpy()), _bits(ref["coords"]))
    # any k-component field, against the oracle's FillPointMask + StreamCompact
    import oracle
    rnd = np.random.default_rng(7).standard_normal((f.size, 4)).astype(np.float32)
    want = oracle.Oracle.threshold_compact_point_field(og, oracle_best.threshold_count(og, f, lo, hi),
                                                       rnd)
    got4 = disp.CompactPointField(torch.from_numpy(rnd).cuda())
    assert np.array_equal(_bits(got4.cpu().numpy()), _bits(want))


@pytest.mark.parametrize("case", cases.threshold_cases(), ids=lambda c: c[0])
def test_threshold_without_point_removal(gb300, oracle_best, case):
    """SetRemoveDuplicatePoints(false): the kept cells' connectivity in the
    input's own point ids (the reference skips FillPointMask and
    ResolveDuplicatePoints), and CompactPointField compacts nothing."""
    name, dims, origin, spacing, emin, f, lo, hi = case
    cont = gb300
    og = _ogrid(dims, origin, spacing, emin)
    count_ref = oracle_best.threshold_count(og, f, lo, hi)
    nx, ny, nz = dims
    cx, cy = nx - 1, ny - 1
    kept = np.nonzero(count_ref)[0]
    p = kept % cx + nx * ((kept // cx) % cy + ny * (kept // (cx * cy)))
    off = np.array([0, 1, nx + 1, nx, nx * ny, nx * ny + 1, nx * ny + nx + 1, nx * ny + nx])
    ref_conn = (p[:, None] + off[None, :]).astype(np.int32)
    grid = _grid(cont, dims, origin, spacing, emin)
    fd = torch.from_numpy(f).cuda()
    w = cont.ThresholdCount(lo, hi)
    disp = cont.DispatcherGenerateTopology(cont.DispatcherMapCell(w).Invoke(grid, fd),
                                           threshold_worklet=w)
    disp.SetRemoveDuplicatePoints(False)
    out = disp.Invoke(grid, fd)
    assert np.array_equal(out.GetCellConnections().cpu().numpy(), ref_conn.reshape(-1, 8))
    assert out.GetNumberOfPoints() == nx * ny * nz
    assert disp.CompactPointField(fd) is None


def test_threshold_compact_point_field_capacity(gb300):
    """Too small an output is refused at the totals, and nothing is written."""
    import ctypes
    from daxtoolkit_gb300 import capi
    cont = gb300
    dims = (26, 26, 26)
    grid = cont.UniformGrid(dims)
    f = torch.from_numpy(cases.linear_field(dims)).cuda()
    g = grid.desc()
    n = capi.lib().dax_gb300_threshold_scratch_bytes(ctypes.byref(g))
    scratch = torch.empty(n, dtype=torch.uint8, device="cuda")
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    capi.call("dax_gb300_threshold_count", ctypes.byref(g), p(f), 70.0, 82.0, p(scratch), n, s)
    out = torch.full((3,), -7.0, device="cuda")
    capi.call("dax_gb300_threshold_compact_point_field", ctypes.byref(g), p(scratch), n, p(f), 1,
              p(out), 3, s)
    K, U = ctypes.c_int64(0), ctypes.c_int64(0)
    st = capi.lib().dax_gb300_threshold_totals(p(scratch), ctypes.byref(K), ctypes.byref(U), s)
    assert st == capi.ERROR_CAPACITY and U.value > 3
    assert bool((out == -7.0).all())


@pytest.mark.parametrize("case", cases.gradient_cases(), ids=lambda c: c[0])
def test_cell_gradient(gb300, oracle_best, case):
    name, dims, origin, spacing, emin, f = case
    cont = gb300
    ref = oracle_best.cell_gradient(_ogrid(dims, origin, spacing, emin), f)
    out = cont.DispatcherMapCell(cont.CellGradient()).Invoke(
        _grid(cont, dims, origin, spacing, emin), torch.from_numpy(f).cuda())
    assert np.array_equal(_bits(out.cpu().numpy()), _bits(ref))


def test_cell_gradient_unaligned_output(gb300, oracle_best):
    """An output pointer that is 4- but not 8-byte aligned (the kernel's
    scalar-store variant) gives the same bits."""
    import ctypes
    from daxtoolkit_gb300 import capi
    name, dims, origin, spacing, emin, f = cases.gradient_cases()[3]
    cont = gb300
    ref = oracle_best.cell_gradient(_ogrid(dims, origin, spacing, emin), f)
    grid = _grid(cont, dims, origin, spacing, emin)
    fd = torch.from_numpy(f).cuda()
    buf = torch.full((ref.size + 2,), -7.0, device="cuda")
    out = buf[1:1 + ref.size]
    assert out.data_ptr() % 8 == 4
    capi.call("dax_gb300_cell_gradient", ctypes.byref(grid.desc()), ctypes.c_void_p(fd.data_ptr()),
              ctypes.c_void_p(out.data_ptr()), None)
    torch.cuda.synchronize()
    assert np.array_equal(_bits(out.cpu().numpy().reshape(ref.shape)), _bits(ref))
    assert buf[0].item() == -7.0 and buf[-1].item() == -7.0


@pytest.mark.parametrize("entry", ["dax_gb300_mc_count", "dax_gb300_threshold_count"])
def test_unaligned_scratch_is_refused(gb300, entry):
    """A scratch pointer off a 16-byte boundary is refused (the count passes
    store 16-byte vectors into it), and nothing is written."""
    import ctypes
    from daxtoolkit_gb300 import capi
    cont = gb300
    dims = (26, 26, 26)
    grid = cont.UniformGrid(dims)
    f = torch.from_numpy(cases.linear_field(dims)).cuda()
    g = grid.desc()
    n = capi.lib().dax_gb300_mc_scratch_bytes(ctypes.byref(g))
    n = max(n, capi.lib().dax_gb300_threshold_scratch_bytes(ctypes.byref(g)))
    buf = torch.full((n + 16,), 0x5a, dtype=torch.uint8, device="cuda")
    scratch = buf[4:]
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    args = (70.0,) if entry == "dax_gb300_mc_count" else (70.0, 82.0)
    st = getattr(capi.lib(), entry)(ctypes.byref(g), p(f), *[ctypes.c_float(a) for a in args],
                                     p(scratch), ctypes.c_size_t(n), s)
    torch.cuda.synchronize()
    assert st == capi.ERROR_BAD_VALUE
    assert bool((buf == 0x5a).all())


def test_capacity_error_writes_nothing(gb300):
    """A too-small output buffer is reported, and nothing is written."""
    import ctypes
    from daxtoolkit_gb300 import capi
    cont = gb300
    dims = (26, 26, 26)
    grid = cont.UniformGrid(dims)
    f = torch.from_numpy(cases.linear_field(dims)).cuda()
    g = grid.desc()
    n = capi.lib().dax_gb300_mc_scratch_bytes(ctypes.byref(g))
    scratch = torch.empty(n, dtype=torch.uint8, device="cuda")
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    capi.call("dax_gb300_mc_count", ctypes.byref(g), p(f), 70.0, p(scratch), n, s)
    verts = torch.full((10, 3), -7.0, device="cuda")
    conn = torch.full((10, 3), -7, dtype=torch.int32, device="cuda")
    capi.call("dax_gb300_mc_generate", ctypes.byref(g), p(f), 70.0, 1, p(scratch), n, p(verts), 10,
              p(conn), 10, None, None, None, s)
    T, V = ctypes.c_int64(0), ctypes.c_int64(0)
    st = capi.lib().dax_gb300_mc_totals(p(scratch), ctypes.byref(T), ctypes.byref(V), s)
    assert st == capi.ERROR_CAPACITY
    assert T.value == 61 and V.value == 45
    assert bool((verts == -7.0).all()) and bool((conn == -7).all())

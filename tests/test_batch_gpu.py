"""Batched marching cubes (many grids of uneven extents and isovalues in one
launch per pass, and the same pipeline replayed from a CUDA graph): every
grid's slice of the concatenated output equals the single-grid pipeline's
output bit for bit, and the single-grid pipeline equals the oracle."""
import numpy as np
import pytest
import torch

from tests import cases

pytestmark = pytest.mark.gpu


def _inputs(cont, count, lo, hi, seed):
    from daxtoolkit_gb300 import synthetic
    dims = synthetic.batch_grid_dims(count, lo, hi, seed)
    isos = synthetic.batch_isovalues(count, 0.3, 0.6, seed)
    grids, fields = [], []
    for n, d in enumerate(dims):
        grids.append(cont.UniformGrid(d, spacing=tuple(1.0 / (x - 1) for x in d)))
        fields.append(torch.from_numpy(cases.random_blobs(d, 4, seed + n, noise=0.05)).cuda())
    return grids, fields, isos


@pytest.mark.parametrize("merge", [True, False], ids=["merged", "unmerged"])
def test_batch_equals_per_grid(gb300, merge):
    cont = gb300
    grids, fields, isos = _inputs(cont, 12, 5, 70, 31)
    batch = cont.MarchingCubesBatch(grids, fields, isos)
    verts, conn, toff, voff = batch.run(merge=merge)
    verts, conn = verts.cpu().numpy(), conn.cpu().numpy()
    for g in range(len(grids)):
        single = cont.marching_cubes(grids[g], fields[g], isos[g], merge=merge)
        sv, sc = single["verts"].cpu().numpy(), single["conn"].cpu().numpy()
        assert np.array_equal(conn[toff[g]:toff[g + 1]], sc), g
        assert np.array_equal(verts[voff[g]:voff[g + 1]].view(np.uint32), sv.view(np.uint32)), g


def test_batch_graph_replay(gb300):
    cont = gb300
    grids, fields, isos = _inputs(cont, 16, 24, 60, 32)
    batch = cont.MarchingCubesBatch(grids, fields, isos)
    verts, conn, toff, voff = batch.run(merge=True)
    gv = torch.full_like(verts, -1.0)
    gc = torch.full_like(conn, -1)
    batch.capture(gv, gc, merge=True)
    for _ in range(3):
        batch.replay()
    torch.cuda.synchronize()
    assert torch.equal(gv, verts) and torch.equal(gc, conn)
    t2, v2 = batch.totals()
    assert t2 == toff and v2 == voff


def test_batch_single_grid_equals_oracle(gb300, oracle_port):
    import oracle
    cont = gb300
    d = (37, 29, 23)
    f = cases.random_blobs(d, 4, 77, noise=0.05)
    grid = cont.UniformGrid(d, spacing=tuple(1.0 / (x - 1) for x in d))
    batch = cont.MarchingCubesBatch([grid], [torch.from_numpy(f).cuda()], [0.45])
    verts, conn, _, _ = batch.run(merge=True)
    og = oracle.make_grid(d, spacing=tuple(1.0 / (x - 1) for x in d))
    count, _ = oracle_port.mc_count(og, f, 0.45)
    ref = oracle_port.mc_generate(og, f, 0.45, count, merge=True)
    assert np.array_equal(conn.cpu().numpy(), ref["conn"])
    assert np.array_equal(verts.cpu().numpy().view(np.uint32), ref["verts"].view(np.uint32))


def test_batch_every_configuration_and_the_autotuner(gb300):
    """The emit batch size and the count pass are performance choices only:
    every configuration writes the same surface; the autotuner keeps one of
    them, and a second plan of the same extent class takes it from the cache."""
    cont = gb300
    grids, fields, isos = _inputs(cont, 10, 20, 90, 33)
    batch = cont.MarchingCubesBatch(grids, fields, isos)
    ref_v, ref_c, toff, voff = batch.run(merge=True)
    for eb in (1, 8, 16, 32):
        for dealt in (0, 1):
            batch.set_config(eb, dealt)
            assert batch.config() == (eb, dealt)
            v, c, t, vo = batch.run(merge=True)
            assert t == toff and vo == voff
            assert torch.equal(c, ref_c) and torch.equal(v.view(torch.int32), ref_v.view(torch.int32))
    v = torch.empty_like(ref_v)
    c = torch.empty_like(ref_c)
    eb, dealt, ms = batch.autotune(v, c, merge=True)
    assert eb in (8, 16, 32) and dealt in (0, 1) and ms > 0
    assert torch.equal(c, ref_c) and torch.equal(v.view(torch.int32), ref_v.view(torch.int32))
    other = cont.MarchingCubesBatch(grids, fields, isos)
    assert other.autotune(v, c, merge=True) == (eb, dealt, -1.0)
    # one grid: always the per-lane count pass
    single = cont.MarchingCubesBatch(grids[:1], fields[:1], isos[:1])
    single.set_config(8, 1)
    assert single.config() == (8, 0)


def _single_adjoint(cont, grid, field, iso, dV, dG):
    """dax_gb300_mc_count then dax_gb300_field_adjoint on one grid."""
    import ctypes
    from daxtoolkit_gb300 import capi
    g = grid.desc()
    nb = capi.lib().dax_gb300_mc_scratch_bytes(ctypes.byref(g))
    scratch = torch.empty(nb, dtype=torch.uint8, device=field.device)
    out = torch.empty_like(field)
    p = lambda t: None if t is None else ctypes.c_void_p(t.data_ptr())
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    capi.call("dax_gb300_mc_count", ctypes.byref(g), p(field), iso, p(scratch), nb, s)
    capi.call("dax_gb300_field_adjoint", ctypes.byref(g), p(field), iso, p(scratch), nb, p(dV),
              p(dG), p(out), s)
    return out


@pytest.mark.parametrize("count,lo,hi,seed", [(1, 41, 41, 90), (14, 2, 47, 91)],
                         ids=["one_grid", "fourteen_grids"])
def test_batch_gradient_and_adjoint_equal_per_grid(gb300, count, lo, hi, seed):
    """The grid-set CellGradient and field adjoint (one launch per pass for
    every grid): each grid's slice of the concatenated per-cell gradients and
    per-point dL/dfield equals the single-grid entry points bit for bit, for
    grids with their own origins, spacings and extents, down to one cell;
    with upstream gradients on the vertices only, on the gradients only, on
    both, and on neither (all zeros)."""
    from daxtoolkit_gb300 import synthetic
    cont = gb300
    dims = synthetic.batch_grid_dims(count, lo, hi, seed)
    isos = synthetic.batch_isovalues(count, 0.3, 0.6, seed)
    rng = np.random.default_rng(seed)
    grids, fields = [], []
    for n, d in enumerate(dims):
        grids.append(cont.UniformGrid(d, origin=tuple(rng.uniform(-2, 2, 3)),
                                      spacing=tuple(rng.uniform(0.01, 0.2, 3)),
                                      extent_min=tuple(int(x) for x in rng.integers(-5, 5, 3))))
        fields.append(torch.from_numpy(cases.random_blobs(d, 4, seed + n, noise=0.05)).cuda())
    batch = cont.MarchingCubesBatch(grids, fields, isos)
    verts, conn, toff, voff = batch.run(merge=True)
    C, P = batch.sizes()
    assert C == sum(g.GetNumberOfCells() for g in grids)
    assert P == sum(g.GetNumberOfPoints() for g in grids)
    grad = batch.cell_gradient()
    torch.cuda.synchronize()
    dV = torch.from_numpy(rng.standard_normal(tuple(verts.shape)).astype(np.float32)).cuda()
    dG = torch.from_numpy(rng.standard_normal((C, 3)).astype(np.float32)).cuda()
    for use_v, use_g in ((True, True), (True, False), (False, True), (False, False)):
        batch.count()
        out = batch.field_adjoint(dV if use_v else None, dG if use_g else None)
        torch.cuda.synchronize()
        if not (use_v or use_g):
            assert not bool(out.any())
            continue
        c0 = p0 = 0
        for q, (gr, f, iso) in enumerate(zip(grids, fields, isos)):
            nc, npts = gr.GetNumberOfCells(), gr.GetNumberOfPoints()
            if use_v and use_g:
                g1 = cont.cell_gradient(gr, f)
                assert torch.equal(g1.view(torch.int32), grad[c0:c0 + nc].view(torch.int32)), q
            o1 = _single_adjoint(cont, gr, f, iso,
                                 dV[voff[q]:voff[q + 1]].contiguous() if use_v else None,
                                 dG[c0:c0 + nc].contiguous() if use_g else None)
            assert torch.equal(o1.view(torch.int32), out[p0:p0 + npts].view(torch.int32)), (q, use_v,
                                                                                           use_g)
            c0 += nc
            p0 += npts

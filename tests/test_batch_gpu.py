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

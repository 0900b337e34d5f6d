"""Parity at the benchmark workloads' own sizes, through the C ABI, against the
reference-built driver (the DaxToolkit's own worklet functors; the C port
where the reference could not be compiled).

* 256^3 and 512^3 points, float32, 8 Gaussian blobs (seed 20260101) on the
  unit cube: merged marching cubes at isovalue 0.5 with its interpolation
  records (dax/cont/DispatcherGenerateInterpolatedCells.h:145-301),
  Threshold [0.3, 0.7] with its compacted coordinates and field
  (dax/cont/DispatcherGenerateTopology.h:128-258), and CellGradient over
  every cell (dax/worklet/CellGradient.h:35-47).
* 64 grids, each dimension U{32..192} points (seed 777), 4 blobs plus
  0.05 U(-1, 1) noise, per-grid isovalue U[0.3, 0.6]: the batched pipeline,
  run directly and replayed from its CUDA graph, grid by grid.

Everything is compared bit for bit: the kernels round every float operation
as the reference does.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

BLOB_SEED = 20260101


def _bits(a):
    """Bit patterns, every NaN mapped to one value (CUDA's canonical NaN
    differs from the host's; no NaN arises from these fields)."""
    a = np.ascontiguousarray(a)
    b = a.view(np.uint32).copy()
    b[np.isnan(a)] = 0x7FC00000
    return b


@pytest.fixture(scope="module", params=[256, 512], ids=["256cube", "512cube"])
def blob8(request):
    """The 8-blob field at n^3 points: one host copy, one device copy of the
    same bytes."""
    from daxtoolkit_gb300 import synthetic
    n = request.param
    dims = (n, n, n)
    fd = synthetic.blob_field(dims, 8, seed=BLOB_SEED, device="cuda")
    return n, dims, (1.0 / (n - 1),) * 3, fd.cpu().numpy(), fd


def _ogrid(dims, spacing):
    import oracle
    return oracle.make_grid(dims, spacing=spacing)


def test_config2_marching_cubes_merged(gb300, oracle_best, blob8):
    cont = gb300
    n, dims, spacing, fh, fd = blob8
    og = _ogrid(dims, spacing)
    count, _ = oracle_best.mc_count(og, fh, 0.5)
    ref = oracle_best.mc_generate(og, fh, 0.5, count, merge=True)
    out = cont.marching_cubes(cont.UniformGrid(dims, spacing=spacing), fd, 0.5, merge=True,
                              records=True)
    assert out["conn"].shape[0] == ref["conn"].shape[0] > 0
    assert np.array_equal(out["conn"].cpu().numpy(), ref["conn"])
    assert np.array_equal(out["rec_first"].cpu().numpy(), ref["rec_a"])
    assert np.array_equal(out["rec_second"].cpu().numpy(), ref["rec_b"])
    assert np.array_equal(_bits(out["rec_weight"].cpu().numpy()), _bits(ref["rec_w"]))
    assert np.array_equal(_bits(out["verts"].cpu().numpy()), _bits(ref["verts"]))


def test_config2_threshold(gb300, oracle_best, blob8):
    cont = gb300
    n, dims, spacing, fh, fd = blob8
    og = _ogrid(dims, spacing)
    count = oracle_best.threshold_count(og, fh, 0.3, 0.7)
    ref = oracle_best.threshold_generate(og, fh, count)
    out = cont.threshold(cont.UniformGrid(dims, spacing=spacing), fd, 0.3, 0.7)
    assert out["conn"].shape[0] == ref["conn"].shape[0] > 0
    assert np.array_equal(out["conn"].cpu().numpy(), ref["conn"])
    assert np.array_equal(_bits(out["coords"].cpu().numpy()), _bits(ref["coords"]))
    assert np.array_equal(_bits(out["field"].cpu().numpy()), _bits(ref["field"]))


def test_config2_cell_gradient(gb300, oracle_best, blob8):
    cont = gb300
    n, dims, spacing, fh, fd = blob8
    ref = oracle_best.cell_gradient(_ogrid(dims, spacing), fh)
    out = cont.cell_gradient(cont.UniformGrid(dims, spacing=spacing), fd)
    assert out.shape == (ref.shape[0], 3)
    got = out.cpu().numpy()
    del out
    assert np.array_equal(_bits(got), _bits(ref))


def test_config3_batch_64_grids(gb300, oracle_best):
    """The 64-grid batch, directly and from its CUDA graph, grid by grid
    against the reference-built driver on the same bytes."""
    import oracle
    from daxtoolkit_gb300 import synthetic
    cont = gb300
    gdims = synthetic.batch_grid_dims(64, 32, 192, 777)
    isos = synthetic.batch_isovalues(64, 0.3, 0.6, 777)
    grids, fields, hosts = [], [], []
    for k, d in enumerate(gdims):
        sp = tuple(1.0 / (x - 1) for x in d)
        grids.append(cont.UniformGrid(d, spacing=sp))
        f = synthetic.blob_field(d, 4, seed=1000 + k, noise=0.05, device="cuda")
        fields.append(f)
        hosts.append(f.cpu().numpy())
    batch = cont.MarchingCubesBatch(grids, fields, isos)
    verts, conn, toff, voff = batch.run(merge=True)
    gv = torch.full_like(verts, -1.0)
    gc = torch.full_like(conn, -1)
    batch.capture(gv, gc, merge=True)
    batch.replay()
    batch.replay()
    torch.cuda.synchronize()
    assert torch.equal(gv, verts) and torch.equal(gc, conn)
    verts, conn = _bits(verts.cpu().numpy()), conn.cpu().numpy()
    for k, d in enumerate(gdims):
        og = oracle.make_grid(d, spacing=tuple(1.0 / (x - 1) for x in d))
        count, _ = oracle_best.mc_count(og, hosts[k], isos[k])
        ref = oracle_best.mc_generate(og, hosts[k], isos[k], count, merge=True)
        assert toff[k + 1] - toff[k] == ref["conn"].shape[0], k
        assert voff[k + 1] - voff[k] == ref["verts"].shape[0], k
        assert np.array_equal(conn[toff[k]:toff[k + 1]], ref["conn"]), k
        assert np.array_equal(verts[voff[k]:voff[k + 1]], _bits(ref["verts"])), k

"""The fused count pass (classification, counts and the decoupled look-back
scan in one persistent launch, dax_gb300_set_fused_count) against the
three-launch pass (classify, count, scan): marching cubes (merged, with
records) and threshold outputs equal bit for bit, on grids whose rows are
shorter than a word, straddle words and 4-word groups, hold one cell, and
span many scan tiles and classification units; for classification units of
1, 2, 16 and 256 stages; an unaligned field takes the three-launch pass;
the pipelined one-slab frame, repeated and replayed from a CUDA graph, on
the fused pass; and the fused pass against the oracle on the benchmark
field."""
import ctypes

import numpy as np
import pytest
import torch

from tests import cases

pytestmark = pytest.mark.gpu

SHAPES = [(2, 2, 2), (3, 5, 7), (33, 17, 9), (31, 64, 40), (100, 37, 23), (129, 64, 41),
          (160, 150, 60), (257, 3, 200), (4, 300, 260)]


@pytest.fixture
def fused():
    from daxtoolkit_gb300 import capi

    def set_fused(enabled, stages=0):
        capi.call("dax_gb300_set_fused_count", int(enabled), int(stages))
    yield set_fused
    capi.call("dax_gb300_set_fused_count", 0, 16)


def _field(dims, seed):
    f = cases.random_blobs(dims, 5, seed, noise=0.05)
    return torch.from_numpy(f).cuda()


def _mc(cont, grid, f, iso):
    out = cont.marching_cubes(grid, f, iso, merge=True, records=True)
    torch.cuda.synchronize()
    return {k: v.cpu() for k, v in out.items()}


def _thr(cont, grid, f, lo, hi):
    out = cont.threshold(grid, f, lo, hi, compact_field=True)
    torch.cuda.synchronize()
    return {k: v.cpu() for k, v in out.items()}


def _same(a, b):
    assert a.keys() == b.keys()
    for k in a:
        x, y = a[k], b[k]
        assert x.shape == y.shape, k
        if x.dtype == torch.float32:
            x, y = x.view(torch.int32), y.view(torch.int32)
        assert torch.equal(x, y), k


@pytest.mark.parametrize("dims", SHAPES, ids=lambda d: "x".join(map(str, d)))
def test_fused_equals_three_launch(gb300, fused, dims):
    cont = gb300
    f = _field(dims, sum(dims))
    grid = cont.UniformGrid(dims, origin=(0.5, -1.0, 2.0), spacing=(0.1, 0.2, 0.3),
                            extent_min=(1, -2, 3))
    fused(0)
    mc0, th0 = _mc(cont, grid, f, 0.45), _thr(cont, grid, f, 0.3, 0.7)
    for stages in (1, 2, 16, 256):
        fused(1, stages)
        _same(_mc(cont, grid, f, 0.45), mc0)
        _same(_thr(cont, grid, f, 0.3, 0.7), th0)


def test_fused_large_grid_many_tiles(gb300, fused):
    """320 x 288 x 200 (18.4 M points): 4,500 scan tiles, 282 units of 16
    stages, rows of 10 words (4-word groups straddle rows)."""
    from daxtoolkit_gb300 import synthetic
    cont = gb300
    dims = (320, 288, 200)
    f = synthetic.blob_field(dims, 8, seed=20260101, device=torch.device("cuda"))
    grid = cont.UniformGrid(dims, spacing=tuple(1.0 / (d - 1) for d in dims))
    fused(0)
    mc0, th0 = _mc(cont, grid, f, 0.5), _thr(cont, grid, f, 0.3, 0.7)
    assert mc0["conn"].shape[0] > 100000 and th0["conn"].shape[0] > 100000
    for stages in (4, 16):
        fused(1, stages)
        _same(_mc(cont, grid, f, 0.5), mc0)
        _same(_thr(cont, grid, f, 0.3, 0.7), th0)


def test_unaligned_field_takes_three_launch_pass(gb300, fused):
    cont = gb300
    dims = (45, 33, 21)
    P = dims[0] * dims[1] * dims[2]
    base = torch.rand(P + 4, generator=torch.Generator().manual_seed(5)).cuda()
    f = base[1:1 + P]  # 4-byte aligned, not 16
    assert f.data_ptr() % 16 != 0
    grid = cont.UniformGrid(dims)
    fused(1)
    a = _mc(cont, grid, f, 0.45)
    fused(0)
    b = _mc(cont, grid, f.clone(), 0.45)
    _same(a, b)


def test_fused_pipeline_frames_and_graph(gb300, fused):
    """dax_gb300_mc_pipeline's one-slab frame (fused count + emit) equals the
    two-call path on the three-launch pass; repeated on one scratch and
    replayed from a CUDA graph."""
    cont = gb300
    dims = (200, 180, 170)
    from daxtoolkit_gb300 import synthetic
    f = synthetic.blob_field(dims, 8, seed=7, device=torch.device("cuda"))
    grid = cont.UniformGrid(dims, spacing=tuple(1.0 / (d - 1) for d in dims))
    fused(0)
    ref = _mc(cont, grid, f, 0.5)
    T, V = ref["conn"].shape[0], ref["verts"].shape[0]
    fused(1)
    verts = torch.empty((V, 3), dtype=torch.float32, device="cuda")
    conn = torch.empty((T, 3), dtype=torch.int32, device="cuda")
    rec = tuple(torch.empty(V, dtype=dt, device="cuda")
                for dt in (torch.int32, torch.int32, torch.float32))
    scratch = cont.Scratch()
    for _ in range(3):
        verts.fill_(-1.0)
        t, v = cont.marching_cubes_pipelined(grid, f, 0.5, verts, conn, merge=True, records=rec,
                                             scratch=scratch)
        assert (t, v) == (T, V)
        torch.cuda.synchronize()
        _same({"verts": verts.cpu(), "conn": conn.cpu()},
              {"verts": ref["verts"], "conn": ref["conn"]})
        assert torch.equal(rec[2].cpu().view(torch.int32), ref["rec_weight"].view(torch.int32))
    stream = torch.cuda.Stream()
    stream.wait_stream(torch.cuda.current_stream())
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream):
        cont.marching_cubes_pipelined(grid, f, 0.5, verts, conn, merge=True, scratch=scratch,
                                      stream=stream, read_sizes=False)
    for _ in range(3):
        verts.fill_(-1.0)
        conn.fill_(-1)
        g.replay()
        torch.cuda.synchronize()
        _same({"verts": verts.cpu(), "conn": conn.cpu()},
              {"verts": ref["verts"], "conn": ref["conn"]})


def test_fused_equals_oracle_on_the_benchmark_field(gb300, fused, oracle_best):
    """256^3, 8 blobs (seed 20260101), isovalue 0.5, merged, on the fused
    pass: triangles and merged vertices equal the reference-built driver's."""
    import oracle
    from daxtoolkit_gb300 import synthetic
    cont = gb300
    dims = (256, 256, 256)
    spacing = (1.0 / 255,) * 3
    f = synthetic.blob_field(dims, 8, seed=20260101, device=torch.device("cuda"))
    fused(1, 16)
    out = _mc(cont, cont.UniformGrid(dims, spacing=spacing), f, 0.5)
    og = oracle.make_grid(dims, (0, 0, 0), spacing, (0, 0, 0))
    fh = f.cpu().numpy()
    count, _ = oracle_best.mc_count(og, fh, 0.5)
    ref = oracle_best.mc_generate(og, fh, 0.5, count, True)
    assert np.array_equal(out["conn"].numpy(), ref["conn"])
    assert np.array_equal(out["verts"].numpy().view(np.uint32), ref["verts"].view(np.uint32))

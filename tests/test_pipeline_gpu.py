"""dax_gb300_mc_pipeline: count + generate in one slab-pipelined call, through
the C ABI, against the reference-built driver (the C port where the
reference could not be compiled), bit for bit, for 1 to 16 slabs; its
capacity check; repeated calls and a CUDA-graph replay on one scratch."""
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


@pytest.fixture
def slabs():
    from daxtoolkit_gb300 import capi

    def set_slabs(n):
        capi.call("dax_gb300_set_pipeline_slabs", n)
    yield set_slabs
    capi.call("dax_gb300_set_pipeline_slabs", 0)


def _plan_slabs(grid, n):
    from daxtoolkit_gb300 import capi
    out = (ctypes.c_int64 * 52)()
    capi.call("dax_gb300_mc_pipeline_plan", ctypes.byref(grid.desc()), n, out)
    return out[0]


def _run(cont, grid, fd, iso, merge, T, V):
    dev = fd.device
    verts = torch.full((V + 3, 3), -7.0, dtype=torch.float32, device=dev)
    conn = torch.full((T + 3, 3), -7, dtype=torch.int32, device=dev)
    rec = (torch.full((V + 3,), -7, dtype=torch.int32, device=dev),
           torch.full((V + 3,), -7, dtype=torch.int32, device=dev),
           torch.full((V + 3,), -7.0, dtype=torch.float32, device=dev))
    t, v = cont.marching_cubes_pipelined(grid, fd, iso, verts, conn, merge=merge, records=rec)
    assert (t, v) == (T, V)
    # nothing past the result
    assert bool((conn[T:] == -7).all()) and bool((verts[V:] == -7.0).all())
    assert all(bool((r[V:] == -7).all()) for r in rec)
    return verts[:V], conn[:T], [r[:V] for r in rec]


def _check(cont, oracle_best, name, dims, origin, spacing, emin, f, iso, merge):
    import oracle
    og = oracle.make_grid(dims, origin, spacing, emin)
    count, _ = oracle_best.mc_count(og, f, iso)
    ref = oracle_best.mc_generate(og, f, iso, count, merge)
    grid = cont.UniformGrid(dims, origin, spacing, emin)
    verts, conn, rec = _run(cont, grid, torch.from_numpy(f).cuda(), iso, merge,
                            ref["conn"].shape[0], ref["verts"].shape[0])
    assert np.array_equal(conn.cpu().numpy(), ref["conn"]), name
    assert np.array_equal(_bits(verts.cpu().numpy()), _bits(ref["verts"])), name
    assert np.array_equal(rec[0].cpu().numpy(), ref["rec_a"]), name
    assert np.array_equal(rec[1].cpu().numpy(), ref["rec_b"]), name
    assert np.array_equal(_bits(rec[2].cpu().numpy()), _bits(ref["rec_w"])), name


@pytest.mark.parametrize("merge", [True, False], ids=["merged", "unmerged"])
@pytest.mark.parametrize("case", cases.mc_cases(), ids=lambda c: c[0])
def test_pipeline_parity_cases(gb300, oracle_best, slabs, case, merge):
    slabs(16)
    _check(gb300, oracle_best, *case, merge)


def _multi_slab_cases():
    out = []
    d = (256, 64, 96)
    out.append(("blobs_256x64x96", d, (0, 0, 0), tuple(1 / (n - 1) for n in d), (0, 0, 0),
                cases.random_blobs(d, 6, 41, noise=0.05), 0.5))
    d = (33, 5, 6000)
    out.append(("long_z_33x5x6000", d, (0.5, -1.0, 2.0), (0.01, 0.02, 0.003), (2, 0, -9),
                cases.random_blobs(d, 8, 42, noise=0.3), 0.45))
    d = (600, 600, 40)
    out.append(("wide_600x600x40", d, (0, 0, 0), tuple(1 / (n - 1) for n in d), (0, 0, 0),
                cases.random_blobs(d, 5, 43, noise=0.02), 0.5))
    d = (130, 70, 400)
    f = cases.random_blobs(d, 5, 44, noise=0.1)
    f[::97] = np.nan
    out.append(("nan_130x70x400", d, (0, 0, 0), (1, 1, 1), (0, 0, 0), f, 0.5))
    return out


@pytest.mark.parametrize("n", [2, 3, 5, 16])
@pytest.mark.parametrize("merge", [True, False], ids=["merged", "unmerged"])
@pytest.mark.parametrize("case", _multi_slab_cases(), ids=lambda c: c[0])
def test_pipeline_parity_many_slabs(gb300, oracle_best, slabs, case, merge, n):
    cont = gb300
    name, dims, origin, spacing, emin = case[:5]
    assert _plan_slabs(cont.UniformGrid(dims, origin, spacing, emin), n) > 1
    slabs(n)
    _check(cont, oracle_best, *case, merge)


def test_pipeline_512cube_equals_two_call_path(gb300, slabs):
    """The headline 512^3 workload: the pipelined call, twice in a row on one
    scratch, equals dax_gb300_mc_count + dax_gb300_mc_generate bit for bit
    (which tests/test_configs_gpu.py checks against the reference)."""
    from daxtoolkit_gb300 import synthetic
    cont = gb300
    slabs(8)
    dims = (512, 512, 512)
    grid = cont.UniformGrid(dims, spacing=(1 / 511,) * 3)
    fd = synthetic.blob_field(dims, 8, seed=20260101, device="cuda")
    ref = cont.marching_cubes(grid, fd, 0.5, merge=True)
    T, V = ref["conn"].shape[0], ref["verts"].shape[0]
    assert _plan_slabs(grid, 8) == 8
    for _ in range(2):
        verts, conn, _ = _run(cont, grid, fd, 0.5, True, T, V)
        assert torch.equal(conn, ref["conn"])
        assert torch.equal(verts.view(torch.int32), ref["verts"].view(torch.int32))


def test_pipeline_capacity_error(gb300, slabs):
    from daxtoolkit_gb300 import capi
    cont = gb300
    slabs(5)
    d = (256, 64, 96)
    grid = cont.UniformGrid(d, spacing=tuple(1 / (n - 1) for n in d))
    fd = torch.from_numpy(cases.random_blobs(d, 6, 41, noise=0.05)).cuda()
    ref = cont.marching_cubes(grid, fd, 0.5, merge=True)
    T, V = ref["conn"].shape[0], ref["verts"].shape[0]
    for tcap, vcap in ((T // 2, V), (T, V - 1), (0, 0)):
        verts = torch.full((vcap + 8, 3), -7.0, dtype=torch.float32, device="cuda")
        conn = torch.full((tcap + 8, 3), -7, dtype=torch.int32, device="cuda")
        with pytest.raises(capi.DaxError) as e:
            cont.marching_cubes_pipelined(grid, fd, 0.5, verts[:vcap], conn[:tcap])
        assert e.value.code == capi.ERROR_CAPACITY
        torch.cuda.synchronize()
        # nothing past the capacities
        assert bool((conn[tcap:] == -7).all()) and bool((verts[vcap:] == -7.0).all())


def test_pipeline_graph_replay(gb300, slabs):
    """Captured once (after a first call outside capture) and replayed: the
    replays write the same surface."""
    cont = gb300
    slabs(6)
    d = (256, 64, 96)
    grid = cont.UniformGrid(d, spacing=tuple(1 / (n - 1) for n in d))
    fd = torch.from_numpy(cases.random_blobs(d, 6, 45, noise=0.05)).cuda()
    ref = cont.marching_cubes(grid, fd, 0.5, merge=True)
    T, V = ref["conn"].shape[0], ref["verts"].shape[0]
    from daxtoolkit_gb300.cont import Scratch
    scratch = Scratch()
    verts = torch.empty((V, 3), dtype=torch.float32, device="cuda")
    conn = torch.empty((T, 3), dtype=torch.int32, device="cuda")
    cont.marching_cubes_pipelined(grid, fd, 0.5, verts, conn, scratch=scratch)
    verts.fill_(-1.0)
    conn.fill_(-1)
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=side, capture_error_mode="thread_local"):
        cont.marching_cubes_pipelined(grid, fd, 0.5, verts, conn, scratch=scratch,
                                      read_sizes=False)
    torch.cuda.synchronize()
    for _ in range(3):
        g.replay()
    torch.cuda.synchronize()
    assert torch.equal(conn, ref["conn"])
    assert torch.equal(verts.view(torch.int32), ref["verts"].view(torch.int32))

"""dax_gb300_mc_noalloc: the marching-cubes entry point for callers that
cannot allocate device memory (a memory budget reserved up front, no
allocator calls allowed on a latency-critical path, or a plugin host that
only hands over its own buffers).  Its scratch is a fixed 32 MiB array inside
the library, so these tests check that it gives exactly what the allocating
entry points give, on two calls in a row through the same shared array, and
that a grid too large for the array is refused before any work is queued.

Collected last (file name), so that a run stopping at the first failure has
already run every other test; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest
import torch

from tests import cases

pytestmark = pytest.mark.gpu


def _desc(cont, dims):
    return cont.UniformGrid(dims, spacing=tuple(1.0 / (n - 1) for n in dims))


def _noalloc(capi, grid, field, iso, merge, vcap, tcap):
    g = grid.desc()
    verts = torch.full((vcap, 3), -1.0, dtype=torch.float32, device="cuda")
    conn = torch.full((tcap, 3), -1, dtype=torch.int32, device="cuda")
    totals = torch.full((3,), -1, dtype=torch.int64, device="cuda")
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    capi.call("dax_gb300_mc_noalloc", ctypes.byref(g), p(field), float(iso), int(merge), p(verts),
              vcap, p(conn), tcap, p(totals), s)
    torch.cuda.synchronize()
    t = totals.cpu().numpy()
    return verts, conn, t


@pytest.mark.parametrize("merge", [True, False], ids=["merged", "unmerged"])
def test_noalloc_matches_allocating_path_twice(gb300, merge):
    from daxtoolkit_gb300 import capi
    cont = gb300
    runs = [((96, 80, 70), 0.5, 101), ((64, 72, 50), 0.45, 102)]
    for dims, iso, seed in runs:  # two calls in a row share the one scratch array
        grid = _desc(cont, dims)
        field = torch.from_numpy(cases.random_blobs(dims, 5, seed, noise=0.05)).cuda()
        ref = cont.marching_cubes(grid, field, iso, merge=merge)
        T, V = ref["conn"].shape[0], ref["verts"].shape[0]
        verts, conn, tot = _noalloc(capi, grid, field, iso, merge, V + 7, T + 5)
        assert tot[2] == 0
        assert tot[0] == T and (tot[1] == V if merge else 3 * tot[0] == V)
        assert torch.equal(conn[:T], ref["conn"])
        assert np.array_equal(verts[:V].cpu().numpy().view(np.uint32),
                              ref["verts"].cpu().numpy().view(np.uint32))
        # nothing written past the result
        assert bool((conn[T:] == -1).all()) and bool((verts[V:] == -1.0).all())


def test_noalloc_capacity_too_small_reports_and_writes_nothing(gb300):
    from daxtoolkit_gb300 import capi
    cont = gb300
    dims = (48, 40, 36)
    grid = _desc(cont, dims)
    field = torch.from_numpy(cases.random_blobs(dims, 4, 11, noise=0.05)).cuda()
    verts, conn, tot = _noalloc(capi, grid, field, 0.5, True, 4, 4)
    assert tot[0] > 4 and tot[2] == 2
    assert bool((conn == -1).all()) and bool((verts == -1.0).all())


def test_noalloc_rejects_grid_beyond_scratch(gb300):
    from daxtoolkit_gb300 import capi
    cont = gb300
    grid = _desc(cont, (512, 512, 512))  # needs far more than 32 MiB of scratch
    g = grid.desc()
    assert capi.lib().dax_gb300_mc_scratch_bytes(ctypes.byref(g)) > (32 << 20)
    st = capi.lib().dax_gb300_mc_noalloc(ctypes.byref(g), None, 0.5, 1, None, 0, None, 0,
                                         ctypes.c_void_p(16), None)
    assert st == capi.ERROR_UNSUPPORTED
    assert b"32 MiB" in capi.lib().dax_gb300_last_error()


def test_noalloc_refuses_totals_it_cannot_write(gb300):
    """d_totals off an 8-byte boundary, or in pageable host memory, is refused
    before any work is queued; the outputs stay untouched."""
    from daxtoolkit_gb300 import capi
    cont = gb300
    dims = (40, 36, 30)
    grid = _desc(cont, dims)
    g = grid.desc()
    field = torch.from_numpy(cases.random_blobs(dims, 3, 12, noise=0.05)).cuda()
    verts = torch.full((4096, 3), -1.0, dtype=torch.float32, device="cuda")
    conn = torch.full((4096, 3), -1, dtype=torch.int32, device="cuda")
    dev_totals = torch.zeros(4, dtype=torch.int64, device="cuda")
    host_totals = np.zeros(3, np.int64)  # pageable: the device cannot write it
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    L = capi.lib()
    for bad in (ctypes.c_void_p(dev_totals.data_ptr() + 4),
                ctypes.c_void_p(host_totals.ctypes.data)):
        st = L.dax_gb300_mc_noalloc(ctypes.byref(g), p(field), 0.5, 1, p(verts), 4096, p(conn),
                                    4096, bad, s)
        assert st == capi.ERROR_BAD_VALUE, L.dax_gb300_last_error()
    torch.cuda.synchronize()
    assert bool((conn == -1).all()) and bool((verts == -1.0).all())
    assert not host_totals.any() and not bool(dev_totals.any())
    # page-locked host memory with a device mapping is accepted
    pinned = torch.full((3,), -1, dtype=torch.int64, pin_memory=True)
    st = L.dax_gb300_mc_noalloc(ctypes.byref(g), p(field), 0.5, 1, p(verts), 4096, p(conn), 4096,
                                ctypes.c_void_p(pinned.data_ptr()), s)
    assert st == 0, L.dax_gb300_last_error()
    torch.cuda.synchronize()
    ref = cont.marching_cubes(grid, field, 0.5, merge=True)
    assert pinned[0].item() == ref["conn"].shape[0] and pinned[2].item() == 0

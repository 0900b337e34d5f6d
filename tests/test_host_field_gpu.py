"""Fields in page-locked host memory: the kernels read them through their
device mapping, and every output equals the one computed from a device copy
of the field bit for bit.  Pageable host memory is refused before any launch."""
import ctypes

import numpy as np
import pytest
import torch

from tests import cases

pytestmark = pytest.mark.gpu

DIMS = [(48, 40, 36), (130, 9, 6), (33, 17, 5)]


def _pair(dims, seed):
    f = cases.random_blobs(dims, 4, seed, noise=0.05)
    host = torch.from_numpy(f).pin_memory()
    return host, host.cuda()


@pytest.mark.parametrize("dims", DIMS, ids=lambda d: "x".join(map(str, d)))
@pytest.mark.parametrize("merge", [True, False])
def test_mc_from_host_field(gb300, dims, merge):
    cont = gb300
    grid = cont.UniformGrid(dims, origin=(0.5, -1.0, 2.0), spacing=(0.1, 0.2, 0.3))
    host, dev = _pair(dims, 41)
    a = cont.marching_cubes(grid, host, 0.45, merge=merge, records=True)
    b = cont.marching_cubes(grid, dev, 0.45, merge=merge, records=True)
    assert a["conn"].is_cuda and a["conn"].shape[0] > 0
    for k in ("verts", "conn", "rec_first", "rec_second", "rec_weight"):
        assert torch.equal(a[k], b[k]), k


@pytest.mark.parametrize("dims", DIMS, ids=lambda d: "x".join(map(str, d)))
def test_threshold_and_gradient_from_host_field(gb300, dims):
    cont = gb300
    grid = cont.UniformGrid(dims, spacing=(0.5, 0.25, 1.0))
    host, dev = _pair(dims, 42)
    a = cont.threshold(grid, host, 0.2, 0.7)
    b = cont.threshold(grid, dev, 0.2, 0.7)
    for k in ("conn", "coords", "field"):
        assert torch.equal(a[k], b[k]), k
    ga = cont.cell_gradient(grid, host)
    gb = cont.cell_gradient(grid, dev)
    assert torch.equal(ga.view(torch.int32), gb.view(torch.int32))


def test_pageable_host_field_is_refused(gb300):
    from daxtoolkit_gb300 import capi
    cont = gb300
    dims = (16, 16, 16)
    grid = cont.UniformGrid(dims)
    g = grid.desc()
    pageable = np.ones(16 ** 3, np.float32)
    L = capi.lib()
    nb = L.dax_gb300_mc_scratch_bytes(ctypes.byref(g))
    scratch = torch.empty(nb, dtype=torch.uint8, device="cuda")
    with pytest.raises(capi.ErrorControlBadValue) as e:
        capi.call("dax_gb300_mc_count", ctypes.byref(g), ctypes.c_void_p(pageable.ctypes.data), 0.5,
                  ctypes.c_void_p(scratch.data_ptr()), nb, None)
    assert "pageable" in str(e.value)
    with pytest.raises(capi.ErrorControlBadValue):
        cont.marching_cubes(grid, torch.ones(16 ** 3), 0.5)

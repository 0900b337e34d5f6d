"""The largest grid dax::Id allows, checked by slab consistency.

A 1290^3 grid (2,146,689,000 points, just below 2^31) is processed whole
and as its two z-slabs that share one point plane; the upper slab carries
its extent offset, so its coordinates are those of the whole grid.  Cells
partition between the slabs and every output is in cell order, so:

  * marching cubes: the lower slab's triangles are the first triangles of
    the whole run and the upper slab's the rest, with identical vertex
    positions (compared through the connectivity, bit for bit);
  * threshold: the same for kept cells, through the compacted coordinates
    and field;
  * CellGradient: the lower and upper cell gradients are the two halves of
    the whole grid's, bit for bit.

No CPU reference is needed at this size: the slabs are ordinary grids whose
results the parity tests pin, and the whole grid must agree with them.
Index arithmetic past 2^31 (CellGradient writes 6.4e9 floats) and offsets
near 2^31 are exercised.
"""
import pytest
import torch

pytestmark = pytest.mark.gpu

N = 1290
SPLIT = 645  # the shared point plane


@pytest.fixture(scope="module")
def big(gb300):
    free, _ = torch.cuda.mem_get_info()
    if free < 120 * 2 ** 30:
        pytest.skip("needs about 120 GB of free device memory")
    from daxtoolkit_gb300 import synthetic
    cont = gb300
    dims = (N, N, N)
    sp = (1.0 / (N - 1),) * 3
    f = synthetic.blob_field(dims, 16, seed=77, device="cuda")
    plane = N * N
    d = dict(cont=cont, f=f,
             f_lo=f[:(SPLIT + 1) * plane], f_hi=f[SPLIT * plane:],
             whole=cont.UniformGrid(dims, spacing=sp),
             lo=cont.UniformGrid((N, N, SPLIT + 1), spacing=sp),
             hi=cont.UniformGrid((N, N, N - SPLIT), spacing=sp, extent_min=(0, 0, SPLIT)))
    yield d
    d.clear()
    torch.cuda.empty_cache()


def _bits(t):
    return t.contiguous().view(torch.int32)


def test_mc_max_grid_slab_consistency(big):
    cont = big["cont"]
    w = cont.marching_cubes(big["whole"], big["f"], 0.5, merge=True)
    a = cont.marching_cubes(big["lo"], big["f_lo"], 0.5, merge=True)
    b = cont.marching_cubes(big["hi"], big["f_hi"], 0.5, merge=True)
    Tw, Ta, Tb = w["conn"].shape[0], a["conn"].shape[0], b["conn"].shape[0]
    assert Ta > 0 and Tb > 0 and Tw == Ta + Tb
    assert torch.equal(_bits(w["verts"][w["conn"][:Ta].long()]),
                       _bits(a["verts"][a["conn"].long()]))
    assert torch.equal(_bits(w["verts"][w["conn"][Ta:].long()]),
                       _bits(b["verts"][b["conn"].long()]))
    # merged ids are dense and every vertex is referenced
    V = w["verts"].shape[0]
    assert int(w["conn"].max()) == V - 1
    used = torch.zeros(V, dtype=torch.bool, device="cuda")
    used[w["conn"].reshape(-1).long()] = True
    assert bool(used.all())


def test_threshold_max_grid_slab_consistency(big):
    cont = big["cont"]
    w = cont.threshold(big["whole"], big["f"], 0.3, 0.7)
    a = cont.threshold(big["lo"], big["f_lo"], 0.3, 0.7)
    b = cont.threshold(big["hi"], big["f_hi"], 0.3, 0.7)
    Kw, Ka, Kb = w["conn"].shape[0], a["conn"].shape[0], b["conn"].shape[0]
    assert Ka > 0 and Kb > 0 and Kw == Ka + Kb
    for part, rng in ((a, slice(0, Ka)), (b, slice(Ka, Kw))):
        idx_w, idx_p = w["conn"][rng].long(), part["conn"].long()
        assert torch.equal(_bits(w["coords"][idx_w]), _bits(part["coords"][idx_p]))
        assert torch.equal(_bits(w["field"][idx_w]), _bits(part["field"][idx_p]))


def test_cell_gradient_max_grid_slab_consistency(big):
    cont = big["cont"]
    cells_lo = (N - 1) * (N - 1) * SPLIT
    w = cont.cell_gradient(big["whole"], big["f"])
    a = cont.cell_gradient(big["lo"], big["f_lo"])
    assert torch.equal(_bits(w[:cells_lo]), _bits(a))
    del a
    b = cont.cell_gradient(big["hi"], big["f_hi"])
    assert torch.equal(_bits(w[cells_lo:]), _bits(b))

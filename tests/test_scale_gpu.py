"""Forward + adjoint at scale (the 1024^3 configuration: 16 Gaussian blobs,
isovalue 0.5, the count pass recomputed in the backward, and a batch of 32
grids with each dimension in U{64..160}; loss = triangle area + enclosed
volume + sum of ||CellGradient||^2).

* 1024^3 (1.07 G points, 4.3 GB field): a point's dL/dfield involves only the
  cells that contain it (their triangles' area and volume terms and their
  gradients), so on a z-slab of 66 point planes cut from the field the FP64
  autograd gradient of the slab's own loss equals the full grid's at every
  point strictly inside the slab.  The GPU adjoint of the whole grid is
  compared there, relative 1e-4 of the slab gradient's max norm.  The FP64
  reference is given the same upstream gradients as the GPU adjoint (float32
  dL/dvertices and 2 x the float32 cell gradients), so it is exactly the
  backward in FP64: at spacing 1/1023 the float32 loss's own rounding on
  nearly degenerate triangles and the float32 forward's cancellation (the
  forward is float32 by contract, bit for bit the reference's) reach
  ~2e-4 of that norm and would otherwise be what is measured, not the
  adjoint.  (The 128^3 test keeps the end-to-end FP64 comparison.)
* The 32-grid batch: every grid's forward (merged MC + CellGradient) and
  adjoint enqueued as one sequence, captured in one CUDA graph and replayed;
  the replay equals the eager run bit for bit, and every fourth grid's
  adjoint is checked against FP64 autograd."""
import ctypes

import numpy as np
import pytest
import torch

from tests.test_adjoint_gpu import cell_gradient_t, mc_loss

pytestmark = pytest.mark.gpu
TOL = 1e-4


def _adjoint(cont, grid, field, iso, dV, dG, scratch, out, stream=None):
    """dL/dfield from dL/dvertices and dL/dgradient: the count pass is run
    again (recompute in backward), then dax_gb300_field_adjoint."""
    from daxtoolkit_gb300 import capi
    g = grid.desc()
    s = ctypes.c_void_p(0 if stream is None else stream.cuda_stream)
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    n = scratch.numel()
    capi.call("dax_gb300_mc_count", ctypes.byref(g), p(field), iso, p(scratch), n, s)
    capi.call("dax_gb300_field_adjoint", ctypes.byref(g), p(field), iso, p(scratch), n, p(dV),
              p(dG), p(out), s)


def _axis(n, spacing, first=0, device="cuda"):
    """The grid's own float32 coordinates spacing * (first + i) (origin 0),
    widened to float64: the cell widths the forward and the adjoint use are
    differences of these, which at spacing 1/1023 differ from the exact
    widths by up to ~6e-5 relative."""
    i = torch.arange(first, first + n, dtype=torch.float32, device=device)
    return (i * torch.tensor(spacing, dtype=torch.float32, device=device)).double()


def _loss_grads(verts, conn, grad):
    """dL/dverts and dL/dgradient of area + volume + sum ||g||^2 (float32)."""
    v = verts.detach().requires_grad_(True)
    L = mc_loss(v, conn)
    (dV,) = torch.autograd.grad(L, v)
    return dV.contiguous(), (2.0 * grad).contiguous()


def _fp64_grad(cont, dims, spacing, z_first, f64, iso, upstream=False):
    """FP64 autograd dL/dfield of a grid's own loss (topology from the GPU
    forward on the float32 values, positions and weights in float64).

    upstream=True: the loss is the linear functional sum(dV . v) +
    sum(dG . g) with dV, dG the float32 upstream gradients the GPU adjoint
    receives (dL/dvertices of area + volume by float32 autograd on the
    float32 forward, and 2 x its float32 cell gradients), so the FP64
    gradient is exactly J^T dV + G^T dG: the backward in FP64, free of the
    float32 forward's and loss's own rounding."""
    grid = cont.UniformGrid(dims, spacing=spacing, extent_min=(0, 0, z_first))
    out = cont.marching_cubes(grid, f64.float().contiguous(), iso, merge=True, records=True)
    a, b = out["rec_first"].long(), out["rec_second"].long()
    nx, ny, nz = dims
    ft = f64.clone().requires_grad_(True)
    # the slab's planes at their place in the full grid, in its float32 coordinates
    cs = [_axis(dims[0], spacing[0]), _axis(dims[1], spacing[1]),
          _axis(dims[2], spacing[2], first=z_first)]

    def xyz(p):
        return torch.stack([cs[0][p % nx], cs[1][(p // nx) % ny], cs[2][p // (nx * ny)]], dim=1)

    w = (iso - ft[a]) / (ft[b] - ft[a])
    ca, cb = xyz(a), xyz(b)
    verts = ca + w[:, None] * (cb - ca)
    widths = [c[1:] - c[:-1] for c in cs]
    g = cell_gradient_t(ft.reshape(nz, ny, nx), widths)
    if upstream:
        conn = out["conn"].long()
        dV, _ = _loss_grads(out["verts"], conn, torch.zeros(1, device=f64.device))
        dG = 2.0 * cont.cell_gradient(grid, f64.float().contiguous())
        L = (dV.double() * verts).sum() + (dG.double().view(g.shape) * g).sum()
    else:
        L = mc_loss(verts, out["conn"]) + (g * g).sum()
    L.backward()
    return ft.grad


def test_forward_adjoint_1024(gb300):
    from daxtoolkit_gb300 import capi, synthetic
    cont = gb300
    n = 1024
    dims = (n, n, n)
    spacing = (1.0 / (n - 1),) * 3
    iso = 0.5
    dev = torch.device("cuda")
    field = synthetic.blob_field(dims, 16, seed=20260105, device=dev)
    grid = cont.UniformGrid(dims, spacing=spacing)
    out = cont.marching_cubes(grid, field, iso, merge=True)
    grad = cont.cell_gradient(grid, field)
    assert out["conn"].shape[0] > 1_000_000
    dV, dG = _loss_grads(out["verts"], out["conn"].long(), grad)
    del grad
    nb = capi.lib().dax_gb300_mc_scratch_bytes(ctypes.byref(grid.desc()))
    scratch = torch.empty(nb, dtype=torch.uint8, device=dev)
    dfield = torch.empty_like(field)
    _adjoint(cont, grid, field, iso, dV, dG, scratch, dfield)
    torch.cuda.synchronize()
    del dV, dG, scratch
    assert bool(torch.isfinite(dfield).all())
    f3 = field.view(n, n, n)
    g3 = dfield.view(n, n, n)
    checked = 0
    for k0 in (300, 700):  # two slabs through the blobs
        sub = f3[k0:k0 + 66].double().contiguous().view(-1)
        ref = _fp64_grad(cont, (n, n, 66), spacing, k0, sub, iso, upstream=True).view(66, n, n)
        inner_ref = ref[1:65]
        inner_gpu = g3[k0 + 1:k0 + 65].double()
        scale = inner_ref.abs().max().item()
        err = (inner_gpu - inner_ref).abs().max().item()
        assert scale > 0 and err <= TOL * scale, (k0, err, scale)
        checked += 1
    assert checked == 2


def test_batch32_forward_adjoint_graph(gb300):
    from daxtoolkit_gb300 import capi, synthetic
    cont = gb300
    dev = torch.device("cuda")
    dims = synthetic.batch_grid_dims(32, 64, 160, 1024)
    isos = synthetic.batch_isovalues(32, 0.3, 0.6, 1024)
    items = []
    for q, (d, iso) in enumerate(zip(dims, isos)):
        grid = cont.UniformGrid(d, spacing=tuple(1.0 / (x - 1) for x in d))
        f = synthetic.blob_field(d, 16, seed=3000 + q, device=dev)
        out = cont.marching_cubes(grid, f, iso, merge=True)
        nb = capi.lib().dax_gb300_mc_scratch_bytes(ctypes.byref(grid.desc()))
        items.append(dict(grid=grid, f=f, iso=iso, T=out["conn"].shape[0], V=out["verts"].shape[0],
                          scratch=torch.empty(nb, dtype=torch.uint8, device=dev),
                          verts=torch.empty_like(out["verts"]), conn=torch.empty_like(out["conn"]),
                          grad=torch.empty((grid.GetNumberOfCells(), 3), device=dev),
                          dV=torch.empty_like(out["verts"]),
                          dfield=torch.empty_like(f)))
    p = lambda t: ctypes.c_void_p(t.data_ptr())

    def pipeline(stream):
        """Every grid's forward and adjoint, enqueued on `stream`, no host sync."""
        s = ctypes.c_void_p(stream.cuda_stream)
        for it in items:
            g = it["grid"].desc()
            nb = it["scratch"].numel()
            capi.call("dax_gb300_mc_count", ctypes.byref(g), p(it["f"]), it["iso"], p(it["scratch"]),
                      nb, s)
            capi.call("dax_gb300_mc_generate", ctypes.byref(g), p(it["f"]), it["iso"], 1,
                      p(it["scratch"]), nb, p(it["verts"]), it["V"], p(it["conn"]), it["T"], None,
                      None, None, s)
            capi.call("dax_gb300_cell_gradient", ctypes.byref(g), p(it["f"]), p(it["grad"]), s)
            # dL/dverts = a fixed smooth weight per vertex, dL/dgrad = 2 g
            with torch.cuda.stream(stream):
                torch.mul(it["verts"], 2.0, out=it["dV"])
                torch.mul(it["grad"], 2.0, out=it["grad"])
            capi.call("dax_gb300_mc_count", ctypes.byref(g), p(it["f"]), it["iso"], p(it["scratch"]),
                      nb, s)
            capi.call("dax_gb300_field_adjoint", ctypes.byref(g), p(it["f"]), it["iso"],
                      p(it["scratch"]), nb, p(it["dV"]), p(it["grad"]), p(it["dfield"]), s)

    stream = torch.cuda.Stream()
    stream.wait_stream(torch.cuda.current_stream())
    pipeline(stream)
    torch.cuda.synchronize()
    eager = [(it["verts"].clone(), it["conn"].clone(), it["dfield"].clone()) for it in items]
    for it in items:
        it["dfield"].zero_()
        it["verts"].zero_()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=stream):
        pipeline(stream)
    graph.replay()
    torch.cuda.synchronize()
    for it, (v, c, df) in zip(items, eager):
        assert torch.equal(it["verts"], v) and torch.equal(it["conn"], c)
        assert torch.equal(it["dfield"].view(torch.int32), df.view(torch.int32))
        for t in (it["scratch"],):  # the totals of the replayed pipeline
            T, V = ctypes.c_int64(0), ctypes.c_int64(0)
            capi.call("dax_gb300_mc_totals", p(t), ctypes.byref(T), ctypes.byref(V), None)
            assert (T.value, V.value) == (it["T"], it["V"])
    # the adjoint of the loss sum(|v|^2) + sum(|g|^2) against FP64 autograd
    for it in items[::4]:
        d = it["grid"].dims
        nx, ny, nz = d
        sp = it["grid"].Spacing
        f64 = it["f"].double().clone().requires_grad_(True)
        out = cont.marching_cubes(it["grid"], it["f"], it["iso"], merge=True, records=True)
        a, b = out["rec_first"].long(), out["rec_second"].long()
        cs = [_axis(n_, s_) for n_, s_ in zip(d, sp)]
        xyz = lambda q: torch.stack([cs[0][q % nx], cs[1][(q // nx) % ny], cs[2][q // (nx * ny)]], 1)
        w = (it["iso"] - f64[a]) / (f64[b] - f64[a])
        verts = xyz(a) + w[:, None] * (xyz(b) - xyz(a))
        g = cell_gradient_t(f64.reshape(nz, ny, nx), [c[1:] - c[:-1] for c in cs])
        ((verts * verts).sum() + (g * g).sum()).backward()
        ref = f64.grad
        scale = ref.abs().max().item()
        err = (it["dfield"].double() - ref).abs().max().item()
        assert err <= TOL * scale, (d, err, scale)


def test_batch32_grid_set_forward_adjoint_graph(gb300):
    """The same 32-grid workload through the grid-set launches: count,
    generate, CellGradient, the count pass again (recompute in backward) and
    the field adjoint of every grid, one launch per pass for all grids,
    captured in one CUDA graph.  Every grid's slice equals the single-grid
    entry points bit for bit (which the test above checks against FP64)."""
    from daxtoolkit_gb300 import capi, synthetic
    cont = gb300
    dev = torch.device("cuda")
    dims = synthetic.batch_grid_dims(32, 64, 160, 1024)
    isos = synthetic.batch_isovalues(32, 0.3, 0.6, 1024)
    grids, fields = [], []
    for q, d in enumerate(dims):
        grids.append(cont.UniformGrid(d, spacing=tuple(1.0 / (x - 1) for x in d)))
        fields.append(synthetic.blob_field(d, 16, seed=3000 + q, device=dev))
    batch = cont.MarchingCubesBatch(grids, fields, isos)
    verts, conn, toff, voff = batch.run(merge=True)
    C, P = batch.sizes()
    grad = torch.empty((C, 3), dtype=torch.float32, device=dev)
    dV = torch.empty_like(verts)
    dfield = torch.empty(P, dtype=torch.float32, device=dev)

    def pipeline(stream):
        batch.count(stream)
        batch.generate(verts, conn, True, stream)
        batch.cell_gradient(grad, stream)
        with torch.cuda.stream(stream):
            torch.mul(verts, 2.0, out=dV)
            torch.mul(grad, 2.0, out=grad)
        batch.count(stream)
        batch.field_adjoint(dV, grad, dfield, stream)

    stream = torch.cuda.Stream()
    stream.wait_stream(torch.cuda.current_stream())
    pipeline(stream)
    torch.cuda.synchronize()
    eager = (verts.clone(), conn.clone(), dfield.clone())
    dfield.zero_()
    verts.zero_()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=stream):
        pipeline(stream)
    graph.replay()
    torch.cuda.synchronize()
    assert torch.equal(verts, eager[0]) and torch.equal(conn, eager[1])
    assert torch.equal(dfield.view(torch.int32), eager[2].view(torch.int32))
    # grid by grid against the single-grid entry points
    c0 = p0 = 0
    for q, (gr, f, iso) in enumerate(zip(grids, fields, isos)):
        nc, npts = gr.GetNumberOfCells(), gr.GetNumberOfPoints()
        g1 = cont.cell_gradient(gr, f)
        assert torch.equal((g1 * 2.0).view(torch.int32), grad[c0:c0 + nc].view(torch.int32)), q
        nb = capi.lib().dax_gb300_mc_scratch_bytes(ctypes.byref(gr.desc()))
        scratch = torch.empty(nb, dtype=torch.uint8, device=dev)
        out1 = torch.empty_like(f)
        dV1 = dV[voff[q]:voff[q + 1]].contiguous()
        dG1 = grad[c0:c0 + nc].contiguous()
        _adjoint(cont, gr, f, iso, dV1, dG1, scratch, out1)
        torch.cuda.synchronize()
        assert torch.equal(out1.view(torch.int32), dfield[p0:p0 + npts].view(torch.int32)), q
        c0 += nc
        p0 += npts
    assert (c0, p0) == (C, P)

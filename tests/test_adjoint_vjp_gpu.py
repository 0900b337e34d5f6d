"""dax_gb300_field_adjoint as a vector-Jacobian product, term by term.

For seeded random cotangents dV (on the merged isosurface vertices) and dG
(on the cell gradients), the adjoint must equal d/df [ <verts(f), dV> +
<CellGradient(f), dG> ], computed here in float64 by torch autograd on the
CPU from the oracle's topology.  The float64 forward uses the float32
coordinates and cell widths the reference computes (origin + spacing *
(ijk + extent_min) rounded to float), so the only differences left are the
adjoint's own float32 rounding.  Each term is checked alone and combined, on
grids whose sizes are not multiples of the kernels' tiles (32 columns,
8 rows, 32 planes) and whose far origins make the widths uneven.
Tolerance: max-norm error / max-norm of the float64 result <= 2e-5.
"""
import ctypes

import numpy as np
import pytest
import torch

import oracle
from tests import cases

pytestmark = pytest.mark.gpu

TOL = 2e-5

CASES = [
    ("ragged_70x19x41_far", (70, 19, 41), (1000.0, -4.1, 250.0), (0.013, 0.7, 0.05), (-5, 2, 100),
     0.5),
    ("exact_33x9x34", (33, 9, 34), (0.0, 0.0, 0.0), (1 / 32, 1 / 8, 1 / 33), (0, 0, 0), 0.45),
    ("x130_words_96x5x3", (130, 5, 3), (-2.0, 0.0, 1.0), (0.1, 0.2, 0.3), (0, 0, 0), 0.4),
]


def _f32_axis(o, s, m, n):
    """Reference coordinates along one axis: float(o) + float(s) * float(i + m)."""
    idx = (np.arange(n) + m).astype(np.float32)
    return (np.float32(o) + np.float32(s) * idx).astype(np.float32).astype(np.float64)


def fp64_vjp(f, dims, origin, spacing, emin, iso, rec_a, rec_b, dV, dG, use_v, use_g):
    nx, ny, nz = dims
    ft = torch.tensor(f.astype(np.float64), requires_grad=True)
    ax = [torch.from_numpy(_f32_axis(origin[a], spacing[a], emin[a], dims[a])) for a in range(3)]
    total = torch.zeros((), dtype=torch.float64)
    if use_v and len(rec_a):
        a = torch.from_numpy(rec_a.astype(np.int64))
        b = torch.from_numpy(rec_b.astype(np.int64))

        def xyz(p):
            return torch.stack([ax[0][p % nx], ax[1][(p // nx) % ny], ax[2][p // (nx * ny)]], dim=1)

        ca, cb = xyz(a), xyz(b)
        w = (iso - ft[a]) / (ft[b] - ft[a])
        verts = ca + w[:, None] * (cb - ca)
        total = total + (verts * torch.from_numpy(dV.astype(np.float64))).sum()
    if use_g:
        f3 = ft.reshape(nz, ny, nx)
        v = [f3[:-1, :-1, :-1], f3[:-1, :-1, 1:], f3[:-1, 1:, 1:], f3[:-1, 1:, :-1],
             f3[1:, :-1, :-1], f3[1:, :-1, 1:], f3[1:, 1:, 1:], f3[1:, 1:, :-1]]
        sx = [-1, 1, 1, -1, -1, 1, 1, -1]
        sy = [-1, -1, 1, 1, -1, -1, 1, 1]
        sz = [-1, -1, -1, -1, 1, 1, 1, 1]
        wx, wy, wz = (t[1:] - t[:-1] for t in ax)
        gx = sum(0.25 * s * t for s, t in zip(sx, v)) / wx[None, None, :]
        gy = sum(0.25 * s * t for s, t in zip(sy, v)) / wy[None, :, None]
        gz = sum(0.25 * s * t for s, t in zip(sz, v)) / wz[:, None, None]
        g = torch.stack([gx, gy, gz], dim=-1).reshape(-1, 3)
        total = total + (g * torch.from_numpy(dG.astype(np.float64))).sum()
    total.backward()
    return ft.grad.numpy() if ft.grad is not None else np.zeros(f.shape, np.float64)


def gpu_adjoint(cont, grid, fd, iso, dV, dG):
    from daxtoolkit_gb300 import capi
    g = grid.desc()
    L = capi.lib()
    n = L.dax_gb300_mc_scratch_bytes(ctypes.byref(g))
    scratch = torch.empty(n, dtype=torch.uint8, device=fd.device)
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    p = lambda t: None if t is None else ctypes.c_void_p(t.data_ptr())
    capi.call("dax_gb300_mc_count", ctypes.byref(g), p(fd), iso, p(scratch), n, s)
    out = torch.full_like(fd, float("nan"))  # every point must be written
    capi.call("dax_gb300_field_adjoint", ctypes.byref(g), p(fd), iso, p(scratch), n, p(dV), p(dG),
              p(out), s)
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.fixture(scope="module", params=CASES, ids=lambda c: c[0])
def vjp_case(request, gb300):
    name, dims, origin, spacing, emin, iso = request.param
    cont = gb300
    f = cases.random_blobs(dims, 4, 31, noise=0.1)
    grid = cont.UniformGrid(dims, origin=origin, spacing=spacing, extent_min=emin)
    fd = torch.from_numpy(f).cuda()
    out = cont.marching_cubes(grid, fd, iso, merge=True)
    V = out["verts"].shape[0]
    C = grid.GetNumberOfCells()
    rng = np.random.default_rng(7)
    dV = rng.standard_normal((V, 3)).astype(np.float32)
    dG = rng.standard_normal((C, 3)).astype(np.float32)
    og = oracle.make_grid(dims, origin=origin, spacing=spacing, extent_min=emin)
    O = oracle.Oracle("port")
    count, _ = O.mc_count(og, f, iso)
    ref = O.mc_generate(og, f, iso, count, merge=True)
    assert len(ref["rec_a"]) == V
    return dict(cont=cont, grid=grid, fd=fd, f=f, dims=dims, origin=origin, spacing=spacing,
                emin=emin, iso=iso, dV=dV, dG=dG, ref=ref)


@pytest.mark.parametrize("terms", ["vertices", "gradient", "both"])
def test_adjoint_vjp(vjp_case, terms):
    c = vjp_case
    use_v, use_g = terms in ("vertices", "both"), terms in ("gradient", "both")
    dV = torch.from_numpy(c["dV"]).cuda() if use_v else None
    dG = torch.from_numpy(c["dG"]).cuda() if use_g else None
    got = gpu_adjoint(c["cont"], c["grid"], c["fd"], c["iso"], dV, dG)
    want = fp64_vjp(c["f"], c["dims"], c["origin"], c["spacing"], c["emin"], c["iso"],
                    c["ref"]["rec_a"], c["ref"]["rec_b"], c["dV"], c["dG"], use_v, use_g)
    assert np.isfinite(got).all()
    scale = np.abs(want).max()
    assert scale > 0
    err = np.abs(got.astype(np.float64) - want).max() / scale
    assert err <= TOL, (terms, err)
    if use_v and not use_g:  # points off the surface get exactly zero
        assert np.array_equal(got == 0, want == 0)


def test_adjoint_deterministic(vjp_case):
    c = vjp_case
    dV = torch.from_numpy(c["dV"]).cuda()
    dG = torch.from_numpy(c["dG"]).cuda()
    a = gpu_adjoint(c["cont"], c["grid"], c["fd"], c["iso"], dV, dG)
    b = gpu_adjoint(c["cont"], c["grid"], c["fd"], c["iso"], dV, dG)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))

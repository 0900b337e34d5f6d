"""Differentiable isosurface + CellGradient: the adjoint kernels against FP64.

Loss (float32 on the GPU): total triangle area + enclosed volume (divergence
form, sum of v0 . (v1 x v2) / 6) + sum over cells of ||CellGradient||^2, on a
merged isosurface of a seeded 8-blob field.  The GPU's dL/dfield is checked
  * against an FP64 host gradient: the same forward written in torch float64
    on the CPU (fixed topology from the oracle) and differentiated by torch
    autograd -- independent of the hand-written adjoint formulas;
  * against FP64 central differences (step 1e-4, Richardson-extrapolated with
    a second step of 5e-5 to remove the O(h^2) truncation term, which is
    large on edges whose two end values are both close to the isovalue) on a
    32^3 sub-grid, each perturbation chosen to keep every case index
    unchanged (|f - iso| > 2e-4).
Tolerance: relative 1e-4, measured in both tests as the max-norm of the
error over the max-norm of the FP64 gradient on the full grid.  (The forward
CellGradient is float32 by contract -- it reproduces the reference's float
arithmetic bit for bit -- and its rounding, ~1e-5 of that norm, is what the
FP64 references see; a per-sample normalisation would measure the forward's
float32 rounding, not the adjoint.)
"""
import ctypes

import numpy as np
import pytest
import torch

import oracle
from tests import cases

pytestmark = pytest.mark.gpu

H = 1e-4
TOL = 1e-4


class IsoSurfaceWithGradient(torch.autograd.Function):
    """Test-harness wrapper: forward = merged marching cubes + CellGradient,
    backward = dax_gb300_field_adjoint (the count pass is recomputed)."""

    @staticmethod
    def forward(ctx, field, grid, iso, cont):
        out = cont.marching_cubes(grid, field, iso, merge=True)
        grad = cont.cell_gradient(grid, field)
        ctx.save_for_backward(field)
        ctx.grid, ctx.iso, ctx.cont = grid, iso, cont
        ctx.mark_non_differentiable(out["conn"])
        return out["verts"], out["conn"], grad

    @staticmethod
    def backward(ctx, gv, gc, gg):
        from daxtoolkit_gb300 import capi
        (field,) = ctx.saved_tensors
        g = ctx.grid.desc()
        L = capi.lib()
        n = L.dax_gb300_mc_scratch_bytes(ctypes.byref(g))
        scratch = torch.empty(n, dtype=torch.uint8, device=field.device)
        s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        p = lambda t: None if t is None else ctypes.c_void_p(t.contiguous().data_ptr())
        capi.call("dax_gb300_mc_count", ctypes.byref(g), p(field), ctx.iso, p(scratch), n, s)
        out = torch.empty_like(field)
        gv = None if gv is None else gv.contiguous()
        gg = None if gg is None else gg.contiguous()
        capi.call("dax_gb300_field_adjoint", ctypes.byref(g), p(field), ctx.iso, p(scratch), n,
                  p(gv), p(gg), p(out), s)
        return out, None, None, None


def mc_loss(verts, conn):
    v0, v1, v2 = verts[conn[:, 0].long()], verts[conn[:, 1].long()], verts[conn[:, 2].long()]
    area = 0.5 * torch.linalg.norm(torch.cross(v1 - v0, v2 - v0, dim=1), dim=1).sum()
    vol = (v0 * torch.cross(v1, v2, dim=1)).sum() / 6.0
    return area + vol


def grad_loss(g):
    return (g * g).sum()


def cell_gradient_t(f3, spacing_axes):
    """CellGradient in torch (any dtype), f3 indexed [k, j, i]."""
    v = [f3[:-1, :-1, :-1], f3[:-1, :-1, 1:], f3[:-1, 1:, 1:], f3[:-1, 1:, :-1],
         f3[1:, :-1, :-1], f3[1:, :-1, 1:], f3[1:, 1:, 1:], f3[1:, 1:, :-1]]
    sx = [-1, 1, 1, -1, -1, 1, 1, -1]
    sy = [-1, -1, 1, 1, -1, -1, 1, 1]
    sz = [-1, -1, -1, -1, 1, 1, 1, 1]
    gx = sum(0.25 * s * t for s, t in zip(sx, v))
    gy = sum(0.25 * s * t for s, t in zip(sy, v))
    gz = sum(0.25 * s * t for s, t in zip(sz, v))
    wx, wy, wz = spacing_axes
    return torch.stack([gx / wx[None, None, :], gy / wy[None, :, None], gz / wz[:, None, None]],
                       dim=-1)


def fp64_loss_and_grad(f, dims, spacing, iso, rec_a, rec_b, conn):
    nx, ny, nz = dims
    ft = torch.tensor(f, dtype=torch.float64, requires_grad=True)
    a = torch.from_numpy(rec_a.astype(np.int64))
    b = torch.from_numpy(rec_b.astype(np.int64))
    coords = [torch.arange(d, dtype=torch.float64) * s for d, s in zip(dims, spacing)]

    def xyz(p):
        return torch.stack([coords[0][p % nx], coords[1][(p // nx) % ny], coords[2][p // (nx * ny)]],
                           dim=1)

    ca, cb = xyz(a), xyz(b)
    fa, fb = ft[a], ft[b]
    w = (iso - fa) / (fb - fa)
    verts = ca + w[:, None] * (cb - ca)
    widths = [c[1:] - c[:-1] for c in coords]
    g = cell_gradient_t(ft.reshape(nz, ny, nx), widths)
    L = mc_loss(verts, torch.from_numpy(conn)) + grad_loss(g)
    L.backward()
    return L.item(), ft.grad.numpy()


@pytest.fixture(scope="module")
def setup(gb300):
    cont = gb300
    n = 128
    dims = (n, n, n)
    spacing = (1.0 / (n - 1),) * 3
    f = cases.random_blobs(dims, 8, 2024)
    iso = 0.5
    grid = cont.UniformGrid(dims, spacing=spacing)
    fd = torch.from_numpy(f).cuda().requires_grad_(True)
    verts, conn, grad = IsoSurfaceWithGradient.apply(fd, grid, iso, cont)
    loss = mc_loss(verts, conn) + grad_loss(grad)
    loss.backward()
    og = oracle.make_grid(dims, spacing=spacing)
    O = oracle.Oracle("port")
    count, _ = O.mc_count(og, f, iso)
    ref = O.mc_generate(og, f, iso, count, merge=True)
    L64, g64 = fp64_loss_and_grad(f, dims, spacing, iso, ref["rec_a"], ref["rec_b"], ref["conn"])
    return dict(cont=cont, dims=dims, spacing=spacing, f=f, iso=iso, loss=loss.item(),
                gpu_grad=fd.grad.cpu().numpy(), ref=ref, L64=L64, g64=g64,
                scale=np.abs(g64).max())


def test_adjoint_matches_fp64_autograd(setup):
    s = setup
    assert abs(s["loss"] - s["L64"]) <= 1e-4 * abs(s["L64"])
    err = np.abs(s["gpu_grad"].astype(np.float64) - s["g64"]).max() / s["scale"]
    assert err <= TOL, err


def test_adjoint_matches_central_differences(setup):
    """FP64 central differences of the same loss on a 32^3 sub-grid."""
    s = setup
    f = s["f"].astype(np.float64)
    nx, ny, nz = s["dims"]
    sp = s["spacing"][0]
    iso = s["iso"]
    ra, rb = s["ref"]["rec_a"].astype(np.int64), s["ref"]["rec_b"].astype(np.int64)
    conn = s["ref"]["conn"].astype(np.int64)
    # vertex -> triangles, point -> vertices
    tri_of_v = {}
    for t, tri in enumerate(conn):
        for v in tri:
            tri_of_v.setdefault(int(v), []).append(t)
    verts_of_p = {}
    for v, (a, b) in enumerate(zip(ra, rb)):
        verts_of_p.setdefault(int(a), []).append(v)
        verts_of_p.setdefault(int(b), []).append(v)

    def xyz(p):
        return np.array([p % nx, (p // nx) % ny, p // (nx * ny)], np.float64) * sp

    def vertex(v, ff):
        a, b = ra[v], rb[v]
        w = (iso - ff(a)) / (ff(b) - ff(a))
        ca, cb = xyz(a), xyz(b)
        return ca + w * (cb - ca)

    def tri_terms(tris, ff):
        tot = 0.0
        for t in tris:
            v0, v1, v2 = (vertex(int(v), ff) for v in conn[t])
            tot += 0.5 * np.linalg.norm(np.cross(v1 - v0, v2 - v0)) + v0 @ np.cross(v1, v2) / 6.0
        return tot

    def cell_terms(p, ff):
        i, j, k = p % nx, (p // nx) % ny, p // (nx * ny)
        tot = 0.0
        for kc in (k - 1, k):
            for jc in (j - 1, j):
                for ic in (i - 1, i):
                    if min(ic, jc, kc) < 0 or ic >= nx - 1 or jc >= ny - 1 or kc >= nz - 1:
                        continue
                    q = ic + nx * (jc + ny * kc)
                    v = [ff(q), ff(q + 1), ff(q + nx + 1), ff(q + nx),
                         ff(q + nx * ny), ff(q + nx * ny + 1), ff(q + nx * ny + nx + 1),
                         ff(q + nx * ny + nx)]
                    gx = 0.25 * (-v[0] + v[1] + v[2] - v[3] - v[4] + v[5] + v[6] - v[7]) / sp
                    gy = 0.25 * (-v[0] - v[1] + v[2] + v[3] - v[4] - v[5] + v[6] + v[7]) / sp
                    gz = 0.25 * (-v[0] - v[1] - v[2] - v[3] + v[4] + v[5] + v[6] + v[7]) / sp
                    tot += gx * gx + gy * gy + gz * gz
        return tot

    lo = (48, 48, 48)  # 32^3 sub-grid crossing the blob surfaces
    pts = [i + nx * (j + ny * k) for k in range(lo[2], lo[2] + 32) for j in range(lo[1], lo[1] + 32)
           for i in range(lo[0], lo[0] + 32)]
    rng = np.random.default_rng(3)
    surf = [p for p in pts if p in verts_of_p]
    other = [p for p in pts if p not in verts_of_p]
    sample = surf[:600] + list(rng.choice(other, size=min(200, len(other)), replace=False))
    assert len(surf) > 50
    fd_vals, gpu_vals = [], []
    for p in sample:
        if abs(f[p] - iso) <= 2 * H:
            continue
        tris = sorted({t for v in verts_of_p.get(p, []) for t in tri_of_v.get(v, [])})

        def central(h, p=p, tris=tris):
            def ff_plus(q):
                return f[q] + (h if q == p else 0.0)

            def ff_minus(q):
                return f[q] - (h if q == p else 0.0)

            lp = tri_terms(tris, ff_plus) + cell_terms(p, ff_plus)
            lm = tri_terms(tris, ff_minus) + cell_terms(p, ff_minus)
            return (lp - lm) / (2 * h)

        fd_vals.append((4.0 * central(H / 2) - central(H)) / 3.0)
        gpu_vals.append(float(s["gpu_grad"][p]))
    fd_vals, gpu_vals = np.array(fd_vals), np.array(gpu_vals)
    err = np.abs(fd_vals - gpu_vals).max() / s["scale"]
    assert err <= TOL, err
    # the finite differences also agree with the FP64 autograd gradient
    idx = [p for p in sample if abs(f[p] - iso) > 2 * H]
    assert np.abs(fd_vals - s["g64"][idx]).max() <= 1e-6 * s["scale"]


def test_adjoint_deterministic(setup):
    """Two backward passes give bit-identical gradients (no atomics)."""
    s = setup
    cont = s["cont"]
    grid = cont.UniformGrid(s["dims"], spacing=s["spacing"])
    outs = []
    for _ in range(2):
        fd = torch.from_numpy(s["f"]).cuda().requires_grad_(True)
        v, c, g = IsoSurfaceWithGradient.apply(fd, grid, s["iso"], cont)
        (mc_loss(v, c) + grad_loss(g)).backward()
        outs.append(fd.grad.cpu().numpy().view(np.uint32))
    assert np.array_equal(outs[0], outs[1])

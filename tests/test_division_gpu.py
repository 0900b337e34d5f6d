"""The reciprocal-based divisions of the stencil kernels (Markstein's
correction step on a correctly rounded reciprocal: div_by_recip with its
range checks, and div_fast on its narrower domain) against CUDA's correctly
rounded division, exhaustively over all 2^32 numerator bit patterns, for
every divisor a gradient launch uses on the bench grid and the gradient test
grids: the differences of neighbouring implicit coordinates along each axis."""
import ctypes

import numpy as np
import pytest
import torch

from tests import cases

pytestmark = pytest.mark.gpu


def _axis_steps(n, origin, spacing, emin):
    f32 = np.float32
    c = f32(origin) + f32(spacing) * (np.arange(n) + emin).astype(f32)
    return (c[1:] - c[:-1]).astype(f32)


def _divisors():
    grids = [((512, 512, 512), (0, 0, 0), (1 / 511,) * 3, (0, 0, 0))]
    grids += [(d, o, s, e) for _, d, o, s, e, _ in cases.gradient_cases()]
    steps = set()
    for dims, origin, spacing, emin in grids:
        for a in range(3):
            if dims[a] > 1:
                w = _axis_steps(dims[a], origin[a], spacing[a], emin[a])
                steps.update(w.view(np.uint32).tolist())
    # plus divisors near the band limits and of every binade's extremes
    extra = [2.0 ** -89, 2.0 ** 89, 1.0, 1.5, 1.9999999, 3.0, 0.1, 1 / 3, 7e-20, 3e19,
             2.0 ** -30, -(2.0 ** -30), np.nextafter(np.float32(2.0 ** 30), np.float32(0)),
             0.75 * 2.0 ** 30, -1.75e-9]
    steps.update(np.asarray(extra, np.float32).view(np.uint32).tolist())
    return np.array(sorted(steps), np.uint32).view(np.float32)


def _check(divisors, first, count, step):
    from daxtoolkit_gb300 import capi
    dev = torch.from_numpy(np.ascontiguousarray(divisors, np.float32)).cuda()
    mism = torch.zeros(1, dtype=torch.int64, device="cuda")
    for b in range(0, dev.numel(), 8):
        part = dev[b:b + 8]
        capi.call("dax_gb300_selfcheck_division", ctypes.c_void_p(part.data_ptr()), part.numel(),
                  first, count, step, ctypes.c_void_p(mism.data_ptr()), None)
    torch.cuda.synchronize()
    return int(mism.item())


def _bits(x):
    return int(np.float32(x).view(np.uint32))


def test_division_exhaustive_for_every_grid_divisor(gb300):
    """Every one of the 2^32 numerator bit patterns for every divisor of the
    bench grid and the gradient test grids, and for divisors at the edges of
    the reciprocal path's band."""
    d = _divisors()
    assert 20 < d.size < 600
    assert _check(d, 0, 1 << 32, 1) == 0


def test_division_sampled_for_every_grid_divisor(gb300):
    """2^28 numerators spread over all bit patterns (odd stride) for every
    divisor of the bench grid and the gradient test grids."""
    d = _divisors()
    assert 20 < d.size < 600
    assert _check(d, 0, 1 << 28, 0x9E3779B1) == 0

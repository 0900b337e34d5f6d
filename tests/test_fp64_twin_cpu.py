"""The FP64 twin of the reference (its worklets built with
DAX_USE_DOUBLE_PRECISION) against the float32 reference on the CPU: the
same topology, and every float32 weight, position and cell gradient within
the float32 rounding bounds of oracle/fp64_error.py.  The GPU results equal
the float32 reference bit for bit, so these bounds hold for them too
(tests/test_fp64_error_gpu.py checks them on the GPU at full size)."""
import numpy as np
import pytest

from tests import cases


@pytest.fixture(scope="module")
def oracles():
    import oracle
    try:
        return oracle.Oracle("reference"), oracle.Fp64Twin()
    except RuntimeError as e:
        pytest.skip(str(e))


FINITE = [c for c in cases.mc_cases() if np.isfinite(c[5]).all()]


@pytest.mark.parametrize("case", FINITE, ids=lambda c: c[0])
def test_twin_marching_cubes_within_bounds(oracles, case):
    import oracle
    from oracle import fp64_error
    R, tw = oracles
    name, dims, origin, spacing, emin, f, iso = case
    g = oracle.make_grid(dims, origin, spacing, emin)
    count, _ = R.mc_count(g, f, iso)
    r32 = R.mc_generate(g, f, iso, count, merge=True)
    r64 = tw.mc_generate(g, f, iso, merge=True)
    assert np.array_equal(r32["conn"], r64["conn"])
    assert np.array_equal(r32["rec_a"], r64["rec_a"]) and np.array_equal(r32["rec_b"], r64["rec_b"])
    if r32["verts"].shape[0] == 0:
        return
    st = fp64_error.mc_error_stats(r32["verts"], r32["rec_w"], r64, origin, spacing, emin, dims)
    assert st["weight_err_over_bound_max"] <= 1.0, st
    assert st["pos_err_max_spacings"] <= st["pos_bound_spacings"], st


@pytest.mark.parametrize("case", FINITE, ids=lambda c: c[0])
def test_twin_cell_gradient_within_bounds(oracles, case):
    import oracle
    from oracle import fp64_error
    R, tw = oracles
    name, dims, origin, spacing, emin, f, iso = case
    if min(dims) < 2:
        return
    g = oracle.make_grid(dims, origin, spacing, emin)
    st = fp64_error.gradient_error_stats(R.cell_gradient(g, f), tw.cell_gradient(g, f), f, origin,
                                         spacing, emin, dims)
    assert st["err_over_bound_max"] <= 1.0, st


def test_twin_blob_field_128(oracles):
    """The 8-blob benchmark field at 128^3: positions within a few 1e-6 of a
    spacing of double, gradients within the bound."""
    import oracle
    from daxtoolkit_gb300 import synthetic
    from oracle import fp64_error
    R, tw = oracles
    n = 128
    dims, spacing = (n, n, n), (1.0 / (n - 1),) * 3
    f = synthetic.blob_field(dims, 8, seed=20260101).numpy()
    g = oracle.make_grid(dims, spacing=spacing)
    count, _ = R.mc_count(g, f, 0.5)
    r32 = R.mc_generate(g, f, 0.5, count, merge=True)
    st = fp64_error.mc_error_stats(r32["verts"], r32["rec_w"], tw.mc_generate(g, f, 0.5), (0, 0, 0),
                                   spacing, (0, 0, 0), dims)
    # float32 positions do differ from double, within the bound
    assert 0 < st["pos_err_max_spacings"] <= st["pos_bound_spacings"] < 1e-4
    gs = fp64_error.gradient_error_stats(R.cell_gradient(g, f), tw.cell_gradient(g, f), f,
                                         (0, 0, 0), spacing, (0, 0, 0), dims)
    assert gs["err_over_bound_max"] <= 1.0

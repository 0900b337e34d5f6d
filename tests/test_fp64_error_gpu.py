"""Error of the float32 results against the FP64 twin of the reference (its
own worklets built with DAX_USE_DOUBLE_PRECISION, on the same float32 field
and grid description), on the benchmark workloads: the sphere at 64^3
(iso 0.35) and the 8-blob field at 256^3 and 512^3 (iso 0.5).  The results
themselves are bit-identical to the float32 reference; these tests state
how far that float32 arithmetic lies from double, and check it against the
float32 rounding bounds of oracle/fp64_error.py:
* every weight within 3.01 u |w| of the FP64 weight (u = 2^-24);
* every vertex within the position bound (a few u of the coordinates'
  magnitude, in spacings);
* every cell gradient within 8 u sum|0.25 f| / width + (width error + 2u)|g|.
The measured figures are printed (pytest -s); bench.py reports the same
statement for the whole 512^3 field as its fp64_error entry."""
import json

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def twin():
    import oracle
    try:
        return oracle.Fp64Twin()
    except RuntimeError as e:
        pytest.skip(str(e))


def _workloads():
    return [("sphere64", 64), ("blobs256", 256), ("blobs512", 512)]


def _field(name, n):
    from daxtoolkit_gb300 import synthetic
    if name.startswith("sphere"):
        return synthetic.sphere_field((n, n, n), noise=0.01, seed=1234).numpy(), 0.35
    return synthetic.blob_field((n, n, n), 8, seed=20260101, device="cuda").cpu().numpy(), 0.5


@pytest.mark.parametrize("name,n", _workloads(), ids=[w[0] for w in _workloads()])
def test_fp64_error_marching_cubes(gb300, twin, name, n):
    import oracle
    from oracle import fp64_error
    cont = gb300
    dims, spacing = (n, n, n), (1.0 / (n - 1),) * 3
    fh, iso = _field(name, n)
    out = cont.marching_cubes(cont.UniformGrid(dims, spacing=spacing), torch.from_numpy(fh).cuda(),
                              iso, merge=True, records=True)
    r64 = twin.mc_generate(oracle.make_grid(dims, spacing=spacing), fh, iso, merge=True)
    # same case decisions in double: the same topology and output order
    assert np.array_equal(out["conn"].cpu().numpy(), r64["conn"])
    assert np.array_equal(out["rec_first"].cpu().numpy(), r64["rec_a"])
    st = fp64_error.mc_error_stats(out["verts"].cpu().numpy(), out["rec_weight"].cpu().numpy(),
                                   r64, (0, 0, 0), spacing, (0, 0, 0), dims)
    print("\nfp64 error, marching cubes,", name, json.dumps(st))
    assert st["weight_err_over_bound_max"] <= 1.0
    assert st["pos_err_max_spacings"] <= st["pos_bound_spacings"]


@pytest.mark.parametrize("name,n", _workloads(), ids=[w[0] for w in _workloads()])
def test_fp64_error_cell_gradient(gb300, twin, name, n):
    import oracle
    from oracle import fp64_error
    cont = gb300
    dims, spacing = (n, n, n), (1.0 / (n - 1),) * 3
    fh, _ = _field(name, n)
    g32 = cont.cell_gradient(cont.UniformGrid(dims, spacing=spacing),
                             torch.from_numpy(fh).cuda()).cpu().numpy()
    g64 = twin.cell_gradient(oracle.make_grid(dims, spacing=spacing), fh)
    st = fp64_error.gradient_error_stats(g32, g64, fh, (0, 0, 0), spacing, (0, 0, 0), dims)
    print("\nfp64 error, cell gradient,", name, json.dumps(st))
    assert st["err_over_bound_max"] <= 1.0

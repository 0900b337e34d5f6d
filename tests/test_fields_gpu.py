"""The reference's own marching-cubes benchmark pipeline on the GPU
(Benchmarks/MarchingCubes/Pipeline.h:100-150: Magnitude of the point
coordinates, then marching cubes at isovalue 100, points merged or not, on a
dim^3 grid of unit spacing) against the oracle, and its VTK dump from device
memory."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import vtk_writer

pytestmark = pytest.mark.gpu


def _bits(a):
    a = np.ascontiguousarray(a)
    b = a.view(np.uint32).copy()
    b[np.isnan(a)] = 0x7FC00000
    return b


@pytest.mark.parametrize("g", [((16, 12, 9), (0, 0, 0), (1, 1, 1), (0, 0, 0)),
                               ((33, 17, 5), (-1.5, 2.25, 0.125), (0.3, 0.7, 1.1), (3, -2, 7)),
                               ((128, 128, 128), (0, 0, 0), (1, 1, 1), (0, 0, 0))])
def test_point_magnitude(gb300, oracle_best, g):
    import oracle
    dims, origin, spacing, emin = g
    f = gb300.point_magnitude(gb300.UniformGrid(dims, origin, spacing, emin)).cpu().numpy()
    ref = oracle_best.point_magnitude(oracle.make_grid(dims, origin, spacing, emin))
    assert np.array_equal(_bits(f), _bits(ref))


@pytest.mark.parametrize("merge", [True, False], ids=["remove_duplicates", "plain"])
def test_reference_mc_benchmark_pipeline(gb300, oracle_best, merge, tmp_path):
    """Pipelines MARCHING_CUBES and MARCHING_CUBES_REMOVE_DUPLICATES at the
    benchmark's default size 128, then the VTK dump from device memory."""
    import oracle
    from daxtoolkit_gb300 import capi
    cont = gb300
    dim = 128
    grid = cont.UniformGrid((dim,) * 3)
    f = cont.point_magnitude(grid)
    out = cont.marching_cubes(grid, f, 100.0, merge=merge)
    g = oracle.make_grid((dim,) * 3)
    fh = f.cpu().numpy()
    count, _ = oracle_best.mc_count(g, fh, 100.0)
    ref = oracle_best.mc_generate(g, fh, 100.0, count, merge)
    assert np.array_equal(out["conn"].cpu().numpy(), ref["conn"])
    assert np.array_equal(_bits(out["verts"].cpu().numpy()), _bits(ref["verts"]))
    path = tmp_path / "MCdaxResult.vtk"
    cont.write_vtk(str(path), cont.UnstructuredGrid(out["verts"], out["conn"]))
    assert path.read_bytes() == vtk_writer.polydata_text(ref["verts"], ref["conn"])

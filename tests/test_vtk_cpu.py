"""The legacy-VTK writer (dax_gb300_write_vtk_polydata, host arrays, no GPU
needed) against the restatement of the reference's PrintContentsToStream
(Benchmarks/MarchingCubes/Pipeline.h:51-98), byte for byte; and the
Magnitude point field of the reference's MC benchmark (port vs the
reference's own functor)."""
import ctypes

import numpy as np
import pytest

import oracle
from oracle import vtk_writer


def _write(tmp_path, pts, conn, V=3):
    from daxtoolkit_gb300 import capi
    pts = np.ascontiguousarray(pts, np.float32)
    conn = np.ascontiguousarray(conn, np.int32)
    path = tmp_path / "out.vtk"
    capi.call("dax_gb300_write_vtk_polydata", str(path).encode(),
              pts.ctypes.data_as(ctypes.c_void_p), pts.shape[0],
              conn.ctypes.data_as(ctypes.c_void_p), conn.shape[0] if conn.size else 0, V)
    return path.read_bytes()


@pytest.fixture(scope="module", autouse=True)
def _lib():
    pytest.importorskip("torch")
    from daxtoolkit_gb300 import build
    build.build()


@pytest.mark.parametrize("n_pts,n_cells", [(0, 0), (1, 0), (7, 2), (9, 3), (3001, 1000)])
def test_vtk_bytes(tmp_path, n_pts, n_cells):
    rng = np.random.default_rng(n_pts)
    pts = (rng.standard_normal((n_pts, 3)) * rng.choice([1e-9, 1e-3, 1, 1e4, 1e9], (n_pts, 3)))
    pts = pts.astype(np.float32)
    conn = rng.integers(0, max(n_pts, 1), size=(n_cells, 3)).astype(np.int32)
    assert _write(tmp_path, pts, conn) == vtk_writer.polydata_text(pts, conn)


def test_vtk_special_values(tmp_path):
    pts = np.array([[0.0, -0.0, 1e-7], [123456789.0, 0.1, 1.0 / 3], [np.inf, -np.inf, 2.5e-45],
                    [100.0, 1e6, 1e-5]], np.float32)
    conn = np.array([[0, 1, 2], [3, 2, 1]], np.int32)
    assert _write(tmp_path, pts, conn) == vtk_writer.polydata_text(pts, conn)


def test_vtk_surface_of_the_reference_benchmark(tmp_path):
    """The 26^3 known-answer surface, merged, as MCdaxResult.vtk would hold it."""
    from tests import cases
    O = oracle.Oracle("port")
    g = oracle.make_grid((26, 26, 26))
    f = cases.linear_field((26, 26, 26))
    count, _ = O.mc_count(g, f, 70.0)
    out = O.mc_generate(g, f, 70.0, count, True)
    data = _write(tmp_path, out["verts"], out["conn"])
    assert data == vtk_writer.polydata_text(out["verts"], out["conn"])
    assert data.startswith(b"# vtk DataFile Version 3.0\nvtk output\nASCII\nDATASET POLYDATA\n"
                           b"POINTS 45 float\n")
    assert b"POLYGONS 61 244\n" in data and data.endswith(b"\n\n")


@pytest.mark.skipif(not oracle.build.reference_available(), reason="reference tree absent")
@pytest.mark.parametrize("g", [((16, 12, 9), (0, 0, 0), (1, 1, 1), (0, 0, 0)),
                               ((33, 17, 5), (-1.5, 2.25, 0.125), (0.3, 0.7, 1.1), (3, -2, 7))])
def test_magnitude_port_matches_reference(g):
    dims, origin, spacing, emin = g
    grid = oracle.make_grid(dims, origin, spacing, emin)
    a = oracle.Oracle("port").point_magnitude(grid)
    b = oracle.Oracle("reference").point_magnitude(grid)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def _ostream_bytes(tmp_path, pts, conn, V=3):
    """The file std::ostream writes (oracle/vtk_ostream.cpp, the reference
    benchmark's stream insertions) for the same points and cells."""
    import subprocess
    pts = np.ascontiguousarray(pts, np.float32)
    conn = np.ascontiguousarray(conn, np.int32)
    pf, cf, out = tmp_path / "p.f32", tmp_path / "c.i32", tmp_path / "ostream.vtk"
    pts.tofile(pf)
    conn.tofile(cf)
    exe = oracle.build.build_vtk_ostream()
    subprocess.check_call([exe, str(pf), str(pts.shape[0]), str(cf),
                           str(conn.shape[0] if conn.size else 0), str(V), str(out)])
    return out.read_bytes()


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_vtk_bytes_equal_std_ostream(tmp_path, seed):
    """The library's writer and the Python restatement both produce the bytes
    that the C++ standard library's operator<< writes: floats of every
    magnitude, signed zeros, infinities, NaNs of both signs, subnormals, and
    ragged counts."""
    rng = np.random.default_rng(seed)
    n_pts, n_cells = 3000 + seed, 1000 + 7 * seed
    pts = (rng.standard_normal((n_pts, 3)) *
           10.0 ** rng.integers(-40, 38, size=(n_pts, 3))).astype(np.float32)
    pts[:8] = np.array([[0.0, -0.0, np.inf], [-np.inf, 1e-45, -1e-45], [1.0, 0.1, 1.0 / 3],
                        [123456.5, 1234567.0, 999999.5], [1e-5, 1e-4, 100000.0],
                        [2.5e-38, 3.4e38, -7.0], [0.5, 65536.0, 1e6], [1e7, 1e-7, 42.0]])[:8]
    pts[8] = [np.nan, -np.nan, 0.0]
    conn = rng.integers(0, 2 ** 31 - 1, size=(n_cells, 3)).astype(np.int32)
    want = _ostream_bytes(tmp_path, pts, conn)
    assert vtk_writer.polydata_text(pts, conn) == want
    assert _write(tmp_path, pts, conn) == want


def test_vtk_benchmark_surface_equals_std_ostream(tmp_path):
    from tests import cases
    O = oracle.Oracle("port")
    g = oracle.make_grid((26, 26, 26))
    f = cases.linear_field((26, 26, 26))
    count, _ = O.mc_count(g, f, 70.0)
    out = O.mc_generate(g, f, 70.0, count, True)
    assert _write(tmp_path, out["verts"], out["conn"]) == _ostream_bytes(tmp_path, out["verts"],
                                                                          out["conn"])

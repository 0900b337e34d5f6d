"""Control-environment surface of the GB300 device adapter, in Python.

Mirrors the part of ``dax::cont`` that the uniform-grid hot path uses --
``UniformGrid`` (dax/cont/UniformGrid.h:114-252), ``DispatcherMapCell``
(dax/cont/DispatcherMapCell.h:27-64), ``DispatcherGenerateInterpolatedCells``
(dax/cont/DispatcherGenerateInterpolatedCells.h:34-301) and
``DispatcherGenerateTopology`` (dax/cont/DispatcherGenerateTopology.h:30-258)
-- with the same names, argument meaning and error types, over the C ABI in
``include/dax_gb300.h``.  Arrays are torch CUDA tensors (the ArrayHandle's
execution-side storage); torch supplies device memory and the current stream,
all arithmetic runs in libdax_gb300.so.
"""
import ctypes

import numpy as np

import torch

from . import capi

__all__ = [
    "UniformGrid", "UnstructuredGrid", "MarchingCubesCount", "MarchingCubesGenerate",
    "ThresholdCount", "ThresholdTopology", "CellGradient", "DispatcherMapCell",
    "DispatcherGenerateInterpolatedCells", "DispatcherGenerateTopology", "marching_cubes",
    "threshold", "cell_gradient", "Scratch", "SliceCount", "SliceGenerate", "slice", "slice_field",
    "MarchingTetrahedraCount", "MarchingTetrahedraGenerate", "marching_tetrahedra",
    "Tetrahedralize", "tetrahedralize", "marching_cubes_counted", "Mandlebulb",
    "MandlebulbClipCount", "MandlebulbVolume", "MandlebulbSurface", "mandlebulb_field",
    "compute_mandlebulb", "colors_and_norms", "extract_surface", "extract_cut", "point_magnitude",
    "write_vtk", "marching_cubes_pipelined",
]


def _ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _stream(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def _require_field(field, grid):
    """A field is a CUDA tensor or a page-locked CPU tensor (the kernels then
    read it over the host link through its device mapping)."""
    if not isinstance(field, torch.Tensor) or not (field.is_cuda or field.is_pinned()):
        raise capi.ErrorControlBadValue(capi.ERROR_BAD_VALUE,
                                        "field must be a CUDA tensor or a page-locked CPU tensor")
    if field.dtype != torch.float32 or not field.is_contiguous():
        raise capi.ErrorControlBadValue(capi.ERROR_BAD_VALUE, "field must be contiguous float32")
    if field.numel() != grid.GetNumberOfPoints():
        raise capi.ErrorControlBadValue(capi.ERROR_BAD_VALUE,
                                        "field has %d values, grid has %d points"
                                        % (field.numel(), grid.GetNumberOfPoints()))


def _out_device(field):
    """Device of the outputs computed from `field`: its own, or the current
    CUDA device for a page-locked CPU field."""
    return field.device if field.is_cuda else torch.device("cuda", torch.cuda.current_device())


class UniformGrid:
    """Axis-aligned grid with implicit coordinates origin + spacing*(ijk+min)."""

    def __init__(self, dims=None, origin=(0.0, 0.0, 0.0), spacing=(1.0, 1.0, 1.0),
                 extent_min=(0, 0, 0)):
        self.Origin = tuple(float(v) for v in origin)
        self.Spacing = tuple(float(v) for v in spacing)
        self.ExtentMin = tuple(int(v) for v in extent_min)
        dims = dims or (1, 1, 1)
        self.ExtentMax = tuple(self.ExtentMin[a] + int(dims[a]) - 1 for a in range(3))

    def SetExtent(self, emin, emax):
        self.ExtentMin, self.ExtentMax = tuple(map(int, emin)), tuple(map(int, emax))

    def SetOrigin(self, o):
        self.Origin = tuple(map(float, o))

    def SetSpacing(self, s):
        self.Spacing = tuple(map(float, s))

    @property
    def dims(self):
        return tuple(self.ExtentMax[a] - self.ExtentMin[a] + 1 for a in range(3))

    def GetNumberOfPoints(self):
        d = self.dims
        return d[0] * d[1] * d[2]

    def GetNumberOfCells(self):
        d = self.dims
        if min(d) < 2:
            return 0
        return (d[0] - 1) * (d[1] - 1) * (d[2] - 1)

    def desc(self):
        g = capi.UniformGridDesc()
        for a in range(3):
            g.origin[a] = self.Origin[a]
            g.spacing[a] = self.Spacing[a]
            g.extent_min[a] = self.ExtentMin[a]
            g.extent_max[a] = self.ExtentMax[a]
        return g


class UnstructuredGrid:
    """Explicit points [N,3] and connectivity [cells, verts]: the output of
    the generate dispatchers, and (with int32 [C,4] tetrahedra) the input of
    marching tetrahedra (dax::cont::UnstructuredGrid<CellTagTetrahedron>)."""

    def __init__(self, points, connectivity):
        self.points = points
        self.connectivity = connectivity

    def GetPointCoordinates(self):
        return self.points

    def GetCellConnections(self):
        return self.connectivity

    def GetNumberOfPoints(self):
        return int(self.points.shape[0])

    def GetNumberOfCells(self):
        return int(self.connectivity.shape[0])


class Scratch:
    """Device scratch for the count/generate passes, grown on demand.

    Allocation happens only when a larger grid is seen, so steady-state
    pipelines allocate nothing.
    """

    def __init__(self, device=None):
        self.device = device
        self.buf = None

    def get(self, nbytes):
        if self.buf is None or self.buf.numel() < nbytes:
            dev = self.device or torch.device("cuda", torch.cuda.current_device())
            self.buf = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=dev)
        return self.buf


_default_scratch = {}


def _scratch_for(kind):
    dev = torch.cuda.current_device()
    key = (kind, dev)
    if key not in _default_scratch:
        _default_scratch[key] = Scratch()
    return _default_scratch[key]


# ---- worklets (descriptors; the arithmetic lives in the CUDA kernels) ----
class MarchingCubesCount:
    """dax/worklet/MarchingCubes.h:53-86."""

    def __init__(self, isovalue):
        self.IsoValue = float(isovalue)


class MarchingCubesGenerate:
    """dax/worklet/MarchingCubes.h:90-169."""

    def __init__(self, isovalue):
        self.IsoValue = float(isovalue)


class SliceCount:
    """dax/worklet/Slice.h:28-77: triangles per cell of the plane through
    `origin` with `normal` (the point field is the grid's coordinates)."""

    def __init__(self, origin, normal):
        self.Origin = tuple(float(v) for v in origin)
        self.Normal = tuple(float(v) for v in normal)


class SliceGenerate(SliceCount):
    """dax/worklet/Slice.h:82-168."""


class MarchingTetrahedraCount:
    """dax/worklet/MarchingTetrahedra.h:49-80."""

    def __init__(self, isovalue):
        self.IsoValue = float(isovalue)


class MarchingTetrahedraGenerate:
    """dax/worklet/MarchingTetrahedra.h:85-161."""

    def __init__(self, isovalue):
        self.IsoValue = float(isovalue)


class ThresholdCount:
    """dax/worklet/Threshold.h:69-96."""

    def __init__(self, thresholdMin, thresholdMax):
        self.ThresholdMin = float(thresholdMin)
        self.ThresholdMax = float(thresholdMax)


class ThresholdTopology:
    """dax/worklet/Threshold.h:98-111."""


class CellGradient:
    """dax/worklet/CellGradient.h:28-48."""


# ---- fused pipelines ------------------------------------------------------
def marching_cubes(grid, field, isovalue, merge=True, records=False, scratch=None, stream=None):
    """Count, size the outputs on the host, generate.  Returns a dict with
    ``verts`` [V,3] f32, ``conn`` [T,3] i32 and, if ``records``, the
    PointAsEdgeInterpolation arrays ``rec_first``, ``rec_second``, ``rec_weight``."""
    _require_field(field, grid)
    g = grid.desc()
    s = _stream(stream)
    nbytes = capi.lib().dax_gb300_mc_scratch_bytes(ctypes.byref(g))
    buf = (scratch or _scratch_for("mc")).get(nbytes)
    capi.call("dax_gb300_mc_count", ctypes.byref(g), _ptr(field), float(isovalue), _ptr(buf),
              buf.numel(), s)
    T, Vm = ctypes.c_int64(0), ctypes.c_int64(0)
    capi.call("dax_gb300_mc_totals", _ptr(buf), ctypes.byref(T), ctypes.byref(Vm), s)
    T = T.value
    V = Vm.value if merge else 3 * T
    dev = _out_device(field)
    verts = torch.empty((V, 3), dtype=torch.float32, device=dev)
    conn = torch.empty((T, 3), dtype=torch.int32, device=dev)
    ra = rb = rw = None
    if records:
        ra = torch.empty(V, dtype=torch.int32, device=dev)
        rb = torch.empty(V, dtype=torch.int32, device=dev)
        rw = torch.empty(V, dtype=torch.float32, device=dev)
    capi.call("dax_gb300_mc_generate", ctypes.byref(g), _ptr(field), float(isovalue),
              int(bool(merge)), _ptr(buf), buf.numel(), _ptr(verts), V, _ptr(conn), T, _ptr(ra),
              _ptr(rb), _ptr(rw), s)
    out = dict(verts=verts, conn=conn)
    if records:
        out.update(rec_first=ra, rec_second=rb, rec_weight=rw)
    return out


def marching_cubes_pipelined(grid, field, isovalue, verts, conn, merge=True, records=None,
                             scratch=None, stream=None, read_sizes=True):
    """Count and generate in one slab-pipelined call (``dax_gb300_mc_pipeline``)
    into caller-held outputs ``verts`` [>= V, 3] and ``conn`` [>= T, 3] (and,
    if given, ``records`` = (first, second, weight) of >= V entries).  With
    ``read_sizes`` the totals are read back (one host sync, which raises
    ErrorControlBadValue-family errors such as the capacity error) and
    (T, V) is returned; otherwise nothing blocks and None is returned."""
    _require_field(field, grid)
    g = grid.desc()
    s = _stream(stream)
    nbytes = capi.lib().dax_gb300_mc_scratch_bytes(ctypes.byref(g))
    buf = (scratch or _scratch_for("mc")).get(nbytes)
    ra, rb, rw = records if records is not None else (None, None, None)
    capi.call("dax_gb300_mc_pipeline", ctypes.byref(g), _ptr(field), float(isovalue),
              int(bool(merge)), _ptr(buf), buf.numel(), _ptr(verts), verts.shape[0], _ptr(conn),
              conn.shape[0], _ptr(ra), _ptr(rb), _ptr(rw), s)
    if not read_sizes:
        return None
    T, Vm = ctypes.c_int64(0), ctypes.c_int64(0)
    capi.call("dax_gb300_mc_totals", _ptr(buf), ctypes.byref(T), ctypes.byref(Vm), s)
    return T.value, (Vm.value if merge else 3 * T.value)


def slice_field(grid, origin, normal, out=None, stream=None):
    """The point field of a slice, dot(normal, coord(p) - origin), and its
    isovalue dot(normal, origin): marching cubes of it is the reference's
    Slice (dax/worklet/Slice.h)."""
    g = grid.desc()
    if out is None:
        out = torch.empty(grid.GetNumberOfPoints(), dtype=torch.float32, device="cuda")
    o = (ctypes.c_float * 3)(*[float(v) for v in origin])
    nrm = (ctypes.c_float * 3)(*[float(v) for v in normal])
    iso = ctypes.c_float(0.0)
    capi.call("dax_gb300_slice_field", ctypes.byref(g), o, nrm, _ptr(out), ctypes.byref(iso),
              _stream(stream))
    return out, iso.value


def slice(grid, origin, normal, merge=True, records=False, scratch=None, stream=None):
    """Triangles of the reference's Slice (SliceCount + SliceGenerate) for the
    plane given by `origin` and `normal`: the same dict as marching_cubes.
    The slice field is evaluated from the grid coordinates; none is stored."""
    g = grid.desc()
    s = _stream(stream)
    o = (ctypes.c_float * 3)(*[float(v) for v in origin])
    nrm = (ctypes.c_float * 3)(*[float(v) for v in normal])
    nbytes = capi.lib().dax_gb300_mc_scratch_bytes(ctypes.byref(g))
    buf = (scratch or _scratch_for("mc")).get(nbytes)
    capi.call("dax_gb300_slice_count", ctypes.byref(g), o, nrm, _ptr(buf), buf.numel(), s)
    T, Vm = ctypes.c_int64(0), ctypes.c_int64(0)
    capi.call("dax_gb300_mc_totals", _ptr(buf), ctypes.byref(T), ctypes.byref(Vm), s)
    T = T.value
    V = Vm.value if merge else 3 * T
    dev = buf.device
    verts = torch.empty((V, 3), dtype=torch.float32, device=dev)
    conn = torch.empty((T, 3), dtype=torch.int32, device=dev)
    ra = rb = rw = None
    if records:
        ra = torch.empty(V, dtype=torch.int32, device=dev)
        rb = torch.empty(V, dtype=torch.int32, device=dev)
        rw = torch.empty(V, dtype=torch.float32, device=dev)
    capi.call("dax_gb300_slice_generate", ctypes.byref(g), o, nrm, int(bool(merge)), _ptr(buf),
              buf.numel(), _ptr(verts), V, _ptr(conn), T, _ptr(ra), _ptr(rb), _ptr(rw), s)
    out = dict(verts=verts, conn=conn)
    if records:
        out.update(rec_first=ra, rec_second=rb, rec_weight=rw)
    return out


class Tetrahedralize:
    """dax/worklet/Tetrahedralize.h:55-82: 5 tetrahedra per voxel."""


def tetrahedralize(grid, stream=None):
    """DispatcherGenerateTopology<Tetrahedralize> (count 5 per cell, points
    not merged) over a UniformGrid: an UnstructuredGrid of tetrahedra whose
    points are the uniform grid's points, in id order."""
    g = grid.desc()
    s = _stream(stream)
    conn = torch.empty((5 * grid.GetNumberOfCells(), 4), dtype=torch.int32, device="cuda")
    capi.call("dax_gb300_tetrahedralize", ctypes.byref(g), _ptr(conn), s)
    pts = torch.empty((grid.GetNumberOfPoints(), 3), dtype=torch.float32, device="cuda")
    capi.call("dax_gb300_point_coordinates", ctypes.byref(g), _ptr(pts), s)
    return UnstructuredGrid(pts, conn)


def _tet_conn(grid):
    conn = grid.GetCellConnections()
    if (not isinstance(conn, torch.Tensor) or not conn.is_cuda or conn.dtype != torch.int32
            or conn.dim() != 2 or conn.shape[1] != 4 or not conn.is_contiguous()):
        raise capi.ErrorControlBadValue(capi.ERROR_BAD_VALUE,
                                        "tetrahedra must be a contiguous int32 CUDA tensor [C, 4]")
    return conn


def marching_tetrahedra(grid, field, isovalue, merge=True, records=False, scratch=None,
                        stream=None):
    """MarchingTetrahedraCount + Generate on an UnstructuredGrid of
    tetrahedra: the same dict as marching_cubes."""
    _require_field(field, grid)
    conn = _tet_conn(grid)
    pts = grid.GetPointCoordinates()
    if (not isinstance(pts, torch.Tensor) or not (pts.is_cuda or pts.is_pinned())
            or pts.dtype != torch.float32 or tuple(pts.shape) != (grid.GetNumberOfPoints(), 3)
            or not pts.is_contiguous()):
        raise capi.ErrorControlBadValue(capi.ERROR_BAD_VALUE,
                                        "points must be a contiguous float32 tensor [P, 3]")
    L = capi.lib()
    s = _stream(stream)
    C, P = conn.shape[0], pts.shape[0]
    iso = float(isovalue)
    nbytes = L.dax_gb300_mt_scratch_bytes(C)
    buf = (scratch or _scratch_for("mt")).get(nbytes)
    capi.call("dax_gb300_mt_count", _ptr(conn), C, _ptr(field), P, iso, _ptr(buf), buf.numel(), s)
    T = ctypes.c_int64(0)
    capi.call("dax_gb300_mc_totals", _ptr(buf), ctypes.byref(T), None, s)
    T = T.value
    mbuf, mbytes = None, 0
    if merge:
        mbytes = L.dax_gb300_mt_merge_scratch_bytes(T, P)
        mbuf = _scratch_for("mt_merge").get(mbytes)
        V = ctypes.c_int64(0)
        capi.call("dax_gb300_mt_merge", _ptr(conn), C, _ptr(field), P, iso, _ptr(buf), buf.numel(),
                  _ptr(mbuf), mbuf.numel(), ctypes.byref(V), s)
        V = V.value
    else:
        V = 3 * T
    dev = conn.device
    verts = torch.empty((V, 3), dtype=torch.float32, device=dev)
    tconn = torch.empty((T, 3), dtype=torch.int32, device=dev)
    ra = rb = rw = None
    if records:
        ra = torch.empty(V, dtype=torch.int32, device=dev)
        rb = torch.empty(V, dtype=torch.int32, device=dev)
        rw = torch.empty(V, dtype=torch.float32, device=dev)
    capi.call("dax_gb300_mt_generate", _ptr(pts), _ptr(conn), C, _ptr(field), P, iso,
              int(bool(merge)), _ptr(buf), buf.numel(), _ptr(mbuf), mbuf.numel() if merge else 0,
              _ptr(verts), V, _ptr(tconn), T, _ptr(ra), _ptr(rb), _ptr(rw), s)
    out = dict(verts=verts, conn=tconn)
    if records:
        out.update(rec_first=ra, rec_second=rb, rec_weight=rw)
    return out


def interpolate_point_field(rec_first, rec_second, rec_weight, field, stream=None):
    """CompactPointField: a scalar field [P] gives [V]; a field of k floats per
    point [P, k] (a dax::Vector3 field has k = 3) gives [V, k]."""
    if field.dim() == 1:
        out = torch.empty(rec_first.numel(), dtype=torch.float32, device=_out_device(field))
        capi.call("dax_gb300_interpolate_point_field", _ptr(rec_first), _ptr(rec_second),
                  _ptr(rec_weight), rec_first.numel(), _ptr(field), _ptr(out), _stream(stream))
        return out
    if field.dim() != 2 or field.dtype != torch.float32 or not field.is_contiguous():
        raise capi.ErrorControlBadValue(capi.ERROR_BAD_VALUE,
                                        "point field must be contiguous float32 [P] or [P, k]")
    k = int(field.shape[1])
    out = torch.empty((rec_first.numel(), k), dtype=torch.float32, device=_out_device(field))
    capi.call("dax_gb300_interpolate_point_field_n", _ptr(rec_first), _ptr(rec_second),
              _ptr(rec_weight), rec_first.numel(), _ptr(field), field.shape[0], k, _ptr(out),
              _stream(stream))
    return out


def marching_cubes_counted(grid, field, isovalue, count, merge=True, records=False,
                           stream=None):
    """DispatcherGenerateInterpolatedCells<MarchingCubesGenerate> driven by an
    arbitrary int32 count per cell: the same dict as marching_cubes."""
    _require_field(field, grid)
    if (not isinstance(count, torch.Tensor) or count.dtype != torch.int32 or not count.is_cuda
            or count.numel() != grid.GetNumberOfCells() or not count.is_contiguous()):
        raise capi.ErrorControlBadValue(capi.ERROR_BAD_VALUE,
                                        "count must be a contiguous int32 CUDA tensor, one per cell")
    L = capi.lib()
    g = grid.desc()
    s = _stream(stream)
    iso = float(isovalue)
    nbytes = L.dax_gb300_mc_counted_scratch_bytes(ctypes.byref(g))
    buf = _scratch_for("counted").get(nbytes)
    T = ctypes.c_int64(0)
    capi.call("dax_gb300_mc_counted_scan", ctypes.byref(g), _ptr(count), _ptr(buf), buf.numel(),
              ctypes.byref(T), s)
    T = T.value
    mbuf = None
    if merge:
        mbytes = L.dax_gb300_mt_merge_scratch_bytes(T, grid.GetNumberOfPoints())
        mbuf = _scratch_for("counted_merge").get(mbytes)
        V = ctypes.c_int64(0)
        capi.call("dax_gb300_mc_counted_merge", ctypes.byref(g), _ptr(field), iso, _ptr(count),
                  _ptr(buf), buf.numel(), _ptr(mbuf), mbuf.numel(), ctypes.byref(V), s)
        V = V.value
    else:
        V = 3 * T
    dev = count.device
    verts = torch.empty((V, 3), dtype=torch.float32, device=dev)
    conn = torch.empty((T, 3), dtype=torch.int32, device=dev)
    ra = rb = rw = None
    if records:
        ra = torch.empty(V, dtype=torch.int32, device=dev)
        rb = torch.empty(V, dtype=torch.int32, device=dev)
        rw = torch.empty(V, dtype=torch.float32, device=dev)
    capi.call("dax_gb300_mc_counted_generate", ctypes.byref(g), _ptr(field), iso, _ptr(count),
              int(bool(merge)), _ptr(buf), buf.numel(), _ptr(mbuf), mbuf.numel() if merge else 0,
              _ptr(verts), V, _ptr(conn), T, _ptr(ra), _ptr(rb), _ptr(rw), s)
    capi.call("dax_gb300_mc_totals", _ptr(buf), None, None, s)  # raises on a bad count array
    out = dict(verts=verts, conn=conn)
    if records:
        out.update(rec_first=ra, rec_second=rb, rec_weight=rw)
    return out


def point_magnitude(grid, stream=None):
    """DispatcherMapField<Magnitude> over the grid's point coordinates
    (dax/worklet/Magnitude.h): |coord(p)| for every point, float32 [P]."""
    g = grid.desc()
    out = torch.empty(grid.GetNumberOfPoints(), dtype=torch.float32, device="cuda")
    capi.call("dax_gb300_point_magnitude", ctypes.byref(g), _ptr(out), _stream(stream))
    return out


def write_vtk(path, grid):
    """The legacy-VTK ASCII POLYDATA file of an UnstructuredGrid of triangles
    (or other cells), as the reference benchmark's PrintContentsToStream
    writes it (Benchmarks/MarchingCubes/Pipeline.h:51-98)."""
    pts = grid.GetPointCoordinates().contiguous()
    conn = grid.GetCellConnections().contiguous()
    if pts.dtype != torch.float32 or conn.dtype != torch.int32:
        raise capi.ErrorControlBadValue(capi.ERROR_BAD_VALUE,
                                        "points must be float32 and connectivity int32")
    if pts.is_cuda or conn.is_cuda:
        torch.cuda.synchronize()
    V = int(conn.shape[1]) if conn.dim() == 2 else 3
    capi.call("dax_gb300_write_vtk_polydata", str(path).encode(), _ptr(pts), int(pts.shape[0]),
              _ptr(conn), int(conn.numel() // V), V)


# ---- the Mandelbulb benchmark pipeline (Benchmarks/Mandlebulb) -------------
class Mandlebulb:
    """worklet::Mandlebulb (Benchmarks/Mandlebulb/Worklets.h:65-109): the
    escape iteration of every grid point."""


class MandlebulbClipCount:
    """worklet::MandlebulbClipCount (Worklets.h:112-170)."""

    def __init__(self, origin, location, normal, isovalue):
        self.Origin = tuple(float(v) for v in origin)
        self.Location = tuple(float(v) for v in location)
        self.Normal = tuple(float(v) for v in normal)
        self.IsoValue = float(isovalue)


class MandlebulbVolume:
    """mandle::MandlebulbVolume (Mandlebulb.h): the grid and its escape
    iteration field."""

    def __init__(self, grid, field):
        self.Grid = grid
        self.EscapeIteration = field


class MandlebulbSurface:
    """mandle::MandlebulbSurface (Mandlebulb.h): the unmerged triangle surface
    with per-point normals [3T, 3] and colours [3T, 4] uint8 -- the device
    buffers the reference hands to OpenGL."""

    def __init__(self, data, norms, colors):
        self.Data = data
        self.Norms = norms
        self.Colors = colors


def mandlebulb_field(grid, stream=None):
    g = grid.desc()
    out = torch.empty(grid.GetNumberOfPoints(), dtype=torch.float32, device="cuda")
    capi.call("dax_gb300_mandelbulb_field", ctypes.byref(g), _ptr(out), _stream(stream))
    return out


def compute_mandlebulb(origin, spacing, extent_max, stream=None):
    """computeMandlebulb (Benchmarks/Mandlebulb/Mandlebulb.cxx:83-102) on the
    grid of points 0 .. extent_max."""
    grid = UniformGrid(tuple(int(e) + 1 for e in extent_max), origin, spacing)
    return MandlebulbVolume(grid, mandlebulb_field(grid, stream=stream))


def colors_and_norms(points, stream=None):
    """worklet::ColorsAndNorms (Worklets.h:177-209) over an unmerged surface's
    points [3T, 3]: (normals [3T, 3], colours [3T, 4] uint8)."""
    n = int(points.shape[0])
    norms = torch.empty((n, 3), dtype=torch.float32, device=points.device)
    colors = torch.empty((n, 4), dtype=torch.uint8, device=points.device)
    capi.call("dax_gb300_colors_and_norms", _ptr(points), n, _ptr(norms), _ptr(colors),
              _stream(stream))
    return norms, colors


def _surface(out, stream):
    norms, colors = colors_and_norms(out["verts"], stream=stream)
    return MandlebulbSurface(UnstructuredGrid(out["verts"], out["conn"]), norms, colors)


def extract_surface(vol, iteration, stream=None):
    """extractSurface (Mandlebulb.cxx:105-123): marching cubes of the escape
    iteration at `iteration`, points not merged, then ColorsAndNorms."""
    out = marching_cubes(vol.Grid, vol.EscapeIteration, iteration, merge=False, stream=stream)
    return _surface(out, stream)


def extract_cut(vol, cut_percent, iteration, stream=None):
    """extractCut (Mandlebulb.cxx:126-157): MandlebulbClipCount against the z
    plane at cut_percent of the grid, the count-driven generate, points not
    merged, then ColorsAndNorms."""
    g = vol.Grid
    o, sp = g.Origin, g.Spacing
    cd = [n - 1 for n in g.dims]
    f32 = np.float32
    # the location as the reference computes it, in float
    loc = (f32(o[0]) + f32(sp[0]) * f32(cd[0]), f32(o[1]) + f32(sp[1]) * f32(cd[1]),
           f32(o[2]) + f32(sp[2]) * f32(f32(cd[2]) * f32(cut_percent)))
    w = MandlebulbClipCount(o, [float(v) for v in loc], (0.0, 0.0, 1.0), iteration)
    count = DispatcherMapCell(w).Invoke(g, vol.EscapeIteration, stream=stream)
    out = marching_cubes_counted(g, vol.EscapeIteration, iteration, count, merge=False,
                                 stream=stream)
    return _surface(out, stream)


def threshold(grid, field, lo, hi, compact_field=True, scratch=None, stream=None):
    """Returns dict(conn [K,8] i32, coords [U,3] f32, field [U] f32 or None)."""
    _require_field(field, grid)
    g = grid.desc()
    s = _stream(stream)
    nbytes = capi.lib().dax_gb300_threshold_scratch_bytes(ctypes.byref(g))
    buf = (scratch or _scratch_for("threshold")).get(nbytes)
    capi.call("dax_gb300_threshold_count", ctypes.byref(g), _ptr(field), float(lo), float(hi),
              _ptr(buf), buf.numel(), s)
    K, U = ctypes.c_int64(0), ctypes.c_int64(0)
    capi.call("dax_gb300_threshold_totals", _ptr(buf), ctypes.byref(K), ctypes.byref(U), s)
    K, U = K.value, U.value
    dev = _out_device(field)
    conn = torch.empty((K, 8), dtype=torch.int32, device=dev)
    coords = torch.empty((U, 3), dtype=torch.float32, device=dev)
    fout = torch.empty(U, dtype=torch.float32, device=dev) if compact_field else None
    capi.call("dax_gb300_threshold_generate", ctypes.byref(g), _ptr(field), float(lo), float(hi),
              _ptr(buf), buf.numel(), _ptr(conn), K, _ptr(coords), _ptr(fout), U, s)
    return dict(conn=conn, coords=coords, field=fout)


def threshold_compact_point_field(grid, scratch, used_points, field, out=None, stream=None):
    """CompactPointField of a threshold (DispatcherGenerateTopology.h:98-113):
    the point field ``field`` ([P] or [P, k] float32) at the used points, in
    the order of the threshold's coordinates.  ``scratch`` holds the
    threshold count pass of the same grid; ``used_points`` is its U."""
    if not isinstance(field, torch.Tensor) or field.dim() not in (1, 2):
        raise capi.ErrorControlBadValue(capi.ERROR_BAD_VALUE, "the point field must be [P] or [P, k]")
    k = 1 if field.dim() == 1 else field.shape[1]
    if (field.dtype != torch.float32 or not field.is_contiguous() or k < 1
            or field.shape[0] != grid.GetNumberOfPoints() or not (field.is_cuda or field.is_pinned())):
        raise capi.ErrorControlBadValue(capi.ERROR_BAD_VALUE,
                                        "the point field must be a contiguous float32 [P] or [P, k] "
                                        "CUDA (or page-locked) tensor")
    if out is None:
        shape = (used_points,) if field.dim() == 1 else (used_points, k)
        out = torch.empty(shape, dtype=torch.float32, device=_out_device(field))
    g = grid.desc()
    capi.call("dax_gb300_threshold_compact_point_field", ctypes.byref(g), _ptr(scratch),
              scratch.numel(), _ptr(field), k, _ptr(out), used_points, _stream(stream))
    return out


def cell_gradient(grid, field, out=None, stream=None):
    _require_field(field, grid)
    g = grid.desc()
    if out is None:
        out = torch.empty((grid.GetNumberOfCells(), 3), dtype=torch.float32,
                          device=_out_device(field))
    capi.call("dax_gb300_cell_gradient", ctypes.byref(g), _ptr(field), _ptr(out), _stream(stream))
    return out


# ---- dispatchers ----------------------------------------------------------
class DispatcherMapCell:
    """DispatcherMapCell<Worklet>: one output value per cell, cell-id order."""

    def __init__(self, worklet):
        self.worklet = worklet

    def Invoke(self, grid, field=None, stream=None):
        w = self.worklet
        if not isinstance(w, SliceCount):  # a slice's point field is the implicit coordinates
            _require_field(field, grid)
        if isinstance(w, MarchingTetrahedraCount):
            conn = _tet_conn(grid)
            count = torch.empty(conn.shape[0], dtype=torch.int32, device=_out_device(field))
            capi.call("dax_gb300_mt_classify_count", _ptr(conn), conn.shape[0], _ptr(field),
                      grid.GetNumberOfPoints(), w.IsoValue, _ptr(count), _stream(stream))
            return count
        g = grid.desc()
        C = grid.GetNumberOfCells()
        if isinstance(w, MarchingCubesCount):
            count = torch.empty(C, dtype=torch.int32, device=_out_device(field))
            capi.call("dax_gb300_mc_classify_count", ctypes.byref(g), _ptr(field), w.IsoValue,
                      _ptr(count), None, _stream(stream))
            count._dax_mc_source = (field.data_ptr(), w.IsoValue)
            return count
        if isinstance(w, MandlebulbClipCount):
            count = torch.empty(C, dtype=torch.int32, device=_out_device(field))
            vec = lambda v: (ctypes.c_float * 3)(*v)
            capi.call("dax_gb300_mandelbulb_clip_count", ctypes.byref(g), _ptr(field), w.IsoValue,
                      vec(w.Origin), vec(w.Location), vec(w.Normal), _ptr(count), _stream(stream))
            return count
        if isinstance(w, SliceCount):
            sf, iso = slice_field(grid, w.Origin, w.Normal, stream=stream)
            count = torch.empty(C, dtype=torch.int32, device=sf.device)
            capi.call("dax_gb300_mc_classify_count", ctypes.byref(g), _ptr(sf), iso, _ptr(count),
                      None, _stream(stream))
            return count
        if isinstance(w, ThresholdCount):
            count = torch.empty(C, dtype=torch.int32, device=_out_device(field))
            capi.call("dax_gb300_threshold_classify_count", ctypes.byref(g), _ptr(field),
                      w.ThresholdMin, w.ThresholdMax, _ptr(count), _stream(stream))
            return count
        if isinstance(w, CellGradient):
            return cell_gradient(grid, field, stream=stream)
        raise capi.ErrorControlBadValue(capi.ERROR_BAD_VALUE,
                                        "worklet %r has no GB300 kernel" % type(w).__name__)

    def classify_cases(self, grid, field, stream=None):
        """MarchingCubesCount with the per-cell case index as a second output."""
        g = grid.desc()
        C = grid.GetNumberOfCells()
        count = torch.empty(C, dtype=torch.int32, device=_out_device(field))
        cases = torch.empty(C, dtype=torch.uint8, device=_out_device(field))
        capi.call("dax_gb300_mc_classify_count", ctypes.byref(g), _ptr(field),
                  self.worklet.IsoValue, _ptr(count), _ptr(cases), _stream(stream))
        return count, cases


class DispatcherGenerateInterpolatedCells:
    """DispatcherGenerateInterpolatedCells<MarchingCubesGenerate | SliceGenerate |
    MarchingTetrahedraGenerate>.

    A count array from MarchingCubesCount on the same field and isovalue
    (tagged when DispatcherMapCell made it) is not read: the generate pass recounts from the field (identical by
    construction), so no per-cell array is scanned.  Any other count array
    (a clip, a mask) drives the generate as the reference's dispatcher does:
    scan, upper bounds, visit index (marching_cubes_counted).
    """

    def __init__(self, count, worklet):
        self.count = count
        self.worklet = worklet
        self.RemoveDuplicatePoints = True
        self.ReleaseCount = True
        self._records = None

    def SetRemoveDuplicatePoints(self, b):
        self.RemoveDuplicatePoints = bool(b)

    def GetRemoveDuplicatePoints(self):
        return self.RemoveDuplicatePoints

    def SetReleaseCount(self, b):
        self.ReleaseCount = bool(b)

    def Invoke(self, grid, field=None, stream=None):
        w = self.worklet
        if isinstance(w, SliceGenerate):
            out = slice(grid, w.Origin, w.Normal, merge=self.RemoveDuplicatePoints, records=True,
                        stream=stream)
        elif isinstance(w, MarchingTetrahedraGenerate):
            out = marching_tetrahedra(grid, field, w.IsoValue, merge=self.RemoveDuplicatePoints,
                                      records=True, stream=stream)
        elif (self.count is not None and isinstance(w, MarchingCubesGenerate)
              and getattr(self.count, "_dax_mc_source", None) != (field.data_ptr(), w.IsoValue)):
            out = marching_cubes_counted(grid, field, w.IsoValue, self.count,
                                         merge=self.RemoveDuplicatePoints, records=True,
                                         stream=stream)
        else:
            out = marching_cubes(grid, field, w.IsoValue, merge=self.RemoveDuplicatePoints,
                                 records=True, stream=stream)
        self._records = (out["rec_first"], out["rec_second"], out["rec_weight"])
        if self.ReleaseCount:
            self.count = None
        return UnstructuredGrid(out["verts"], out["conn"])

    def CompactPointField(self, field, stream=None):
        if self._records is None:
            raise capi.ErrorControlBadValue(capi.ERROR_BAD_VALUE, "Invoke before CompactPointField")
        return interpolate_point_field(*self._records, field, stream=stream)


class DispatcherGenerateTopology:
    """DispatcherGenerateTopology<ThresholdTopology> driven by a ThresholdCount."""

    def __init__(self, count, worklet=None, threshold_worklet=None):
        self.count = count
        self.worklet = worklet or ThresholdTopology()
        self.threshold = threshold_worklet
        self.RemoveDuplicatePoints = True
        self._field = None

    def SetRemoveDuplicatePoints(self, b):
        self.RemoveDuplicatePoints = bool(b)

    def Invoke(self, grid, field, stream=None):
        if self.threshold is None:
            raise capi.ErrorControlBadValue(capi.ERROR_BAD_VALUE,
                                            "the GB300 path needs the ThresholdCount worklet")
        self._scratch = Scratch()  # kept: CompactPointField reads its count pass
        out = threshold(grid, field, self.threshold.ThresholdMin, self.threshold.ThresholdMax,
                        scratch=self._scratch, stream=stream)
        self._field = out["field"]
        self._grid = grid
        self._used = out["coords"].shape[0]
        if self.RemoveDuplicatePoints:
            return UnstructuredGrid(out["coords"], out["conn"])
        # without point removal the connectivity keeps the input's point ids
        # (DispatcherGenerateTopology.h:199-203 skips FillPointMask and
        # ResolveDuplicatePoints): the used points' own ids, compacted as raw
        # 32-bit words, map the compacted ids back
        P = grid.GetNumberOfPoints()
        dev = out["conn"].device
        buf = self._scratch.get(capi.lib().dax_gb300_threshold_scratch_bytes(
            ctypes.byref(grid.desc())))
        ids = torch.arange(P, dtype=torch.int32, device=dev).view(torch.float32)
        used = threshold_compact_point_field(grid, buf, self._used, ids, stream=stream)
        conn = used.view(torch.int32)[out["conn"].long()]
        pts = torch.empty((P, 3), dtype=torch.float32, device=dev)
        capi.call("dax_gb300_point_coordinates", ctypes.byref(grid.desc()), _ptr(pts), _stream(stream))
        return UnstructuredGrid(pts, conn)

    def CompactPointField(self, field=None, stream=None):
        """The input point field ([P] or [P, k]) at the used points, in the
        order of the output coordinates (DispatcherGenerateTopology.h:98-113);
        with no argument, the thresholded field itself.  Without point
        removal nothing is compacted (the reference returns false): None."""
        if not self.RemoveDuplicatePoints:
            return None
        if field is None:
            return self._field
        buf = self._scratch.get(capi.lib().dax_gb300_threshold_scratch_bytes(
            ctypes.byref(self._grid.desc())))
        return threshold_compact_point_field(self._grid, buf, self._used, field, stream=stream)


class MarchingCubesBatch:
    """Many uniform grids (own extents, fields, isovalues) through one launch
    per pass: ``dax_gb300_mc_batch_*``.  Outputs are concatenated; grid g's
    triangles are ``conn[tri_offsets[g]:tri_offsets[g+1]]`` and index the
    grid's own vertices ``verts[vert_offsets[g]:vert_offsets[g+1]]`` (merged)."""

    def __init__(self, grids, fields, isovalues):
        self.grids = list(grids)
        self.fields = list(fields)
        for gr, f in zip(self.grids, self.fields):
            _require_field(f, gr)
        n = len(self.grids)
        descs = (capi.UniformGridDesc * n)(*[gr.desc() for gr in self.grids])
        ptrs = (ctypes.c_void_p * n)(*[f.data_ptr() for f in self.fields])
        isos = (ctypes.c_float * n)(*[float(v) for v in isovalues])
        h = ctypes.c_void_p()
        capi.call("dax_gb300_mc_batch_create", n, descs, ptrs, isos, ctypes.byref(h))
        self.handle = h
        self.n = n
        nbytes = capi.lib().dax_gb300_mc_batch_scratch_bytes(h)
        self.scratch = torch.empty(nbytes, dtype=torch.uint8, device=self.fields[0].device)
        self.graph = None

    def __del__(self):
        try:
            if self.graph:
                capi.lib().dax_gb300_graph_destroy(self.graph)
            if self.handle:
                capi.lib().dax_gb300_mc_batch_destroy(self.handle)
        except Exception:
            pass

    def count(self, stream=None):
        capi.call("dax_gb300_mc_batch_count", self.handle, _ptr(self.scratch), self.scratch.numel(),
                  _stream(stream))

    def totals(self, stream=None):
        t = (ctypes.c_int64 * (self.n + 1))()
        v = (ctypes.c_int64 * (self.n + 1))()
        capi.call("dax_gb300_mc_batch_totals", self.handle, _ptr(self.scratch), t, v,
                  _stream(stream))
        return list(t), list(v)

    def generate(self, verts, conn, merge=True, stream=None):
        capi.call("dax_gb300_mc_batch_generate", self.handle, int(bool(merge)), _ptr(self.scratch),
                  self.scratch.numel(), _ptr(verts), verts.shape[0], _ptr(conn), conn.shape[0],
                  _stream(stream))

    def run(self, merge=True, stream=None):
        """count, size on the host, generate; returns (verts, conn, tri_off, vert_off)."""
        self.count(stream)
        t, v = self.totals(stream)
        dev = self.fields[0].device
        V = v[-1] if merge else 3 * t[-1]
        verts = torch.empty((V, 3), dtype=torch.float32, device=dev)
        conn = torch.empty((t[-1], 3), dtype=torch.int32, device=dev)
        self.generate(verts, conn, merge, stream)
        if not merge:
            v = [3 * x for x in t]
        return verts, conn, t, v

    def sizes(self):
        """(cells, points) of all grids: the lengths of the concatenated
        per-cell and per-point arrays."""
        c, pnt = ctypes.c_int64(), ctypes.c_int64()
        capi.call("dax_gb300_mc_batch_sizes", self.handle, ctypes.byref(c), ctypes.byref(pnt))
        return c.value, pnt.value

    def cell_gradient(self, out=None, stream=None):
        """Every grid's cell gradients in one launch, grid after grid."""
        if out is None:
            out = torch.empty((self.sizes()[0], 3), dtype=torch.float32,
                              device=self.fields[0].device)
        capi.call("dax_gb300_mc_batch_cell_gradient", self.handle, _ptr(out), _stream(stream))
        return out

    def field_adjoint(self, grad_vertices=None, grad_cell_gradients=None, out=None, stream=None):
        """dL/dfield of every grid (concatenated) from dL/d(merged vertices)
        of this plan's last count pass and/or dL/d(cell gradients)."""
        if out is None:
            out = torch.empty(self.sizes()[1], dtype=torch.float32, device=self.fields[0].device)
        capi.call("dax_gb300_mc_batch_field_adjoint", self.handle, _ptr(self.scratch),
                  self.scratch.numel(), _ptr(grad_vertices), _ptr(grad_cell_gradients), _ptr(out),
                  _stream(stream))
        return out

    def autotune(self, verts, conn, merge=True, stream=None):
        """dax_gb300_mc_batch_autotune on these outputs: keeps the fastest
        emit batch / count pass in the plan; returns (emit_batch, dealt,
        best_ms), best_ms -1 when the extent class was tuned before."""
        ms = ctypes.c_float()
        capi.call("dax_gb300_mc_batch_autotune", self.handle, int(bool(merge)), _ptr(self.scratch),
                  self.scratch.numel(), _ptr(verts), verts.shape[0], _ptr(conn), conn.shape[0],
                  _stream(stream), ctypes.byref(ms))
        return self.config() + (ms.value,)

    def set_config(self, emit_batch=0, dealt=-1):
        capi.call("dax_gb300_mc_batch_set_config", self.handle, int(emit_batch), int(dealt))

    def config(self):
        eb, dc = ctypes.c_int(), ctypes.c_int()
        capi.call("dax_gb300_mc_batch_get_config", self.handle, ctypes.byref(eb), ctypes.byref(dc))
        return eb.value, dc.value

    def capture(self, verts, conn, merge=True):
        """Capture count + generate into a CUDA graph writing into verts/conn."""
        g = ctypes.c_void_p()
        capi.call("dax_gb300_mc_batch_capture", self.handle, int(bool(merge)), _ptr(self.scratch),
                  self.scratch.numel(), _ptr(verts), verts.shape[0], _ptr(conn), conn.shape[0],
                  ctypes.byref(g))
        if self.graph:
            capi.lib().dax_gb300_graph_destroy(self.graph)
        self.graph = g

    def replay(self, stream=None):
        capi.call("dax_gb300_graph_launch", self.graph, _stream(stream))


# ---- generic primitives: dax::cont::internal::DeviceAdapterAlgorithm -------
class SortLess:
    """dax::math::SortLess: ascending order (the default)."""


class SortGreater:
    """dax::math::SortGreater: descending order."""


_TYPES = {torch.int32: capi.TYPE_I32, torch.float32: capi.TYPE_F32, torch.int64: capi.TYPE_I64}
if hasattr(torch, "uint32"):
    _TYPES[torch.uint32] = capi.TYPE_U32
if hasattr(torch, "uint64"):
    _TYPES[torch.uint64] = capi.TYPE_U64


def _elem_type(t, what):
    if not isinstance(t, torch.Tensor) or not t.is_cuda or not t.is_contiguous():
        raise capi.ErrorControlBadValue(capi.ERROR_BAD_VALUE, "%s must be a contiguous CUDA tensor"
                                        % what)
    if t.dtype not in _TYPES:
        raise capi.ErrorControlBadValue(capi.ERROR_BAD_VALUE, "unsupported %s type %s"
                                        % (what, t.dtype))
    return _TYPES[t.dtype]


def _row_bytes(t):
    return t[0].numel() * t.element_size() if t.dim() > 1 else t.element_size()


class Algorithm:
    """The device adapter's generic algorithms (DeviceAdapterAlgorithm.h:44-331)
    on torch CUDA tensors, with the reference's names and argument meanings."""

    @staticmethod
    def Copy(src, dst=None):
        if dst is None:
            return src.clone()
        dst.resize_(src.shape).copy_(src)
        return dst

    @staticmethod
    def _scan(inp, out, exclusive, stream):
        t = _elem_type(inp, "array")
        if out is None:
            out = torch.empty_like(inp)
        n = inp.numel()
        nb = capi.lib().dax_gb300_scan_scratch_bytes(n)
        scratch = torch.empty(nb, dtype=torch.uint8, device=inp.device)
        total = torch.zeros(1, dtype=inp.dtype)
        capi.call("dax_gb300_scan", _ptr(inp), _ptr(out), n, t, int(exclusive), _ptr(scratch), nb,
                  ctypes.c_void_p(total.data_ptr()), _stream(stream))
        return total.item(), out

    @staticmethod
    def ScanInclusive(inp, out=None, stream=None):
        """Returns (total, out); out may be inp (in place)."""
        return Algorithm._scan(inp, out, False, stream)

    @staticmethod
    def ScanExclusive(inp, out=None, stream=None):
        return Algorithm._scan(inp, out, True, stream)

    @staticmethod
    def SortByKey(keys, values, comp=None, stream=None):
        """Sorts keys in place (stable), carrying values ([n] or [n, k] rows of
        up to 16 bytes).  Keys of shape [n, k] sort lexicographically, as the
        reference's tuple keys do (first component most significant)."""
        desc = isinstance(comp, SortGreater) or comp is SortGreater
        if keys.dim() > 1:
            return Algorithm._sort_rows(keys, values, desc, stream)
        t = _elem_type(keys, "keys")
        n = keys.numel()
        vb = 0
        if values is not None:
            if not values.is_cuda or not values.is_contiguous() or values.shape[0] != n:
                raise capi.ErrorControlBadValue(capi.ERROR_BAD_VALUE,
                                                "values must be contiguous, one row per key")
            vb = _row_bytes(values) if n else 0
        nb = capi.lib().dax_gb300_sort_scratch_bytes(n, t, vb)
        if nb == 0:
            raise capi.ErrorControlBadValue(capi.ERROR_BAD_VALUE, "value rows must be 4..16 bytes")
        scratch = torch.empty(nb, dtype=torch.uint8, device=keys.device)
        capi.call("dax_gb300_sort_by_key", _ptr(keys), _ptr(values) if vb else None, n, t, vb,
                  int(desc), _ptr(scratch), nb, _stream(stream))
        return keys, values

    @staticmethod
    def _sort_rows(keys, values, desc, stream):
        n = keys.shape[0]
        perm = torch.arange(n, dtype=torch.int32, device=keys.device)
        for c in reversed(range(keys.shape[1])):  # least significant component first
            col = keys[:, c][perm.long()].contiguous()
            Algorithm.SortByKey(col, perm, SortGreater() if desc else None, stream)
        idx = perm.long()
        keys.copy_(keys[idx])
        if values is not None:
            values.copy_(values[idx])
        return keys, values

    @staticmethod
    def Sort(array, comp=None, stream=None):
        return Algorithm.SortByKey(array, None, comp, stream)[0]

    @staticmethod
    def Unique(array, stream=None):
        """Keeps the first of every run of equal adjacent values; returns the
        shrunk view of `array`."""
        t = _elem_type(array, "array")
        n = array.numel()
        nb = capi.lib().dax_gb300_compact_scratch_bytes(n, array.element_size())
        scratch = torch.empty(nb, dtype=torch.uint8, device=array.device)
        cnt = ctypes.c_int64(0)
        capi.call("dax_gb300_unique", _ptr(array), n, t, _ptr(scratch), nb, ctypes.byref(cnt),
                  _stream(stream))
        return array[:cnt.value]

    @staticmethod
    def _bounds(sorted_, values, out, upper, stream):
        t = _elem_type(sorted_, "input")
        if values.dtype != sorted_.dtype:
            raise capi.ErrorControlBadValue(capi.ERROR_BAD_VALUE, "values must match the input type")
        if out is None:
            out = torch.empty(values.numel(), dtype=torch.int32, device=values.device)
        capi.call("dax_gb300_bounds", _ptr(sorted_), sorted_.numel(), _ptr(values), values.numel(),
                  t, int(upper), _ptr(out), _stream(stream))
        return out

    @staticmethod
    def LowerBounds(inp, values, out=None, comp=None, stream=None):
        return Algorithm._bounds(inp, values, out, False, stream)

    @staticmethod
    def UpperBounds(inp, values, out=None, comp=None, stream=None):
        return Algorithm._bounds(inp, values, out, True, stream)

    @staticmethod
    def StreamCompact(inp, stencil=None, stream=None):
        """StreamCompact(input, stencil): the rows of input whose stencil entry
        is non-zero.  StreamCompact(stencil): the int32 indices of the non-zero
        entries."""
        if stencil is None:
            stencil, inp = inp, None
        st = _elem_type(stencil, "stencil")
        if st not in (capi.TYPE_I32, capi.TYPE_F32):
            raise capi.ErrorControlBadValue(capi.ERROR_BAD_VALUE, "stencil must be int32 or float32")
        n = stencil.numel()
        if inp is None:
            out = torch.empty(n, dtype=torch.int32, device=stencil.device)
            vb = 4
        else:
            if not inp.is_cuda or not inp.is_contiguous() or inp.shape[0] != n:
                raise capi.ErrorControlBadValue(capi.ERROR_BAD_VALUE,
                                                "input must be contiguous, one row per stencil entry")
            out = torch.empty_like(inp)
            vb = _row_bytes(inp) if n else 4
        nb = capi.lib().dax_gb300_compact_scratch_bytes(n, 0)
        scratch = torch.empty(nb, dtype=torch.uint8, device=stencil.device)
        cnt = ctypes.c_int64(0)
        capi.call("dax_gb300_stream_compact", _ptr(inp), vb, _ptr(stencil), st, n, _ptr(out),
                  _ptr(scratch), nb, ctypes.byref(cnt), _stream(stream))
        return out[:cnt.value]

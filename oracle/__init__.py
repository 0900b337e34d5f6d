"""numpy front end for the CPU oracle (test infrastructure only).

``Oracle("port")`` loads the C restatement (``dax_oracle.c``);
``Oracle("reference")`` loads ``ref_driver.cpp`` built against the DaxToolkit's
own worklet headers (present only where the reference tree could be compiled).
Both expose the same calls with the same argument meaning, so a test can run
one against the other.  Nothing in the product package imports this module.
"""
import ctypes
import os

import numpy as np

from . import build as _build


class GridDesc(ctypes.Structure):
    """Uniform grid: origin, spacing, point extent [min, max] (inclusive)."""

    _fields_ = [("origin", ctypes.c_float * 3), ("spacing", ctypes.c_float * 3),
                ("extent_min", ctypes.c_int32 * 3), ("extent_max", ctypes.c_int32 * 3)]


def make_grid(dims, origin=(0.0, 0.0, 0.0), spacing=(1.0, 1.0, 1.0), extent_min=(0, 0, 0)):
    g = GridDesc()
    for a in range(3):
        g.origin[a] = origin[a]
        g.spacing[a] = spacing[a]
        g.extent_min[a] = extent_min[a]
        g.extent_max[a] = extent_min[a] + dims[a] - 1
    return g


def grid_dims(g):
    return tuple(int(g.extent_max[a] - g.extent_min[a] + 1) for a in range(3))


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class Oracle:
    def __init__(self, kind="port"):
        self.kind = kind
        if kind == "port":
            path, prefix = _build.build_oracle(), "orc_"
        elif kind == "reference":
            path, prefix = _build.build_ref(), "ref_"
            if path is None or not os.path.exists(path):
                raise RuntimeError("reference oracle not built (DaxToolkit tree unavailable)")
        else:
            raise ValueError(kind)
        self.lib = ctypes.CDLL(path)
        self._p = prefix
        L = self.lib
        vp, f32, i64 = ctypes.c_void_p, ctypes.c_float, ctypes.c_int64
        gp = ctypes.POINTER(GridDesc)
        self._count = getattr(L, prefix + "mc_count")
        self._count.argtypes = [gp, vp, f32, vp, vp]
        self._gen = getattr(L, prefix + "mc_generate")
        self._gen.argtypes = [gp, vp, f32, vp, ctypes.c_int, vp, vp, vp, vp, vp,
                              ctypes.POINTER(i64)]
        self._gen.restype = i64
        self._interp = getattr(L, prefix + "interpolate_point_field")
        self._interp.argtypes = [vp, vp, vp, i64, vp, vp]
        self._thr_count = getattr(L, prefix + "threshold_count")
        self._thr_count.argtypes = [gp, vp, f32, f32, vp]
        self._thr_gen = getattr(L, prefix + "threshold_generate")
        self._thr_gen.argtypes = [gp, vp, vp, vp, vp, vp, ctypes.POINTER(i64)]
        self._thr_gen.restype = i64
        self._grad = getattr(L, prefix + "cell_gradient")
        self._grad.argtypes = [gp, vp, vp]
        self._slice_count = getattr(L, prefix + "slice_count")
        self._slice_count.argtypes = [gp, vp, vp, vp]
        self._slice_gen = getattr(L, prefix + "slice_generate")
        self._slice_gen.argtypes = [gp, vp, vp, vp, ctypes.c_int, vp, vp, vp, vp, vp,
                                    ctypes.POINTER(i64)]
        self._slice_gen.restype = i64
        self._magnitude = getattr(L, prefix + "point_magnitude")
        self._magnitude.argtypes = [gp, vp]
        self._tetra = getattr(L, prefix + "tetrahedralize")
        self._tetra.argtypes = [gp, vp]
        if kind == "port":
            L.orc_mandelbulb_field.argtypes = [gp, vp]
            L.orc_colors_and_norms.argtypes = [vp, i64, vp, vp]
            L.orc_mandelbulb_clip_count.argtypes = [gp, vp, ctypes.c_float, vp, vp, vp, vp]
        self._mt_count = getattr(L, prefix + "mt_count")
        self._mt_count.argtypes = [vp, i64, vp, ctypes.c_float, vp]
        self._mt_gen = getattr(L, prefix + "mt_generate")
        self._mt_gen.argtypes = [vp, vp, i64, vp, ctypes.c_float, vp, ctypes.c_int, vp, vp, vp, vp,
                                 vp, ctypes.POINTER(i64)]
        self._mt_gen.restype = i64
        if kind == "reference":
            L.ref_set_threads.argtypes = [ctypes.c_int]
            L.ref_max_threads.restype = ctypes.c_int

    # -- threading (reference driver only; the C port is single-threaded) --
    def set_threads(self, n):
        if self.kind == "reference":
            self.lib.ref_set_threads(int(n))
            return int(n)
        return 1

    def max_threads(self):
        return int(self.lib.ref_max_threads()) if self.kind == "reference" else 1

    @staticmethod
    def _points(g):
        d = grid_dims(g)
        return d[0] * d[1] * d[2]

    @staticmethod
    def _cells(g):
        d = grid_dims(g)
        return 0 if min(d) < 2 else (d[0] - 1) * (d[1] - 1) * (d[2] - 1)

    def mc_count(self, g, field, iso):
        field = np.ascontiguousarray(field, dtype=np.float32).ravel()
        C = self._cells(g)
        count = np.zeros(C, np.int32)
        cases = np.zeros(C, np.uint8)
        self._count(ctypes.byref(g), _ptr(field), float(iso), _ptr(count), _ptr(cases))
        return count, cases

    def mc_generate(self, g, field, iso, count, merge=True):
        """Returns dict(verts [V,3] f32, conn [T,3] i32, rec_a, rec_b, rec_w)."""
        field = np.ascontiguousarray(field, dtype=np.float32).ravel()
        count = np.ascontiguousarray(count, dtype=np.int32)
        T = int(count.astype(np.int64).sum())
        cap = max(3 * T, 1)
        verts = np.zeros((cap, 3), np.float32)
        conn = np.zeros(cap, np.int32)
        ra = np.zeros(cap, np.int32)
        rb = np.zeros(cap, np.int32)
        rw = np.zeros(cap, np.float32)
        nv = ctypes.c_int64(0)
        t = self._gen(ctypes.byref(g), _ptr(field), float(iso), _ptr(count), int(bool(merge)),
                      _ptr(verts), _ptr(conn), _ptr(ra), _ptr(rb), _ptr(rw), ctypes.byref(nv))
        assert t == T
        V = nv.value
        return dict(verts=verts[:V], conn=conn[:3 * T].reshape(T, 3), rec_a=ra[:V], rec_b=rb[:V],
                    rec_w=rw[:V])

    def interpolate_point_field(self, rec_a, rec_b, rec_w, field):
        field = np.ascontiguousarray(field, dtype=np.float32).ravel()
        out = np.zeros(len(rec_a), np.float32)
        self._interp(_ptr(np.ascontiguousarray(rec_a)), _ptr(np.ascontiguousarray(rec_b)),
                     _ptr(np.ascontiguousarray(rec_w)), len(rec_a), _ptr(field), _ptr(out))
        return out

    def threshold_count(self, g, field, lo, hi):
        field = np.ascontiguousarray(field, dtype=np.float32).ravel()
        count = np.zeros(self._cells(g), np.int32)
        self._thr_count(ctypes.byref(g), _ptr(field), float(lo), float(hi), _ptr(count))
        return count

    def threshold_generate(self, g, field, count):
        """Returns dict(conn [K,8] i32, coords [U,3] f32, field [U] f32)."""
        field = np.ascontiguousarray(field, dtype=np.float32).ravel()
        count = np.ascontiguousarray(count, dtype=np.int32)
        K = int(count.astype(np.int64).sum())
        P = field.size
        conn = np.zeros(max(8 * K, 1), np.int32)
        coords = np.zeros((max(P, 1), 3), np.float32)
        fout = np.zeros(max(P, 1), np.float32)
        pu = ctypes.c_int64(0)
        k = self._thr_gen(ctypes.byref(g), _ptr(field), _ptr(count), _ptr(conn), _ptr(coords),
                          _ptr(fout), ctypes.byref(pu))
        assert k == K
        U = pu.value
        return dict(conn=conn[:8 * K].reshape(K, 8), coords=coords[:U], field=fout[:U])

    @staticmethod
    def threshold_compact_point_field(g, count, field):
        """CompactPointField of the threshold dispatcher
        (dax/cont/DispatcherGenerateTopology.h:98-113): FillPointMask over the
        kept cells' 8 corner ids (:206-227, corners in TopologyUniform order,
        dax/exec/internal/TopologyUniform.h:150-157), then StreamCompact of
        the point field ([P] or [P, k]) with that mask
        (DeviceAdapterAlgorithmGeneral.h:769-830): the used points' values
        in point order."""
        nx, ny, nz = grid_dims(g)
        cx, cy = nx - 1, ny - 1
        kept = np.nonzero(np.asarray(count))[0].astype(np.int64)
        p = kept % cx + nx * ((kept // cx) % cy + ny * (kept // (cx * cy)))
        off = np.array([0, 1, nx + 1, nx, nx * ny, nx * ny + 1, nx * ny + nx + 1, nx * ny + nx],
                       np.int64)
        mask = np.zeros(nx * ny * nz, bool)
        mask[(p[:, None] + off[None, :]).ravel()] = True
        return np.asarray(field)[mask]

    def slice_count(self, g, origin, normal):
        o = np.asarray(origin, np.float32)
        nrm = np.asarray(normal, np.float32)
        count = np.zeros(self._cells(g), np.int32)
        self._slice_count(ctypes.byref(g), _ptr(o), _ptr(nrm), _ptr(count))
        return count

    def slice_generate(self, g, origin, normal, count, merge=True):
        """Returns dict(verts, conn, rec_a, rec_b, rec_w) as mc_generate."""
        o = np.asarray(origin, np.float32)
        nrm = np.asarray(normal, np.float32)
        count = np.ascontiguousarray(count, dtype=np.int32)
        T = int(count.astype(np.int64).sum())
        cap = max(3 * T, 1)
        verts = np.zeros((cap, 3), np.float32)
        conn = np.zeros(cap, np.int32)
        ra = np.zeros(cap, np.int32)
        rb = np.zeros(cap, np.int32)
        rw = np.zeros(cap, np.float32)
        nv = ctypes.c_int64(0)
        t = self._slice_gen(ctypes.byref(g), _ptr(o), _ptr(nrm), _ptr(count), int(bool(merge)),
                            _ptr(verts), _ptr(conn), _ptr(ra), _ptr(rb), _ptr(rw), ctypes.byref(nv))
        assert t == T
        V = nv.value
        return dict(verts=verts[:V], conn=conn[:3 * T].reshape(T, 3), rec_a=ra[:V], rec_b=rb[:V],
                    rec_w=rw[:V])

    def point_magnitude(self, g):
        """Magnitude of every grid point's coordinates."""
        out = np.zeros(self._points(g), np.float32)
        self._magnitude(ctypes.byref(g), _ptr(out))
        return out

    def tetrahedralize(self, g):
        """Tetrahedralize over the grid: int32 [5 * cells, 4]."""
        conn = np.zeros((5 * self._cells(g), 4), np.int32)
        self._tetra(ctypes.byref(g), _ptr(conn))
        return conn

    # -- Mandelbulb benchmark pipeline (C restatement only: the reference's
    #    worklets there need Boost.Preprocessor, absent from this image) --
    def mandelbulb_field(self, g):
        out = np.zeros(self._points(g), np.float32)
        self._port().orc_mandelbulb_field(ctypes.byref(g), _ptr(out))
        return out

    def colors_and_norms(self, verts):
        verts = np.ascontiguousarray(verts, dtype=np.float32).reshape(-1, 3)
        norms = np.zeros_like(verts)
        colors = np.zeros((verts.shape[0], 4), np.uint8)
        self._port().orc_colors_and_norms(_ptr(verts), verts.shape[0], _ptr(norms), _ptr(colors))
        return norms, colors

    def mandelbulb_clip_count(self, g, field, iso, origin, location, normal):
        field = np.ascontiguousarray(field, dtype=np.float32).ravel()
        vec = lambda v: np.asarray(v, np.float32)
        o, l, n = vec(origin), vec(location), vec(normal)
        count = np.zeros(self._cells(g), np.int32)
        self._port().orc_mandelbulb_clip_count(ctypes.byref(g), _ptr(field), float(iso), _ptr(o),
                                               _ptr(l), _ptr(n), _ptr(count))
        return count

    def _port(self):
        if self.kind == "port":
            return self.lib
        if not hasattr(self, "_port_lib"):
            self._port_lib = Oracle("port").lib
        return self._port_lib

    def mt_count(self, conn, field, iso):
        """MarchingTetrahedraCount per tetrahedron; conn is int32 [C, 4]."""
        conn = np.ascontiguousarray(conn, dtype=np.int32).reshape(-1, 4)
        field = np.ascontiguousarray(field, dtype=np.float32).ravel()
        count = np.zeros(conn.shape[0], np.int32)
        self._mt_count(_ptr(conn), conn.shape[0], _ptr(field), float(iso), _ptr(count))
        return count

    def mt_generate(self, points, conn, field, iso, count, merge=True):
        """Returns dict(verts, conn, rec_a, rec_b, rec_w) as mc_generate."""
        points = np.ascontiguousarray(points, dtype=np.float32).reshape(-1, 3)
        conn = np.ascontiguousarray(conn, dtype=np.int32).reshape(-1, 4)
        field = np.ascontiguousarray(field, dtype=np.float32).ravel()
        count = np.ascontiguousarray(count, dtype=np.int32)
        T = int(count.astype(np.int64).sum())
        cap = max(3 * T, 1)
        verts = np.zeros((cap, 3), np.float32)
        tconn = np.zeros(cap, np.int32)
        ra = np.zeros(cap, np.int32)
        rb = np.zeros(cap, np.int32)
        rw = np.zeros(cap, np.float32)
        nv = ctypes.c_int64(0)
        t = self._mt_gen(_ptr(points), _ptr(conn), conn.shape[0], _ptr(field), float(iso),
                         _ptr(count), int(bool(merge)), _ptr(verts), _ptr(tconn), _ptr(ra),
                         _ptr(rb), _ptr(rw), ctypes.byref(nv))
        assert t == T
        V = nv.value
        return dict(verts=verts[:V], conn=tconn[:3 * T].reshape(T, 3), rec_a=ra[:V],
                    rec_b=rb[:V], rec_w=rw[:V])

    def cell_gradient(self, g, field):
        field = np.ascontiguousarray(field, dtype=np.float32).ravel()
        out = np.zeros((self._cells(g), 3), np.float32)
        self._grad(ctypes.byref(g), _ptr(field), _ptr(out))
        return out


class Fp64Twin:
    """The reference-built driver compiled with the DaxToolkit's own
    DAX_USE_DOUBLE_PRECISION option (dax::Scalar = double): the same worklets
    on the same float32 field and grid description, evaluated in double.  Its
    marching-cubes weights and positions and its cell gradients are returned
    as float64 -- the FP64 values that the float32 results' errors are stated
    against.  Topology and output order equal the float32 driver's whenever
    the case decisions do (they compare the same float32 values)."""

    def __init__(self):
        path = _build.build_ref(variant="f64")
        if path is None or not os.path.exists(path):
            raise RuntimeError("FP64 reference twin not built (DaxToolkit tree unavailable)")
        L = self.lib = ctypes.CDLL(path)
        vp, f32, i64 = ctypes.c_void_p, ctypes.c_float, ctypes.c_int64
        gp = ctypes.POINTER(GridDesc)
        L.ref64_mc_count.argtypes = [gp, vp, f32, vp, vp]
        L.ref64_mc_generate.argtypes = [gp, vp, f32, vp, ctypes.c_int, vp, vp, vp, vp, vp,
                                        ctypes.POINTER(i64)]
        L.ref64_mc_generate.restype = i64
        L.ref64_cell_gradient.argtypes = [gp, vp, vp]
        L.ref64_set_threads.argtypes = [ctypes.c_int]
        L.ref64_max_threads.restype = ctypes.c_int
        L.ref64_set_threads(int(L.ref64_max_threads()))

    def mc_generate(self, g, field, iso, merge=True):
        """Count and generate in FP64: dict(verts [V,3] f64, conn [T,3] i32,
        rec_a, rec_b, rec_w f64)."""
        field = np.ascontiguousarray(field, dtype=np.float32).ravel()
        C = Oracle._cells(g)
        count = np.zeros(C, np.int32)
        self.lib.ref64_mc_count(ctypes.byref(g), _ptr(field), float(iso), _ptr(count), None)
        T = int(count.astype(np.int64).sum())
        cap = max(3 * T, 1)
        verts = np.zeros((cap, 3), np.float64)
        conn = np.zeros(cap, np.int32)
        ra = np.zeros(cap, np.int32)
        rb = np.zeros(cap, np.int32)
        rw = np.zeros(cap, np.float64)
        nv = ctypes.c_int64(0)
        t = self.lib.ref64_mc_generate(ctypes.byref(g), _ptr(field), float(iso), _ptr(count),
                                       int(bool(merge)), _ptr(verts), _ptr(conn), _ptr(ra),
                                       _ptr(rb), _ptr(rw), ctypes.byref(nv))
        assert t == T
        V = nv.value
        return dict(verts=verts[:V], conn=conn[:3 * T].reshape(T, 3), rec_a=ra[:V], rec_b=rb[:V],
                    rec_w=rw[:V])

    def cell_gradient(self, g, field):
        field = np.ascontiguousarray(field, dtype=np.float32).ravel()
        out = np.zeros((Oracle._cells(g), 3), np.float64)
        self.lib.ref64_cell_gradient(ctypes.byref(g), _ptr(field), _ptr(out))
        return out

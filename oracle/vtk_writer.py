"""Legacy-VTK POLYDATA text as the reference's PrintContentsToStream writes it
(Benchmarks/MarchingCubes/Pipeline.h:51-98) -- TEST INFRASTRUCTURE ONLY, the
checker for dax_gb300_write_vtk_polydata.

std::ostream prints a float as printf's %g of its double value with precision
6 and an int in decimal; std::endl is a newline.  Python's "%g" rounds the
same way; only the sign of a NaN needs care (glibc prints "-nan")."""
import math

import numpy as np


def _g(x):
    x = float(x)
    if math.isnan(x):
        return "-nan" if math.copysign(1.0, x) < 0 else "nan"
    return "%g" % x


def polydata_text(points, conn):
    """points [P, 3] float32, conn [C, V] int: the file's bytes."""
    points = np.asarray(points, np.float32).reshape(-1, 3)
    conn = np.asarray(conn)
    if conn.ndim == 1:
        conn = conn.reshape(-1, 3)
    out = ["# vtk DataFile Version 3.0\n", "vtk output\n", "ASCII\n", "DATASET POLYDATA\n",
           "POINTS %d float\n" % points.shape[0]]
    for i, p in enumerate(points):
        out.append("%s %s %s " % (_g(p[0]), _g(p[1]), _g(p[2])))
        if i % 3 == 2:
            out.append("\n")
    if points.shape[0] % 3:
        out.append("\n")
    V = conn.shape[1]
    out.append("POLYGONS %d %d\n" % (conn.shape[0], conn.shape[0] * (V + 1)))
    for c in conn:
        out.append("%d %s\n" % (V, " ".join("%d" % int(v) for v in c)))
    out.append("\n")
    return "".join(out).encode()

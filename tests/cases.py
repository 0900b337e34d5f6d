"""Seeded parity cases shared by the CPU and GPU tests (small enough for the
CPU oracle to finish in well under a second each)."""
import numpy as np


def linear_field(dims, grad=(1.0, 1.0, 1.0), origin=(0, 0, 0), spacing=(1, 1, 1), emin=(0, 0, 0)):
    """x*gx + y*gy + z*gz on the grid's float coordinates (the reference's
    unit-test fields, e.g. UnitTestWorkletMarchingCubes.cxx:94-101)."""
    nx, ny, nz = dims
    ax = [np.float32(origin[a]) + np.float32(spacing[a]) *
          (np.arange(dims[a]) + emin[a]).astype(np.float32) for a in range(3)]
    z, y, x = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    return (x * np.float32(grad[0]) + y * np.float32(grad[1]) + z * np.float32(grad[2])) \
        .astype(np.float32).ravel()


def all_cases_strip(iso=0.0, seed=5):
    """A 769 x 2 x 2 grid whose cells at i = 3c have case index c for all 256
    marching-cubes cases (other cells get whatever their points give)."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = 3 * 256 + 1, 2, 2
    f = rng.uniform(-1, 1, size=(nz, ny, nx)).astype(np.float32)
    corners = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
    for c in range(256):
        for n, (di, dj, dk) in enumerate(corners):
            f[dk, dj, 3 * c + di] = iso + (0.5 if (c >> n) & 1 else -0.5)
    return (nx, ny, nz), f.ravel()


def random_blobs(dims, nblobs, seed, noise=0.0):
    rng = np.random.default_rng(seed)
    c = rng.uniform(0.1, 0.9, size=(nblobs, 3))
    s = rng.uniform(0.05, 0.15, size=nblobs)
    ax = [np.arange(dims[a]) / max(dims[a] - 1, 1) for a in range(3)]
    z, y, x = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    f = np.zeros_like(x)
    for b in range(nblobs):
        f += np.exp(-((x - c[b, 0]) ** 2 + (y - c[b, 1]) ** 2 + (z - c[b, 2]) ** 2) / (2 * s[b] ** 2))
    if noise:
        f += noise * rng.uniform(-1, 1, size=f.shape)
    return f.astype(np.float32).ravel()


def sphere(dims, noise=0.01, seed=1234):
    rng = np.random.default_rng(seed)
    ax = [np.arange(dims[a]) / (dims[a] - 1) for a in range(3)]
    z, y, x = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    r = np.sqrt((x - 0.5) ** 2 + (y - 0.5) ** 2 + (z - 0.5) ** 2)
    return (r + noise * rng.uniform(-1, 1, size=r.shape)).astype(np.float32).ravel()


def wide_exponent_field(dims, seed):
    """Values of random sign whose exponents spread over the whole float32
    range, by thirds of the z-planes: magnitudes in [2^-60, 2^86) (the band in
    which the GPU gradient takes its fused path), then down to subnormals,
    then up to 2^128 with infinities and NaNs; +0 and -0 throughout, and the
    band's edge values 2^-60, 2^86 and their neighbours placed explicitly."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = dims
    n = nx * ny
    third = max(nz // 3, 1)
    f = np.empty((nz, n), np.float32)
    for k in range(nz):
        lo, hi = (-60, 86) if k < third else ((-150, -40) if k < 2 * third else (40, 128))
        m = np.exp2(rng.uniform(lo, hi, n)).astype(np.float32)
        m = np.where(rng.uniform(size=n) < 0.5, -m, m).astype(np.float32)
        z = rng.uniform(size=n)
        m[z < 0.08] = 0.0
        m[(z >= 0.08) & (z < 0.11)] = -0.0
        f[k] = m
    edges = np.array([2.0 ** -60, -(2.0 ** -60), np.nextafter(np.float32(2.0 ** 86), np.float32(0))],
                     np.float32)
    f[1, :edges.size] = edges
    f[third, :4] = np.array([np.nextafter(np.float32(2.0 ** -60), np.float32(0)), 2.0 ** 86,
                             -(2.0 ** 86), 2.0 ** -126], np.float32)
    if nz > 2 * third:
        f[2 * third, :3] = np.array([np.inf, -np.inf, np.nan], np.float32)
    return f.ravel()


def mc_cases():
    """(name, dims, origin, spacing, extent_min, field, isovalue)."""
    out = []
    out.append(("kat26_linear", (26, 26, 26), (0, 0, 0), (1, 1, 1), (0, 0, 0),
                linear_field((26, 26, 26)), 70.0))
    out.append(("sphere64", (64, 64, 64), (0, 0, 0), (1 / 63,) * 3, (0, 0, 0),
                sphere((64, 64, 64)), 0.35))
    d = (48, 40, 36)
    out.append(("blobs_48x40x36", d, (0, 0, 0), tuple(1 / (n - 1) for n in d), (0, 0, 0),
                random_blobs(d, 4, 11, noise=0.05), 0.5))
    d = (33, 17, 5)
    out.append(("odd_33x17x5_offset", d, (-1.5, 2.25, 0.125), (0.3, 0.7, 1.1), (3, -2, 7),
                random_blobs(d, 3, 12), 0.4))
    d, f = all_cases_strip()
    out.append(("all256_strip", d, (0, 0, 0), (1, 1, 1), (0, 0, 0), f, 0.0))
    d = (70, 3, 4)
    out.append(("wide_x_70x3x4", d, (0, 0, 0), (0.1, 0.2, 0.3), (0, 0, 0),
                random_blobs(d, 2, 13, noise=0.3), 0.5))
    d = (2, 2, 2)
    out.append(("single_cell", d, (0, 0, 0), (1, 1, 1), (0, 0, 0),
                np.array([1, -1, 1, -1, -1, 1, 1, -1], np.float32), 0.0))
    d = (20, 20, 20)
    f = random_blobs(d, 3, 14)
    f[::7] = np.nan
    out.append(("nan_sprinkled", d, (0, 0, 0), (1, 1, 1), (0, 0, 0), f, 0.5))
    out.append(("all_inside", (9, 8, 7), (0, 0, 0), (1, 1, 1), (0, 0, 0),
                np.ones(9 * 8 * 7, np.float32), 0.0))
    out.append(("flat_no_cells", (16, 16, 1), (0, 0, 0), (1, 1, 1), (0, 0, 0),
                random_blobs((16, 16, 1), 2, 15), 0.3))
    d = (130, 9, 6)
    out.append(("x130_two_words_tail", d, (0, 0, 0), (1, 1, 1), (0, 0, 0),
                random_blobs(d, 5, 16, noise=0.2), 0.45))
    return out


def threshold_cases():
    out = []
    out.append(("kat26_linear", (26, 26, 26), (0, 0, 0), (1, 1, 1), (0, 0, 0),
                linear_field((26, 26, 26)), 70.0, 82.0))
    d = (48, 40, 36)
    out.append(("blobs_48x40x36", d, (0, 0, 0), tuple(1 / (n - 1) for n in d), (0, 0, 0),
                random_blobs(d, 4, 11, noise=0.05), 0.3, 0.7))
    d = (33, 17, 5)
    out.append(("odd_33x17x5_offset", d, (-1.5, 2.25, 0.125), (0.3, 0.7, 1.1), (3, -2, 7),
                random_blobs(d, 3, 12), 0.1, 0.6))
    d = (130, 9, 6)
    out.append(("x130", d, (0, 0, 0), (1, 1, 1), (0, 0, 0), random_blobs(d, 5, 16, noise=0.2),
                0.2, 0.8))
    # rows of exactly 4 and of 8 bit words (the count passes take four words
    # of one row at a time), with an extent offset; and a row of 3 words,
    # whose 4-word groups all straddle rows
    d = (100, 11, 7)
    out.append(("wr4_100x11x7_offset", d, (0.5, -1.0, 2.0), (0.01, 0.1, 0.2), (-7, 3, 1),
                random_blobs(d, 4, 21, noise=0.1), -0.2, 0.5))
    d = (250, 6, 5)
    out.append(("wr8_250x6x5", d, (0, 0, 0), (1, 1, 1), (0, 0, 0), random_blobs(d, 6, 22, noise=0.1),
                -0.05, 0.4))
    d = (70, 13, 9)
    out.append(("wr3_70x13x9", d, (0, 0, 0), (1, 1, 1), (0, 0, 0), random_blobs(d, 3, 23, noise=0.1),
                -0.2, 0.5))
    out.append(("none_kept", (9, 8, 7), (0, 0, 0), (1, 1, 1), (0, 0, 0),
                np.ones(9 * 8 * 7, np.float32), 2.0, 3.0))
    out.append(("all_kept", (9, 8, 7), (0, 0, 0), (1, 1, 1), (0, 0, 0),
                np.ones(9 * 8 * 7, np.float32), 0.0, 3.0))
    return out


def gradient_cases():
    out = []
    out.append(("kat8_linear", (8, 8, 8), (0, 0, 0), (1, 1, 1), (0, 0, 0),
                linear_field((8, 8, 8))))
    out.append(("sphere64", (64, 64, 64), (0, 0, 0), (1 / 63,) * 3, (0, 0, 0), sphere((64, 64, 64))))
    d = (33, 17, 5)
    out.append(("odd_33x17x5_offset", d, (-1.5, 2.25, 0.125), (0.3, 0.7, 1.1), (3, -2, 7),
                random_blobs(d, 3, 12)))
    # ragged tiles in every direction (69 cells in x, 18 rows, 40 planes) and a
    # far origin, so the cell widths differ by rounding from column to column
    d = (70, 19, 41)
    out.append(("ragged_70x19x41_far", d, (1000.0, -4.1, 250.0), (0.013, 0.7, 0.05), (-5, 2, 100),
                random_blobs(d, 4, 17, noise=0.1)))
    # exact tiles: 32 cells in x, 8 rows, 33 planes (one plane past a segment)
    d = (33, 9, 34)
    out.append(("exact_tiles_33x9x34", d, (0, 0, 0), (1, 1, 1), (0, 0, 0), random_blobs(d, 3, 18)))
    out.append(("single_cell", (2, 2, 2), (0.5, 0.5, 0.5), (2.0, 3.0, 4.0), (0, 0, 0),
                np.arange(8, dtype=np.float32) ** 2))
    # exponents over the whole float32 range: both of the GPU kernel's paths,
    # chosen plane by plane, within one grid (2 column tiles, ragged bands, 2
    # plane segments)
    d = (40, 11, 37)
    out.append(("wide_exponents_40x11x37", d, (0, 0, 0), (1, 1, 1), (0, 0, 0),
                wide_exponent_field(d, 29)))
    # cell widths at the edges of the fused path's width band [2^-30, 2^30)
    # and outside it (1e-12 in x, 3e9 in y, exactly 2^30 in z)
    d = (35, 9, 6)
    out.append(("widths_in_band_edges", d, (0, 0, 0), (2.0 ** -30, 0.75 * 2.0 ** 30, 1.0), (0, 0, 0),
                random_blobs(d, 3, 31, noise=0.05)))
    out.append(("widths_outside_band", d, (0, 0, 0), (1e-12, 3e9, 2.0 ** 30), (0, 0, 0),
                random_blobs(d, 3, 32, noise=0.05)))
    return out


def slice_cases():
    """(name, dims, origin, spacing, extent_min, plane_origin, plane_normal).

    dax::worklet::Slice compares dot(N, x - O) against dot(N, O)
    (Slice.h:60-70), so the surface cut is the plane dot(N, x) = 2 dot(N, O);
    the cases are chosen against that plane."""
    out = []
    # UnitTestWorkletSlice.cxx:22-24 -- 8^3 unit grid, O=(3,2,1), N=(1,0,0):
    # the cut x = 6 runs through grid points; 98 triangles, 64 merged points
    out.append(("kat8_axis_x", (8, 8, 8), (0, 0, 0), (1, 1, 1), (0, 0, 0), (3, 2, 1), (1, 0, 0)))
    out.append(("axis_z_between", (12, 10, 9), (0, 0, 0), (1, 1, 1), (0, 0, 0),
                (0, 0, 1.7), (0, 0, 1)))
    out.append(("oblique_offset", (30, 24, 18), (-1, 0.5, 2), (0.1, 0.13, 0.2), (2, -3, 1),
                (0.7, 0.9, 3.1), (0.3, -0.5, 0.81)))
    out.append(("nonunit_normal", (41, 33, 20), (0, 0, 0), (0.05, 0.05, 0.05), (0, 0, 0),
                (0.4, 0.3, 0.2), (2.5, 1.25, -3.0)))
    out.append(("misses_grid", (10, 10, 10), (0, 0, 0), (1, 1, 1), (0, 0, 0), (50, 0, 0), (1, 0, 0)))
    out.append(("single_cell", (2, 2, 2), (0, 0, 0), (1, 1, 1), (0, 0, 0),
                (0.2, 0.25, 0.3), (1, 1, 1)))
    out.append(("diagonal_x130", (130, 9, 6), (-3, -1, -1), (0.05, 0.25, 0.4), (0, 0, 0),
                (0.5, 0.2, 0.1), (1, 1, 1)))
    out.append(("far_origin", (37, 21, 25), (1000.0, -4.1, 250.0), (0.013, 0.7, 0.05), (-5, 2, 100),
                (500.1, -1.0, 127.6), (0.6, 0.0, -0.8)))
    # a normal with zero x component: every row is all inside or all outside
    out.append(("rows_constant", (45, 12, 11), (0, 0, 0), (0.1, 0.1, 0.1), (0, 0, 0),
                (0.2, 0.31, 0.4), (0.0, 0.6, 0.8)))
    # negative spacing along x and a negative normal: the inside part of each
    # row is a prefix, then a suffix
    out.append(("negative_spacing", (50, 13, 9), (5, 0, 0), (-0.2, 0.25, 0.5), (1, 0, 0),
                (1.0, 1.1, 1.2), (0.7, -0.2, 0.3)))
    out.append(("negative_normal", (50, 13, 9), (0, 0, 0), (0.2, 0.25, 0.5), (0, 0, 0),
                (1.0, 1.1, 1.2), (-0.7, -0.2, 0.3)))
    # values that overflow to infinity, and a NaN normal: the per-point path
    out.append(("overflow_inf", (9, 7, 5), (0, 0, 0), (3e37, 1, 1), (0, 0, 0),
                (1e38, 0.0, 0.0), (3.0, 0.5, 0.25)))
    out.append(("nan_normal", (9, 7, 5), (0, 0, 0), (1, 1, 1), (0, 0, 0),
                (1.0, 2.0, 3.0), (float("nan"), 0.0, 1.0)))
    return out


# Freudenthal subdivision of each hexahedron into 6 tetrahedra, in the
# reference test grid's order (dax/cont/testing/TestingGridGenerator.h:
# 301-330): voxel corner lists, corners in TopologyUniform order.
_FREUDENTHAL = ((0, 2, 3, 6), (0, 3, 7, 6), (0, 7, 4, 6), (0, 5, 6, 4), (1, 5, 6, 0), (1, 6, 2, 0))
_CORNER = ((0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1))


def tetrahedralize(dims):
    """int32 [6*C, 4] connectivity of the uniform grid `dims` (points x
    fastest), cells in id order, 6 tetrahedra per cell."""
    nx, ny, nz = dims
    k, j, i = np.meshgrid(np.arange(nz - 1), np.arange(ny - 1), np.arange(nx - 1), indexing="ij")
    first = (i + nx * (j + ny * k)).ravel().astype(np.int64)
    off = np.array([dx + nx * (dy + ny * dz) for dx, dy, dz in _CORNER], np.int64)
    tets = np.array(_FREUDENTHAL, np.int64)  # [6, 4] corner ids
    conn = first[:, None, None] + off[tets][None, :, :]
    return conn.reshape(-1, 4).astype(np.int32)


def grid_points(dims, origin=(0, 0, 0), spacing=(1, 1, 1)):
    """float32 [P, 3] coordinates origin + spacing * ijk, x fastest."""
    f32 = np.float32
    ax = [f32(origin[a]) + f32(spacing[a]) * np.arange(dims[a]).astype(f32) for a in range(3)]
    z, y, x = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    return np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1).astype(f32)


def shuffle_mesh(points, conn, field, seed):
    """The same mesh with point ids permuted, cells reordered and each
    cell's vertex list rotated (an even permutation)."""
    rng = np.random.default_rng(seed)
    P = points.shape[0]
    perm = rng.permutation(P)           # new id of old point p is inv[p]
    inv = np.empty(P, np.int64)
    inv[perm] = np.arange(P)
    pts = points[perm]
    fld = field[perm]
    c = inv[conn.astype(np.int64)]
    c = c[rng.permutation(c.shape[0])]
    rot = rng.integers(0, 3, size=c.shape[0])
    out = c.copy()
    for r in (1, 2):  # cycle vertices 1..3, which keeps the orientation
        m = rot == r
        out[m, 1:] = np.roll(c[m, 1:], r, axis=1)
    return pts, out.astype(np.int32), fld


def all_tet_cases():
    """16 separate tetrahedra, tetrahedron c in marching case c."""
    pts, conn, f = [], [], []
    base = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], np.float32)
    for c in range(16):
        pts.append(base + np.float32(2 * c))
        conn.append(np.arange(4) + 4 * c)
        f.extend(1.0 if (c >> n) & 1 else -1.0 for n in range(4))
    return (np.concatenate(pts).astype(np.float32), np.array(conn, np.int32),
            np.array(f, np.float32))


def mt_cases():
    """(name, points [P,3] f32, conn [C,4] i32, field [P] f32, isovalue)."""
    out = []
    # UnitTestWorkletMarchingTetrahedra.cxx:33-34, :50-60 -- 26^3 grid split
    # 6 ways, field x+y+z, isovalue 70: 151 merged points
    d = (26, 26, 26)
    out.append(("kat26_linear", grid_points(d), tetrahedralize(d), linear_field(d), 70.0))
    d = (20, 17, 13)
    sp = tuple(1 / (n - 1) for n in d)
    bl = random_blobs(d, 3, 21, noise=0.05)
    out.append(("blobs_20x17x13", grid_points(d, spacing=sp), tetrahedralize(d), bl, 0.5))
    pts, conn, fld = shuffle_mesh(grid_points(d, spacing=sp), tetrahedralize(d), bl, 22)
    out.append(("blobs_shuffled", pts, conn, fld, 0.5))
    pts, conn, fld = all_tet_cases()
    out.append(("all16_cases", pts, conn, fld, 0.0))
    d = (12, 11, 10)
    f = random_blobs(d, 2, 23)
    f[::5] = np.nan
    out.append(("nan_sprinkled", grid_points(d), tetrahedralize(d), f, 0.4))
    out.append(("all_inside", grid_points((5, 4, 3)), tetrahedralize((5, 4, 3)),
                np.ones(60, np.float32), 0.0))
    # tetrahedra with a repeated point id: zero-length edges, 0/0 weights
    pts = grid_points((3, 3, 2))
    f = np.linspace(-1, 1, 18).astype(np.float32)
    conn = np.array([[0, 0, 4, 13], [1, 5, 5, 9], [2, 3, 14, 14], [4, 10, 11, 12]], np.int32)
    out.append(("degenerate_ids", pts, conn, f, 0.05))
    d = (48, 40, 36)
    sp = tuple(1 / (n - 1) for n in d)
    out.append(("blobs_48x40x36", grid_points(d, spacing=sp), tetrahedralize(d),
                random_blobs(d, 4, 11, noise=0.05), 0.5))
    return out

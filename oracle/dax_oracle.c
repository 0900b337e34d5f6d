/*
 * CPU oracle for the uniform-grid isosurface / threshold / gradient path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, step by step, what the Dax
 * Serial device adapter computes for the hot path so that the CUDA kernels can
 * be checked against it.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg may load it; the product library never links it.
 *
 * Every function follows the reference's control flow literally (inclusive
 * scan, upper bounds, visit index, per-output-cell worklet, sort/unique/
 * lower-bounds merge) rather than the sort-free formulation the GPU uses, so
 * that agreement between the two is evidence and not a tautology.
 *
 * Build: gcc -O2 -ffp-contract=off -fPIC -shared (no FMA contraction, so that
 * the float arithmetic rounds exactly like the reference's Serial adapter).
 *
 * Citations are paths inside the DaxToolkit source tree.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../daxtoolkit_gb300/csrc/mc_tables.h"

typedef struct {
  float origin[3];
  float spacing[3];
  int32_t extent_min[3];
  int32_t extent_max[3];
} orc_grid;

static const uint64_t kCase[256] = DAX_GB300_MC_CASE_WORDS;

/* NumFaces[case]: dax/worklet/internal/MarchingCubesTable.h:28-45 */
static int num_faces(int c) { return (int)(kCase[c] >> 60); }
/* TriTable[case][n]: dax/worklet/internal/MarchingCubesTable.h:48-306 */
static int tri_edge(int c, int n) { return (int)((kCase[c] >> (4 * n)) & 0xF); }

/* cellVertEdges: dax/worklet/MarchingCubes.h:131-135 */
static const unsigned char kCellVertEdges[12][2] = {
    {0, 1}, {1, 2}, {3, 2}, {0, 3}, {4, 5}, {5, 6},
    {7, 6}, {4, 7}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};

static void dims_of(const orc_grid* g, int64_t d[3]) {
  /* extentDimensions: dax/Extent.h:55-61 */
  for (int a = 0; a < 3; ++a) d[a] = (int64_t)g->extent_max[a] - g->extent_min[a] + 1;
}

/* TopologyUniform::GetCellConnections: dax/exec/internal/TopologyUniform.h:139-159
 * with indexToConnectivityIndex: dax/Extent.h:128-137 */
static void cell_vertices(const int64_t d[3], int64_t cell, int64_t v[8]) {
  const int64_t cx = d[0] - 1, cy = d[1] - 1;
  const int64_t i = cell % cx, j = (cell / cx) % cy, k = cell / (cx * cy);
  const int64_t first = i + d[0] * (j + d[1] * k);
  const int64_t second = first + d[0] * d[1];
  v[0] = first;
  v[1] = first + 1;
  v[2] = first + d[0] + 1;
  v[3] = first + d[0];
  v[4] = second;
  v[5] = second + 1;
  v[6] = second + d[0] + 1;
  v[7] = second + d[0];
}

/* ArrayPortalFromUniformGridPointCoordinates::Get: dax/cont/UniformGrid.h:82-89
 * (flatIndexToIndex3 adds the extent minimum: dax/Extent.h:76-85). */
static void point_coords(const orc_grid* g, const int64_t d[3], int64_t p, float c[3]) {
  const int64_t loc[3] = {p % d[0] + g->extent_min[0], (p / d[0]) % d[1] + g->extent_min[1],
                          p / (d[0] * d[1]) + g->extent_min[2]};
  for (int a = 0; a < 3; ++a) c[a] = g->origin[a] + g->spacing[a] * (float)loc[a];
}

/* GetHexahedronClassification: dax/worklet/MarchingCubes.h:36-48 */
static int classify(const float val[8], float iso) {
  int c = 0;
  for (int n = 0; n < 8; ++n) c |= (val[n] > iso) << n;
  return c;
}

static int64_t num_cells(const int64_t d[3]) {
  if (d[0] < 2 || d[1] < 2 || d[2] < 2) return 0;
  return (d[0] - 1) * (d[1] - 1) * (d[2] - 1);
}

/* DispatcherMapCell<MarchingCubesCount>: Serial Schedule(Id3) visits cells in
 * k/j/i order (dax/cont/internal/DeviceAdapterAlgorithmSerial.h:146-176);
 * MarchingCubesCount::operator(): dax/worklet/MarchingCubes.h:62-85. */
void orc_mc_count(const orc_grid* g, const float* field, float iso, int32_t* count,
                  uint8_t* cases) {
  int64_t d[3];
  dims_of(g, d);
  const int64_t C = num_cells(d);
  for (int64_t c = 0; c < C; ++c) {
    int64_t v[8];
    float val[8];
    cell_vertices(d, c, v);
    for (int n = 0; n < 8; ++n) val[n] = field[v[n]];
    const int cs = classify(val, iso);
    count[c] = num_faces(cs);
    if (cases) cases[c] = (uint8_t)cs;
  }
}

/* PointAsEdgeInterpolation: dax/cont/internal/EdgeInterpolatedGrid.h:28-74
 * (== and < compare the two point ids only). */
typedef struct {
  int32_t a, b;
  float w;
} orc_edge_rec;

static int rec_less(const orc_edge_rec* x, const orc_edge_rec* y) {
  return x->a < y->a || (x->a == y->a && x->b < y->b);
}
static int rec_cmp(const void* x, const void* y) {
  const orc_edge_rec* p = (const orc_edge_rec*)x;
  const orc_edge_rec* q = (const orc_edge_rec*)y;
  if (rec_less(p, q)) return -1;
  if (rec_less(q, p)) return 1;
  return 0;
}

/* std::upper_bound / std::lower_bound over an ascending int64 array. */
static int64_t upper_bound_i64(const int64_t* a, int64_t n, int64_t key) {
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    int64_t mid = lo + (hi - lo) / 2;
    if (a[mid] <= key) lo = mid + 1; else hi = mid;
  }
  return lo;
}
static int64_t lower_bound_i64(const int64_t* a, int64_t n, int64_t key) {
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    int64_t mid = lo + (hi - lo) / 2;
    if (a[mid] < key) lo = mid + 1; else hi = mid;
  }
  return lo;
}

/* Lerp of two implicit grid coordinates: InterpolateFieldToField,
 * dax/exec/internal/kernel/GenerateWorklets.h:79-92, with
 * dax::math::Lerp = a + w*(b-a), dax/math/VectorAnalysis.h:35-50. */
static void lerp_coords(const orc_grid* g, const int64_t d[3], const orc_edge_rec* r,
                        float out[3]) {
  float ca[3], cb[3];
  point_coords(g, d, r->a, ca);
  point_coords(g, d, r->b, cb);
  for (int a = 0; a < 3; ++a) out[a] = ca[a] + r->w * (cb[a] - ca[a]);
}

/*
 * DispatcherGenerateInterpolatedCells<MarchingCubesGenerate>::Invoke with the
 * Serial adapter: GenerateNewTopology + ResolveCoordinates,
 * dax/cont/DispatcherGenerateInterpolatedCells.h:158-301.
 *
 *  - ScanInclusive(count) -> T                     (:180-183, std::partial_sum)
 *  - UpperBounds(scan, 0..T-1) -> input cell id    (:199-202)
 *  - visit = t - LowerBounds(cellIds, cellIds[t])  (dax/cont/dispatcher/AddVisitIndexArg.h:55-62)
 *  - MarchingCubesGenerate::BuildTriangle per t    (dax/worklet/MarchingCubes.h:121-168)
 *  - merge: Copy -> Sort -> Unique -> LowerBounds  (:276-291)
 *  - coordinates: CompactPointField = Lerp          (:107-141)
 *
 * Outputs (caller capacity 3*T for verts/conn/records): verts [V][3],
 * conn [3T], and the interpolation records (rec_a, rec_b, rec_w) [V] that
 * CompactPointField uses for any other point field.  Returns T; *nverts = V.
 */
int64_t orc_mc_generate(const orc_grid* g, const float* field, float iso, const int32_t* count,
                        int merge, float* verts, int32_t* conn, int32_t* rec_a, int32_t* rec_b,
                        float* rec_w, int64_t* nverts) {
  int64_t d[3];
  dims_of(g, d);
  const int64_t C = num_cells(d);
  *nverts = 0;
  if (C == 0) return 0;
  int64_t* scan = (int64_t*)malloc(sizeof(int64_t) * C);
  int64_t acc = 0;
  for (int64_t c = 0; c < C; ++c) { acc += count[c]; scan[c] = acc; }
  const int64_t T = acc;
  if (T == 0) { free(scan); return 0; }
  int64_t* cell_of = (int64_t*)malloc(sizeof(int64_t) * T);
  for (int64_t t = 0; t < T; ++t) cell_of[t] = upper_bound_i64(scan, C, t);
  free(scan);
  orc_edge_rec* recs = (orc_edge_rec*)malloc(sizeof(orc_edge_rec) * 3 * T);
  for (int64_t t = 0; t < T; ++t) {
    const int64_t visit = t - lower_bound_i64(cell_of, T, cell_of[t]);
    int64_t v[8];
    float val[8];
    cell_vertices(d, cell_of[t], v);
    for (int n = 0; n < 8; ++n) val[n] = field[v[n]];
    const int cs = classify(val, iso);
    for (int m = 0; m < 3; ++m) {
      const int e = tri_edge(cs, (int)(visit * 3 + m));
      int va, vb;
      if (v[kCellVertEdges[e][0]] < v[kCellVertEdges[e][1]]) {
        va = kCellVertEdges[e][0];
        vb = kCellVertEdges[e][1];
      } else {
        va = kCellVertEdges[e][1];
        vb = kCellVertEdges[e][0];
      }
      const float w = (iso - val[va]) / (val[vb] - val[va]);
      recs[3 * t + m].a = (int32_t)v[va];
      recs[3 * t + m].b = (int32_t)v[vb];
      recs[3 * t + m].w = w;
    }
  }
  int64_t V;
  if (merge) {
    orc_edge_rec* uniq = (orc_edge_rec*)malloc(sizeof(orc_edge_rec) * 3 * T);
    memcpy(uniq, recs, sizeof(orc_edge_rec) * 3 * T);
    qsort(uniq, (size_t)(3 * T), sizeof(orc_edge_rec), rec_cmp);
    /* std::unique keeps the first of each run of equal (a, b). */
    V = 0;
    for (int64_t i = 0; i < 3 * T; ++i)
      if (V == 0 || rec_cmp(&uniq[V - 1], &uniq[i]) != 0) uniq[V++] = uniq[i];
    for (int64_t i = 0; i < 3 * T; ++i) {
      int64_t lo = 0, hi = V;
      while (lo < hi) {
        int64_t mid = lo + (hi - lo) / 2;
        if (rec_less(&uniq[mid], &recs[i])) lo = mid + 1; else hi = mid;
      }
      conn[i] = (int32_t)lo;
    }
    for (int64_t i = 0; i < V; ++i) {
      lerp_coords(g, d, &uniq[i], verts + 3 * i);
      if (rec_a) { rec_a[i] = uniq[i].a; rec_b[i] = uniq[i].b; rec_w[i] = uniq[i].w; }
    }
    free(uniq);
  } else {
    V = 3 * T;
    for (int64_t i = 0; i < V; ++i) {
      lerp_coords(g, d, &recs[i], verts + 3 * i);
      conn[i] = (int32_t)i;
      if (rec_a) { rec_a[i] = recs[i].a; rec_b[i] = recs[i].b; rec_w[i] = recs[i].w; }
    }
  }
  free(recs);
  free(cell_of);
  *nverts = V;
  return T;
}

/* DispatcherGenerateInterpolatedCells::CompactPointField for an arbitrary
 * scalar point field: dax/cont/DispatcherGenerateInterpolatedCells.h:107-141. */
void orc_interpolate_point_field(const int32_t* rec_a, const int32_t* rec_b, const float* rec_w,
                                 int64_t n, const float* in, float* out) {
  for (int64_t i = 0; i < n; ++i) {
    const float x = in[rec_a[i]], y = in[rec_b[i]];
    out[i] = x + rec_w[i] * (y - x);
  }
}

/* ThresholdCount: all 8 point values in [lo, hi] (inclusive),
 * dax/worklet/Threshold.h:30-96. */
void orc_threshold_count(const orc_grid* g, const float* field, float lo, float hi,
                         int32_t* count) {
  int64_t d[3];
  dims_of(g, d);
  const int64_t C = num_cells(d);
  for (int64_t c = 0; c < C; ++c) {
    int64_t v[8];
    cell_vertices(d, c, v);
    int valid = 1;
    for (int n = 0; n < 8; ++n) {
      const float x = field[v[n]];
      valid &= x >= lo && x <= hi;
    }
    count[c] = valid;
  }
}

static int cmp_i64(const void* x, const void* y) {
  const int64_t a = *(const int64_t*)x, b = *(const int64_t*)y;
  return a < b ? -1 : (a > b ? 1 : 0);
}

/*
 * DispatcherGenerateTopology<ThresholdTopology>::Invoke followed by
 * CompactPointField(field), dax/cont/DispatcherGenerateTopology.h:98-258:
 *  - ScanInclusive -> K; UpperBounds -> kept cell ids          (:142-165)
 *  - ThresholdTopology copies the cell's 8 point ids            (dax/worklet/Threshold.h:98-111)
 *  - FillPointMask                                              (:206-227)
 *  - StreamCompact(coords, mask)                                (:237-239)
 *  - Copy / Sort / Unique / LowerBounds of the connectivity     (:244-257)
 *  - CompactPointField = StreamCompact(field, mask)             (:98-113)
 * Capacities: conn 8*C, coords 3*P, field_out P.  Returns K; *p_used set.
 */
int64_t orc_threshold_generate(const orc_grid* g, const float* field, const int32_t* count,
                               int32_t* conn, float* coords, float* field_out, int64_t* p_used) {
  int64_t d[3];
  dims_of(g, d);
  const int64_t C = num_cells(d), P = d[0] * d[1] * d[2];
  *p_used = 0;
  if (C == 0) return 0;
  int64_t* scan = (int64_t*)malloc(sizeof(int64_t) * C);
  int64_t acc = 0;
  for (int64_t c = 0; c < C; ++c) { acc += count[c]; scan[c] = acc; }
  const int64_t K = acc;
  if (K == 0) { free(scan); return 0; }
  int64_t* ids = (int64_t*)malloc(sizeof(int64_t) * 8 * K);
  for (int64_t t = 0; t < K; ++t) {
    int64_t v[8];
    cell_vertices(d, upper_bound_i64(scan, C, t), v);
    for (int n = 0; n < 8; ++n) ids[8 * t + n] = v[n];
  }
  free(scan);
  unsigned char* mask = (unsigned char*)calloc((size_t)P, 1);
  for (int64_t i = 0; i < 8 * K; ++i) mask[ids[i]] = 1;
  int64_t U = 0;
  for (int64_t p = 0; p < P; ++p) {
    if (!mask[p]) continue;
    point_coords(g, d, p, coords + 3 * U);
    field_out[U] = field[p];
    ++U;
  }
  free(mask);
  int64_t* used = (int64_t*)malloc(sizeof(int64_t) * 8 * K);
  memcpy(used, ids, sizeof(int64_t) * 8 * K);
  qsort(used, (size_t)(8 * K), sizeof(int64_t), cmp_i64);
  int64_t nu = 0;
  for (int64_t i = 0; i < 8 * K; ++i)
    if (nu == 0 || used[nu - 1] != used[i]) used[nu++] = used[i];
  for (int64_t i = 0; i < 8 * K; ++i) conn[i] = (int32_t)lower_bound_i64(used, nu, ids[i]);
  free(used);
  free(ids);
  *p_used = U;
  return K;
}

/* CellGradient on voxels: dax/worklet/CellGradient.h:35-47 ->
 * CellDerivative(Voxel), dax/exec/Derivative.h:64-75 ->
 * CellDerivativeAxisAligned, :37-58, with DerivativeWeights at the
 * parametric centre (0.5,0.5,0.5), dax/exec/internal/DerivativeWeights.h:30-69.
 * Every weight is +-0.25; the signs per vertex and component follow. */
static const float kDW[8][3] = {
    {-0.25f, -0.25f, -0.25f}, {0.25f, -0.25f, -0.25f}, {0.25f, 0.25f, -0.25f},
    {-0.25f, 0.25f, -0.25f},  {-0.25f, -0.25f, 0.25f}, {0.25f, -0.25f, 0.25f},
    {0.25f, 0.25f, 0.25f},    {-0.25f, 0.25f, 0.25f}};

void orc_cell_gradient(const orc_grid* g, const float* field, float* out) {
  int64_t d[3];
  dims_of(g, d);
  const int64_t C = num_cells(d);
  for (int64_t c = 0; c < C; ++c) {
    int64_t v[8];
    cell_vertices(d, c, v);
    float c0[3], c6[3];
    point_coords(g, d, v[0], c0);
    point_coords(g, d, v[6], c6);
    float sum[3] = {0.0f, 0.0f, 0.0f};
    for (int n = 0; n < 8; ++n) {
      const float f = field[v[n]];
      for (int a = 0; a < 3; ++a) sum[a] = sum[a] + f * kDW[n][a];
    }
    for (int a = 0; a < 3; ++a) out[3 * c + a] = sum[a] / (c6[a] - c0[a]);
  }
}

/*
 * Slice on a uniform grid (dax/worklet/Slice.h:28-168).  SliceCount and
 * SliceGenerate classify and interpolate each cell with
 * s = dot(normal, coords[v] - origin) per vertex against the isovalue
 * dot(normal, origin), with the voxel edges listed lower point first
 * (Slice.h:143-148) and the same TriTable, weight and merge as marching
 * cubes.  s depends only on the point, so the slice is the marching-cubes
 * dispatch on the point field s(p) with that isovalue.  dax::dot accumulates
 * in component order, a0*b0 + a1*b1 + a2*b2 (dax/Types.h:611-620).
 */
static float dot3(const float a[3], const float b[3]) {
  float r = a[0] * b[0];
  r += a[1] * b[1];
  r += a[2] * b[2];
  return r;
}

static float* slice_field(const orc_grid* g, const float origin[3], const float normal[3],
                          float* iso) {
  int64_t d[3];
  dims_of(g, d);
  const int64_t P = d[0] * d[1] * d[2];
  float* f = (float*)malloc(sizeof(float) * (P > 0 ? P : 1));
  for (int64_t p = 0; p < P; ++p) {
    float c[3], r[3];
    point_coords(g, d, p, c);
    for (int a = 0; a < 3; ++a) r[a] = c[a] - origin[a];
    f[p] = dot3(normal, r);
  }
  *iso = dot3(normal, origin);
  return f;
}

void orc_slice_count(const orc_grid* g, const float* origin, const float* normal, int32_t* count) {
  float iso;
  float* f = slice_field(g, origin, normal, &iso);
  orc_mc_count(g, f, iso, count, NULL);
  free(f);
}

int64_t orc_slice_generate(const orc_grid* g, const float* origin, const float* normal,
                           const int32_t* count, int merge, float* verts, int32_t* conn,
                           int32_t* rec_a, int32_t* rec_b, float* rec_w, int64_t* nverts) {
  float iso;
  float* f = slice_field(g, origin, normal, &iso);
  const int64_t T = orc_mc_generate(g, f, iso, count, merge, verts, conn, rec_a, rec_b, rec_w,
                                    nverts);
  free(f);
  return T;
}

/* ---- Marching tetrahedra on an unstructured tetrahedral grid ------------- */

#include "../daxtoolkit_gb300/csrc/mt_tables.h"

static const uint32_t kMtCase[16] = DAX_GB300_MT_CASE_WORDS;
/* NumFaces / TriTable: dax/worklet/internal/MarchingTetrahedraTable.h:28-53 */
static int mt_num_faces(int c) { return (int)(kMtCase[c] >> 28); }
static int mt_tri_edge(int c, int n) { return (int)((kMtCase[c] >> (4 * n)) & 0xF); }
/* cellVertEdges: dax/worklet/MarchingTetrahedra.h:126-129 */
static const unsigned char kTetVertEdges[6][2] = {{0, 1}, {1, 2}, {2, 0}, {3, 0}, {3, 1}, {3, 2}};

/* GetTetrahedronClassification: dax/worklet/MarchingTetrahedra.h:36-46 */
static int mt_classify(const float val[4], float iso) {
  int c = 0;
  for (int n = 0; n < 4; ++n) c |= (val[n] > iso) << n;
  return c;
}

/* DispatcherMapCell<MarchingTetrahedraCount> (MarchingTetrahedra.h:49-80):
 * conn holds 4 point ids per tetrahedron. */
void orc_mt_count(const int32_t* conn, int64_t C, const float* field, float iso, int32_t* count) {
  for (int64_t c = 0; c < C; ++c) {
    float val[4];
    for (int n = 0; n < 4; ++n) val[n] = field[conn[4 * c + n]];
    count[c] = mt_num_faces(mt_classify(val, iso));
  }
}

/* Lerp of two explicit point coordinates (points [P][3]). */
static void lerp_points(const float* pts, const orc_edge_rec* r, float out[3]) {
  const float* ca = pts + 3 * (int64_t)r->a;
  const float* cb = pts + 3 * (int64_t)r->b;
  for (int a = 0; a < 3; ++a) out[a] = ca[a] + r->w * (cb[a] - ca[a]);
}

/*
 * DispatcherGenerateInterpolatedCells<MarchingTetrahedraGenerate> with the
 * Serial adapter: the same scan / upper bounds / visit index / sort-unique-
 * lower-bounds steps as orc_mc_generate, with MarchingTetrahedraGenerate::
 * BuildTriangle (MarchingTetrahedra.h:117-161) per output triangle and the
 * grid's explicit point coordinates.  Returns T; *nverts = V.
 */
int64_t orc_mt_generate(const float* pts, const int32_t* conn, int64_t C, const float* field,
                        float iso, const int32_t* count, int merge, float* verts, int32_t* tconn,
                        int32_t* rec_a, int32_t* rec_b, float* rec_w, int64_t* nverts) {
  *nverts = 0;
  if (C == 0) return 0;
  int64_t* scan = (int64_t*)malloc(sizeof(int64_t) * C);
  int64_t acc = 0;
  for (int64_t c = 0; c < C; ++c) { acc += count[c]; scan[c] = acc; }
  const int64_t T = acc;
  if (T == 0) { free(scan); return 0; }
  int64_t* cell_of = (int64_t*)malloc(sizeof(int64_t) * T);
  for (int64_t t = 0; t < T; ++t) cell_of[t] = upper_bound_i64(scan, C, t);
  free(scan);
  orc_edge_rec* recs = (orc_edge_rec*)malloc(sizeof(orc_edge_rec) * 3 * T);
  for (int64_t t = 0; t < T; ++t) {
    const int64_t visit = t - lower_bound_i64(cell_of, T, cell_of[t]);
    const int32_t* v = conn + 4 * cell_of[t];
    float val[4];
    for (int n = 0; n < 4; ++n) val[n] = field[v[n]];
    const int cs = mt_classify(val, iso);
    for (int m = 0; m < 3; ++m) {
      const int e = mt_tri_edge(cs, (int)(visit * 3 + m));
      int va, vb;
      if (v[kTetVertEdges[e][0]] < v[kTetVertEdges[e][1]]) {
        va = kTetVertEdges[e][0];
        vb = kTetVertEdges[e][1];
      } else {
        va = kTetVertEdges[e][1];
        vb = kTetVertEdges[e][0];
      }
      recs[3 * t + m].a = v[va];
      recs[3 * t + m].b = v[vb];
      recs[3 * t + m].w = (iso - val[va]) / (val[vb] - val[va]);
    }
  }
  int64_t V;
  if (merge) {
    orc_edge_rec* uniq = (orc_edge_rec*)malloc(sizeof(orc_edge_rec) * 3 * T);
    memcpy(uniq, recs, sizeof(orc_edge_rec) * 3 * T);
    qsort(uniq, (size_t)(3 * T), sizeof(orc_edge_rec), rec_cmp);
    V = 0;
    for (int64_t i = 0; i < 3 * T; ++i)
      if (V == 0 || rec_cmp(&uniq[V - 1], &uniq[i]) != 0) uniq[V++] = uniq[i];
    for (int64_t i = 0; i < 3 * T; ++i) {
      int64_t lo = 0, hi = V;
      while (lo < hi) {
        int64_t mid = lo + (hi - lo) / 2;
        if (rec_less(&uniq[mid], &recs[i])) lo = mid + 1; else hi = mid;
      }
      tconn[i] = (int32_t)lo;
    }
    for (int64_t i = 0; i < V; ++i) {
      lerp_points(pts, &uniq[i], verts + 3 * i);
      if (rec_a) { rec_a[i] = uniq[i].a; rec_b[i] = uniq[i].b; rec_w[i] = uniq[i].w; }
    }
    free(uniq);
  } else {
    V = 3 * T;
    for (int64_t i = 0; i < V; ++i) {
      lerp_points(pts, &recs[i], verts + 3 * i);
      tconn[i] = (int32_t)i;
      if (rec_a) { rec_a[i] = recs[i].a; rec_b[i] = recs[i].b; rec_w[i] = recs[i].w; }
    }
  }
  free(recs);
  free(cell_of);
  *nverts = V;
  return T;
}

/* ---- Tetrahedralize: 5 tetrahedra per voxel -------------------------------- */

/* PossibleTetraSplitCases (dax/worklet/Tetrahedralize.h:36-48): rows 0-4 for
 * even cell ids, 5-9 for odd, voxel corners in TopologyUniform order. */
static const unsigned char kTetSplit[10][4] = {
    {2, 1, 5, 0}, {0, 2, 3, 7}, {2, 5, 6, 7}, {0, 7, 4, 5}, {0, 2, 7, 5},
    {1, 3, 6, 2}, {0, 1, 3, 4}, {1, 4, 5, 6}, {3, 6, 7, 4}, {1, 4, 6, 3}};

/* DispatcherGenerateTopology<Tetrahedralize> with a constant count of 5 and
 * no point merging (UnitTestWorkletTetrahedralize.cxx:73-90): output cell o
 * comes from input cell o / 5 with visit index o % 5 (Tetrahedralize.h:71-80).
 * conn gets [5C][4] point ids. */
void orc_tetrahedralize(const orc_grid* g, int32_t* conn) {
  int64_t d[3];
  dims_of(g, d);
  const int64_t C = num_cells(d);
  for (int64_t o = 0; o < 5 * C; ++o) {
    const int64_t cell = o / 5, visit = o % 5;
    int64_t v[8];
    cell_vertices(d, cell, v);
    const unsigned char* row = kTetSplit[visit + 5 * (cell % 2)];
    for (int n = 0; n < 4; ++n) conn[4 * o + n] = (int32_t)v[row[n]];
  }
}

/* ---- Mandelbulb benchmark pipeline (Benchmarks/Mandlebulb) ----------------- */

#include <math.h>

#include "../daxtoolkit_gb300/csrc/coolwarm_table.h"

static const unsigned char kCoolWarm[3 * DAX_GB300_COOLWARM_ENTRIES] = DAX_GB300_COOLWARM_RGB;

/* dax::math::MagnitudeSquared = dot(p, p), components in order. */
static float magsq3(const float p[3]) {
  float r = p[0] * p[0];
  r += p[1] * p[1];
  r += p[2] * p[2];
  return r;
}

/* worklet::Mandlebulb::PowerN (Benchmarks/Mandlebulb/Worklets.h:92-108): the
 * 10th power of White and Nylander's formula, in float with libm's float
 * functions (dax::math maps Sqrt, ATan2, Pow, Sin, Tan, Cos to sqrtf ...). */
static void mandelbulb_power(const float pos[3], float out[3]) {
  const float squareR = magsq3(pos);
  const float t = sqrtf(pos[0] * pos[0] + pos[1] * pos[1]);
  const float thetaN = 10 * atan2f(t, pos[2]);
  const float phiN = 10 * atan2f(pos[1], pos[2]);
  const float powR = powf(squareR, 5.0f);
  out[0] = powR * (sinf(thetaN) * tanf(phiN));
  out[1] = powR * (sinf(thetaN) * sinf(phiN));
  out[2] = powR * cosf(thetaN);
}

/* worklet::Mandlebulb::operator() (Worklets.h:70-90): the escape iteration of
 * pos -> pos^10 + c, 0 when c itself lies outside radius sqrt(2), at most 35. */
static float mandelbulb_value(const float c[3]) {
  float pos[3] = {c[0], c[1], c[2]};
  if (magsq3(pos) > 2) return 0;
  for (int i = 1; i < 35; ++i) {
    float q[3];
    mandelbulb_power(pos, q);
    for (int a = 0; a < 3; ++a) pos[a] = q[a] + c[a];
    if (magsq3(pos) > 2) return (float)i;
  }
  return 35;
}

/* DispatcherMapField<Mandlebulb> over the grid's point coordinates
 * (Benchmarks/Mandlebulb/Mandlebulb.cxx:83-102). */
void orc_mandelbulb_field(const orc_grid* g, float* out) {
  int64_t d[3];
  dims_of(g, d);
  const int64_t P = d[0] * d[1] * d[2];
  for (int64_t p = 0; p < P; ++p) {
    float c[3];
    point_coords(g, d, p, c);
    out[p] = mandelbulb_value(c);
  }
}

/* worklet::ColorsAndNorms (Worklets.h:177-209) over the points of an unmerged
 * triangle surface (point v belongs to triangle v / 3): the normal
 * Normal(Cross(b - a, c - a)) = (1 / sqrt(dot)) * cross, and the cool-warm
 * colour of |dot(point, (0.09, 0.09, 0.9))| (CoolWarmColorMap.h:38-45) with
 * alpha 255.  norms [nv][3], colors [nv][4]. */
void orc_colors_and_norms(const float* verts, int64_t nv, float* norms, uint8_t* colors) {
  for (int64_t v = 0; v < nv; ++v) {
    const float* c0 = verts + 3 * (3 * (v / 3));
    const float* c1 = c0 + 3;
    const float* c2 = c0 + 6;
    float a[3], b[3], x[3];
    for (int k = 0; k < 3; ++k) {
      a[k] = c1[k] - c0[k];
      b[k] = c2[k] - c0[k];
    }
    x[0] = a[1] * b[2] - a[2] * b[1];
    x[1] = a[2] * b[0] - a[0] * b[2];
    x[2] = a[0] * b[1] - a[1] * b[0];
    const float r = 1 / sqrtf(magsq3(x));
    for (int k = 0; k < 3; ++k) norms[3 * v + k] = r * x[k];
    const float* p = verts + 3 * v;
    float s = p[0] * 0.09f;
    s += p[1] * 0.09f;
    s += p[2] * 0.9f;
    s = fabsf(s);
    s = fmaxf(0.0f, s);
    s = fminf(0.9999f, s);
    const int idx = (int)(257 * s);
    for (int k = 0; k < 3; ++k) colors[4 * v + k] = kCoolWarm[3 * idx + k];
    colors[4 * v + 3] = 255;
  }
}

/* worklet::MandlebulbClipCount (Worklets.h:112-170): a cell counts its
 * marching-cubes triangles only when one of its points lies beyond the plane,
 * dot(N, p - O) > dot(N, L); otherwise 0. */
void orc_mandelbulb_clip_count(const orc_grid* g, const float* field, float iso,
                               const float* origin, const float* location, const float* normal,
                               int32_t* count) {
  int64_t d[3];
  dims_of(g, d);
  const int64_t C = num_cells(d);
  const float loc = dot3(normal, location);
  for (int64_t c = 0; c < C; ++c) {
    int64_t v[8];
    float val[8];
    cell_vertices(d, c, v);
    int in = 0;
    for (int n = 0; n < 8; ++n) {
      float p[3], r[3];
      point_coords(g, d, v[n], p);
      for (int a = 0; a < 3; ++a) r[a] = p[a] - origin[a];
      in |= dot3(normal, r) > loc;
      val[n] = field[v[n]];
    }
    count[c] = in ? num_faces(classify(val, iso)) : 0;
  }
}

/* DispatcherMapField<Magnitude> over the grid's point coordinates
 * (dax/worklet/Magnitude.h:27-38): Sqrt(dot(p, p)). */
void orc_point_magnitude(const orc_grid* g, float* out) {
  int64_t d[3];
  dims_of(g, d);
  const int64_t P = d[0] * d[1] * d[2];
  for (int64_t p = 0; p < P; ++p) {
    float c[3];
    point_coords(g, d, p, c);
    out[p] = sqrtf(magsq3(c));
  }
}


// Reference-side CPU driver: runs the DaxToolkit's OWN worklet functors
// (MarchingCubesCount, MarchingCubesGenerate, SliceCount, SliceGenerate,
// MarchingTetrahedraCount, MarchingTetrahedraGenerate, Tetrahedralize, Magnitude, ThresholdCount,
// ThresholdTopology, CellGradient), its TopologyUniform connectivity and
// point coordinates, its PointAsEdgeInterpolation ordering and dax::math::Lerp, compiled from the reference's headers.  Only the dispatcher
// layer is restated here (the full dispatcher stack needs Boost.MPL and is not
// buildable in this environment): it follows the Serial adapter's std::
// algorithms step by step.
//
// TEST INFRASTRUCTURE ONLY: used to pin the C oracle (dax_oracle.c) and as
// the timed CPU baseline.  Built by oracle/build.py into oracle/_ref/.
//
// With threads > 1 the per-cell / per-output loops run under OpenMP and the
// scan and sort use libstdc++'s parallel mode, the CPU analogue of the
// reference's OpenMP device adapter (dax/openmp/cont/internal/
// DeviceAdapterAlgorithmOpenMP.h:34-139, Thrust's OMP backend).
#include <dax/cont/internal/EdgeInterpolatedGrid.h>
#include <dax/exec/internal/TopologyUniform.h>
#include <dax/math/VectorAnalysis.h>
#include <dax/worklet/CellGradient.h>
#include <dax/worklet/Magnitude.h>
#include <dax/worklet/MarchingCubes.h>
#include <dax/worklet/MarchingTetrahedra.h>
#include <dax/worklet/Slice.h>
#include <dax/worklet/Tetrahedralize.h>
#include <dax/worklet/Threshold.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#include <parallel/algorithm>
#include <parallel/numeric>
#endif

// DAXREF_F64: the FP64 twin.  Built with the reference's own
// DAX_USE_DOUBLE_PRECISION option (CMakeLists.txt:69, dax::Scalar = double),
// so every worklet evaluates in double from the same float32 field and grid
// description; the marching-cubes positions and weights and the cell
// gradients come out as double, and every entry point is named ref64_*.
#ifdef DAXREF_F64
#define REF_API(name) ref64_##name
typedef double RefReal;
#else
#define REF_API(name) ref_##name
typedef float RefReal;
#endif

namespace {

struct RefGrid {
  float origin[3];
  float spacing[3];
  int32_t extent_min[3];
  int32_t extent_max[3];
};

int g_threads = 1;

struct Ctx {
  dax::exec::internal::TopologyUniform topo;
  dax::Id numCells;
  dax::Id numPoints;
  explicit Ctx(const RefGrid* g) {
    topo.Origin = dax::make_Vector3(g->origin[0], g->origin[1], g->origin[2]);
    topo.Spacing = dax::make_Vector3(g->spacing[0], g->spacing[1], g->spacing[2]);
    topo.Extent = dax::Extent3(dax::make_Id3(g->extent_min[0], g->extent_min[1], g->extent_min[2]),
                               dax::make_Id3(g->extent_max[0], g->extent_max[1], g->extent_max[2]));
    dax::Id3 d = dax::extentDimensions(topo.Extent);
    numPoints = d[0] * d[1] * d[2];
    numCells = (d[0] < 2 || d[1] < 2 || d[2] < 2) ? 0 : topo.GetNumberOfCells();
  }
  // Point coordinates of the uniform grid, origin + spacing * ijk with the
  // extent minimum added (TopologyUniform::GetPointCoordiantes).
  dax::Vector3 Coord(dax::Id p) const { return topo.GetPointCoordiantes(p); }
  dax::exec::CellVertices<dax::CellTagVoxel> Verts(dax::Id cell) const {
    return topo.GetCellConnections(cell);
  }
  // The cell's point coordinates, as BindCellPoints gathers them for a
  // Vector3 point field.
  dax::exec::CellField<dax::Vector3, dax::CellTagVoxel> Coords(
      const dax::exec::CellVertices<dax::CellTagVoxel>& v) const {
    dax::exec::CellField<dax::Vector3, dax::CellTagVoxel> c;
    for (int n = 0; n < 8; ++n) c[n] = Coord(v[n]);
    return c;
  }
  // A float32 point field gathered as dax::Scalar (exact widening in the
  // FP64 twin).
  dax::exec::CellField<dax::Scalar, dax::CellTagVoxel> Gather(
      const dax::exec::CellVertices<dax::CellTagVoxel>& v, const float* f) const {
    dax::exec::CellField<dax::Scalar, dax::CellTagVoxel> vals;
    for (int n = 0; n < 8; ++n) vals[n] = f[v[n]];
    return vals;
  }
};

template <typename It, typename Out>
void partial_sum_any(It b, It e, Out o) {
#ifdef _OPENMP
  if (g_threads > 1) { __gnu_parallel::partial_sum(b, e, o); return; }
#endif
  std::partial_sum(b, e, o);
}

template <typename It>
void sort_any(It b, It e) {
#ifdef _OPENMP
  if (g_threads > 1) { __gnu_parallel::sort(b, e); return; }
#endif
  std::sort(b, e);
}

// ScanInclusive + UpperBounds(counting) of DispatcherGenerateInterpolatedCells
// / DispatcherGenerateTopology (GenerateNewTopology).
dax::Id ScanAndUpperBounds(const int32_t* count, dax::Id C, std::vector<dax::Id>& cellOf) {
  std::vector<dax::Id> scan(C);
  partial_sum_any(count, count + C, scan.begin());
  const dax::Id T = C ? scan[C - 1] : 0;
  cellOf.resize(T);
#pragma omp parallel for schedule(static) if (g_threads > 1)
  for (dax::Id t = 0; t < T; ++t)
    cellOf[t] = std::upper_bound(scan.begin(), scan.end(), t) - scan.begin();
  return T;
}

// DispatcherGenerateInterpolatedCells with the Serial adapter
// (dax/cont/DispatcherGenerateInterpolatedCells.h:158-301): ScanInclusive +
// UpperBounds -> input cell of every output triangle, visit index, the
// worklet's interpolated triangle, then (merge) Sort/Unique/LowerBounds of
// the PointAsEdgeInterpolation records and the coordinates by Lerp.
// An unstructured tetrahedral grid: explicit point coordinates [P][3] and
// four point ids per cell (dax::cont::UnstructuredGrid<CellTagTetrahedron>).
struct TetCtx {
  const float* pts;
  const int32_t* conn;
  dax::Id numCells;
  dax::Vector3 Coord(dax::Id p) const {
    return dax::make_Vector3(pts[3 * p], pts[3 * p + 1], pts[3 * p + 2]);
  }
  dax::exec::CellVertices<dax::CellTagTetrahedron> Verts(dax::Id cell) const {
    dax::exec::CellVertices<dax::CellTagTetrahedron> v;
    for (int n = 0; n < 4; ++n) v[n] = conn[4 * cell + n];
    return v;
  }
  dax::exec::CellField<dax::Scalar, dax::CellTagTetrahedron> Gather(
      const dax::exec::CellVertices<dax::CellTagTetrahedron>& v, const float* f) const {
    dax::exec::CellField<dax::Scalar, dax::CellTagTetrahedron> vals;
    for (int n = 0; n < 4; ++n) vals[n] = f[v[n]];
    return vals;
  }
};

template <typename Grid, typename Real, typename Build>
int64_t GenerateInterpolated(const Grid& ctx, const int32_t* count, int merge, Real* verts,
                             int32_t* conn, int32_t* rec_a, int32_t* rec_b, Real* rec_w,
                             int64_t* nverts, Build build) {
  *nverts = 0;
  std::vector<dax::Id> cellOf;
  const dax::Id T = ScanAndUpperBounds(count, ctx.numCells, cellOf);
  if (T == 0) return 0;
  std::vector<dax::PointAsEdgeInterpolation> recs(3 * T);
#pragma omp parallel for schedule(static) if (g_threads > 1)
  for (dax::Id t = 0; t < T; ++t) {
    // ComputeVisitIndex: workId - LowerBounds(cellIds, cellIds[t])
    const dax::Id visit =
        t - (std::lower_bound(cellOf.begin(), cellOf.end(), cellOf[t]) - cellOf.begin());
    dax::exec::InterpolatedCellPoints<dax::CellTagTriangle> out;
    build(cellOf[t], visit, out);
    for (int m = 0; m < 3; ++m) recs[3 * t + m] = out[m];
  }
  std::vector<dax::PointAsEdgeInterpolation> weights(recs);
  if (merge) {
    sort_any(weights.begin(), weights.end());
    weights.erase(std::unique(weights.begin(), weights.end()), weights.end());
#pragma omp parallel for schedule(static) if (g_threads > 1)
    for (dax::Id i = 0; i < 3 * T; ++i)
      conn[i] = (int32_t)(std::lower_bound(weights.begin(), weights.end(), recs[i]) -
                          weights.begin());
  } else {
#pragma omp parallel for schedule(static) if (g_threads > 1)
    for (dax::Id i = 0; i < 3 * T; ++i) conn[i] = (int32_t)i;
  }
  const dax::Id V = (dax::Id)weights.size();
#pragma omp parallel for schedule(static) if (g_threads > 1)
  for (dax::Id i = 0; i < V; ++i) {
    const dax::PointAsEdgeInterpolation& r = weights[i];
    dax::Vector3 p = dax::math::Lerp(ctx.Coord(r.EdgeIdFirst), ctx.Coord(r.EdgeIdSecond),
                                     r.Weight);
    verts[3 * i + 0] = p[0];
    verts[3 * i + 1] = p[1];
    verts[3 * i + 2] = p[2];
    if (rec_a) {
      rec_a[i] = r.EdgeIdFirst;
      rec_b[i] = r.EdgeIdSecond;
      rec_w[i] = r.Weight;
    }
  }
  *nverts = V;
  return T;
}

}  // namespace

extern "C" {

void REF_API(set_threads)(int n) {
  g_threads = n < 1 ? 1 : n;
#ifdef _OPENMP
  omp_set_num_threads(g_threads);
#endif
}

int REF_API(max_threads)() {
#ifdef _OPENMP
  return omp_get_num_procs();
#else
  return 1;
#endif
}

void REF_API(mc_count)(const RefGrid* g, const float* field, float iso, int32_t* count,
                  uint8_t* cases) {
  Ctx ctx(g);
  dax::worklet::MarchingCubesCount worklet(iso);
#pragma omp parallel for schedule(static) if (g_threads > 1)
  for (dax::Id c = 0; c < ctx.numCells; ++c) {
    dax::exec::CellVertices<dax::CellTagVoxel> v = ctx.Verts(c);
    dax::exec::CellField<dax::Scalar, dax::CellTagVoxel> vals = ctx.Gather(v, field);
    count[c] = (int32_t)worklet(vals);
    if (cases)
      cases[c] = (uint8_t)dax::worklet::internal::marchingcubes::GetHexahedronClassification(
          dax::Scalar(iso), vals);
  }
}

int64_t REF_API(mc_generate)(const RefGrid* g, const float* field, float iso,
                             const int32_t* count, int merge, RefReal* verts, int32_t* conn,
                             int32_t* rec_a, int32_t* rec_b, RefReal* rec_w, int64_t* nverts) {
  Ctx ctx(g);
  dax::worklet::MarchingCubesGenerate worklet(iso);
  return GenerateInterpolated(
      ctx, count, merge, verts, conn, rec_a, rec_b, rec_w, nverts,
      [&](dax::Id cell, dax::Id visit, dax::exec::InterpolatedCellPoints<dax::CellTagTriangle>& out) {
        dax::exec::CellVertices<dax::CellTagVoxel> v = ctx.Verts(cell);
        dax::exec::CellField<dax::Scalar, dax::CellTagVoxel> vals = ctx.Gather(v, field);
        worklet(v, out, vals, visit);
      });
}

// SliceCount over all cells: the cell's point coordinates against the plane
// (dax/worklet/Slice.h:28-77).
void REF_API(slice_count)(const RefGrid* g, const float* origin, const float* normal, int32_t* count) {
  Ctx ctx(g);
  dax::worklet::SliceCount worklet(dax::make_Vector3(origin[0], origin[1], origin[2]),
                                   dax::make_Vector3(normal[0], normal[1], normal[2]));
#pragma omp parallel for schedule(static) if (g_threads > 1)
  for (dax::Id c = 0; c < ctx.numCells; ++c) count[c] = (int32_t)worklet(ctx.Coords(ctx.Verts(c)));
}

// DispatcherGenerateInterpolatedCells<SliceGenerate> (Slice.h:82-168).
int64_t REF_API(slice_generate)(const RefGrid* g, const float* origin, const float* normal,
                           const int32_t* count, int merge, float* verts, int32_t* conn,
                           int32_t* rec_a, int32_t* rec_b, float* rec_w, int64_t* nverts) {
  Ctx ctx(g);
  dax::worklet::SliceGenerate worklet(dax::make_Vector3(origin[0], origin[1], origin[2]),
                                      dax::make_Vector3(normal[0], normal[1], normal[2]));
  return GenerateInterpolated(
      ctx, count, merge, verts, conn, rec_a, rec_b, rec_w, nverts,
      [&](dax::Id cell, dax::Id visit, dax::exec::InterpolatedCellPoints<dax::CellTagTriangle>& out) {
        dax::exec::CellVertices<dax::CellTagVoxel> v = ctx.Verts(cell);
        worklet(v, out, ctx.Coords(v), visit);
      });
}

// DispatcherMapField<Magnitude> over the grid's point coordinates
// (dax/worklet/Magnitude.h:27-38).
void REF_API(point_magnitude)(const RefGrid* g, float* out) {
  Ctx ctx(g);
  dax::worklet::Magnitude worklet;
#pragma omp parallel for schedule(static) if (g_threads > 1)
  for (dax::Id p = 0; p < ctx.numPoints; ++p) {
    dax::Scalar v;
    worklet(ctx.Coord(p), v);
    out[p] = v;
  }
}

// DispatcherGenerateTopology<Tetrahedralize> with a constant count of 5 and
// no point merging (UnitTestWorkletTetrahedralize.cxx:73-90): output cell o
// is the worklet's visit o % 5 of input cell o / 5.
void REF_API(tetrahedralize)(const RefGrid* g, int32_t* conn) {
  Ctx ctx(g);
  dax::worklet::Tetrahedralize worklet;
#pragma omp parallel for schedule(static) if (g_threads > 1)
  for (dax::Id o = 0; o < 5 * ctx.numCells; ++o) {
    dax::exec::CellVertices<dax::CellTagTetrahedron> out;
    worklet(ctx.Verts(o / 5), out, o, o % 5);
    for (int n = 0; n < 4; ++n) conn[4 * o + n] = (int32_t)out[n];
  }
}

// DispatcherMapCell<MarchingTetrahedraCount> over a tetrahedral grid
// (dax/worklet/MarchingTetrahedra.h:49-80).
void REF_API(mt_count)(const int32_t* conn, int64_t C, const float* field, float iso, int32_t* count) {
  TetCtx ctx{nullptr, conn, (dax::Id)C};
  dax::worklet::MarchingTetrahedraCount worklet(iso);
#pragma omp parallel for schedule(static) if (g_threads > 1)
  for (dax::Id c = 0; c < ctx.numCells; ++c)
    count[c] = (int32_t)worklet(ctx.Gather(ctx.Verts(c), field));
}

// DispatcherGenerateInterpolatedCells<MarchingTetrahedraGenerate>
// (MarchingTetrahedra.h:85-161) with the grid's explicit coordinates.
int64_t REF_API(mt_generate)(const float* pts, const int32_t* conn, int64_t C, const float* field,
                        float iso, const int32_t* count, int merge, float* verts, int32_t* tconn,
                        int32_t* rec_a, int32_t* rec_b, float* rec_w, int64_t* nverts) {
  TetCtx ctx{pts, conn, (dax::Id)C};
  dax::worklet::MarchingTetrahedraGenerate worklet(iso);
  return GenerateInterpolated(
      ctx, count, merge, verts, tconn, rec_a, rec_b, rec_w, nverts,
      [&](dax::Id cell, dax::Id visit, dax::exec::InterpolatedCellPoints<dax::CellTagTriangle>& out) {
        dax::exec::CellVertices<dax::CellTagTetrahedron> v = ctx.Verts(cell);
        worklet(v, out, ctx.Gather(v, field), visit);
      });
}

void REF_API(interpolate_point_field)(const int32_t* rec_a, const int32_t* rec_b, const float* rec_w,
                                 int64_t n, const float* in, float* out) {
#pragma omp parallel for schedule(static) if (g_threads > 1)
  for (int64_t i = 0; i < n; ++i) out[i] = dax::math::Lerp(in[rec_a[i]], in[rec_b[i]], rec_w[i]);
}

void REF_API(threshold_count)(const RefGrid* g, const float* field, float lo, float hi,
                         int32_t* count) {
  Ctx ctx(g);
  dax::worklet::ThresholdCount<dax::Scalar> worklet(lo, hi);
#pragma omp parallel for schedule(static) if (g_threads > 1)
  for (dax::Id c = 0; c < ctx.numCells; ++c)
    count[c] = (int32_t)worklet(ctx.Gather(ctx.Verts(c), field));
}

int64_t REF_API(threshold_generate)(const RefGrid* g, const float* field, const int32_t* count,
                               int32_t* conn, float* coords, float* field_out, int64_t* p_used) {
  Ctx ctx(g);
  *p_used = 0;
  std::vector<dax::Id> cellOf;
  const dax::Id K = ScanAndUpperBounds(count, ctx.numCells, cellOf);
  if (K == 0) return 0;
  dax::worklet::ThresholdTopology worklet;
  std::vector<dax::Id> ids(8 * K);
#pragma omp parallel for schedule(static) if (g_threads > 1)
  for (dax::Id t = 0; t < K; ++t) {
    dax::exec::CellVertices<dax::CellTagHexahedron> out;
    worklet(ctx.Verts(cellOf[t]), out);
    for (int n = 0; n < 8; ++n) ids[8 * t + n] = out[n];
  }
  // FillPointMask: ClearUsedPoints then GetUsedPoints through a permutation.
  std::vector<dax::Id> mask(ctx.numPoints, 0);
  for (dax::Id i = 0; i < 8 * K; ++i) mask[ids[i]] = 1;
  // StreamCompact(coords, mask) and CompactPointField(field) in point order.
  dax::Id U = 0;
  for (dax::Id p = 0; p < ctx.numPoints; ++p) {
    if (!mask[p]) continue;
    dax::Vector3 c = ctx.Coord(p);
    coords[3 * U + 0] = c[0];
    coords[3 * U + 1] = c[1];
    coords[3 * U + 2] = c[2];
    field_out[U] = field[p];
    ++U;
  }
  // ResolveDuplicatePoints: Copy, Sort, Unique, LowerBounds.
  std::vector<dax::Id> used(ids);
  sort_any(used.begin(), used.end());
  used.erase(std::unique(used.begin(), used.end()), used.end());
#pragma omp parallel for schedule(static) if (g_threads > 1)
  for (dax::Id i = 0; i < 8 * K; ++i)
    conn[i] = (int32_t)(std::lower_bound(used.begin(), used.end(), ids[i]) - used.begin());
  *p_used = U;
  return K;
}

void REF_API(cell_gradient)(const RefGrid* g, const float* field, RefReal* out) {
  Ctx ctx(g);
  dax::worklet::CellGradient worklet;
#pragma omp parallel for schedule(static) if (g_threads > 1)
  for (dax::Id c = 0; c < ctx.numCells; ++c) {
    dax::exec::CellVertices<dax::CellTagVoxel> v = ctx.Verts(c);
    dax::exec::CellField<dax::Vector3, dax::CellTagVoxel> xyz;
    for (int n = 0; n < 8; ++n) xyz[n] = ctx.Coord(v[n]);
    dax::Vector3 grad = worklet(xyz, ctx.Gather(v, field));
    out[3 * c + 0] = grad[0];
    out[3 * c + 1] = grad[1];
    out[3 * c + 2] = grad[2];
  }
}

}  // extern "C"

/*
 * dax_gb300.h -- C ABI of the GB300 (sm_103a) device adapter for the Dax
 * uniform-grid isosurface / threshold / gradient path.
 *
 * Plain C: raw device pointers, sizes, a POD grid descriptor and an opaque
 * CUDA stream (cudaStream_t passed as void*; NULL = legacy default stream).
 * Every call returns a dax_gb300_status; dax_gb300_last_error() returns the
 * message of the last failing call on the calling thread.
 *
 * Work is stream-ordered and asynchronous unless the comment says "blocks".
 * The only calls that block are the *_totals readers and the *_pipeline
 * conveniences, mirroring the places where the Dax control environment needs
 * a size on the host (ScanInclusive's return value,
 * dax/cont/DispatcherGenerateInterpolatedCells.h:180-183, and
 * dax/cont/DispatcherGenerateTopology.h:142-145).
 *
 * Ids follow dax::Id (int32, dax/Types.h:246-249).  Point fields are float32
 * (dax::Scalar, dax/Types.h:265-268), one value per point, x fastest.
 */
#ifndef DAX_GB300_H
#define DAX_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DAX_GB300_ABI_VERSION 1

typedef enum dax_gb300_status {
  DAX_GB300_SUCCESS = 0,
  /* dax::cont::ErrorControlBadValue (dax/cont/ArrayHandle.h:110-123) */
  DAX_GB300_ERROR_BAD_VALUE = 1,
  /* dax::cont::ErrorControlOutOfMemory
     (dax/thrust/cont/internal/ArrayManagerExecutionThrustDevice.h:97-100) */
  DAX_GB300_ERROR_OUT_OF_MEMORY = 2,
  /* dax::cont::ErrorExecution: an error raised on the device
     (dax/exec/internal/ErrorMessageBuffer.h:46-66) */
  DAX_GB300_ERROR_EXECUTION = 3,
  /* a CUDA runtime call failed */
  DAX_GB300_ERROR_CUDA = 4,
  /* an output buffer is smaller than the result; nothing was written */
  DAX_GB300_ERROR_CAPACITY = 5,
  /* a bounded device-side wait gave up (the fused count pass's blocks wait
     on one another; the staged count waits for its bulk copies); the count
     pass has no result and the generate pass writes nothing.  The single-pass
     integer scan, StreamCompact and Unique (whose tiles wait on the sums of
     earlier tiles) report it when their total or count is read */
  DAX_GB300_ERROR_TIMEOUT = 6,
  /* grid shape outside what the kernels support (see each call) */
  DAX_GB300_ERROR_UNSUPPORTED = 7
} dax_gb300_status;

/* A dax::cont::UniformGrid (dax/cont/UniformGrid.h:114-252): point extent
 * [extent_min, extent_max] inclusive, coordinates
 * origin + spacing * (ijk + extent_min), computed in float. */
typedef struct dax_gb300_uniform_grid {
  float origin[3];
  float spacing[3];
  int32_t extent_min[3];
  int32_t extent_max[3];
} dax_gb300_uniform_grid;

int dax_gb300_abi_version(void);

/* Per-SM block limit of one marching-cubes pass for later launches in this
 * process: pass 0 = classification (K1), 1 = count (K2a), 2 = generate (K3);
 * inside dax_gb300_mc_pipeline 3 = classification (default 3), 4 = count
 * (default: no limit), 5 = generate (default 1); 6 = the fused count pass;
 * blocks = 0 restores "as many as fit".  A limit leaves room on every SM for
 * the passes of other frames, or other slabs, running on other streams. */
int dax_gb300_set_blocks_per_sm(int pass, int blocks);

/* The count passes of one grid (dax_gb300_mc_count, dax_gb300_threshold_count,
 * dax_gb300_mc_pipeline's one-slab frame) on a 16-byte aligned device field,
 * with enabled = 1, run the classification (the field streamed into shared
 * memory by bulk TMA copies) and the counts of the row words behind it as ONE
 * persistent launch, then the scan; 0 (the default: separate classify, count
 * and scan launches, which measure faster at 512^3); -1 leaves it.
 * unit_stages = 16 KB field stages per classification work item, rounded
 * down to a power of 2 (default 16; <= 0 leaves it).  Both forms give the
 * same bytes.  Process-wide tuning knob. */
int dax_gb300_set_fused_count(int enabled, int unit_stages);
int dax_gb300_get_fused_count(int* enabled, int* unit_stages);

/* Slabs dax_gb300_mc_pipeline cuts a grid into (1..16; 0 restores the
 * default, 1: no overlap, the passes take the whole device).  Fewer are used
 * where a grid is too small for them.  Process-wide tuning knob; results do
 * not depend on it. */
int dax_gb300_set_pipeline_slabs(int slabs);

/* Further dax_gb300_mc_pipeline tuning knobs, process-wide; results do not
 * depend on them.  emit_batch: active row words a warp of the emit pass takes
 * at a time (1..32; 0 = default 8).  emit_streams: internal streams the
 * slabs' emit passes are dealt to (1..4; 0 = default 2).  keep_field_in_l2:
 * 1 = the classification reads the field with the default cache policy so
 * that a slab's values are still in L2 when its emit gathers them, 0 =
 * evict-first, -1 = default (1). */
int dax_gb300_set_pipeline_options(int emit_batch, int emit_streams, int keep_field_in_l2);

/* Timeline of dax_gb300_mc_pipeline calls on the current device, for
 * profiling: enable = 1 records CUDA timing events in the calls that follow,
 * 0 stops, -1 leaves the setting.  h_ms (n floats, may be NULL) receives,
 * for the last recorded call, per slab the milliseconds from the call's
 * start to the ends of: the classification, the wait before the count, the
 * count, the scan, the wait before the emit, the emit (6 per slab); the call
 * waits for those events.  *h_slabs (may be NULL) receives its slab count. */
int dax_gb300_pipeline_timeline(int enable, float* h_ms, int n, int* h_slabs);

/* The slabs a dax_gb300_mc_pipeline call on this grid uses with `slabs`
 * requested (0 = the current setting), computed on the host: out (int64[52])
 * receives S, then 17 count/scan boundaries (row words), 17 emit boundaries
 * (row words) and 17 classification boundaries (128-point chunks), each list
 * S + 1 long and padded with -1. */
int dax_gb300_mc_pipeline_plan(const dax_gb300_uniform_grid* grid, int slabs, int64_t* out);

/* Self-check of the reciprocal-based division the stencil kernels use
 * (Markstein's correction step) against CUDA's correctly rounded division:
 * the numerators with bit patterns first + i * step (i < count <= 2^32,
 * modulo 2^32) against each of the num_divisors divisors (device memory);
 * *d_mismatches (device, caller-zeroed) gets the number of results whose bits
 * differ.  Asynchronous. */
int dax_gb300_selfcheck_division(const float* d_divisors, int num_divisors, uint32_t first,
                                 uint64_t count, uint32_t step, unsigned long long* d_mismatches,
                                 void* stream);
const char* dax_gb300_last_error(void);

/* Sets the message dax_gb300_last_error() returns on this thread and returns
 * code: the error path of the header-only parts of the adapter
 * (dax_gb300_schedule.cuh). */
int dax_gb300_report_error(int code, const char* message);

/* Blocks until all work on `stream` is done and reports any sticky CUDA
 * error.  Replaces DeviceAdapterAlgorithm<Tag>::Synchronize
 * (dax/cuda/cont/internal/DeviceAdapterAlgorithmCuda.h:40-43). */
int dax_gb300_synchronize(void* stream);

/* ------------------------------------------------------------------------ */
/* Point classification                                                      */
/* ------------------------------------------------------------------------ */

#define DAX_GB300_CLASSIFY_ABOVE 0    /* bit = value > a        (MarchingCubes.h:40-47) */
#define DAX_GB300_CLASSIFY_IN_RANGE 1 /* bit = a <= value <= b  (Threshold.h:40-43)     */

/* Number of uint32 words dax_gb300_classify_points writes for n points. */
int64_t dax_gb300_classify_words(int64_t n);

/* One bit per point, point i in bit (i % 32) of word i / 32, the first pass
 * of the marching-cubes and threshold pipelines (the per-point half of
 * GetHexahedronClassification / ThresholdFunction).  d_bits:
 * uint32[dax_gb300_classify_words(n)]; the words after the last point are
 * zero.  Asynchronous. */
int dax_gb300_classify_points(const float* d_field, int64_t n, int mode, float a, float b,
                              uint32_t* d_bits, void* stream);

/* ------------------------------------------------------------------------ */
/* Marching cubes                                                            */
/* ------------------------------------------------------------------------ */

/* Per-cell triangle count (and optionally the 8-bit case index) for every
 * cell, in cell-id order: DispatcherMapCell<MarchingCubesCount>::Invoke
 * (dax/cont/DispatcherMapCell.h:27-64 with dax/worklet/MarchingCubes.h:53-86).
 * d_count: int32[cells]; d_cases: uint8[cells] or NULL. */
int dax_gb300_mc_classify_count(const dax_gb300_uniform_grid* grid, const float* d_field,
                                float isovalue, int32_t* d_count, uint8_t* d_cases,
                                void* stream);

/* Device scratch the fused pipeline needs for this grid (bytes).  Every
 * scratch buffer passed to this library must start on a 16-byte boundary
 * (cudaMalloc's are); others are refused with DAX_GB300_ERROR_BAD_VALUE. */
size_t dax_gb300_mc_scratch_bytes(const dax_gb300_uniform_grid* grid);

/* Classify every point, count triangles and crossing edges per row word and
 * scan them (a classification, a staged count and a reduce-then-scan
 * launch; or the fused count, dax_gb300_set_fused_count): everything
 * DispatcherGenerateInterpolatedCells::GenerateNewTopology does before its
 * generate worklet (dax/cont/DispatcherGenerateInterpolatedCells.h:178-223).
 * Asynchronous; results stay in d_scratch. */
int dax_gb300_mc_count(const dax_gb300_uniform_grid* grid, const float* d_field, float isovalue,
                       void* d_scratch, size_t scratch_bytes, void* stream);

/* Blocks on `stream`, then returns the triangle count and the number of
 * merged (unique-edge) vertices found by dax_gb300_mc_count, and any device
 * error it raised.  Unmerged output has 3 * num_triangles vertices. */
int dax_gb300_mc_totals(const void* d_scratch, int64_t* num_triangles,
                        int64_t* num_merged_vertices, void* stream);

/* Write the isosurface: the MarchingCubesGenerate worklet plus
 * ResolveCoordinates (dax/cont/DispatcherGenerateInterpolatedCells.h:225-301,
 * dax/worklet/MarchingCubes.h:121-168).
 *   merge != 0 : SetRemoveDuplicatePoints(true)  -- vertices are the unique
 *                crossing edges in ascending (first id, second id) order and
 *                d_conn holds their indices;
 *   merge == 0 : one vertex per triangle corner, d_conn = 0..3T-1.
 * d_verts: float[vert_capacity][3]; d_conn: int32[tri_capacity][3].
 * d_rec_first/d_rec_second/d_rec_weight (int32/int32/float [vert_capacity],
 * any may be NULL) receive the PointAsEdgeInterpolation record of each
 * vertex (dax/cont/internal/EdgeInterpolatedGrid.h:28-74), the input of
 * dax_gb300_interpolate_point_field.  If a capacity is too small the call
 * writes nothing and dax_gb300_mc_totals reports DAX_GB300_ERROR_CAPACITY.
 * Must follow dax_gb300_mc_count on the same scratch, grid, field, isovalue
 * and stream.  Asynchronous. */
int dax_gb300_mc_generate(const dax_gb300_uniform_grid* grid, const float* d_field,
                          float isovalue, int merge, void* d_scratch, size_t scratch_bytes,
                          float* d_verts, int64_t vert_capacity, int32_t* d_conn,
                          int64_t tri_capacity, int32_t* d_rec_first, int32_t* d_rec_second,
                          float* d_rec_weight, void* stream);

/* dax_gb300_mc_count followed by dax_gb300_mc_generate in one call, for a
 * caller that already holds output buffers large enough (from an earlier
 * frame, or the upper bounds 5 x cells triangles and 3 x triangles
 * vertices): DispatcherMapCell<MarchingCubesCount> and
 * DispatcherGenerateInterpolatedCells<MarchingCubesGenerate>
 * (dax/cont/DispatcherGenerateInterpolatedCells.h:145-301) without the host
 * reading the sizes in between.  The grid is cut into z-ordered slabs whose
 * passes overlap: the classification of one slab streams the field while
 * the earlier slabs are counted, scanned and emitted, on two internal
 * streams that fork from `stream` and join back into it, so work queued on
 * `stream` afterwards sees the complete result.  Same outputs, bit for bit,
 * as the two calls; the same scratch (dax_gb300_mc_scratch_bytes); the
 * totals and error bits are read afterwards with dax_gb300_mc_totals.  When
 * a capacity is too small, DAX_GB300_ERROR_CAPACITY is reported there and
 * nothing is written past the capacities, but the slabs before the first
 * one that did not fit may have been written.  The first call on a device
 * creates the internal streams and events: make it outside any stream
 * capture.  Calls from several host threads are serialised.  Asynchronous. */
int dax_gb300_mc_pipeline(const dax_gb300_uniform_grid* grid, const float* d_field,
                          float isovalue, int merge, void* d_scratch, size_t scratch_bytes,
                          float* d_verts, int64_t vert_capacity, int32_t* d_conn,
                          int64_t tri_capacity, int32_t* d_rec_first, int32_t* d_rec_second,
                          float* d_rec_weight, void* stream);

/* CompactPointField for any scalar point field
 * (dax/cont/DispatcherGenerateInterpolatedCells.h:107-141): out[v] =
 * Lerp(in[first[v]], in[second[v]], weight[v]).  Asynchronous. */
int dax_gb300_interpolate_point_field(const int32_t* d_rec_first, const int32_t* d_rec_second,
                                      const float* d_rec_weight, int64_t n, const float* d_in,
                                      float* d_out, void* stream);

/* Marching cubes that allocates nothing.  No counterpart in the reference:
 * it exists for callers that cannot allocate device memory where they need
 * the isosurface -- code that runs inside a memory budget reserved up front
 * (its own pool owns the device), code that must not take allocator locks or
 * risk an out-of-memory failure on a latency-critical path, and plugin hosts
 * that hand a plugin only the buffers they pass in.  Same results as
 * dax_gb300_mc_count + dax_gb300_mc_generate (merge as there), but the
 * scratch is a 32 MiB array compiled into this library, held by every GPU
 * that loads it until the process exits; grids whose scratch
 * (dax_gb300_mc_scratch_bytes) exceeds 32 MiB -- about 360^3 points -- are
 * rejected with DAX_GB300_ERROR_UNSUPPORTED before any work is queued.  Calls
 * no cudaMalloc, cudaFree or other allocating routine.  All calls on a
 * device share that one array, and each call leaves its contents behind
 * (the count pass clears what must start at zero): calls whose work overlaps
 * on the GPU -- on different streams, or from different host threads -- race
 * and must be serialised by the caller.  The first call on each device looks
 * up the array's device address; make that first call outside any stream
 * capture, and do not reset the device (cudaDeviceReset) after it: the
 * looked-up address is kept for the life of the process.  d_totals (int64[3],
 * 8-byte aligned, in device or managed memory or in page-locked host memory
 * with a device mapping; anything else is refused with
 * DAX_GB300_ERROR_BAD_VALUE before any work is queued) receives the triangle
 * count, the vertex count of the merged output, and the device error bits
 * (0 = ok; 2 = an output capacity was too small and nothing was written).
 * Asynchronous. */
int dax_gb300_mc_noalloc(const dax_gb300_uniform_grid* grid, const float* d_field, float isovalue,
                         int merge, float* d_verts, int64_t vert_capacity, int32_t* d_conn,
                         int64_t tri_capacity, int64_t* d_totals, void* stream);

/* ------------------------------------------------------------------------ */
/* Slice (dax/worklet/Slice.h)                                               */
/* ------------------------------------------------------------------------ */

/* SliceCount + SliceGenerate (Slice.h:28-77, :82-168) as one count pass and
 * one generate pass, with the scratch and totals of marching cubes:
 * dax_gb300_mc_scratch_bytes(grid) bytes of scratch, dax_gb300_mc_totals()
 * between the passes, outputs and merge exactly as dax_gb300_mc_generate.
 * The cell values are s = dot(normal, coord - origin) against the isovalue
 * dot(normal, origin), as Slice.h:64-73 computes them (the surface is the
 * plane dot(normal, x) = 2 dot(normal, origin)); they are evaluated from the
 * grid coordinates, so no field is read or stored.  origin and normal are
 * host float[3].  Asynchronous. */
int dax_gb300_slice_count(const dax_gb300_uniform_grid* grid, const float* origin,
                          const float* normal, void* d_scratch, size_t scratch_bytes,
                          void* stream);
int dax_gb300_slice_generate(const dax_gb300_uniform_grid* grid, const float* origin,
                             const float* normal, int merge, void* d_scratch,
                             size_t scratch_bytes, float* d_verts, int64_t vert_capacity,
                             int32_t* d_conn, int64_t tri_capacity, int32_t* d_rec_first,
                             int32_t* d_rec_second, float* d_rec_weight, void* stream);

/* The slice's point field itself: d_field[p] = dot(normal, coord(p) - origin)
 * (float[P], device memory) and *h_isovalue = dot(normal, origin) if
 * h_isovalue is not NULL.  Marching cubes of this field at this isovalue
 * equals the slice; the per-cell SliceCount handle is
 * dax_gb300_mc_classify_count of it.  Asynchronous. */
int dax_gb300_slice_field(const dax_gb300_uniform_grid* grid, const float* origin,
                          const float* normal, float* d_field, float* h_isovalue, void* stream);

/* ------------------------------------------------------------------------ */
/* Marching tetrahedra (dax/worklet/MarchingTetrahedra.h)                    */
/* ------------------------------------------------------------------------ */

/* DispatcherGenerateTopology<Tetrahedralize> over a uniform grid with a count
 * of 5 per cell and no point merging (dax/worklet/Tetrahedralize.h:36-82):
 * d_conn int32[5 * cells][4], output cell o from cell o / 5, split pattern by
 * the parity of the cell id.  Point ids index the grid's points, whose
 * coordinates dax_gb300_point_coordinates writes as float[P][3]
 * (UniformGrid::ComputePointCoordinates).  Asynchronous. */
int dax_gb300_tetrahedralize(const dax_gb300_uniform_grid* grid, int32_t* d_conn, void* stream);
int dax_gb300_point_coordinates(const dax_gb300_uniform_grid* grid, float* d_points,
                                void* stream);

/* An unstructured tetrahedral grid, dax::cont::UnstructuredGrid<
 * CellTagTetrahedron>: d_conn int32[num_cells][4] point ids, d_points
 * float[num_points][3], d_field float[num_points] (device memory; the field
 * and points may also be page-locked host memory).  Results are the
 * reference's MarchingTetrahedraCount + DispatcherGenerateInterpolatedCells
 * <MarchingTetrahedraGenerate> (MarchingTetrahedra.h:49-161,
 * DispatcherGenerateInterpolatedCells.h:158-301) bit for bit: triangles in
 * cell order then TriTable order, edges lower point id first, merged points
 * in ascending (first, second) order.  A cell with a point id outside
 * [0, num_points) yields DAX_GB300_ERROR_BAD_VALUE from the totals; no such
 * id is dereferenced.
 *
 * DispatcherMapCell<MarchingTetrahedraCount>: int32 count per cell.
 * Blocking (reads the error word back). */
int dax_gb300_mt_classify_count(const int32_t* d_conn, int64_t num_cells, const float* d_field,
                                int64_t num_points, float isovalue, int32_t* d_count,
                                void* stream);

/* Count pass (asynchronous); dax_gb300_mc_totals(d_scratch, &T, NULL, s)
 * then returns the triangle count. */
size_t dax_gb300_mt_scratch_bytes(int64_t num_cells);
int dax_gb300_mt_count(const int32_t* d_conn, int64_t num_cells, const float* d_field,
                       int64_t num_points, float isovalue, void* d_scratch, size_t scratch_bytes,
                       void* stream);

/* Merging (RemoveDuplicatePoints): after the count pass, Sort + Unique of the
 * interpolation records in d_merge (dax_gb300_mt_merge_scratch_bytes(T, P)
 * bytes).  Blocking; *h_num_merged = the number of merged points. */
size_t dax_gb300_mt_merge_scratch_bytes(int64_t num_triangles, int64_t num_points);
int dax_gb300_mt_merge(const int32_t* d_conn, int64_t num_cells, const float* d_field,
                       int64_t num_points, float isovalue, void* d_scratch, size_t scratch_bytes,
                       void* d_merge, size_t merge_bytes, int64_t* h_num_merged, void* stream);

/* Generate pass (asynchronous).  merge = 0: 3T points, connectivity 0..3T-1,
 * d_merge unused.  merge = 1: the points of dax_gb300_mt_merge on the same
 * scratch and d_merge.  Records (first, second, weight) per output point are
 * optional (all three or none).  If a capacity is too small nothing is
 * written and dax_gb300_mc_totals then returns DAX_GB300_ERROR_CAPACITY. */
int dax_gb300_mt_generate(const float* d_points, const int32_t* d_conn, int64_t num_cells,
                          const float* d_field, int64_t num_points, float isovalue, int merge,
                          void* d_scratch, size_t scratch_bytes, void* d_merge,
                          size_t merge_bytes, float* d_verts, int64_t vert_capacity,
                          int32_t* d_tri_conn, int64_t tri_capacity, int32_t* d_rec_first,
                          int32_t* d_rec_second, float* d_rec_weight, void* stream);

/* ------------------------------------------------------------------------ */
/* Marching cubes driven by an arbitrary count array                          */
/* ------------------------------------------------------------------------ */

/* DispatcherGenerateInterpolatedCells<MarchingCubesGenerate> with any int32
 * per-cell count array d_count (DispatcherGenerateInterpolatedCells.h:158-301):
 * ScanInclusive of the counts, UpperBounds for each output triangle's cell, the
 * visit index, the worklet's triangle; merging by Sort + Unique + LowerBounds
 * of the interpolation records.  A count of 0 drops a cell (e.g. the
 * Mandelbulb cut, below); a count above the cell's NumFaces yields
 * DAX_GB300_ERROR_BAD_VALUE from the totals and writes nothing for it.
 *   dax_gb300_mc_counted_scan     (blocking) -> *h_num_triangles = T
 *   dax_gb300_mc_counted_merge    (blocking, merge only) -> *h_num_merged = V;
 *                                 d_merge: dax_gb300_mt_merge_scratch_bytes(T, P)
 *   dax_gb300_mc_counted_generate (asynchronous), outputs as dax_gb300_mc_generate;
 *                                 dax_gb300_mc_totals(d_scratch, ...) reports errors. */
size_t dax_gb300_mc_counted_scratch_bytes(const dax_gb300_uniform_grid* grid);
int dax_gb300_mc_counted_scan(const dax_gb300_uniform_grid* grid, const int32_t* d_count,
                              void* d_scratch, size_t scratch_bytes, int64_t* h_num_triangles,
                              void* stream);
int dax_gb300_mc_counted_merge(const dax_gb300_uniform_grid* grid, const float* d_field,
                               float isovalue, const int32_t* d_count, void* d_scratch,
                               size_t scratch_bytes, void* d_merge, size_t merge_bytes,
                               int64_t* h_num_merged, void* stream);
int dax_gb300_mc_counted_generate(const dax_gb300_uniform_grid* grid, const float* d_field,
                                  float isovalue, const int32_t* d_count, int merge,
                                  void* d_scratch, size_t scratch_bytes, void* d_merge,
                                  size_t merge_bytes, float* d_verts, int64_t vert_capacity,
                                  int32_t* d_conn, int64_t tri_capacity, int32_t* d_rec_first,
                                  int32_t* d_rec_second, float* d_rec_weight, void* stream);

/* CompactPointField for a point field of `components` floats per point (a
 * dax::Vector3 field has 3): d_out[v][c] = Lerp(d_in[first[v]][c],
 * d_in[second[v]][c], weight[v]); record ids outside [0, num_points) give
 * NaN and are not read.  Asynchronous. */
int dax_gb300_interpolate_point_field_n(const int32_t* d_rec_first, const int32_t* d_rec_second,
                                        const float* d_rec_weight, int64_t n, const float* d_in,
                                        int64_t num_points, int components, float* d_out,
                                        void* stream);

/* ------------------------------------------------------------------------ */
/* Point fields and output                                                    */
/* ------------------------------------------------------------------------ */

/* DispatcherMapField<Magnitude> over the grid's point coordinates
 * (dax/worklet/Magnitude.h:27-38): float[P] = |coord(p)|, bit for bit; the
 * field of the reference's marching-cubes benchmark
 * (Benchmarks/MarchingCubes/Pipeline.h:100-106).  Asynchronous. */
int dax_gb300_point_magnitude(const dax_gb300_uniform_grid* grid, float* d_field, void* stream);

/* Legacy-VTK ASCII POLYDATA file of a cell set, byte for byte as the
 * reference's PrintContentsToStream writes it
 * (Benchmarks/MarchingCubes/Pipeline.h:51-98): points float[num_points][3],
 * conn int32[num_cells][verts_per_cell] (3 for triangles), each in device or
 * host memory.  Blocking; formats on the host cores. */
int dax_gb300_write_vtk_polydata(const char* path, const float* points, int64_t num_points,
                                 const int32_t* conn, int64_t num_cells, int verts_per_cell);

/* ------------------------------------------------------------------------ */
/* The Mandelbulb benchmark's compute pipeline (Benchmarks/Mandlebulb)        */
/* ------------------------------------------------------------------------ */

/* worklet::Mandlebulb (Worklets.h:65-109) over the grid's points: the escape
 * iteration (0 .. 35) of pos -> pos^10 + c, as float[P].  The transcendental
 * functions are CUDA's; a point on the fractal's boundary may escape one
 * iteration apart from a host C library's evaluation.  Asynchronous. */
int dax_gb300_mandelbulb_field(const dax_gb300_uniform_grid* grid, float* d_field, void* stream);

/* worklet::MandlebulbClipCount (Worklets.h:112-170): per cell the
 * marching-cubes triangle count at isovalue when a cell point lies beyond the
 * plane (dot(normal, p - origin) > dot(normal, location)), else 0; int32 per
 * cell, for dax_gb300_mc_counted_*.  Asynchronous. */
int dax_gb300_mandelbulb_clip_count(const dax_gb300_uniform_grid* grid, const float* d_field,
                                    float isovalue, const float* origin, const float* location,
                                    const float* normal, int32_t* d_count, void* stream);

/* worklet::ColorsAndNorms (Worklets.h:177-209) on an unmerged triangle surface
 * (3 points per triangle, num_points = 3T): per point the unit normal of its
 * triangle (float[3]) and its cool-warm colour, r g b 255 (uint8[4], 4-byte
 * aligned), bit for bit as the reference computes them on the CPU.
 * Asynchronous. */
int dax_gb300_colors_and_norms(const float* d_verts, int64_t num_points, float* d_norms,
                               uint8_t* d_colors, void* stream);

/* ------------------------------------------------------------------------ */
/* Batched marching cubes: many grids, one launch per pass                   */
/* ------------------------------------------------------------------------ */

/* A batch of uniform grids with their own extents, fields and isovalues.
 * The plan owns a small device table (one entry per grid), uploaded at
 * creation; it allocates nothing else.  The reference runs one dispatcher
 * invocation per grid (dax/cont/DispatcherGenerateInterpolatedCells.h:145-254),
 * so the batch has no direct counterpart; per grid the results equal
 * dax_gb300_mc_count/generate on that grid alone. */
typedef struct dax_gb300_mc_batch dax_gb300_mc_batch;

/* d_fields: host array of num_grids device pointers; isovalues: host array. Blocks. */
int dax_gb300_mc_batch_create(int num_grids, const dax_gb300_uniform_grid* grids,
                              const float* const* d_fields, const float* isovalues,
                              dax_gb300_mc_batch** out);
int dax_gb300_mc_batch_destroy(dax_gb300_mc_batch* batch);
size_t dax_gb300_mc_batch_scratch_bytes(const dax_gb300_mc_batch* batch);

/* Classify + count + scan all grids (3 launches in total).  Asynchronous. */
int dax_gb300_mc_batch_count(dax_gb300_mc_batch* batch, void* d_scratch, size_t scratch_bytes,
                             void* stream);

/* Blocks; per-grid triangle and merged-vertex offsets into the concatenated
 * outputs (host int64[num_grids + 1] each; the last entry is the total). */
int dax_gb300_mc_batch_totals(const dax_gb300_mc_batch* batch, const void* d_scratch,
                              int64_t* tri_offsets, int64_t* vert_offsets, void* stream);

/* Generate all grids into concatenated outputs: grid g's triangles are
 * d_conn[tri_offsets[g] .. tri_offsets[g+1]) and index its own vertices
 * (0-based within the grid), which are d_verts[vert_offsets[g] ..) when
 * merged, d_verts[3 * tri_offsets[g] ..) when not.  Capacity rules as
 * dax_gb300_mc_generate.  Asynchronous. */
int dax_gb300_mc_batch_generate(dax_gb300_mc_batch* batch, int merge, void* d_scratch,
                                size_t scratch_bytes, float* d_verts, int64_t vert_capacity,
                                int32_t* d_conn, int64_t tri_capacity, void* stream);

/* Capture count + generate of the batch into a CUDA graph (instantiated);
 * *graph receives an opaque executable-graph handle.  Output buffers and
 * scratch are baked into the graph.  Blocks while capturing. */
int dax_gb300_mc_batch_capture(dax_gb300_mc_batch* batch, int merge, void* d_scratch,
                               size_t scratch_bytes, float* d_verts, int64_t vert_capacity,
                               int32_t* d_conn, int64_t tri_capacity, void** graph);

/* Autotuner of a batch plan (no counterpart in the reference; its batching
 * is per grid).  Times the plan's count + generate on the caller's buffers
 * (three timed runs after one warm-up) for every candidate configuration --
 * an emit pass taking 8, 16 or 32 active row words per warp batch, and for
 * grid sets the count pass that deals a warp's active cells to its lanes or
 * the per-lane one -- and keeps the fastest in the plan, which later count,
 * generate and capture calls use.  Outputs do not depend on the choice.  The
 * choice is cached per extent class (the log2 of the number of grids and of
 * their mean point count, and merge), so a plan of a class already tuned
 * takes it without timing (*h_best_ms = -1).  Synchronous; the outputs hold
 * the last candidate's (identical) result. */
int dax_gb300_mc_batch_autotune(dax_gb300_mc_batch* batch, int merge, void* d_scratch,
                                size_t scratch_bytes, float* d_verts, int64_t vert_capacity,
                                int32_t* d_conn, int64_t tri_capacity, void* stream,
                                float* h_best_ms);
/* Sizes of the arrays the grid-set CellGradient and adjoint concatenate over
 * the batch's grids, in the order the grids were given: cells and points. */
int dax_gb300_mc_batch_sizes(const dax_gb300_mc_batch* batch, int64_t* num_cells,
                             int64_t* num_points);

/* DispatcherMapCell<CellGradient> (dax/worklet/CellGradient.h:28-48) on every
 * grid of the batch in one launch: d_out (float[num_cells][3]) holds grid 0's
 * cell gradients, then grid 1's, ...; each grid's are those of
 * dax_gb300_cell_gradient.  Asynchronous. */
int dax_gb300_mc_batch_cell_gradient(const dax_gb300_mc_batch* batch, float* d_out, void* stream);

/* dax_gb300_field_adjoint on every grid of the batch in two launches (no
 * counterpart in the reference): d_grad_fields (float[num_points], grids
 * concatenated) = dL/dfield from d_grad_vertices (float[V][3], the batch's
 * merged vertices as dax_gb300_mc_batch_generate wrote them; needs the
 * batch's count pass on d_scratch, which may be recomputed) and/or
 * d_grad_cell_gradients (float[num_cells][3] in the order of
 * dax_gb300_mc_batch_cell_gradient); either may be NULL.  Each grid's slice
 * equals dax_gb300_field_adjoint's result for that grid bit for bit.
 * Deterministic, no atomics.  Asynchronous. */
int dax_gb300_mc_batch_field_adjoint(const dax_gb300_mc_batch* batch, const void* d_scratch,
                                     size_t scratch_bytes, const float* d_grad_vertices,
                                     const float* d_grad_cell_gradients, float* d_grad_fields,
                                     void* stream);

/* Sets (emit_batch 1..32, 0 = default 16; dealt_count 1, 0, -1 = default)
 * or reads a plan's configuration. */
int dax_gb300_mc_batch_set_config(dax_gb300_mc_batch* batch, int emit_batch, int dealt_count);
int dax_gb300_mc_batch_get_config(const dax_gb300_mc_batch* batch, int* emit_batch,
                                  int* dealt_count);
int dax_gb300_graph_launch(void* graph, void* stream);
int dax_gb300_graph_destroy(void* graph);

/* ------------------------------------------------------------------------ */
/* Threshold                                                                 */
/* ------------------------------------------------------------------------ */

/* Per-cell 0/1 keep flag (all 8 point values in [lo, hi]):
 * DispatcherMapCell<ThresholdCount<Scalar>> (dax/worklet/Threshold.h:69-96). */
int dax_gb300_threshold_classify_count(const dax_gb300_uniform_grid* grid, const float* d_field,
                                       float lo, float hi, int32_t* d_count, void* stream);

size_t dax_gb300_threshold_scratch_bytes(const dax_gb300_uniform_grid* grid);

/* Classify, count kept cells and used points per row, scan (single pass).
 * The front half of DispatcherGenerateTopology::GenerateNewTopology
 * (dax/cont/DispatcherGenerateTopology.h:128-165).  Asynchronous. */
int dax_gb300_threshold_count(const dax_gb300_uniform_grid* grid, const float* d_field, float lo,
                              float hi, void* d_scratch, size_t scratch_bytes, void* stream);

/* Blocks; kept cells K and used points (the compacted point count). */
int dax_gb300_threshold_totals(const void* d_scratch, int64_t* kept_cells, int64_t* used_points,
                               void* stream);

/* Kept cells' connectivity into the compacted point list (int32[K][8], hex
 * vertex order), the compacted coordinates (float[U][3]) and the compacted
 * field (float[U], may be NULL): ThresholdTopology + FillPointMask +
 * ResolveDuplicatePoints + CompactPointField
 * (dax/cont/DispatcherGenerateTopology.h:98-258).  Asynchronous. */
int dax_gb300_threshold_generate(const dax_gb300_uniform_grid* grid, const float* d_field,
                                 float lo, float hi, void* d_scratch, size_t scratch_bytes,
                                 int32_t* d_conn, int64_t cell_capacity, float* d_coords,
                                 float* d_field_out, int64_t point_capacity, void* stream);

/* CompactPointField(input, output) of the threshold dispatcher
 * (dax/cont/DispatcherGenerateTopology.h:98-113, a StreamCompact of the
 * point field with the used-point mask): `components` floats per point of
 * d_in, written for the used points in point order -- the order of the
 * compacted coordinates -- to d_out (float[U][components]).  Needs
 * dax_gb300_threshold_count on the same scratch and grid; independent of
 * dax_gb300_threshold_generate.  A capacity below U writes nothing and
 * reports DAX_GB300_ERROR_CAPACITY at the next dax_gb300_threshold_totals.
 * Asynchronous. */
int dax_gb300_threshold_compact_point_field(const dax_gb300_uniform_grid* grid,
                                            void* d_scratch, size_t scratch_bytes,
                                            const float* d_in, int components, float* d_out,
                                            int64_t point_capacity, void* stream);

/* ------------------------------------------------------------------------ */
/* CellGradient                                                              */
/* ------------------------------------------------------------------------ */

/* Per-cell gradient of a point scalar on voxels, float[cells][3]:
 * DispatcherMapCell<CellGradient> (dax/worklet/CellGradient.h:28-48,
 * dax/exec/Derivative.h:37-75).  Asynchronous. */
int dax_gb300_cell_gradient(const dax_gb300_uniform_grid* grid, const float* d_field,
                            float* d_gradient, void* stream);

/* ------------------------------------------------------------------------ */
/* Adjoints (differentiable isosurface and gradient)                         */
/* ------------------------------------------------------------------------ */

/* dL/dfield (float[points]) from dL/d(merged isosurface vertices)
 * (float[V][3], or NULL) and/or dL/d(cell gradients) (float[cells][3], or
 * NULL): the adjoint of the edge interpolation
 * (dax/worklet/MarchingCubes.h:160-161 with dax/math/VectorAnalysis.h:35-50)
 * and of CellGradient (dax/exec/Derivative.h:37-58).  Each point gathers its
 * incident edges and cells in a fixed order: deterministic, no atomics.
 * When d_grad_vertices is given, d_scratch must hold a dax_gb300_mc_count of
 * the same grid, field and isovalue (re-run it in the backward pass rather
 * than keeping it).  Every point is written.  No reference counterpart (the
 * reference has no adjoints).  Asynchronous. */
int dax_gb300_field_adjoint(const dax_gb300_uniform_grid* grid, const float* d_field,
                            float isovalue, const void* d_scratch, size_t scratch_bytes,
                            const float* d_grad_vertices, const float* d_grad_cell_gradient,
                            float* d_grad_field, void* stream);

/* ------------------------------------------------------------------------ */
/* Generic primitives of the device adapter                                  */
/* (dax::cont::internal::DeviceAdapterAlgorithm<Tag>,                         */
/*  dax/cont/internal/DeviceAdapterAlgorithm.h:44-331; generic versions in    */
/*  dax/cont/internal/DeviceAdapterAlgorithmGeneral.h)                        */
/* ------------------------------------------------------------------------ */

/* Element types.  dax::Id is DAX_GB300_TYPE_I32, dax::Scalar F32. */
#define DAX_GB300_TYPE_I32 0
#define DAX_GB300_TYPE_U32 1
#define DAX_GB300_TYPE_F32 2
#define DAX_GB300_TYPE_I64 3
#define DAX_GB300_TYPE_U64 4

/* Scratch bytes for dax_gb300_scan on n elements (any type). */
size_t dax_gb300_scan_scratch_bytes(int64_t n);

/* ScanInclusive / ScanExclusive (DeviceAdapterAlgorithm.h ScanInclusive,
 * ScanExclusive; DeviceAdapterAlgorithmGeneral.h:337-448): d_out[i] = sum of
 * d_in[0..i] (inclusive) or d_in[0..i-1] (exclusive), any type above; d_out
 * may equal d_in.  Integer sums wrap in the element width.  If h_total is
 * not NULL it receives the sum of all elements (one element of the type; the
 * stream is synchronised for it), which is what the reference returns.
 * Integer scans run in one pass whose tiles wait, bounded, on the sums of the
 * tiles before them; a wait that ran out is reported as
 * DAX_GB300_ERROR_TIMEOUT when h_total is read. */
int dax_gb300_scan(const void* d_in, void* d_out, int64_t n, int type, int exclusive,
                   void* d_scratch, size_t scratch_bytes, void* h_total, void* stream);

/* Scratch bytes for dax_gb300_sort_by_key (0 for an unsupported shape). */
size_t dax_gb300_sort_scratch_bytes(int64_t n, int key_type, int value_bytes);

/* Sort / SortByKey (DeviceAdapterAlgorithm.h Sort, SortByKey;
 * DeviceAdapterAlgorithmGeneral.h:658-695): sorts d_keys in place, ascending
 * (descending = 0, the reference's default and SortLess) or descending
 * (SortGreater), carrying d_values (value_bytes = 0 for Sort, else 4, 8, 12
 * or 16 bytes per element: a dax::Vector3 is 12).  Stable: equal keys keep
 * their order (the reference leaves it unspecified).  Float keys sort by
 * IEEE order with -0 before +0; NaN keys are not supported. */
int dax_gb300_sort_by_key(void* d_keys, void* d_values, int64_t n, int key_type, int value_bytes,
                          int descending, void* d_scratch, size_t scratch_bytes, void* stream);

/* Scratch bytes for dax_gb300_unique (element_bytes = key bytes) and
 * dax_gb300_stream_compact (element_bytes = 0). */
size_t dax_gb300_compact_scratch_bytes(int64_t n, int element_bytes);

/* Unique (DeviceAdapterAlgorithmGeneral.h:905-927): keeps the first of every
 * run of equal adjacent keys, in place, in order.  h_count (if not NULL, the
 * stream is synchronised) receives the new length -- the reference shrinks
 * the array to it. */
int dax_gb300_unique(void* d_keys, int64_t n, int key_type, void* d_scratch, size_t scratch_bytes,
                     int64_t* h_count, void* stream);

/* StreamCompact (DeviceAdapterAlgorithmGeneral.h:770-830): the elements of
 * d_input (value_bytes each: 4, 8, 12 or 16) whose stencil entry differs from
 * zero, in order; with d_input NULL, the int32 indices of those entries (the
 * reference's one-argument form).  Stencil: int32 or float.  h_count as for
 * dax_gb300_unique.  d_output holds n elements at most. */
int dax_gb300_stream_compact(const void* d_input, int value_bytes, const void* d_stencil,
                             int stencil_type, int64_t n, void* d_output, void* d_scratch,
                             size_t scratch_bytes, int64_t* h_count, void* stream);

/* LowerBounds / UpperBounds (DeviceAdapterAlgorithmGeneral.h:175-308,
 * :961-1091): for each of the m values, the first index of the sorted array
 * (n elements) whose element is not less than (upper = 0) or greater than
 * (upper = 1) the value, as int32.  d_out may equal d_values for 4-byte keys. */
int dax_gb300_bounds(const void* d_sorted, int64_t n, const void* d_values, int64_t m,
                     int key_type, int upper, int32_t* d_out, void* stream);

/* ------------------------------------------------------------------------ */
/* Device memory, copies and timers (the ArrayManagerExecution and Timer of  */
/* the device-adapter tag, include/dax_gb300_tag.h)                          */
/* ------------------------------------------------------------------------ */

/* Allocates `bytes` of device memory on the current device (NULL for 0
 * bytes): ArrayManagerExecution::AllocateArrayForOutput / LoadDataForInput
 * (dax/cont/internal/ArrayManagerExecution.h:44-143; the CUDA adapter's
 * device_vector, dax/thrust/cont/internal/ArrayManagerExecutionThrustDevice.h:
 * 65-186).  Failure is DAX_GB300_ERROR_OUT_OF_MEMORY, the reference's
 * ErrorControlOutOfMemory (:97-100), with *d_ptr = NULL. */
int dax_gb300_device_alloc(void** d_ptr, uint64_t bytes);
int dax_gb300_device_free(void* d_ptr);

/* Allocations above `bytes` fail with DAX_GB300_ERROR_OUT_OF_MEMORY without
 * reaching the device (0 = no limit): a way to exercise a caller's
 * out-of-memory path. */
int dax_gb300_set_alloc_limit(uint64_t bytes);

/* Synchronous copy of `bytes` (ArrayManagerExecution LoadDataForInput,
 * RetrieveOutputData, CopyInto). */
#define DAX_GB300_HOST_TO_DEVICE 0
#define DAX_GB300_DEVICE_TO_HOST 1
#define DAX_GB300_DEVICE_TO_DEVICE 2
int dax_gb300_memcpy(void* dst, const void* src, uint64_t bytes, int kind);

/* A device timer, dax::cont::Timer<Tag> (dax/cont/Timer.h:39-75;
 * DeviceAdapterTimerImplementation, DeviceAdapterAlgorithm.h:343-406; the
 * CUDA adapter's events, DeviceAdapterAlgorithmCuda.h:49-88): start records
 * an event on `stream`, elapsed records a second one, waits for it and
 * returns the seconds between them. */
int dax_gb300_timer_create(void** timer);
int dax_gb300_timer_start(void* timer, void* stream);
int dax_gb300_timer_elapsed(void* timer, void* stream, double* seconds);
int dax_gb300_timer_destroy(void* timer);

#ifdef __cplusplus
}
#endif

#endif /* DAX_GB300_H */

// Launchers shared between the kernel translation units and the C ABI.
#pragma once

#include <cstdint>
#include <string>
#include <cuda_runtime.h>

#include "common.cuh"

namespace daxgb {

// Sets the message dax_gb300_last_error() returns on this thread.
void set_last_error(const std::string& msg);

// Bits words allocated for P points: whole 128-point chunks plus padding
// that unaligned 64-bit fetches may touch.
inline long long bit_words(long long P) { return ((P + 127) / 128) * 4 + 8; }

// A GridSet holding one grid (no device table).
inline GridSet single_set(const Grid& g, const float* field, float a, float b) {
  GridSet S{};
  S.slots = nullptr;
  S.count = 1;
  S.rows = g.R;
  S.chunks = (g.P + 127) / 128;
  S.rowwords = g.R * g.wr;
  S.one.g = g;
  S.one.field = field;
  S.one.iso = a;
  S.one.iso_hi = b;
  S.one.chunk0 = 0;
  S.one.word0 = 0;
  S.one.row0 = 0;
  S.one.rw0 = 0;
  return S;
}

void launch_classify_bits(int mode, const GridSet& S, bool all_aligned, uint32_t* bits,
                          long long nwords, int num_sms, cudaStream_t s);
// One grid's chunks [c_begin, c_end) only; init != NULL clears that Info
// block's error words and emit counters first; `pass` selects the per-SM
// limit; keep (mode 0) reads the field with the default cache policy
// instead of evict-first.
void launch_classify_range(int mode, const GridSet& S, bool all_aligned, uint32_t* bits,
                           long long nwords, long long c_begin, long long c_end, Info* init,
                           int pass, bool keep, int num_sms, cudaStream_t s);
void launch_cell_count(int mode, const Grid& g, const float* f, float a, float b, int32_t* count,
                       uint8_t* cases, int num_sms, cudaStream_t s);

// Per-SM block limits of the marching-cubes passes (dax_gb300_set_blocks_per_sm):
// 0 = as many as fit.  Below that, a pass leaves room on every SM for the
// kernels of other frames in flight on other streams.  kPassPipeClassify is
// the classification inside the pipelined call (default 3 blocks per SM),
// which leaves room for the count, scan and emit passes of earlier slabs.
enum TunedPass {
  kPassClassify = 0,
  kPassCount = 1,
  kPassEmit = 2,
  kPassPipeClassify = 3,
  kPassPipeCount = 4,
  kPassPipeEmit = 5,
  kPassFused = 6,  // the fused count pass (classify + count + scan, one launch)
  kTunedPasses = 7
};
int tuned_blocks_per_sm(int pass);

// Blocks of a grid-stride kernel that are resident at once on `num_sms` SMs
// (never more than `want`): one wave, no tail.  `pass` >= 0 applies that
// pass's per-SM limit.
// Occupancy of a kernel (blocks per SM at `threads` and `smem`) on the current
// device, queried once per (device, kernel, shape) and cached: the query
// costs microseconds of host time, which the many launches of a pipelined
// call would otherwise pay each time.
int cached_occupancy(const void* kernel, int threads, size_t smem);

// Launches `kernel` with programmatic stream serialization: it may begin
// (its blocks run up to pdl_wait) while the previous kernel on `s` finishes.
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), unsigned grid, unsigned block, size_t smem,
                              cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

template <typename K>
inline int resident_blocks(K kernel, int threads, size_t smem, int num_sms, long long want,
                           int pass = -1) {
  int per_sm = cached_occupancy(reinterpret_cast<const void*>(kernel), threads, smem);
  if (per_sm < 1) per_sm = 1;
  if (pass >= 0) {
    const int lim = tuned_blocks_per_sm(pass);
    if (lim > 0 && lim < per_sm) per_sm = lim;
  }
  const long long cap = (long long)num_sms * per_sm;
  return (int)(want < 1 ? 1 : (want < cap ? want : cap));
}

// Row-word count passes write packed per-word counts wc = (a << 16) | b and,
// per tile of kScanTile words, the totals of a, of b and of non-zero words
// (tile[0 / 1 / 2][tiles]); launch_word_scan turns them into per-word
// exclusive offsets wt (a), wv (b) (uint32[rowwords + 1]; entry rowwords
// holds the totals), the compacted list act of the non-zero words, and the
// totals and error word in Info.
constexpr int kScanItems = 16;               // words per thread in a tile
constexpr int kScanTile = 256 * kScanItems;  // words per tile
struct WordOffsets {
  uint32_t* wc;    // [rowwords] packed counts
  uint32_t* wt;    // [rowwords + 1]
  uint32_t* wv;    // [rowwords + 1]
  uint32_t* act;   // [rowwords]
  uint32_t* tile;  // [3][tiles] per-tile totals
};

// Slab boundaries of the pipelined marching cubes (pipeline.cu): n
// boundary row words e[0..n) whose active-word prefixes the scan records.
constexpr int kMaxSlabs = 16;
struct SlabBounds {
  int n;
  long long e[kMaxSlabs];
};
// S slabs: count/scan slab s covers tiles [tile[s], tile[s+1]) = row words
// [W[s], W[s+1]); its emit covers the active words in [E[s], E[s+1]); its
// classification covers chunks [K[s], K[s+1]).
struct SlabPlan {
  int S;
  int tile[kMaxSlabs + 1];
  long long W[kMaxSlabs + 1];
  long long E[kMaxSlabs + 1];
  long long K[kMaxSlabs + 1];
};
SlabPlan plan_slabs(const Grid& g, int wanted);
void set_pipeline_slabs(int slabs);
int pipeline_slabs();
// The slab section of the marching-cubes scratch: slab_act[kMaxSlabs + 1],
// then at kSlabCounters each slab's emit ticket and done counters.
constexpr int kSlabCounters = 32;
constexpr int kSlabWords = kSlabCounters + 2 * kMaxSlabs;
// Pipelined call options: active words per emit batch (1..32), streams the
// slabs' emits are dealt to (1..kMaxEmitStreams), and whether the
// classification keeps the field in L2 for the emit's gathers.
constexpr int kMaxEmitStreams = 4;
// Timeline of a pipelined call, per slab: ends of K1, of the wait before the
// count, of the count, of the scan, of the wait before the emit, of the emit.
constexpr int kTimelinePoints = 6;
// enable: 1 records the timeline of later calls, 0 stops, -1 leaves it; out
// (n floats): ms since the last recorded call's start, kTimelinePoints per
// slab; *slabs: that call's slab count.
int pipeline_timeline(int enable, float* out, int n, int* slabs);
struct PipeOptions {
  int emit_batch = 8;
  int emit_streams = 2;
  bool keep_field = true;
};
void set_pipeline_options(const PipeOptions& o);
PipeOptions pipeline_options();

int word_scan_tiles(long long rowwords);

// The fused count pass of one grid (marching cubes: mode 0; threshold:
// mode 1): classification and per-word counts in one persistent launch,
// then the scan -- the bits, wc / tile totals, wt / wv / act, the totals in
// Info and (mode 1) the kept / used masks, bit for bit as the separate
// passes write them.  The field must be 16-byte aligned device memory.  Its
// control words (fctl, fused_ctl_bytes(g) bytes) are cleared first.
// Returns a cudaError_t.
int launch_fused_count(int mode, const Grid& g, const float* f, float a, float b, uint32_t* bits,
                       long long nwords, const WordOffsets& o, Info* info, uint32_t* kept,
                       uint32_t* used, uint32_t* fctl, int num_sms, cudaStream_t s);
size_t fused_ctl_bytes(const Grid& g);
// enabled: 1 / 0 (-1 keeps it); unit_stages: 16 KB stages per classify unit,
// rounded down to a power of 2 (<= 0 keeps it).
void set_fused_count(int enabled, int unit_stages);
int fused_count_enabled();
int fused_unit_stages();
// abort (optional): a word that, when non-zero, makes the scan report
// kErrTimeout (the fused count pass's abort word).
void launch_word_scan(long long rowwords, const uint32_t* wc, const uint32_t* tile_tot,
                      uint32_t* wt, uint32_t* wv, uint32_t* act, Info* info, cudaStream_t s,
                      const uint32_t* abort = nullptr);
// Marching-cubes K2a of one grid with each scan tile's bits staged in
// shared memory by bulk TMA copies (staged.cu): k_mc_count's outputs, bit
// for bit.  False (nothing launched) when a tile's ranges do not fit the
// shared memory.  A copy that does not arrive sets info->aborted, which the
// scan reports as kErrTimeout.
bool launch_mc_count_staged(const Grid& g, const uint32_t* bits, long long nwords,
                            const WordOffsets& o, Info* info, int num_sms, cudaStream_t s);
// Marching cubes K2a (counts: triangles, crossing edges) + K2b.
// dealt != 0: for a grid set, the count pass that deals a warp's active cells
// to its lanes (the default); 0: the per-lane count pass.  One grid always
// takes the per-lane pass.
void launch_mc_scan(const GridSet& S, const uint32_t* bits, const WordOffsets& o, Info* info,
                    int num_sms, cudaStream_t s, int dealt = -1);
void launch_mc_emit(const GridSet& S, bool merge, const uint32_t* bits, const WordOffsets& o,
                    Info* info, float* verts, long long vcap, int32_t* conn, long long tcap,
                    int32_t* ra, int32_t* rb, float* rw, int num_sms, cudaStream_t s);
// One slab of the pipelined marching cubes (one grid): counts and scan of
// tiles [tile_begin, tile_end); the scan records the active-word prefixes of
// the boundaries B in slab_act.
void launch_mc_scan_slab(const GridSet& S, const uint32_t* bits, const WordOffsets& o, Info* info,
                         int tile_begin, int tile_end, const SlabBounds& B, uint32_t* slab_act,
                         int pass, int num_sms, cudaStream_t s,
                         cudaEvent_t after_count = nullptr);
// The emit of the active words act[slab_act[0] .. slab_act[1]) of row words
// [word_begin, word_end), capacity-checked at the offsets of range_end
// (range_end < 0: every active word, after a complete count pass).
// Warps take `batch` active words at a time from *ticket (reset to 0 with
// *done by the launch's last block).  kEmitBatch: the batch of a whole-grid
// emit.
constexpr int kEmitBatch = 16;
void launch_mc_emit_range(const GridSet& S, bool merge, const uint32_t* bits, const WordOffsets& o,
                          Info* info, float* verts, long long vcap, int32_t* conn, long long tcap,
                          int32_t* ra, int32_t* rb, float* rw, long long word_begin,
                          long long word_end, long long range_end, const uint32_t* slab_act,
                          unsigned* ticket, unsigned* done, int batch, int pass, int num_sms,
                          cudaStream_t s, bool pdl = false);
// The whole count + generate of one grid, slab-pipelined (pipeline.cu).
// fused: a one-slab frame runs the fused count pass (fctl: its control
// words) and the emit, on the caller's stream.
int launch_mc_pipeline(const Grid& g, const float* f, bool aligned, float iso, bool merge,
                       uint32_t* bits, long long nwords, const WordOffsets& o, Info* info,
                       uint32_t* slab_act, float* verts, long long vcap, int32_t* conn,
                       long long tcap, int32_t* ra, int32_t* rb, float* rw, uint32_t* fctl,
                       bool fused, int num_sms, cudaStream_t s);
// goff[2g], goff[2g+1]: first triangle / merged vertex of grid g; then totals.
void launch_grid_offsets(const GridSet& S, const WordOffsets& o, long long* goff,
                         cudaStream_t s);
void launch_interpolate(const int32_t* ra, const int32_t* rb, const float* rw, long long n,
                        const float* in, float* out, int num_sms, cudaStream_t s);
void launch_interpolate_n(const int32_t* ra, const int32_t* rb, const float* rw, long long n,
                          long long P, int k, const float* in, float* out, int num_sms,
                          cudaStream_t s);

// Threshold over row words: per word the kept-cell and used-point masks, the
// packed counts (kept << 16) | used and the tile totals for
// launch_word_scan; then the emit.
void launch_thr_count(const Grid& g, const uint32_t* bits, uint32_t* kept, uint32_t* used,
                      uint32_t* wc, uint32_t* tile_tot, int num_sms, cudaStream_t s);
// CompactPointField of the threshold: `comps` floats per point of `in`,
// compacted to the used points (after the count pass on the same scratch).
void launch_thr_compact_field(const Grid& g, const uint32_t* used, const uint32_t* wv, Info* info,
                              const float* in, int comps, float* out, long long cap, int num_sms,
                              cudaStream_t s);
void launch_thr_emit(const Grid& g, const float* f, const WordOffsets& o, const uint32_t* kept,
                     const uint32_t* used, Info* info, int32_t* conn, long long kcap,
                     float* coords, float* fout, long long ucap, int num_sms, cudaStream_t s);

// z-marching stencil kernels (the adjoint; CellGradient has its own tile
// constants below): one warp per
// tile of kMarchCols columns in x (the 32nd lane supplies the +x/-x
// neighbour column), a band of rows in y and kSeg planes in z, marched
// along z; kMarchWarps warps (independent tiles) per block.  Band heights
// and register budgets (blocks per SM) were chosen by timing on GB300.
constexpr int kMarchCols = 31;
constexpr int kSeg = 32;
constexpr int kMarchWarps = 8;
constexpr int kGradBand = 4;        // cell rows per CellGradient tile
constexpr int kGradSeg = 16;        // cell planes per CellGradient tile
constexpr int kGradWarps = 4;       // CellGradient tiles (warps) per block
constexpr int kGradMinBlocks = 4;
constexpr int kAdjBand = 8;         // point rows per adjoint tile
constexpr int kAdjMinBlocks = 3;

struct MarchTiles {
  int nxw, nband, nseg;  // tiles along x, y, z
  long long tasks;       // nxw * nband * nseg, x fastest
};
// Tiles covering an nx x ny x nz box of cells or points, `band` rows each.
__host__ __device__ inline MarchTiles march_tiles(int nx, int ny, int nz, int band) {
  MarchTiles mt;
  mt.nxw = (nx + kMarchCols - 1) / kMarchCols;
  mt.nband = (ny + band - 1) / band;
  mt.nseg = (nz + kSeg - 1) / kSeg;
  mt.tasks = (long long)mt.nxw * mt.nband * mt.nseg;
  return mt;
}

// dL/dfield from dL/d(merged vertices) (needs the count pass's bits and
// word offsets) and/or dL/d(cell gradients); out is fully written.
void launch_field_adjoint(const Grid& g, const float* f, float iso, const uint32_t* bits,
                          const WordOffsets* o, const float* dverts, const float* dgrad,
                          float* out, int num_sms, cudaStream_t s);

void launch_cell_gradient(const Grid& g, const float* f, float* out, int num_sms, cudaStream_t s);

// Grid sets (one launch for all grids; block0[slot] = the grid's first block,
// from the per-grid block counts below; per-cell and per-point arrays are
// concatenated over the set at the slots' cell0 / point0).
long long grad_blocks(const Grid& g);
long long adjoint_grad_blocks(const Grid& g);
long long adjoint_edge_blocks(const Grid& g);
// vec: every grid's output 8-byte aligned; loadv: every grid's nx even and
// field 8-byte aligned (the single-grid kernel's fast paths).
void launch_cell_gradient_set(const GridSet& S, const long long* block0, long long blocks,
                              bool vec, bool loadv, float* out, cudaStream_t s);
// dL/dfield of every grid, out[points]: the gradient term from dgrad (or
// zero) then the vertex term from dverts (the set's merged vertices; needs
// the set's count pass: bits and word offsets wv).
void launch_field_adjoint_set(const GridSet& S, const long long* grad_block0,
                              long long grad_blocks, const long long* edge_block0,
                              long long edge_blocks, long long points, const uint32_t* bits,
                              const uint32_t* wv, const float* dverts, const float* dgrad,
                              float* out, cudaStream_t s);

// Slice: the isovalue dot(normal, origin); the classification bits of the
// implicit field dot(normal, coord - origin) > iso (bit_words(P) words, the
// layout launch_classify_bits writes; row_scratch: uint32[R] for the
// per-row splits, or NULL to test every point); the field itself (float[P]).
float slice_isovalue(const float origin[3], const float normal[3]);
bool slice_rows_exact(const Grid& g, float3 o, float3 n);
void launch_slice_bits(const Grid& g, float3 o, float3 n, float iso, uint32_t* bits,
                       long long nwords, uint32_t* row_scratch, int num_sms, cudaStream_t s);
void launch_slice_field(const Grid& g, float3 o, float3 n, float* out, int num_sms,
                        cudaStream_t s);

// Ascending radix sort of unsigned keys (32- or 64-bit) whose set bits all lie
// below `bits`: only those digits are sorted.  scratch as
// dax_gb300_sort_scratch_bytes(n, U32 / U64, 0) (primitives.cu).
void sort_unsigned_bits(void* keys, long long n, bool wide, int bits, void* scratch,
                        cudaStream_t s);

// Tetrahedralize: int32[5 * cells][4] (mt.cu); the uniform grid's point
// coordinates as float[P][3].
void launch_tetrahedralize(const Grid& g, int32_t* out, int num_sms, cudaStream_t s);
void launch_point_coordinates(const Grid& g, float* out, int num_sms, cudaStream_t s);

// Marching tetrahedra on an unstructured tetrahedral grid (mt.cu).
// Count scratch: [Info][tile totals u32][tile offsets u64][chunk totals u32]
// [case byte per cell].  A tile is kMtTile cells, a chunk kMtChunk cells (one
// warp of the count and emit passes, 16 cells per lane in the emit).
constexpr int kMtThreads = 256;
constexpr int kMtPerLane = 16;
constexpr int kMtChunk = 32 * kMtPerLane;                 // cells per chunk
constexpr int kMtTile = (kMtThreads / 32) * kMtChunk;     // cells per tile
struct MtLayout {
  int tiles;
  size_t info, tile_tot, tile_off, chunk_tot, cases, total;
};
MtLayout mt_layout(long long C);
// Bits of the B half of a merge key (A << bits) | B: P <= 2^bits.  Keys are
// 32-bit when 2 * bits <= 32, else 64-bit.
int mt_key_bits(long long P);
void launch_mt_count(const int32_t* conn, long long C, const float* f, long long P, float iso,
                     char* scratch, int num_sms, cudaStream_t s);
void launch_mt_cell_count(const int32_t* conn, long long C, const float* f, long long P,
                          float iso, int32_t* count, int* err, int num_sms, cudaStream_t s);
void launch_mt_emit_direct(const float* pts, const int32_t* conn, long long C, const float* f,
                           long long P, float iso, char* scratch, float* verts, long long vcap,
                           int32_t* tconn, long long tcap, int32_t* ra, int32_t* rb, float* rw,
                           int num_sms, cudaStream_t s);
void launch_mt_emit_keys(const int32_t* conn, long long C, const float* f, long long P, float iso,
                         char* scratch, void* keys, int num_sms, cudaStream_t s);
// The merge scratch begins with a header (a marker, the unique-key count,
// the byte offsets of the record keys and of the unique keys, the triangle
// count it was built for) that the merged kernels check and read.
void launch_mt_set_merged(void* merge, long long T, long long V, size_t keys_off,
                          size_t uniq_off, cudaStream_t s);
// Merged outputs from the merge scratch: points are pts[P][3], or the uniform
// grid's when grid is not NULL.
void launch_mt_merged(const float* pts, const Grid* grid, Info* info, const float* f,
                      long long P, float iso, const void* merge, size_t merge_bytes, float* verts,
                      long long vcap, int32_t* tconn, long long tcap, int32_t* ra, int32_t* rb,
                      float* rw, int num_sms, cudaStream_t s);

// Marching cubes driven by an int32 count per cell (mt.cu): scan = its
// inclusive scan, Info.total_a = T.  keys != NULL writes the merge keys of
// the 3T records (mt_key_bits(P) format), else vertices / connectivity /
// records directly.
void launch_set_total(Info* info, long long T, int error, cudaStream_t s);
void launch_mc_counted(const Grid& g, const float* f, float iso, const int32_t* count,
                       const int32_t* scan, Info* info, void* keys, float* verts, long long vcap,
                       int32_t* tconn, long long tcap, int32_t* ra, int32_t* rb, float* rw,
                       long long T_hint, int num_sms, cudaStream_t s);

// Magnitude of the grid's point coordinates (fields.cu).
void launch_point_magnitude(const Grid& g, float* out, int num_sms, cudaStream_t s);

// Mandelbulb benchmark pipeline (mandelbulb.cu).
void launch_mandelbulb_field(const Grid& g, float* out, int num_sms, cudaStream_t s);
void launch_colors_and_norms(const float* verts, long long nv, float* norms, uint8_t* colors,
                             int num_sms, cudaStream_t s);
void launch_mandelbulb_clip_count(const Grid& g, const float* f, float iso, float3 o, float3 n,
                                  float loc, int32_t* count, int num_sms, cudaStream_t s);

}  // namespace daxgb

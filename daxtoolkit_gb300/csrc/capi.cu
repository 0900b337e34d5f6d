// C ABI over the sm_103a kernels (declared in include/dax_gb300.h).
//
// Scratch layout (one buffer, caller-owned, 256-byte aligned sections), with
// W = R x wr row words:
//   marching cubes: [Info][tile totals: 3 x tiles x u32][wc: W x u32]
//                   [wt: (W+1) x u32][wv: (W+1) x u32][act: W x u32]
//                   [slab: 64 x u32][bits: bit_words(P) x u32]
//   threshold:      the same, then [kept: W x u32][used: W x u32]
// Nothing is cleared per call: every byte, the Info block included, is
// written by the count pass before anything reads it.
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/dax_gb300.h"
#include "common.cuh"
#include "kernels.cuh"

namespace {

using daxgb::Grid;
using daxgb::Info;

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char* where) {
  return fail(DAX_GB300_ERROR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

int num_sms() {
  int dev = 0;
  cudaGetDevice(&dev);
  static int cache[64] = {0};
  if (dev < 0 || dev >= 64) dev = 0;
  if (!cache[dev]) {
    int n = 0;
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    cache[dev] = n > 0 ? n : 1;
  }
  return cache[dev];
}

constexpr int kMaxRowWords = 256;  // nx <= 8192 (shared-memory row staging in K3)

// Validates and converts the ABI grid.  Point ids are int32 (dax::Id), so the
// grid may hold at most 2^31 - 1 points.
int make_grid(const dax_gb300_uniform_grid* in, Grid& g) {
  if (!in) return fail(DAX_GB300_ERROR_BAD_VALUE, "grid is NULL");
  long long d[3];
  for (int a = 0; a < 3; ++a) {
    d[a] = (long long)in->extent_max[a] - in->extent_min[a] + 1;
    if (d[a] < 1) return fail(DAX_GB300_ERROR_BAD_VALUE, "extent_max < extent_min");
  }
  const long long P = d[0] * d[1] * d[2];
  if (P > 2147483647ll)
    return fail(DAX_GB300_ERROR_UNSUPPORTED, "grid has more than 2^31-1 points (dax::Id is int32)");
  g.nx = (int)d[0];
  g.ny = (int)d[1];
  g.nz = (int)d[2];
  g.wr = (g.nx + 31) / 32;
  if (g.wr > kMaxRowWords)
    return fail(DAX_GB300_ERROR_UNSUPPORTED, "x dimension above 8192 points is not supported");
  g.ox = in->origin[0];
  g.oy = in->origin[1];
  g.oz = in->origin[2];
  g.sx = in->spacing[0];
  g.sy = in->spacing[1];
  g.sz = in->spacing[2];
  g.mx = in->extent_min[0];
  g.my = in->extent_min[1];
  g.mz = in->extent_min[2];
  g.P = P;
  g.R = d[1] * d[2];
  g.mwr = daxgb::div_multiplier((unsigned)g.wr);
  g.mny = daxgb::div_multiplier((unsigned)g.ny);
  return DAX_GB300_SUCCESS;
}

bool has_cells(const Grid& g) { return g.nx >= 2 && g.ny >= 2 && g.nz >= 2; }

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Marching-cubes scratch: [Info][fused count control words][tile totals
// 3 x tiles][wc][wt][wv][act][slab: active-word prefixes of the pipelined
// call's slabs][bits].
struct McLayout {
  long long rowwords;
  int tiles;
  size_t info, fctl, tile, wc, wt, wv, act, slab, bits, total;
  daxgb::WordOffsets offsets(void* base) const;
};

// fctl_bytes: the control words of the fused count pass (one grid).
McLayout mc_layout_words(long long rowwords, long long bitwords, size_t head, size_t fctl_bytes = 0) {
  McLayout L;
  L.rowwords = rowwords;
  L.tiles = daxgb::word_scan_tiles(rowwords);
  L.info = 0;
  L.fctl = align256(head);
  L.tile = align256(L.fctl + fctl_bytes);
  L.wc = align256(L.tile + 3 * 4 * (size_t)L.tiles);
  L.wt = align256(L.wc + 4 * (size_t)rowwords);
  L.wv = align256(L.wt + 4 * (size_t)(rowwords + 1));
  L.act = align256(L.wv + 4 * (size_t)(rowwords + 1));
  L.slab = align256(L.act + 4 * (size_t)rowwords);
  L.bits = align256(L.slab + 4 * (size_t)daxgb::kSlabWords);
  L.total = align256(L.bits + 4 * (size_t)bitwords);
  return L;
}

McLayout mc_layout(const Grid& g) {
  return mc_layout_words(g.R * g.wr, daxgb::bit_words(g.P), sizeof(Info), daxgb::fused_ctl_bytes(g));
}

// Threshold scratch: the marching-cubes sections, then the per-word kept-cell
// and used-point masks.
struct Layout {
  McLayout m;
  size_t kept, used, total;
};

Layout layout(const Grid& g) {
  Layout L;
  const long long W = g.R * g.wr;
  L.m = mc_layout_words(W, daxgb::bit_words(g.P), sizeof(Info), daxgb::fused_ctl_bytes(g));
  L.kept = L.m.total;
  L.used = align256(L.kept + 4 * (size_t)W);
  L.total = align256(L.used + 4 * (size_t)W);
  return L;
}

template <typename T>
T* at(void* base, size_t off) {
  return reinterpret_cast<T*>(static_cast<char*>(base) + off);
}

daxgb::WordOffsets McLayout::offsets(void* base) const {
  daxgb::WordOffsets o;
  o.wc = at<uint32_t>(base, wc);
  o.wt = at<uint32_t>(base, wt);
  o.wv = at<uint32_t>(base, wv);
  o.act = at<uint32_t>(base, act);
  o.tile = at<uint32_t>(base, tile);
  return o;
}

int check_launch(const char* where) {
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? DAX_GB300_SUCCESS : cuda_fail(e, where);
}

// A field may be device memory or page-locked host memory (cudaHostAlloc,
// cudaHostRegister); host memory is read by the kernels through its device
// mapping, over the host link.  Pageable host memory is refused: the device
// cannot address it through the CUDA runtime.
int device_view(const float*& p, const char* what) {
  if (!p) return DAX_GB300_SUCCESS;  // the callers report NULL themselves
  cudaPointerAttributes a;
  cudaError_t e = cudaPointerGetAttributes(&a, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(DAX_GB300_ERROR_BAD_VALUE, std::string(what) + " pointer is not known to CUDA");
  }
  if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return DAX_GB300_SUCCESS;
  if (a.type == cudaMemoryTypeHost && a.devicePointer) {
    p = static_cast<const float*>(a.devicePointer);
    return DAX_GB300_SUCCESS;
  }
  return fail(DAX_GB300_ERROR_BAD_VALUE,
              std::string(what) + " is pageable host memory: page-lock it or copy it to the device");
}

int read_totals(const void* scratch, int64_t* a, int64_t* b, cudaStream_t s) {
  if (!scratch) return fail(DAX_GB300_ERROR_BAD_VALUE, "scratch is NULL");
  Info h;
  cudaError_t e = cudaMemcpyAsync(&h, scratch, sizeof(Info), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "reading totals");
  if (a) *a = h.total_a;
  if (b) *b = h.total_b;
  if (h.error & daxgb::kErrOverflow)
    return fail(DAX_GB300_ERROR_UNSUPPORTED, "more than 2^31-1 triangles or vertices");
  if (h.error & daxgb::kErrBadCount)
    return fail(DAX_GB300_ERROR_BAD_VALUE,
                "the count array asks a cell for more triangles than its case has");
  if (h.error & daxgb::kErrState)
    return fail(DAX_GB300_ERROR_BAD_VALUE,
                "the merge scratch does not hold dax_gb300_mt_merge's result for this count pass");
  if (h.error & daxgb::kErrTimeout)
    return fail(DAX_GB300_ERROR_TIMEOUT,
                "a bounded device-side wait of the count pass ran out; no result");
  if (h.error & daxgb::kErrBadIndex)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "a cell lists a point id outside [0, num_points)");
  if (h.error & daxgb::kErrCapacity)
    return fail(DAX_GB300_ERROR_CAPACITY, "output capacity smaller than the result; nothing written");
  return DAX_GB300_SUCCESS;
}

// The fused count pass streams the field with bulk TMA copies: it takes
// 16-byte aligned device memory (page-locked host and managed fields take
// the three-launch pass).
bool fused_ok(const float* field) {
  if (!daxgb::fused_count_enabled() || !aligned16(field)) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, field) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice;
}

int count_pass(int mode, const dax_gb300_uniform_grid* grid, const float* field, float a, float b,
               void* scratch, size_t bytes, cudaStream_t s) {
  Grid g;
  int st = make_grid(grid, g);
  if (st) return st;
  if (!field || !scratch) return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL field or scratch");
  if (!aligned16(scratch)) return fail(DAX_GB300_ERROR_BAD_VALUE, "scratch must be 16-byte aligned");
  if ((st = device_view(field, "field"))) return st;
  const size_t need = mode == 0 ? mc_layout(g).total : layout(g).total;
  if (bytes < need) return fail(DAX_GB300_ERROR_BAD_VALUE, "scratch smaller than *_scratch_bytes()");
  if (!has_cells(g)) {  // no cells: totals stay 0
    cudaError_t e = cudaMemsetAsync(scratch, 0, sizeof(Info), s);
    return e == cudaSuccess ? DAX_GB300_SUCCESS : cuda_fail(e, "clearing scratch");
  }
  const int sms = num_sms();
  if (fused_ok(field)) {
    // classification and counts in one launch, then the scan
    const McLayout M = mode == 0 ? mc_layout(g) : layout(g).m;
    uint32_t* kept = mode == 0 ? nullptr : at<uint32_t>(scratch, layout(g).kept);
    uint32_t* used = mode == 0 ? nullptr : at<uint32_t>(scratch, layout(g).used);
    const int e = daxgb::launch_fused_count(mode, g, field, a, b, at<uint32_t>(scratch, M.bits),
                                            daxgb::bit_words(g.P), M.offsets(scratch),
                                            at<Info>(scratch, M.info), kept, used,
                                            at<uint32_t>(scratch, M.fctl), sms, s);
    if (e != 0) return cuda_fail(static_cast<cudaError_t>(e), "fused count kernel");
    return check_launch("fused count kernel");
  }
  const daxgb::GridSet S = daxgb::single_set(g, field, a, b);
  if (mode == 0) {
    const McLayout L = mc_layout(g);
    uint32_t* bits = at<uint32_t>(scratch, L.bits);
    // the classification clears Info's error words first
    daxgb::launch_classify_range(0, S, aligned16(field), bits, daxgb::bit_words(g.P), 0, S.chunks,
                                 at<Info>(scratch, L.info), daxgb::kPassClassify, false, sms, s);
    if ((st = check_launch("classify kernel"))) return st;
    const daxgb::WordOffsets o = L.offsets(scratch);
    daxgb::launch_mc_scan(S, bits, o, at<Info>(scratch, L.info), sms, s);
    return check_launch("count/scan kernels");
  }
  const Layout L = layout(g);
  uint32_t* bits = at<uint32_t>(scratch, L.m.bits);
  daxgb::launch_classify_range(1, S, aligned16(field), bits, daxgb::bit_words(g.P), 0, S.chunks,
                               at<Info>(scratch, L.m.info), daxgb::kPassClassify, false, sms, s);
  if ((st = check_launch("classify kernel"))) return st;
  const daxgb::WordOffsets o = L.m.offsets(scratch);
  daxgb::launch_thr_count(g, bits, at<uint32_t>(scratch, L.kept), at<uint32_t>(scratch, L.used),
                          o.wc, o.tile, sms, s);
  daxgb::launch_word_scan(g.R * g.wr, o.wc, o.tile, o.wt, o.wv, o.act, at<Info>(scratch, L.m.info),
                          s);
  return check_launch("threshold count/scan kernels");
}

}  // namespace

namespace daxgb {
void set_last_error(const std::string& msg) { g_last_error = msg; }

int cached_occupancy(const void* kernel, int threads, size_t smem) {
  static std::mutex m;
  static std::map<std::tuple<int, const void*, int, size_t>, int> cache;
  int dev = 0;
  cudaGetDevice(&dev);
  const auto key = std::make_tuple(dev, kernel, threads, smem);
  std::lock_guard<std::mutex> lock(m);
  const auto it = cache.find(key);
  if (it != cache.end()) return it->second;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) != cudaSuccess) {
    cudaGetLastError();
    per_sm = 1;
  }
  cache[key] = per_sm;
  return per_sm;
}

namespace {
int g_blocks_per_sm[kTunedPasses] = {0, 0, 0, 3, 0, 1, 0};
}
int tuned_blocks_per_sm(int pass) {
  return pass >= 0 && pass < kTunedPasses ? g_blocks_per_sm[pass] : 0;
}
}  // namespace daxgb

// Batched marching cubes plan (host side of dax_gb300_mc_batch).
struct dax_gb300_mc_batch {
  int count = 0;
  std::vector<daxgb::GridSlot> slots;
  daxgb::GridSlot* d_slots = nullptr;
  long long rows = 0, chunks = 0, words = 0, rowwords = 0;
  int max_wr = 1;
  bool aligned = true;
  size_t off_goff = 0;
  McLayout L;
  // tuned by dax_gb300_mc_batch_autotune (or set): active words per emit
  // warp batch, and the dealt (1) or per-lane (0) count pass
  int emit_batch = daxgb::kEmitBatch;
  int dealt = 1;
  // grid-set CellGradient and adjoint: totals of the concatenated per-cell
  // and per-point arrays, and per grid the first block of each set launch
  // (d_blk: [gradient][adjoint gradient term][adjoint vertex term], count + 1
  // each)
  long long cells = 0, points = 0;
  long long* d_blk = nullptr;
  long long blk_total[3] = {0, 0, 0};
  bool grad_vec = true, grad_loadv = true;

  daxgb::GridSet set() const {
    daxgb::GridSet S{};
    S.slots = count > 1 ? d_slots : nullptr;
    S.count = count;
    S.rows = rows;
    S.chunks = chunks;
    S.rowwords = rowwords;
    if (count == 1) S.one = slots[0];
    return S;
  }
  // the set for the grid-set launches, which always read the slot table
  daxgb::GridSet set_for_sets() const {
    daxgb::GridSet S = set();
    S.slots = d_slots;
    return S;
  }
};

extern "C" {

int dax_gb300_abi_version(void) { return DAX_GB300_ABI_VERSION; }

int dax_gb300_set_blocks_per_sm(int pass, int blocks) {
  if (pass < 0 || pass >= daxgb::kTunedPasses || blocks < 0)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "unknown pass or negative block count");
  daxgb::g_blocks_per_sm[pass] = blocks;
  return DAX_GB300_SUCCESS;
}

int dax_gb300_set_fused_count(int enabled, int unit_stages) {
  if (enabled < -1 || enabled > 1) return fail(DAX_GB300_ERROR_BAD_VALUE, "enabled must be -1, 0 or 1");
  daxgb::set_fused_count(enabled, unit_stages);
  return DAX_GB300_SUCCESS;
}

int dax_gb300_get_fused_count(int* enabled, int* unit_stages) {
  if (enabled) *enabled = daxgb::fused_count_enabled();
  if (unit_stages) *unit_stages = daxgb::fused_unit_stages();
  return DAX_GB300_SUCCESS;
}

const char* dax_gb300_last_error(void) { return g_last_error.c_str(); }

int dax_gb300_report_error(int code, const char* message) {
  g_last_error = message ? message : "";
  return code;
}

int dax_gb300_synchronize(void* stream) {
  cudaError_t e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
  if (e == cudaSuccess) e = cudaGetLastError();
  return e == cudaSuccess ? DAX_GB300_SUCCESS : cuda_fail(e, "synchronize");
}

int64_t dax_gb300_classify_words(int64_t n) { return n <= 0 ? 0 : daxgb::bit_words(n); }

int dax_gb300_classify_points(const float* d_field, int64_t n, int mode, float a, float b,
                              uint32_t* d_bits, void* stream) {
  if (n <= 0) return DAX_GB300_SUCCESS;
  if (!d_field || !d_bits) return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL field or bits");
  if (int st = device_view(d_field, "field")) return st;
  if (mode != DAX_GB300_CLASSIFY_ABOVE && mode != DAX_GB300_CLASSIFY_IN_RANGE)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "unknown classification mode");
  Grid g{};
  g.P = n;
  g.nx = 1;
  g.ny = 1;
  g.nz = 1;
  const daxgb::GridSet S = daxgb::single_set(g, d_field, a, b);
  daxgb::launch_classify_bits(mode, S, aligned16(d_field), d_bits, daxgb::bit_words(n), num_sms(),
                              static_cast<cudaStream_t>(stream));
  return check_launch("classify kernel");
}

int dax_gb300_mc_classify_count(const dax_gb300_uniform_grid* grid, const float* d_field,
                                float isovalue, int32_t* d_count, uint8_t* d_cases,
                                void* stream) {
  Grid g;
  int st = make_grid(grid, g);
  if (st) return st;
  if (!has_cells(g)) return DAX_GB300_SUCCESS;
  if (!d_field || !d_count) return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL field or count");
  if ((st = device_view(d_field, "field"))) return st;
  daxgb::launch_cell_count(0, g, d_field, isovalue, 0.0f, d_count, d_cases, num_sms(),
                           static_cast<cudaStream_t>(stream));
  return check_launch("mc classify-count kernel");
}

size_t dax_gb300_mc_scratch_bytes(const dax_gb300_uniform_grid* grid) {
  Grid g;
  if (make_grid(grid, g)) return 0;
  return mc_layout(g).total;
}

int dax_gb300_mc_count(const dax_gb300_uniform_grid* grid, const float* d_field, float isovalue,
                       void* d_scratch, size_t scratch_bytes, void* stream) {
  return count_pass(0, grid, d_field, isovalue, 0.0f, d_scratch, scratch_bytes,
                    static_cast<cudaStream_t>(stream));
}

int dax_gb300_mc_totals(const void* d_scratch, int64_t* num_triangles,
                        int64_t* num_merged_vertices, void* stream) {
  return read_totals(d_scratch, num_triangles, num_merged_vertices,
                     static_cast<cudaStream_t>(stream));
}

int dax_gb300_mc_generate(const dax_gb300_uniform_grid* grid, const float* d_field,
                          float isovalue, int merge, void* d_scratch, size_t scratch_bytes,
                          float* d_verts, int64_t vert_capacity, int32_t* d_conn,
                          int64_t tri_capacity, int32_t* d_rec_first, int32_t* d_rec_second,
                          float* d_rec_weight, void* stream) {
  Grid g;
  int st = make_grid(grid, g);
  if (st) return st;
  if (!has_cells(g)) return DAX_GB300_SUCCESS;
  if (!d_field || !d_scratch) return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL field or scratch");
  if (!aligned16(d_scratch)) return fail(DAX_GB300_ERROR_BAD_VALUE, "scratch must be 16-byte aligned");
  if ((st = device_view(d_field, "field"))) return st;
  if ((!d_verts && vert_capacity > 0) || (!d_conn && tri_capacity > 0) || vert_capacity < 0 ||
      tri_capacity < 0)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL output with nonzero capacity");
  const McLayout L = mc_layout(g);
  if (scratch_bytes < L.total)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "scratch smaller than dax_gb300_mc_scratch_bytes()");
  daxgb::launch_mc_emit(daxgb::single_set(g, d_field, isovalue, 0.0f), merge != 0,
                        at<uint32_t>(d_scratch, L.bits), L.offsets(d_scratch),
                        at<Info>(d_scratch, L.info), d_verts, vert_capacity, d_conn, tri_capacity,
                        d_rec_first, d_rec_second, d_rec_weight, num_sms(),
                        static_cast<cudaStream_t>(stream));
  return check_launch("mc generate kernel");
}

int dax_gb300_mc_pipeline(const dax_gb300_uniform_grid* grid, const float* d_field,
                          float isovalue, int merge, void* d_scratch, size_t scratch_bytes,
                          float* d_verts, int64_t vert_capacity, int32_t* d_conn,
                          int64_t tri_capacity, int32_t* d_rec_first, int32_t* d_rec_second,
                          float* d_rec_weight, void* stream) {
  Grid g;
  int st = make_grid(grid, g);
  if (st) return st;
  if (!d_field || !d_scratch) return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL field or scratch");
  if (!aligned16(d_scratch)) return fail(DAX_GB300_ERROR_BAD_VALUE, "scratch must be 16-byte aligned");
  if ((st = device_view(d_field, "field"))) return st;
  if ((!d_verts && vert_capacity > 0) || (!d_conn && tri_capacity > 0) || vert_capacity < 0 ||
      tri_capacity < 0)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL output with nonzero capacity");
  const McLayout L = mc_layout(g);
  if (scratch_bytes < L.total)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "scratch smaller than dax_gb300_mc_scratch_bytes()");
  const cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!has_cells(g)) {  // no cells: totals stay 0
    cudaError_t e = cudaMemsetAsync(d_scratch, 0, sizeof(Info), s);
    return e == cudaSuccess ? DAX_GB300_SUCCESS : cuda_fail(e, "clearing scratch");
  }
  return daxgb::launch_mc_pipeline(g, d_field, aligned16(d_field), isovalue, merge != 0,
                                   at<uint32_t>(d_scratch, L.bits), daxgb::bit_words(g.P),
                                   L.offsets(d_scratch), at<Info>(d_scratch, L.info),
                                   at<uint32_t>(d_scratch, L.slab), d_verts, vert_capacity, d_conn,
                                   tri_capacity, d_rec_first, d_rec_second, d_rec_weight,
                                   at<uint32_t>(d_scratch, L.fctl), fused_ok(d_field), num_sms(),
                                   s);
}

int dax_gb300_mc_pipeline_plan(const dax_gb300_uniform_grid* grid, int slabs, int64_t* out) {
  Grid g;
  int st = make_grid(grid, g);
  if (st) return st;
  if (!out) return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL output");
  const daxgb::SlabPlan p = daxgb::plan_slabs(g, slabs > 0 ? slabs : daxgb::pipeline_slabs());
  const int n = daxgb::kMaxSlabs + 1;
  out[0] = p.S;
  for (int i = 0; i < n; ++i) {
    const bool in = i <= p.S;
    out[1 + i] = in ? p.W[i] : -1;
    out[1 + n + i] = in ? p.E[i] : -1;
    out[1 + 2 * n + i] = in ? p.K[i] : -1;
  }
  return DAX_GB300_SUCCESS;
}

int dax_gb300_set_pipeline_options(int emit_batch, int emit_streams, int keep_field_in_l2) {
  if (emit_batch < 0 || emit_batch > 32 || emit_streams < 0 ||
      emit_streams > daxgb::kMaxEmitStreams || keep_field_in_l2 < -1 || keep_field_in_l2 > 1)
    return fail(DAX_GB300_ERROR_BAD_VALUE,
                "emit_batch in [0, 32], emit_streams in [0, 4], keep_field_in_l2 in [-1, 1]");
  daxgb::PipeOptions o;
  if (emit_batch > 0) o.emit_batch = emit_batch;
  if (emit_streams > 0) o.emit_streams = emit_streams;
  if (keep_field_in_l2 >= 0) o.keep_field = keep_field_in_l2 != 0;
  daxgb::set_pipeline_options(o);
  return DAX_GB300_SUCCESS;
}

int dax_gb300_pipeline_timeline(int enable, float* h_ms, int n, int* h_slabs) {
  return daxgb::pipeline_timeline(enable, h_ms, n, h_slabs);
}

int dax_gb300_set_pipeline_slabs(int slabs) {
  if (slabs < 0 || slabs > daxgb::kMaxSlabs)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "slabs must be in [0, 16]");
  daxgb::set_pipeline_slabs(slabs);
  return DAX_GB300_SUCCESS;
}

int dax_gb300_slice_field(const dax_gb300_uniform_grid* grid, const float* origin,
                          const float* normal, float* d_field, float* h_isovalue, void* stream) {
  Grid g;
  int st = make_grid(grid, g);
  if (st) return st;
  if (!origin || !normal || !d_field)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL origin, normal or field");
  if (h_isovalue) *h_isovalue = daxgb::slice_isovalue(origin, normal);
  daxgb::launch_slice_field(g, make_float3(origin[0], origin[1], origin[2]),
                            make_float3(normal[0], normal[1], normal[2]), d_field, num_sms(),
                            static_cast<cudaStream_t>(stream));
  return check_launch("slice field kernel");
}

int dax_gb300_slice_count(const dax_gb300_uniform_grid* grid, const float* origin,
                          const float* normal, void* d_scratch, size_t scratch_bytes,
                          void* stream) {
  Grid g;
  int st = make_grid(grid, g);
  if (st) return st;
  if (!origin || !normal || !d_scratch)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL origin, normal or scratch");
  if (!aligned16(d_scratch)) return fail(DAX_GB300_ERROR_BAD_VALUE, "scratch must be 16-byte aligned");
  const McLayout L = mc_layout(g);
  if (scratch_bytes < L.total)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "scratch smaller than dax_gb300_mc_scratch_bytes()");
  const cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!has_cells(g)) {
    cudaError_t e = cudaMemsetAsync(d_scratch, 0, sizeof(Info), s);
    return e == cudaSuccess ? DAX_GB300_SUCCESS : cuda_fail(e, "clearing scratch");
  }
  const int sms = num_sms();
  const float iso = daxgb::slice_isovalue(origin, normal);
  daxgb::GridSet S = daxgb::single_set(g, nullptr, iso, 0.0f);
  S.one.plane_o = make_float3(origin[0], origin[1], origin[2]);
  S.one.plane_n = make_float3(normal[0], normal[1], normal[2]);
  uint32_t* bits = at<uint32_t>(d_scratch, L.bits);
  const daxgb::WordOffsets wo = L.offsets(d_scratch);
  // the row splits live in the active-word list (R <= R * wr entries), which
  // the scan rewrites afterwards
  cudaMemsetAsync(at<Info>(d_scratch, L.info), 0, sizeof(Info), s);  // the error words
  daxgb::launch_slice_bits(g, S.one.plane_o, S.one.plane_n, iso, bits, daxgb::bit_words(g.P),
                           wo.act, sms, s);
  if ((st = check_launch("slice classify kernels"))) return st;
  daxgb::launch_mc_scan(S, bits, wo, at<Info>(d_scratch, L.info), sms, s);
  return check_launch("count/scan kernels");
}

int dax_gb300_slice_generate(const dax_gb300_uniform_grid* grid, const float* origin,
                             const float* normal, int merge, void* d_scratch,
                             size_t scratch_bytes, float* d_verts, int64_t vert_capacity,
                             int32_t* d_conn, int64_t tri_capacity, int32_t* d_rec_first,
                             int32_t* d_rec_second, float* d_rec_weight, void* stream) {
  Grid g;
  int st = make_grid(grid, g);
  if (st) return st;
  if (!has_cells(g)) return DAX_GB300_SUCCESS;
  if (!origin || !normal || !d_scratch)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL origin, normal or scratch");
  if (!aligned16(d_scratch)) return fail(DAX_GB300_ERROR_BAD_VALUE, "scratch must be 16-byte aligned");
  if ((!d_verts && vert_capacity > 0) || (!d_conn && tri_capacity > 0) || vert_capacity < 0 ||
      tri_capacity < 0)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL output with nonzero capacity");
  const McLayout L = mc_layout(g);
  if (scratch_bytes < L.total)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "scratch smaller than dax_gb300_mc_scratch_bytes()");
  daxgb::GridSet S = daxgb::single_set(g, nullptr, daxgb::slice_isovalue(origin, normal), 0.0f);
  S.one.plane_o = make_float3(origin[0], origin[1], origin[2]);
  S.one.plane_n = make_float3(normal[0], normal[1], normal[2]);
  daxgb::launch_mc_emit(S, merge != 0, at<uint32_t>(d_scratch, L.bits), L.offsets(d_scratch),
                        at<Info>(d_scratch, L.info), d_verts, vert_capacity, d_conn, tri_capacity,
                        d_rec_first, d_rec_second, d_rec_weight, num_sms(),
                        static_cast<cudaStream_t>(stream));
  return check_launch("slice generate kernel");
}

int dax_gb300_tetrahedralize(const dax_gb300_uniform_grid* grid, int32_t* d_conn, void* stream) {
  Grid g;
  int st = make_grid(grid, g);
  if (st) return st;
  if (!has_cells(g)) return DAX_GB300_SUCCESS;
  if (!d_conn) return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL connectivity");
  const long long C = (long long)(g.nx - 1) * (g.ny - 1) * (g.nz - 1);
  if (5 * C > 2147483647ll)
    return fail(DAX_GB300_ERROR_UNSUPPORTED, "more than 2^31 - 1 tetrahedra (dax::Id is int32)");
  daxgb::launch_tetrahedralize(g, d_conn, num_sms(), static_cast<cudaStream_t>(stream));
  return check_launch("tetrahedralize kernel");
}

int dax_gb300_point_coordinates(const dax_gb300_uniform_grid* grid, float* d_points,
                                void* stream) {
  Grid g;
  int st = make_grid(grid, g);
  if (st) return st;
  if (!d_points) return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL points");
  daxgb::launch_point_coordinates(g, d_points, num_sms(), static_cast<cudaStream_t>(stream));
  return check_launch("point coordinates kernel");
}

size_t dax_gb300_mt_scratch_bytes(int64_t num_cells) {
  return num_cells < 0 ? 0 : daxgb::mt_layout(num_cells).total;
}

namespace {

int mt_args(const int32_t* conn, int64_t C, const float*& f, int64_t P, const void* scratch,
            size_t bytes) {
  if (C < 0 || P < 0 || C > 2147483647ll || P > 2147483647ll)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "cell and point counts must be in [0, 2^31 - 1]");
  if (C > 0 && (!conn || !f || !scratch))
    return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL connectivity, field or scratch");
  if (bytes < daxgb::mt_layout(C).total)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "scratch smaller than dax_gb300_mt_scratch_bytes()");
  if (reinterpret_cast<uintptr_t>(scratch) & 15)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "scratch must be 16-byte aligned");
  return device_view(f, "field");
}

// Merge scratch: [header: V][keys: 3T][unique keys: 3T][primitive scratch].
struct MtMerge {
  size_t hdr, keys, uniq, prim, prim_bytes, total;
  int type, kb;
};
MtMerge mt_merge_layout(int64_t T, int64_t P) {
  MtMerge M;
  const int bits = daxgb::mt_key_bits(P);
  M.type = 2 * bits > 32 ? DAX_GB300_TYPE_U64 : DAX_GB300_TYPE_U32;
  M.kb = 2 * bits > 32 ? 8 : 4;
  const int64_t n = T > 0 ? 3 * T : 1;
  const size_t sb = dax_gb300_sort_scratch_bytes(n, M.type, 0);
  const size_t cb = dax_gb300_compact_scratch_bytes(n, M.kb);
  M.prim_bytes = sb > cb ? sb : cb;
  M.hdr = 0;
  M.keys = 256;
  M.uniq = align256(M.keys + (size_t)n * M.kb);
  M.prim = align256(M.uniq + (size_t)n * M.kb);
  M.total = align256(M.prim + M.prim_bytes);
  return M;
}

// The keys of the 3T records, written at M.keys: sorted and made unique at
// M.uniq (the reference's Sort + Unique), then the header the merged kernels
// read.  Blocking (the unique count comes back to the host).
int sort_unique_keys(const MtMerge& M, char* m, int64_t T, int64_t P, int64_t* h_num_merged,
                     cudaStream_t s) {
  int64_t V = 0;
  if (T > 0) {
    cudaError_t e = cudaMemcpyAsync(m + M.uniq, m + M.keys, (size_t)(3 * T) * M.kb,
                                    cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return cuda_fail(e, "copying merge keys");
    daxgb::sort_unsigned_bits(m + M.uniq, 3 * T, M.kb == 8, 2 * daxgb::mt_key_bits(P), m + M.prim,
                              s);
    int st = check_launch("merge key sort");
    if (st) return st;
    if ((st = dax_gb300_unique(m + M.uniq, 3 * T, M.type, m + M.prim, M.prim_bytes, &V, s)))
      return st;
  }
  daxgb::launch_mt_set_merged(m + M.hdr, T, V, M.keys, M.uniq, s);
  if (h_num_merged) *h_num_merged = V;
  return check_launch("merge header");
}

// Count-array-driven marching cubes scratch: [Info][inclusive scan: C x i32]
// [scan scratch].
struct CountedLayout {
  size_t info, scan, prim, prim_bytes, total;
};
CountedLayout counted_layout(long long C) {
  CountedLayout L;
  L.info = 0;
  L.scan = align256(sizeof(Info));
  L.prim = align256(L.scan + 4 * (size_t)(C > 0 ? C : 1));
  L.prim_bytes = dax_gb300_scan_scratch_bytes(C > 0 ? C : 1);
  L.total = align256(L.prim + L.prim_bytes);
  return L;
}

long long num_cells_of(const Grid& g) {
  return has_cells(g) ? (long long)(g.nx - 1) * (g.ny - 1) * (g.nz - 1) : 0;
}

}  // namespace

int dax_gb300_mt_count(const int32_t* d_conn, int64_t num_cells, const float* d_field,
                       int64_t num_points, float isovalue, void* d_scratch, size_t scratch_bytes,
                       void* stream) {
  int st = mt_args(d_conn, num_cells, d_field, num_points, d_scratch, scratch_bytes);
  if (st) return st;
  const cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (num_cells == 0) {
    if (!d_scratch) return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL scratch");
    cudaError_t e = cudaMemsetAsync(d_scratch, 0, sizeof(Info), s);
    return e == cudaSuccess ? DAX_GB300_SUCCESS : cuda_fail(e, "clearing scratch");
  }
  daxgb::launch_mt_count(d_conn, num_cells, d_field, num_points, isovalue,
                         static_cast<char*>(d_scratch), num_sms(), s);
  return check_launch("marching tetrahedra count kernels");
}

int dax_gb300_mt_classify_count(const int32_t* d_conn, int64_t num_cells, const float* d_field,
                                int64_t num_points, float isovalue, int32_t* d_count,
                                void* stream) {
  if (num_cells == 0) return DAX_GB300_SUCCESS;
  if (num_cells < 0 || num_points < 0 || num_cells > 2147483647ll || num_points > 2147483647ll)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "cell and point counts must be in [0, 2^31 - 1]");
  if (!d_conn || !d_field || !d_count)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL connectivity, field or count");
  int st = device_view(d_field, "field");
  if (st) return st;
  const cudaStream_t s = static_cast<cudaStream_t>(stream);
  int* err = nullptr;
  cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&err), sizeof(int), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(err, 0, sizeof(int), s);
  if (e != cudaSuccess) return cuda_fail(e, "allocating the error word");
  daxgb::launch_mt_cell_count(d_conn, num_cells, d_field, num_points, isovalue, d_count, err,
                              num_sms(), s);
  int h = 0;
  e = cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaFreeAsync(err, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "marching tetrahedra count kernel");
  if (h & daxgb::kErrBadIndex)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "a cell lists a point id outside [0, num_points)");
  return DAX_GB300_SUCCESS;
}

size_t dax_gb300_mt_merge_scratch_bytes(int64_t num_triangles, int64_t num_points) {
  if (num_triangles < 0 || num_points < 0) return 0;
  return mt_merge_layout(num_triangles, num_points).total;
}

int dax_gb300_mt_merge(const int32_t* d_conn, int64_t num_cells, const float* d_field,
                       int64_t num_points, float isovalue, void* d_scratch, size_t scratch_bytes,
                       void* d_merge, size_t merge_bytes, int64_t* h_num_merged, void* stream) {
  int st = mt_args(d_conn, num_cells, d_field, num_points, d_scratch, scratch_bytes);
  if (st) return st;
  const cudaStream_t s = static_cast<cudaStream_t>(stream);
  int64_t T = 0;
  if (num_cells > 0 && (st = read_totals(d_scratch, &T, nullptr, s))) return st;
  const MtMerge M = mt_merge_layout(T, num_points);
  if (!d_merge || merge_bytes < M.total)
    return fail(DAX_GB300_ERROR_BAD_VALUE,
                "merge scratch smaller than dax_gb300_mt_merge_scratch_bytes()");
  char* m = static_cast<char*>(d_merge);
  if (T > 0) {
    daxgb::launch_mt_emit_keys(d_conn, num_cells, d_field, num_points, isovalue,
                               static_cast<char*>(d_scratch), m + M.keys, num_sms(), s);
    if ((st = check_launch("marching tetrahedra key kernel"))) return st;
  }
  return sort_unique_keys(M, m, T, num_points, h_num_merged, s);
}

int dax_gb300_mt_generate(const float* d_points, const int32_t* d_conn, int64_t num_cells,
                          const float* d_field, int64_t num_points, float isovalue, int merge,
                          void* d_scratch, size_t scratch_bytes, void* d_merge,
                          size_t merge_bytes, float* d_verts, int64_t vert_capacity,
                          int32_t* d_tri_conn, int64_t tri_capacity, int32_t* d_rec_first,
                          int32_t* d_rec_second, float* d_rec_weight, void* stream) {
  int st = mt_args(d_conn, num_cells, d_field, num_points, d_scratch, scratch_bytes);
  if (st) return st;
  if (num_cells == 0) return DAX_GB300_SUCCESS;
  if (!d_points) return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL points");
  if ((st = device_view(d_points, "points"))) return st;
  if ((!d_verts && vert_capacity > 0) || (!d_tri_conn && tri_capacity > 0) || vert_capacity < 0 ||
      tri_capacity < 0)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL output with nonzero capacity");
  if ((d_rec_first || d_rec_second || d_rec_weight) &&
      !(d_rec_first && d_rec_second && d_rec_weight))
    return fail(DAX_GB300_ERROR_BAD_VALUE, "give all three record arrays or none");
  const cudaStream_t s = static_cast<cudaStream_t>(stream);
  char* sc = static_cast<char*>(d_scratch);
  if (!merge) {
    daxgb::launch_mt_emit_direct(d_points, d_conn, num_cells, d_field, num_points, isovalue, sc,
                                 d_verts, vert_capacity, d_tri_conn, tri_capacity, d_rec_first,
                                 d_rec_second, d_rec_weight, num_sms(), s);
    return check_launch("marching tetrahedra emit kernel");
  }
  // the keys, their count and their offsets come from dax_gb300_mt_merge on
  // this scratch (its header); the kernels check the capacities on the device
  if (!d_merge || merge_bytes < 256)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "merge needs the dax_gb300_mt_merge scratch");
  daxgb::launch_mt_merged(d_points, nullptr, at<Info>(sc, daxgb::mt_layout(num_cells).info),
                          d_field, num_points, isovalue, d_merge, merge_bytes, d_verts,
                          vert_capacity, d_tri_conn, tri_capacity, d_rec_first, d_rec_second,
                          d_rec_weight, num_sms(), s);
  return check_launch("marching tetrahedra merged kernels");
}

size_t dax_gb300_mc_counted_scratch_bytes(const dax_gb300_uniform_grid* grid) {
  Grid g;
  if (make_grid(grid, g)) return 0;
  return counted_layout(num_cells_of(g)).total;
}

int dax_gb300_mc_counted_scan(const dax_gb300_uniform_grid* grid, const int32_t* d_count,
                              void* d_scratch, size_t scratch_bytes, int64_t* h_num_triangles,
                              void* stream) {
  Grid g;
  int st = make_grid(grid, g);
  if (st) return st;
  const long long C = num_cells_of(g);
  const CountedLayout L = counted_layout(C);
  if (!d_scratch || scratch_bytes < L.total)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "scratch smaller than dax_gb300_mc_counted_scratch_bytes()");
  if (!aligned16(d_scratch)) return fail(DAX_GB300_ERROR_BAD_VALUE, "scratch must be 16-byte aligned");
  if (C > 0 && !d_count) return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL count array");
  const cudaStream_t s = static_cast<cudaStream_t>(stream);
  char* sc = static_cast<char*>(d_scratch);
  int32_t T32 = 0;
  if (C > 0 && (st = dax_gb300_scan(d_count, sc + L.scan, C, DAX_GB300_TYPE_I32, 0, sc + L.prim,
                                    L.prim_bytes, &T32, stream)))
    return st;
  // the scan wraps like dax::Id; a negative or oversized total cannot be honoured
  const int error = (T32 < 0) ? daxgb::kErrBadCount
                              : (3ll * T32 > 2147483647ll ? daxgb::kErrOverflow : 0);
  daxgb::launch_set_total(at<Info>(sc, L.info), T32 < 0 ? 0 : T32, error, s);
  if ((st = check_launch("counted totals"))) return st;
  if (h_num_triangles) *h_num_triangles = T32 < 0 ? 0 : T32;
  if (error & daxgb::kErrBadCount)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "the count array sums to a negative total");
  if (error) return fail(DAX_GB300_ERROR_UNSUPPORTED, "more than 2^31-1 vertex records");
  return DAX_GB300_SUCCESS;
}

int dax_gb300_mc_counted_merge(const dax_gb300_uniform_grid* grid, const float* d_field,
                               float isovalue, const int32_t* d_count, void* d_scratch,
                               size_t scratch_bytes, void* d_merge, size_t merge_bytes,
                               int64_t* h_num_merged, void* stream) {
  Grid g;
  int st = make_grid(grid, g);
  if (st) return st;
  const long long C = num_cells_of(g);
  const CountedLayout L = counted_layout(C);
  if (!d_scratch || scratch_bytes < L.total)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "scratch smaller than dax_gb300_mc_counted_scratch_bytes()");
  if (!aligned16(d_scratch)) return fail(DAX_GB300_ERROR_BAD_VALUE, "scratch must be 16-byte aligned");
  if (C > 0 && (!d_count || !d_field)) return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL count or field");
  if ((st = device_view(d_field, "field"))) return st;
  const cudaStream_t s = static_cast<cudaStream_t>(stream);
  char* sc = static_cast<char*>(d_scratch);
  int64_t T = 0;
  if ((st = read_totals(sc, &T, nullptr, s))) return st;
  const MtMerge M = mt_merge_layout(T, g.P);
  if (!d_merge || merge_bytes < M.total)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "merge scratch smaller than dax_gb300_mt_merge_scratch_bytes(T, P)");
  char* m = static_cast<char*>(d_merge);
  if (T > 0) {
    daxgb::launch_mc_counted(g, d_field, isovalue, d_count, at<int32_t>(sc, L.scan),
                             at<Info>(sc, L.info), m + M.keys, nullptr, 0, nullptr, 0, nullptr,
                             nullptr, nullptr, T, num_sms(), s);
    if ((st = check_launch("counted key kernel"))) return st;
    // a count the worklet cannot honour shows here, before the keys are used
    if ((st = read_totals(sc, nullptr, nullptr, s))) return st;
  }
  return sort_unique_keys(M, m, T, g.P, h_num_merged, s);
}

int dax_gb300_mc_counted_generate(const dax_gb300_uniform_grid* grid, const float* d_field,
                                  float isovalue, const int32_t* d_count, int merge,
                                  void* d_scratch, size_t scratch_bytes, void* d_merge,
                                  size_t merge_bytes, float* d_verts, int64_t vert_capacity,
                                  int32_t* d_conn, int64_t tri_capacity, int32_t* d_rec_first,
                                  int32_t* d_rec_second, float* d_rec_weight, void* stream) {
  Grid g;
  int st = make_grid(grid, g);
  if (st) return st;
  const long long C = num_cells_of(g);
  if (C == 0) return DAX_GB300_SUCCESS;
  const CountedLayout L = counted_layout(C);
  if (!d_scratch || scratch_bytes < L.total)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "scratch smaller than dax_gb300_mc_counted_scratch_bytes()");
  if (!aligned16(d_scratch)) return fail(DAX_GB300_ERROR_BAD_VALUE, "scratch must be 16-byte aligned");
  if (!d_count || !d_field) return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL count or field");
  if ((st = device_view(d_field, "field"))) return st;
  if ((!d_verts && vert_capacity > 0) || (!d_conn && tri_capacity > 0) || vert_capacity < 0 ||
      tri_capacity < 0)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL output with nonzero capacity");
  if ((d_rec_first || d_rec_second || d_rec_weight) &&
      !(d_rec_first && d_rec_second && d_rec_weight))
    return fail(DAX_GB300_ERROR_BAD_VALUE, "give all three record arrays or none");
  const cudaStream_t s = static_cast<cudaStream_t>(stream);
  char* sc = static_cast<char*>(d_scratch);
  Info* info = at<Info>(sc, L.info);
  if (!merge) {
    daxgb::launch_mc_counted(g, d_field, isovalue, d_count, at<int32_t>(sc, L.scan), info,
                             nullptr, d_verts, vert_capacity, d_conn, tri_capacity, d_rec_first,
                             d_rec_second, d_rec_weight, tri_capacity, num_sms(), s);
    return check_launch("counted generate kernel");
  }
  if (!d_merge || merge_bytes < 256)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "merge needs the dax_gb300_mc_counted_merge scratch");
  daxgb::launch_mt_merged(nullptr, &g, info, d_field, g.P, isovalue, d_merge, merge_bytes,
                          d_verts, vert_capacity, d_conn, tri_capacity, d_rec_first, d_rec_second,
                          d_rec_weight, num_sms(), s);
  return check_launch("counted merged kernels");
}

int dax_gb300_point_magnitude(const dax_gb300_uniform_grid* grid, float* d_field, void* stream) {
  Grid g;
  int st = make_grid(grid, g);
  if (st) return st;
  if (!d_field) return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL field");
  daxgb::launch_point_magnitude(g, d_field, num_sms(), static_cast<cudaStream_t>(stream));
  return check_launch("point magnitude kernel");
}

int dax_gb300_mandelbulb_field(const dax_gb300_uniform_grid* grid, float* d_field, void* stream) {
  Grid g;
  int st = make_grid(grid, g);
  if (st) return st;
  if (!d_field) return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL field");
  daxgb::launch_mandelbulb_field(g, d_field, num_sms(), static_cast<cudaStream_t>(stream));
  return check_launch("mandelbulb field kernel");
}

int dax_gb300_mandelbulb_clip_count(const dax_gb300_uniform_grid* grid, const float* d_field,
                                    float isovalue, const float* origin, const float* location,
                                    const float* normal, int32_t* d_count, void* stream) {
  Grid g;
  int st = make_grid(grid, g);
  if (st) return st;
  if (!has_cells(g)) return DAX_GB300_SUCCESS;
  if (!d_field || !d_count || !origin || !location || !normal)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL argument");
  if ((st = device_view(d_field, "field"))) return st;
  daxgb::launch_mandelbulb_clip_count(
      g, d_field, isovalue, make_float3(origin[0], origin[1], origin[2]),
      make_float3(normal[0], normal[1], normal[2]), daxgb::slice_isovalue(location, normal),
      d_count, num_sms(), static_cast<cudaStream_t>(stream));
  return check_launch("mandelbulb clip count kernel");
}

int dax_gb300_colors_and_norms(const float* d_verts, int64_t num_points, float* d_norms,
                               uint8_t* d_colors, void* stream) {
  if (num_points <= 0) return DAX_GB300_SUCCESS;
  if (num_points % 3) return fail(DAX_GB300_ERROR_BAD_VALUE, "points must come 3 per triangle");
  if (!d_verts || !d_norms || !d_colors) return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL argument");
  if (reinterpret_cast<uintptr_t>(d_colors) & 3)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "colors must be 4-byte aligned");
  daxgb::launch_colors_and_norms(d_verts, num_points, d_norms, d_colors, num_sms(),
                                 static_cast<cudaStream_t>(stream));
  return check_launch("colors and norms kernel");
}

int dax_gb300_interpolate_point_field_n(const int32_t* d_rec_first, const int32_t* d_rec_second,
                                        const float* d_rec_weight, int64_t n, const float* d_in,
                                        int64_t num_points, int components, float* d_out,
                                        void* stream) {
  if (n <= 0) return DAX_GB300_SUCCESS;
  if (components < 1 || components > 16)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "components must be in [1, 16]");
  if (!d_rec_first || !d_rec_second || !d_rec_weight || !d_in || !d_out)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL argument");
  int st = device_view(d_in, "point field");
  if (st) return st;
  daxgb::launch_interpolate_n(d_rec_first, d_rec_second, d_rec_weight, n, num_points, components,
                              d_in, d_out, num_sms(), static_cast<cudaStream_t>(stream));
  return check_launch("interpolate kernel");
}

int dax_gb300_interpolate_point_field(const int32_t* d_rec_first, const int32_t* d_rec_second,
                                      const float* d_rec_weight, int64_t n, const float* d_in,
                                      float* d_out, void* stream) {
  if (n <= 0) return DAX_GB300_SUCCESS;
  if (!d_rec_first || !d_rec_second || !d_rec_weight || !d_in || !d_out)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL argument");
  daxgb::launch_interpolate(d_rec_first, d_rec_second, d_rec_weight, n, d_in, d_out, num_sms(),
                            static_cast<cudaStream_t>(stream));
  return check_launch("interpolate kernel");
}

int dax_gb300_threshold_classify_count(const dax_gb300_uniform_grid* grid, const float* d_field,
                                       float lo, float hi, int32_t* d_count, void* stream) {
  Grid g;
  int st = make_grid(grid, g);
  if (st) return st;
  if (!has_cells(g)) return DAX_GB300_SUCCESS;
  if (!d_field || !d_count) return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL field or count");
  if ((st = device_view(d_field, "field"))) return st;
  daxgb::launch_cell_count(1, g, d_field, lo, hi, d_count, nullptr, num_sms(),
                           static_cast<cudaStream_t>(stream));
  return check_launch("threshold classify-count kernel");
}

size_t dax_gb300_threshold_scratch_bytes(const dax_gb300_uniform_grid* grid) {
  Grid g;
  if (make_grid(grid, g)) return 0;
  return layout(g).total;
}

int dax_gb300_threshold_count(const dax_gb300_uniform_grid* grid, const float* d_field, float lo,
                              float hi, void* d_scratch, size_t scratch_bytes, void* stream) {
  return count_pass(1, grid, d_field, lo, hi, d_scratch, scratch_bytes,
                    static_cast<cudaStream_t>(stream));
}

int dax_gb300_threshold_totals(const void* d_scratch, int64_t* kept_cells, int64_t* used_points,
                               void* stream) {
  return read_totals(d_scratch, kept_cells, used_points, static_cast<cudaStream_t>(stream));
}

int dax_gb300_threshold_compact_point_field(const dax_gb300_uniform_grid* grid,
                                            void* d_scratch, size_t scratch_bytes,
                                            const float* d_in, int components, float* d_out,
                                            int64_t point_capacity, void* stream) {
  Grid g;
  int st = make_grid(grid, g);
  if (st) return st;
  if (!has_cells(g)) return DAX_GB300_SUCCESS;
  if (!d_scratch || !d_in || (!d_out && point_capacity > 0))
    return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL scratch, input or output");
  if (components < 1 || point_capacity < 0)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "components must be >= 1 and the capacity >= 0");
  if (!aligned16(d_scratch)) return fail(DAX_GB300_ERROR_BAD_VALUE, "scratch must be 16-byte aligned");
  if ((st = device_view(d_in, "point field"))) return st;
  const Layout L = layout(g);
  if (scratch_bytes < L.total)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "scratch smaller than dax_gb300_threshold_scratch_bytes()");
  void* sc = d_scratch;  // the kernel raises kErrCapacity in the Info block
  daxgb::launch_thr_compact_field(g, at<uint32_t>(sc, L.used), L.m.offsets(sc).wv,
                                  at<Info>(sc, L.m.info), d_in, components, d_out, point_capacity,
                                  num_sms(), static_cast<cudaStream_t>(stream));
  return check_launch("threshold point-field compaction kernel");
}

int dax_gb300_threshold_generate(const dax_gb300_uniform_grid* grid, const float* d_field,
                                 float lo, float hi, void* d_scratch, size_t scratch_bytes,
                                 int32_t* d_conn, int64_t cell_capacity, float* d_coords,
                                 float* d_field_out, int64_t point_capacity, void* stream) {
  (void)lo;
  (void)hi;
  Grid g;
  int st = make_grid(grid, g);
  if (st) return st;
  if (!has_cells(g)) return DAX_GB300_SUCCESS;
  if (!d_field || !d_scratch) return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL field or scratch");
  if (!aligned16(d_scratch)) return fail(DAX_GB300_ERROR_BAD_VALUE, "scratch must be 16-byte aligned");
  if ((st = device_view(d_field, "field"))) return st;
  if ((!d_conn && cell_capacity > 0) || (!d_coords && point_capacity > 0) || cell_capacity < 0 ||
      point_capacity < 0)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL output with nonzero capacity");
  const Layout L = layout(g);
  if (scratch_bytes < L.total)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "scratch smaller than dax_gb300_threshold_scratch_bytes()");
  daxgb::launch_thr_emit(g, d_field, L.m.offsets(d_scratch), at<uint32_t>(d_scratch, L.kept),
                         at<uint32_t>(d_scratch, L.used), at<Info>(d_scratch, L.m.info), d_conn,
                         cell_capacity, d_coords, d_field_out, point_capacity, num_sms(),
                         static_cast<cudaStream_t>(stream));
  return check_launch("threshold generate kernel");
}

int dax_gb300_cell_gradient(const dax_gb300_uniform_grid* grid, const float* d_field,
                            float* d_gradient, void* stream) {
  Grid g;
  int st = make_grid(grid, g);
  if (st) return st;
  if (!has_cells(g)) return DAX_GB300_SUCCESS;
  if (!d_field || !d_gradient) return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL field or gradient");
  if ((st = device_view(d_field, "field"))) return st;
  daxgb::launch_cell_gradient(g, d_field, d_gradient, num_sms(), static_cast<cudaStream_t>(stream));
  return check_launch("cell gradient kernel");
}

int dax_gb300_field_adjoint(const dax_gb300_uniform_grid* grid, const float* d_field,
                            float isovalue, const void* d_scratch, size_t scratch_bytes,
                            const float* d_grad_vertices, const float* d_grad_cell_gradient,
                            float* d_grad_field, void* stream) {
  Grid g;
  int st = make_grid(grid, g);
  if (st) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!d_grad_field) return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL output");
  if (!has_cells(g) || (!d_grad_vertices && !d_grad_cell_gradient)) {
    cudaError_t e = cudaMemsetAsync(d_grad_field, 0, (size_t)g.P * sizeof(float), s);
    return e == cudaSuccess ? DAX_GB300_SUCCESS : cuda_fail(e, "clearing adjoint");
  }
  if (!d_field) return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL field");
  if ((st = device_view(d_field, "field"))) return st;
  const McLayout L = mc_layout(g);
  if (d_grad_vertices && (!d_scratch || scratch_bytes < L.total))
    return fail(DAX_GB300_ERROR_BAD_VALUE, "vertex adjoint needs the dax_gb300_mc_count scratch");
  void* sc = const_cast<void*>(d_scratch);
  const daxgb::WordOffsets wo = L.offsets(sc);
  daxgb::launch_field_adjoint(g, d_field, isovalue, d_grad_vertices ? at<uint32_t>(sc, L.bits) : nullptr,
                              d_grad_vertices ? &wo : nullptr,
                              d_grad_vertices, d_grad_cell_gradient, d_grad_field, num_sms(), s);
  return check_launch("field adjoint kernel");
}

int dax_gb300_mc_batch_create(int num_grids, const dax_gb300_uniform_grid* grids,
                              const float* const* d_fields, const float* isovalues,
                              dax_gb300_mc_batch** out) {
  if (!out || num_grids < 1 || !grids || !d_fields || !isovalues)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "bad batch arguments");
  *out = nullptr;
  auto* b = new dax_gb300_mc_batch();
  b->count = num_grids;
  b->slots.resize(num_grids);
  for (int i = 0; i < num_grids; ++i) {
    Grid g;
    int st = make_grid(&grids[i], g);
    if (st) { delete b; return st; }
    if (!has_cells(g)) { delete b; return fail(DAX_GB300_ERROR_BAD_VALUE, "batch grid without cells"); }
    if (!d_fields[i]) { delete b; return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL field in batch"); }
    const float* fi = d_fields[i];
    if ((st = device_view(fi, "batch field"))) { delete b; return st; }
    daxgb::GridSlot& sl = b->slots[i];
    sl.g = g;
    sl.field = fi;
    sl.iso = isovalues[i];
    sl.iso_hi = 0.0f;
    sl.chunk0 = b->chunks;
    sl.word0 = 4 * b->chunks;
    sl.row0 = b->rows;
    sl.rw0 = b->rowwords;
    sl.cell0 = b->cells;
    sl.point0 = b->points;
    b->cells += (long long)(g.nx - 1) * (g.ny - 1) * (g.nz - 1);
    b->points += g.P;
    b->grad_vec = b->grad_vec && (sl.cell0 % 2 == 0);
    b->grad_loadv = b->grad_loadv && (g.nx % 2 == 0) && ((reinterpret_cast<uintptr_t>(fi) & 7) == 0);
    b->rowwords += g.R * g.wr;
    b->chunks += (g.P + 127) / 128;
    b->rows += g.R;
    if (g.wr > b->max_wr) b->max_wr = g.wr;
    b->aligned = b->aligned && aligned16(fi);
  }
  b->words = 4 * b->chunks + 8;
  b->off_goff = align256(sizeof(Info));
  b->L = mc_layout_words(b->rowwords, b->words, b->off_goff + 16 * (size_t)(num_grids + 1));
  // per grid, the first block of each grid-set launch
  std::vector<long long> blk(3 * (size_t)(num_grids + 1), 0);
  for (int i = 0; i < num_grids; ++i) {
    const Grid& g = b->slots[i].g;
    const long long n[3] = {daxgb::grad_blocks(g), daxgb::adjoint_grad_blocks(g),
                            daxgb::adjoint_edge_blocks(g)};
    for (int k = 0; k < 3; ++k) blk[k * (num_grids + 1) + i + 1] = blk[k * (num_grids + 1) + i] + n[k];
  }
  for (int k = 0; k < 3; ++k) b->blk_total[k] = blk[k * (num_grids + 1) + num_grids];
  // the slot table (also for one grid: the grid-set launches read it)
  cudaError_t e = cudaMalloc(&b->d_slots, sizeof(daxgb::GridSlot) * num_grids);
  if (e == cudaSuccess)
    e = cudaMemcpy(b->d_slots, b->slots.data(), sizeof(daxgb::GridSlot) * num_grids,
                   cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_blk, blk.size() * sizeof(long long));
  if (e == cudaSuccess)
    e = cudaMemcpy(b->d_blk, blk.data(), blk.size() * sizeof(long long), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    if (b->d_slots) cudaFree(b->d_slots);
    if (b->d_blk) cudaFree(b->d_blk);
    delete b;
    return e == cudaErrorMemoryAllocation ? fail(DAX_GB300_ERROR_OUT_OF_MEMORY, "batch table")
                                          : cuda_fail(e, "uploading batch table");
  }
  *out = b;
  return DAX_GB300_SUCCESS;
}

int dax_gb300_mc_batch_destroy(dax_gb300_mc_batch* b) {
  if (!b) return DAX_GB300_SUCCESS;
  if (b->d_slots) cudaFree(b->d_slots);
  if (b->d_blk) cudaFree(b->d_blk);
  delete b;
  return DAX_GB300_SUCCESS;
}

size_t dax_gb300_mc_batch_scratch_bytes(const dax_gb300_mc_batch* b) { return b ? b->L.total : 0; }

int dax_gb300_mc_batch_count(dax_gb300_mc_batch* b, void* d_scratch, size_t scratch_bytes,
                             void* stream) {
  if (!b || !d_scratch) return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL batch or scratch");
  if (scratch_bytes < b->L.total) return fail(DAX_GB300_ERROR_BAD_VALUE, "batch scratch too small");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const daxgb::GridSet S = b->set();
  uint32_t* bits = at<uint32_t>(d_scratch, b->L.bits);
  // the classification clears Info's error words first
  daxgb::launch_classify_range(0, S, b->aligned, bits, b->words, 0, S.chunks, at<Info>(d_scratch, 0),
                               daxgb::kPassClassify, false, num_sms(), s);
  int st = check_launch("batch classify kernel");
  if (st) return st;
  const daxgb::WordOffsets o = b->L.offsets(d_scratch);
  daxgb::launch_mc_scan(S, bits, o, at<Info>(d_scratch, 0), num_sms(), s, b->dealt);
  if ((st = check_launch("batch count/scan kernels"))) return st;
  daxgb::launch_grid_offsets(S, b->L.offsets(d_scratch), at<long long>(d_scratch, b->off_goff), s);
  return check_launch("batch offsets kernel");
}

int dax_gb300_mc_batch_totals(const dax_gb300_mc_batch* b, const void* d_scratch,
                              int64_t* tri_offsets, int64_t* vert_offsets, void* stream) {
  if (!b || !d_scratch) return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL batch or scratch");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  std::vector<long long> h(2 * (size_t)(b->count + 1));
  cudaError_t e = cudaMemcpyAsync(h.data(), static_cast<const char*>(d_scratch) + b->off_goff,
                                  h.size() * 8, cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return cuda_fail(e, "reading batch offsets");
  int st = read_totals(d_scratch, nullptr, nullptr, s);
  for (int i = 0; i <= b->count; ++i) {
    if (tri_offsets) tri_offsets[i] = h[2 * i];
    if (vert_offsets) vert_offsets[i] = h[2 * i + 1];
  }
  return st;
}

int dax_gb300_mc_batch_generate(dax_gb300_mc_batch* b, int merge, void* d_scratch,
                                size_t scratch_bytes, float* d_verts, int64_t vert_capacity,
                                int32_t* d_conn, int64_t tri_capacity, void* stream) {
  if (!b || !d_scratch) return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL batch or scratch");
  if (scratch_bytes < b->L.total) return fail(DAX_GB300_ERROR_BAD_VALUE, "batch scratch too small");
  if ((!d_verts && vert_capacity > 0) || (!d_conn && tri_capacity > 0))
    return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL output with nonzero capacity");
  const daxgb::GridSet S = b->set();
  Info* info = at<Info>(d_scratch, 0);
  daxgb::launch_mc_emit_range(S, merge != 0, at<uint32_t>(d_scratch, b->L.bits),
                              b->L.offsets(d_scratch), info, d_verts, vert_capacity, d_conn,
                              tri_capacity, nullptr, nullptr, nullptr, 0, S.rowwords, -1, nullptr,
                              &info->ticket, &info->done, b->emit_batch, daxgb::kPassEmit,
                              num_sms(), static_cast<cudaStream_t>(stream));
  return check_launch("batch generate kernel");
}

int dax_gb300_mc_batch_sizes(const dax_gb300_mc_batch* b, int64_t* num_cells,
                             int64_t* num_points) {
  if (!b) return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL batch");
  if (num_cells) *num_cells = b->cells;
  if (num_points) *num_points = b->points;
  return DAX_GB300_SUCCESS;
}

int dax_gb300_mc_batch_cell_gradient(const dax_gb300_mc_batch* b, float* d_out, void* stream) {
  if (!b || (!d_out && b->cells > 0)) return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL batch or output");
  const bool vec = b->grad_vec && (reinterpret_cast<uintptr_t>(d_out) & 7) == 0;
  daxgb::launch_cell_gradient_set(b->set_for_sets(), b->d_blk, b->blk_total[0], vec, b->grad_loadv,
                                  d_out, static_cast<cudaStream_t>(stream));
  return check_launch("batch cell gradient kernel");
}

int dax_gb300_mc_batch_field_adjoint(const dax_gb300_mc_batch* b, const void* d_scratch,
                                     size_t scratch_bytes, const float* d_grad_vertices,
                                     const float* d_grad_cell_gradients, float* d_grad_fields,
                                     void* stream) {
  if (!b || !d_grad_fields) return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL batch or output");
  if (d_grad_vertices && (!d_scratch || scratch_bytes < b->L.total))
    return fail(DAX_GB300_ERROR_BAD_VALUE, "the vertex term needs the batch's count scratch");
  const int n = b->count + 1;
  void* sc = const_cast<void*>(d_scratch);
  const daxgb::WordOffsets wo = d_scratch ? b->L.offsets(sc) : daxgb::WordOffsets{};
  daxgb::launch_field_adjoint_set(b->set_for_sets(), b->d_blk + n, b->blk_total[1],
                                  b->d_blk + 2 * n, b->blk_total[2], b->points,
                                  d_scratch ? at<uint32_t>(sc, b->L.bits) : nullptr, wo.wv,
                                  d_grad_vertices, d_grad_cell_gradients, d_grad_fields,
                                  static_cast<cudaStream_t>(stream));
  return check_launch("batch field adjoint kernels");
}

int dax_gb300_mc_batch_set_config(dax_gb300_mc_batch* b, int emit_batch, int dealt_count) {
  if (!b) return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL batch");
  if (emit_batch < 0 || emit_batch > 32 || dealt_count < -1 || dealt_count > 1)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "emit_batch in [0, 32], dealt_count in [-1, 1]");
  b->emit_batch = emit_batch ? emit_batch : daxgb::kEmitBatch;
  b->dealt = dealt_count < 0 ? 1 : dealt_count;
  return DAX_GB300_SUCCESS;
}

int dax_gb300_mc_batch_get_config(const dax_gb300_mc_batch* b, int* emit_batch, int* dealt_count) {
  if (!b) return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL batch");
  if (emit_batch) *emit_batch = b->emit_batch;
  if (dealt_count) *dealt_count = b->count > 1 ? b->dealt : 0;
  return DAX_GB300_SUCCESS;
}

int dax_gb300_mc_batch_autotune(dax_gb300_mc_batch* b, int merge, void* d_scratch,
                                size_t scratch_bytes, float* d_verts, int64_t vert_capacity,
                                int32_t* d_conn, int64_t tri_capacity, void* stream,
                                float* h_best_ms) {
  if (!b || !d_scratch) return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL batch or scratch");
  // extent class: the number of grids and the log2 of their mean point count
  long long pts = 0;
  for (const auto& sl : b->slots) pts += sl.g.P;
  int lg = 0;
  for (long long m = pts / b->count; m > 1; m >>= 1) ++lg;
  int lc = 0;
  for (int c = b->count; c > 1; c >>= 1) ++lc;
  const long long key = ((long long)lc << 16) | ((long long)lg << 1) | (merge != 0);
  static std::mutex m;
  static std::map<long long, std::pair<int, int>> cache;
  {
    std::lock_guard<std::mutex> lock(m);
    auto it = cache.find(key);
    if (it != cache.end()) {
      b->emit_batch = it->second.first;
      b->dealt = it->second.second;
      if (h_best_ms) *h_best_ms = -1.0f;  // taken from the cache, not timed
      return DAX_GB300_SUCCESS;
    }
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e != cudaSuccess) return cuda_fail(e, "autotune events");
  float best = 1e30f;
  int best_batch = b->emit_batch, best_dealt = b->dealt, st = DAX_GB300_SUCCESS;
  const int batches[3] = {8, 16, 32};
  for (int d = (b->count > 1 ? 1 : 0); d >= 0 && !st; --d)
    for (int bi = 0; bi < 3 && !st; ++bi) {
      b->emit_batch = batches[bi];
      b->dealt = d;
      float total = 0.0f;
      for (int rep = 0; rep < 4 && !st; ++rep) {  // the first run warms up
        e = cudaEventRecord(e0, s);
        st = e == cudaSuccess ? dax_gb300_mc_batch_count(b, d_scratch, scratch_bytes, s)
                              : cuda_fail(e, "autotune");
        if (!st)
          st = dax_gb300_mc_batch_generate(b, merge, d_scratch, scratch_bytes, d_verts,
                                           vert_capacity, d_conn, tri_capacity, s);
        if (!st) e = cudaEventRecord(e1, s);
        if (!st && e == cudaSuccess) e = cudaEventSynchronize(e1);
        float ms = 0.0f;
        if (!st && e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (!st && e != cudaSuccess) st = cuda_fail(e, "autotune timing");
        if (!st && rep > 0) total += ms;
      }
      if (!st) st = read_totals(d_scratch, nullptr, nullptr, s);
      if (!st && total / 3 < best) {
        best = total / 3;
        best_batch = batches[bi];
        best_dealt = d;
      }
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  b->emit_batch = best_batch;
  b->dealt = best_dealt;
  if (st) return st;
  {
    std::lock_guard<std::mutex> lock(m);
    cache[key] = std::make_pair(best_batch, best_dealt);
  }
  if (h_best_ms) *h_best_ms = best;
  return DAX_GB300_SUCCESS;
}

int dax_gb300_mc_batch_capture(dax_gb300_mc_batch* b, int merge, void* d_scratch,
                               size_t scratch_bytes, float* d_verts, int64_t vert_capacity,
                               int32_t* d_conn, int64_t tri_capacity, void** graph) {
  if (!graph) return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL graph handle");
  *graph = nullptr;
  cudaStream_t s;
  cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  if (e != cudaSuccess) return cuda_fail(e, "creating capture stream");
  e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) {
    cudaStreamDestroy(s);
    return cuda_fail(e, "begin capture");
  }
  int st = dax_gb300_mc_batch_count(b, d_scratch, scratch_bytes, s);
  if (!st)
    st = dax_gb300_mc_batch_generate(b, merge, d_scratch, scratch_bytes, d_verts, vert_capacity,
                                     d_conn, tri_capacity, s);
  cudaGraph_t g = nullptr;
  e = cudaStreamEndCapture(s, &g);
  cudaStreamDestroy(s);
  if (st) {
    if (g) cudaGraphDestroy(g);
    return st;
  }
  if (e != cudaSuccess) return cuda_fail(e, "end capture");
  cudaGraphExec_t ex = nullptr;
  e = cudaGraphInstantiate(&ex, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_fail(e, "instantiate graph");
  *graph = ex;
  return DAX_GB300_SUCCESS;
}

int dax_gb300_graph_launch(void* graph, void* stream) {
  if (!graph) return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL graph");
  cudaError_t e = cudaGraphLaunch(static_cast<cudaGraphExec_t>(graph),
                                  static_cast<cudaStream_t>(stream));
  return e == cudaSuccess ? DAX_GB300_SUCCESS : cuda_fail(e, "graph launch");
}

int dax_gb300_graph_destroy(void* graph) {
  if (graph) cudaGraphExecDestroy(static_cast<cudaGraphExec_t>(graph));
  return DAX_GB300_SUCCESS;
}

}  // extern "C"

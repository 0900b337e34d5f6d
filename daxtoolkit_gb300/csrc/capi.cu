// C ABI over the sm_103a kernels (declared in include/dax_gb300.h).
//
// Scratch layout (one buffer, caller-owned, 256-byte aligned sections):
//   [Info][look-back status: 2 x tiles x u64][row_a: (R+1) x i64]
//   [row_b: (R+1) x i64][bits: bit_words(P) x u32][used: R x wr x u32 (threshold)]
// Only the Info block and the status words are cleared per call (a few KB);
// every other byte is fully rewritten by the kernels before it is read.
#include <cstdio>
#include <cstring>
#include <string>

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
  return DAX_GB300_SUCCESS;
}

bool has_cells(const Grid& g) { return g.nx >= 2 && g.ny >= 2 && g.nz >= 2; }

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

struct Layout {
  int tiles;
  size_t info, status, row_a, row_b, bits, used, total, clear;
};

Layout layout(const Grid& g, bool with_used) {
  Layout L;
  L.tiles = (int)((g.R + daxgb::kRowsPerTile - 1) / daxgb::kRowsPerTile);
  L.info = 0;
  L.status = align256(sizeof(Info));
  L.row_a = align256(L.status + 2 * (size_t)L.tiles * 8);
  L.clear = L.row_a;
  L.row_b = align256(L.row_a + (size_t)(g.R + 1) * 8);
  L.bits = align256(L.row_b + (size_t)(g.R + 1) * 8);
  L.used = align256(L.bits + (size_t)daxgb::bit_words(g.P) * 4);
  L.total = with_used ? align256(L.used + (size_t)g.R * g.wr * 4) : L.used;
  return L;
}

template <typename T>
T* at(void* base, size_t off) {
  return reinterpret_cast<T*>(static_cast<char*>(base) + off);
}

int check_launch(const char* where) {
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? DAX_GB300_SUCCESS : cuda_fail(e, where);
}

int read_totals(const void* scratch, int64_t* a, int64_t* b, cudaStream_t s) {
  if (!scratch) return fail(DAX_GB300_ERROR_BAD_VALUE, "scratch is NULL");
  Info h;
  cudaError_t e = cudaMemcpyAsync(&h, scratch, sizeof(Info), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "reading totals");
  if (a) *a = h.total_a;
  if (b) *b = h.total_b;
  if (h.error & daxgb::kErrTimeout)
    return fail(DAX_GB300_ERROR_TIMEOUT, "scan look-back wait expired on the device");
  if (h.error & daxgb::kErrCapacity)
    return fail(DAX_GB300_ERROR_CAPACITY, "output capacity smaller than the result; nothing written");
  return DAX_GB300_SUCCESS;
}

int count_pass(int mode, const dax_gb300_uniform_grid* grid, const float* field, float a, float b,
               void* scratch, size_t bytes, cudaStream_t s) {
  Grid g;
  int st = make_grid(grid, g);
  if (st) return st;
  if (!field || !scratch) return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL field or scratch");
  const Layout L = layout(g, mode == 1);
  if (bytes < L.total) return fail(DAX_GB300_ERROR_BAD_VALUE, "scratch smaller than *_scratch_bytes()");
  cudaError_t e = cudaMemsetAsync(scratch, 0, has_cells(g) ? L.clear : sizeof(Info), s);
  if (e != cudaSuccess) return cuda_fail(e, "clearing scratch");
  if (!has_cells(g)) return DAX_GB300_SUCCESS;  // no cells: totals stay 0
  const int sms = num_sms();
  uint32_t* bits = at<uint32_t>(scratch, L.bits);
  daxgb::launch_classify_bits(mode, field, g.P, a, b, bits, daxgb::bit_words(g.P), sms, s);
  if ((st = check_launch("classify kernel"))) return st;
  Info* info = at<Info>(scratch, L.info);
  auto* status = at<unsigned long long>(scratch, L.status);
  if (mode == 0)
    daxgb::launch_mc_rows(g, bits, at<long long>(scratch, L.row_a), at<long long>(scratch, L.row_b),
                          status, info, L.tiles, s);
  else
    daxgb::launch_thr_rows(g, bits, at<uint32_t>(scratch, L.used), at<long long>(scratch, L.row_a),
                           at<long long>(scratch, L.row_b), status, info, L.tiles, s);
  return check_launch("row count/scan kernel");
}

}  // namespace

extern "C" {

int dax_gb300_abi_version(void) { return DAX_GB300_ABI_VERSION; }

const char* dax_gb300_last_error(void) { return g_last_error.c_str(); }

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
  if (mode != DAX_GB300_CLASSIFY_ABOVE && mode != DAX_GB300_CLASSIFY_IN_RANGE)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "unknown classification mode");
  daxgb::launch_classify_bits(mode, d_field, n, a, b, d_bits, daxgb::bit_words(n), num_sms(),
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
  daxgb::launch_cell_count(0, g, d_field, isovalue, 0.0f, d_count, d_cases, num_sms(),
                           static_cast<cudaStream_t>(stream));
  return check_launch("mc classify-count kernel");
}

size_t dax_gb300_mc_scratch_bytes(const dax_gb300_uniform_grid* grid) {
  Grid g;
  if (make_grid(grid, g)) return 0;
  return layout(g, false).total;
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
  if ((!d_verts && vert_capacity > 0) || (!d_conn && tri_capacity > 0) || vert_capacity < 0 ||
      tri_capacity < 0)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL output with nonzero capacity");
  const Layout L = layout(g, false);
  if (scratch_bytes < L.total)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "scratch smaller than dax_gb300_mc_scratch_bytes()");
  daxgb::launch_mc_emit(g, d_field, isovalue, merge != 0, at<uint32_t>(d_scratch, L.bits),
                        at<long long>(d_scratch, L.row_a), at<long long>(d_scratch, L.row_b),
                        at<Info>(d_scratch, L.info), d_verts, vert_capacity, d_conn, tri_capacity,
                        d_rec_first, d_rec_second, d_rec_weight, num_sms(),
                        static_cast<cudaStream_t>(stream));
  return check_launch("mc generate kernel");
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
  daxgb::launch_cell_count(1, g, d_field, lo, hi, d_count, nullptr, num_sms(),
                           static_cast<cudaStream_t>(stream));
  return check_launch("threshold classify-count kernel");
}

size_t dax_gb300_threshold_scratch_bytes(const dax_gb300_uniform_grid* grid) {
  Grid g;
  if (make_grid(grid, g)) return 0;
  return layout(g, true).total;
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
  if ((!d_conn && cell_capacity > 0) || (!d_coords && point_capacity > 0) || cell_capacity < 0 ||
      point_capacity < 0)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "NULL output with nonzero capacity");
  const Layout L = layout(g, true);
  if (scratch_bytes < L.total)
    return fail(DAX_GB300_ERROR_BAD_VALUE, "scratch smaller than dax_gb300_threshold_scratch_bytes()");
  daxgb::launch_thr_emit(g, d_field, at<uint32_t>(d_scratch, L.bits),
                         at<uint32_t>(d_scratch, L.used), at<long long>(d_scratch, L.row_a),
                         at<long long>(d_scratch, L.row_b), at<Info>(d_scratch, L.info), d_conn,
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
  daxgb::launch_cell_gradient(g, d_field, d_gradient, num_sms(), static_cast<cudaStream_t>(stream));
  return check_launch("cell gradient kernel");
}

}  // extern "C"

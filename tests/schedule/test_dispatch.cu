// TestDispatcher and the worklet checks of the reference's device-adapter
// suite (dax/cont/testing/TestingDeviceAdapter.h:468-560 and :1038-1200),
// restated on dax_gb300::Schedule, which is what a DispatcherMapField /
// DispatcherMapCell of the GB300 tag schedules:
//   * a no-op map-field worklet on one value copies it (NGNoOp);
//   * a multiply worklet on two arrays, then on a constant and an array
//     (NGMult);
//   * a clear worklet scheduled on a subset through a permutation of the
//     even indices (Schedule on Subset);
//   * the Square map-field worklet on a DIM^3 grid's linear field
//     (TestWorkletMapField);
//   * a map-field worklet and a map-cell worklet (an Id3 range of cells) that
//     raise an error, reported as ErrorExecution with the message
//     (TestWorkletFieldMapError, TestWorkletCellMapError);
//   * a map-cell worklet on the DIM^3 grid: the difference of each cell's x
//     corners of the linear field is one spacing (TestWorkletMapCell's
//     gradient, here its x component on the grid's voxels).
// Built and run by tests/test_schedule_gpu.py; prints one line per check and
// exits with the number of failures.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "dax_gb300_schedule.cuh"

namespace {

constexpr int ARRAY_SIZE = 500;
constexpr int OFFSET = 1000;
constexpr int DIM = 8;
constexpr const char* ERROR_MESSAGE = "Got an error.";
int failures = 0;

void check(bool ok, const char* what) {
  std::printf("%s %s\n", ok ? "PASS" : "FAIL", what);
  if (!ok) ++failures;
}

template <typename T>
T* to_device(const std::vector<T>& h) {
  T* d = nullptr;
  cudaMalloc(&d, sizeof(T) * (h.size() ? h.size() : 1));
  cudaMemcpy(d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice);
  return d;
}

template <typename T>
std::vector<T> to_host(const T* d, size_t n) {
  std::vector<T> h(n);
  cudaMemcpy(h.data(), d, sizeof(T) * n, cudaMemcpyDeviceToHost);
  return h;
}

bool near(float a, float b) { return std::fabs(a - b) <= 1e-5f * (1.0f + std::fabs(b)); }

// map-field worklets: one call per value
struct NoOp {
  const int* in;
  int* out;
  __device__ void operator()(long long i) const { out[i] = in[i]; }
};
struct Mult {
  const float* a;
  const float* b;
  float c;  // used when a is null: constant * b
  float* out;
  __device__ void operator()(long long i) const { out[i] = (a ? a[i] : c) * b[i]; }
};
struct ClearPermuted {
  const int* lookup;
  float* full;
  __device__ void operator()(long long i) const { full[lookup[i]] = (float)OFFSET; }
};
struct Square {
  const float* in;
  float* out;
  __device__ void operator()(long long i) const { out[i] = in[i] * in[i]; }
};
struct FieldMapError {
  dax_gb300::ErrorMessageBuffer Errors;
  __device__ void operator()(long long) const { Errors.RaiseError(ERROR_MESSAGE); }
  void SetErrorMessageBuffer(const dax_gb300::ErrorMessageBuffer& b) { Errors = b; }
};
// map-cell worklets: one call per voxel of a DIM^3 point grid
struct CellDx {
  const float* field;
  float* out;
  __device__ void operator()(dax_gb300::IJKIndex c) const {
    const int3 p = c.GetIJK();
    const long long p0 = p.x + (long long)DIM * (p.y + (long long)DIM * p.z);
    out[(long long)c] = field[p0 + 1] - field[p0];
  }
};
struct CellMapError {
  dax_gb300::ErrorMessageBuffer Errors;
  __device__ void operator()(dax_gb300::IJKIndex c) const {
    if ((long long)c == 3) Errors.RaiseError(ERROR_MESSAGE);
  }
  void SetErrorMessageBuffer(const dax_gb300::ErrorMessageBuffer& b) { Errors = b; }
};

}  // namespace

int main() {
  // Dispatcher with one value (NGNoOp)
  {
    int* in = to_device(std::vector<int>{1234});
    int* out = to_device(std::vector<int>{0});
    const int st = dax_gb300::Schedule(NoOp{in, out}, 1);
    check(st == DAX_GB300_SUCCESS && to_host(out, 1)[0] == 1234, "no-op map field of one value");
    cudaFree(in);
    cudaFree(out);
  }
  // NGMult with two arrays, then a constant and an array
  std::vector<float> field(ARRAY_SIZE);
  for (int i = 0; i < ARRAY_SIZE; ++i) field[i] = (float)i;
  float* f = to_device(field);
  float* m = to_device(std::vector<float>(ARRAY_SIZE, 0.0f));
  {
    int st = dax_gb300::Schedule(Mult{f, f, 0.0f, m}, ARRAY_SIZE);
    std::vector<float> h = to_host(m, ARRAY_SIZE);
    bool ok = st == DAX_GB300_SUCCESS;
    for (int i = 0; i < ARRAY_SIZE; ++i) ok = ok && near(h[i], field[i] * field[i]);
    check(ok, "multiply worklet on two arrays");
    st = dax_gb300::Schedule(Mult{nullptr, f, 4.0f, m}, ARRAY_SIZE);
    h = to_host(m, ARRAY_SIZE);
    ok = st == DAX_GB300_SUCCESS;
    for (int i = 0; i < ARRAY_SIZE; ++i) ok = ok && near(h[i], field[i] * 4.0f);
    check(ok, "multiply worklet on a constant and an array");
  }
  // Schedule on a subset through a permutation of the even indices
  {
    std::vector<int> lookup(ARRAY_SIZE / 2);
    for (int i = 0; i < ARRAY_SIZE; i += 2) lookup[i / 2] = i;
    int* d_lookup = to_device(lookup);
    float* full = to_device(std::vector<float>(ARRAY_SIZE, 0.0f));
    const int st = dax_gb300::Schedule(ClearPermuted{d_lookup, full}, ARRAY_SIZE / 2);
    const std::vector<float> h = to_host(full, ARRAY_SIZE);
    bool ok = st == DAX_GB300_SUCCESS;
    for (int i = 0; i < ARRAY_SIZE; ++i) ok = ok && h[i] == (i % 2 == 0 ? (float)OFFSET : 0.0f);
    check(ok, "clear scheduled on the even subset");
    cudaFree(d_lookup);
    cudaFree(full);
  }
  // Square on a DIM^3 grid of dot(coordinates, (1, 1, 1))
  const int P = DIM * DIM * DIM;
  std::vector<float> lin(P);
  for (int k = 0; k < DIM; ++k)
    for (int j = 0; j < DIM; ++j)
      for (int i = 0; i < DIM; ++i) lin[i + DIM * (j + DIM * k)] = (float)(i + j + k);
  float* d_lin = to_device(lin);
  float* sq = to_device(std::vector<float>(P, 0.0f));
  {
    const int st = dax_gb300::Schedule(Square{d_lin, sq}, P);
    const std::vector<float> h = to_host(sq, P);
    bool ok = st == DAX_GB300_SUCCESS;
    for (int p = 0; p < P; ++p) ok = ok && near(h[p], lin[p] * lin[p]);
    check(ok, "square map-field worklet");
  }
  {
    const int st = dax_gb300::Schedule(FieldMapError{}, P);
    check(st == DAX_GB300_ERROR_EXECUTION && std::strcmp(dax_gb300_last_error(), ERROR_MESSAGE) == 0,
          "map-field worklet error reported with its message");
  }
  // map-cell worklets on the DIM^3 grid's voxels
  const int C = (DIM - 1) * (DIM - 1) * (DIM - 1);
  float* dx = to_device(std::vector<float>(C, 0.0f));
  {
    const int st = dax_gb300::Schedule(CellDx{d_lin, dx}, make_int3(DIM - 1, DIM - 1, DIM - 1));
    const std::vector<float> h = to_host(dx, C);
    bool ok = st == DAX_GB300_SUCCESS;
    for (int c = 0; c < C; ++c) ok = ok && h[c] == 1.0f;
    check(ok, "map-cell worklet on the voxels");
  }
  {
    const int st = dax_gb300::Schedule(CellMapError{}, make_int3(DIM - 1, DIM - 1, DIM - 1));
    check(st == DAX_GB300_ERROR_EXECUTION && std::strcmp(dax_gb300_last_error(), ERROR_MESSAGE) == 0,
          "map-cell worklet error reported with its message");
  }
  cudaFree(f);
  cudaFree(m);
  cudaFree(d_lin);
  cudaFree(sq);
  cudaFree(dx);
  std::printf("%d failures\n", failures);
  return failures;
}

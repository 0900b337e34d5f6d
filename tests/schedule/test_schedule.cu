// TestAlgorithmSchedule and TestErrorExecution of the reference's device
// adapter suite (dax/cont/testing/TestingDeviceAdapter.h:382-466, :1003-1036),
// restated for dax_gb300::Schedule: ClearArrayKernel then AddArrayKernel on 1
// and on ARRAY_SIZE instances and on an Id3 range of ceil(cbrt(ARRAY_SIZE))^3;
// a kernel that raises one error and one where every instance raises, both
// reported with their message; a schedule after an error runs clean.  Built
// and run by tests/test_schedule_gpu.py; prints one line per check and exits
// with the number of failures.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "dax_gb300_schedule.cuh"

namespace {

constexpr int ARRAY_SIZE = 500;
constexpr int OFFSET = 1000;
constexpr const char* ERROR_MESSAGE = "Got an error.";
int failures = 0;

void check(bool ok, const char* what) {
  std::printf("%s %s\n", ok ? "PASS" : "FAIL", what);
  if (!ok) ++failures;
}

struct ClearArrayKernel {
  int* array;
  __device__ void operator()(long long index) const { array[index] = OFFSET; }
};

struct AddArrayKernel {
  int* array;
  __device__ void operator()(long long index) const { array[index] = array[index] + (int)index; }
};

struct OneErrorKernel {
  dax_gb300::ErrorMessageBuffer Errors;
  __device__ void operator()(long long index) const {
    if (index == ARRAY_SIZE / 2) Errors.RaiseError(ERROR_MESSAGE);
  }
  void SetErrorMessageBuffer(const dax_gb300::ErrorMessageBuffer& b) { Errors = b; }
};

struct AllErrorKernel {
  dax_gb300::ErrorMessageBuffer Errors;
  __device__ void operator()(long long) const { Errors.RaiseError(ERROR_MESSAGE); }
  void SetErrorMessageBuffer(const dax_gb300::ErrorMessageBuffer& b) { Errors = b; }
};

// Writes i + 10 j + 100 k at the flat index, checking the flat id itself.
struct IJKKernel {
  int* array;
  int3 range;
  int* bad;
  __device__ void operator()(dax_gb300::IJKIndex index) const {
    const int3 p = index.GetIJK();
    if ((long long)index != p.x + (long long)range.x * (p.y + (long long)range.y * p.z)) atomicAdd(bad, 1);
    array[(long long)index] = p.x + 10 * p.y + 100 * p.z;
  }
};

std::vector<int> fetch(const int* d, int n) {
  std::vector<int> h(n);
  cudaMemcpy(h.data(), d, sizeof(int) * n, cudaMemcpyDeviceToHost);
  return h;
}

}  // namespace

int main() {
  int* d = nullptr;
  const int dim = (int)std::ceil(std::cbrt((double)ARRAY_SIZE));
  const int n3 = dim * dim * dim;
  cudaMalloc(&d, sizeof(int) * n3);

  // single instance, then ARRAY_SIZE instances
  for (int n : {1, ARRAY_SIZE}) {
    int st = dax_gb300::Schedule(ClearArrayKernel{d}, n);
    st |= dax_gb300::Schedule(AddArrayKernel{d}, n);
    const std::vector<int> h = fetch(d, n);
    bool ok = st == DAX_GB300_SUCCESS;
    for (int i = 0; i < n; ++i) ok = ok && h[i] == i + OFFSET;
    check(ok, n == 1 ? "schedule one instance" : "schedule ARRAY_SIZE instances");
  }

  // an Id3 range: the same kernels see the flat index
  {
    const int3 r = make_int3(dim, dim, dim);
    int st = dax_gb300::Schedule(ClearArrayKernel{d}, r);
    st |= dax_gb300::Schedule(AddArrayKernel{d}, r);
    const std::vector<int> h = fetch(d, n3);
    bool ok = st == DAX_GB300_SUCCESS;
    for (int i = 0; i < n3; ++i) ok = ok && h[i] == i + OFFSET;
    check(ok, "schedule an Id3 range");
  }

  // IJK indices of a ragged range
  {
    const int3 r = make_int3(7, 5, 3);
    int* bad = nullptr;
    cudaMalloc(&bad, sizeof(int));
    cudaMemset(bad, 0, sizeof(int));
    const int st = dax_gb300::Schedule(IJKKernel{d, r, bad}, r);
    const std::vector<int> h = fetch(d, 105);
    bool ok = st == DAX_GB300_SUCCESS && fetch(bad, 1)[0] == 0;
    for (int k = 0; k < 3; ++k)
      for (int j = 0; j < 5; ++j)
        for (int i = 0; i < 7; ++i) ok = ok && h[i + 7 * (j + 5 * k)] == i + 10 * j + 100 * k;
    check(ok, "schedule IJK indices of a 7 x 5 x 3 range");
    cudaFree(bad);
  }

  // errors raised in the execution environment
  {
    const int st = dax_gb300::Schedule(OneErrorKernel{}, ARRAY_SIZE);
    check(st == DAX_GB300_ERROR_EXECUTION && std::strcmp(dax_gb300_last_error(), ERROR_MESSAGE) == 0,
          "one raised error reported with its message");
  }
  {
    const int st = dax_gb300::Schedule(AllErrorKernel{}, ARRAY_SIZE);
    check(st == DAX_GB300_ERROR_EXECUTION && std::strcmp(dax_gb300_last_error(), ERROR_MESSAGE) == 0,
          "every instance raising reported once with its message");
  }
  {
    const int st = dax_gb300::Schedule(ClearArrayKernel{d}, ARRAY_SIZE);
    check(st == DAX_GB300_SUCCESS, "a schedule after an error runs clean");
  }
  {
    const int st = dax_gb300::Schedule(ClearArrayKernel{d}, 0);
    check(st == DAX_GB300_SUCCESS, "an empty schedule");
  }
  cudaFree(d);
  std::printf("%d failures\n", failures);
  return failures;
}

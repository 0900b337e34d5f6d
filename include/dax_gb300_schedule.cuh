/* Schedule of arbitrary functors on the GB300 device adapter: the
 * DeviceAdapterAlgorithm::Schedule(functor, numInstances) and
 * Schedule(functor, Id3 rangeMax) of dax/cont/internal/DeviceAdapterAlgorithm.h
 * for CUDA C++ callers (the reference's own interface is a template, so this
 * part of the adapter is a header, compiled with the caller's functors).
 *
 *   struct Kernel {
 *     __device__ void operator()(long long index) const { ... }
 *     // optional, as in the reference: receives the error buffer
 *     void SetErrorMessageBuffer(const dax_gb300::ErrorMessageBuffer& b) { Errors = b; }
 *     dax_gb300::ErrorMessageBuffer Errors;
 *   };
 *   int st = dax_gb300::Schedule(Kernel{...}, n);          // index = 0 .. n-1
 *   int st = dax_gb300::Schedule(Kernel{...}, make_int3(nx, ny, nz));
 *
 * With an int3 range the functor is called with an IJKIndex, which converts
 * to the flat index i + nx * (j + ny * k) and carries (i, j, k)
 * (dax/exec/internal/IJKIndex.h).  Schedule is synchronous, like the
 * reference's: after the launch it returns DAX_GB300_ERROR_EXECUTION when a
 * functor raised an error, and dax_gb300_last_error() then holds the first
 * message raised (DeviceAdapterAlgorithmSerial.h:121-176).  Launch failures
 * return DAX_GB300_ERROR_CUDA.  Link with libdax_gb300. */
#ifndef DAX_GB300_SCHEDULE_CUH
#define DAX_GB300_SCHEDULE_CUH

#include <stdint.h>

#include <mutex>

#include <cuda_runtime.h>

#include "dax_gb300.h"

namespace dax_gb300 {

/* Device error buffer (dax/exec/internal/ErrorMessageBuffer.h): a claim word
 * then the message.  The first RaiseError of a launch claims the word
 * atomically and writes its message; later ones return. */
class ErrorMessageBuffer {
 public:
  __host__ __device__ ErrorMessageBuffer() : Claim(nullptr), Message(nullptr), Size(0) {}
  __host__ __device__ ErrorMessageBuffer(int* claim, char* message, int size)
      : Claim(claim), Message(message), Size(size) {}

  __device__ void RaiseError(const char* message) const {
    if (!Claim || atomicCAS(Claim, 0, 1) != 0) return;
    int n = 0;
    for (; n < Size - 1 && message[n] != '\0'; ++n) Message[n] = message[n];
    Message[n] = '\0';
    __threadfence();
  }

  __device__ bool IsErrorRaised() const {
    return Claim && *static_cast<volatile int*>(Claim) != 0;
  }

 private:
  int* Claim;
  char* Message;
  int Size;
};

/* Index of a 3D schedule: (i, j, k) and its flat id. */
struct IJKIndex {
  int3 ijk;
  long long flat;
  __device__ operator long long() const { return flat; }
  __device__ int3 GetIJK() const { return ijk; }
};

namespace detail {

constexpr int kMessageSize = 1024;

template <class F>
__global__ void __launch_bounds__(256) schedule_flat(F functor, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    functor(i);
}

template <class F>
__global__ void __launch_bounds__(256) schedule_ijk(F functor, int3 range) {
  const long long n = (long long)range.x * range.y * range.z;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    const long long row = p / range.x;
    IJKIndex index;
    index.ijk = make_int3((int)(p - row * range.x), (int)(row % range.y), (int)(row / range.y));
    index.flat = p;
    functor(index);
  }
}

// SetErrorMessageBuffer when the functor declares it.
template <class F>
auto give_buffer(F& f, const ErrorMessageBuffer& b, int) -> decltype(f.SetErrorMessageBuffer(b), void()) {
  f.SetErrorMessageBuffer(b);
}
template <class F>
void give_buffer(F&, const ErrorMessageBuffer&, long) {}

// The calling device's claim word and message, allocated once per device
// (under a lock, so that host threads starting at once allocate it once).
// Schedules on one device share it: as in the reference, whose control
// environment is single-threaded, one host thread schedules on a device at
// a time.
inline int device_buffer(int** claim, char** message) {
  static int* claims[64] = {nullptr};
  static std::mutex lock;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return DAX_GB300_ERROR_CUDA;
  std::lock_guard<std::mutex> guard(lock);
  if (!claims[dev]) {
    void* p = nullptr;
    if (cudaMalloc(&p, sizeof(int) + kMessageSize) != cudaSuccess) return DAX_GB300_ERROR_OUT_OF_MEMORY;
    claims[dev] = static_cast<int*>(p);
  }
  *claim = claims[dev];
  *message = reinterpret_cast<char*>(claims[dev] + 1);
  return DAX_GB300_SUCCESS;
}

template <class K>
inline int resident_grid(K kernel, long long work) {
  int dev = 0, sms = 1, per = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, 256, 0) != cudaSuccess || per < 1)
    per = 1;
  const long long want = (work + 255) / 256, cap = (long long)sms * per;
  return (int)(want < 1 ? 1 : (want < cap ? want : cap));
}

// Clears the claim word, launches, waits, and turns a raised error into
// DAX_GB300_ERROR_EXECUTION with its message as the library's last error.
template <class K, class F, class R>
inline int run(K kernel, F functor, R range, long long work, cudaStream_t s) {
  int* claim = nullptr;
  char* message = nullptr;
  int st = device_buffer(&claim, &message);
  if (st) return dax_gb300_report_error(st, "no device error buffer");
  give_buffer(functor, ErrorMessageBuffer(claim, message, kMessageSize), 0);
  if (cudaMemsetAsync(claim, 0, sizeof(int) + 1, s) != cudaSuccess)
    return dax_gb300_report_error(DAX_GB300_ERROR_CUDA, "clearing the error buffer");
  if (work > 0) kernel<<<resident_grid(kernel, work), 256, 0, s>>>(functor, range);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return dax_gb300_report_error(DAX_GB300_ERROR_CUDA, cudaGetErrorString(e));
  int raised = 0;
  char text[kMessageSize];
  if (cudaMemcpy(&raised, claim, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess ||
      (raised && cudaMemcpy(text, message, kMessageSize, cudaMemcpyDeviceToHost) != cudaSuccess))
    return dax_gb300_report_error(DAX_GB300_ERROR_CUDA, "reading the error buffer");
  if (!raised) return DAX_GB300_SUCCESS;
  text[kMessageSize - 1] = '\0';
  return dax_gb300_report_error(DAX_GB300_ERROR_EXECUTION, text);
}

}  // namespace detail

/* functor(index) for index = 0 .. numInstances - 1. */
template <class F>
inline int Schedule(F functor, long long numInstances, cudaStream_t stream = 0) {
  return detail::run(detail::schedule_flat<F>, functor, numInstances,
                     numInstances > 0 ? numInstances : 0, stream);
}

/* functor(IJKIndex) over 0 .. rangeMax - 1 in each dimension, i fastest. */
template <class F>
inline int Schedule(F functor, int3 rangeMax, cudaStream_t stream = 0) {
  const long long n = (rangeMax.x > 0 && rangeMax.y > 0 && rangeMax.z > 0)
                          ? (long long)rangeMax.x * rangeMax.y * rangeMax.z
                          : 0;
  return detail::run(detail::schedule_ijk<F>, functor, rangeMax, n, stream);
}

}  // namespace dax_gb300

#endif  // DAX_GB300_SCHEDULE_CUH

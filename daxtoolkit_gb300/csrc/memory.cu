// Device memory, copies and timers behind the C ABI, for a host side that
// links only this library: the ArrayManagerExecution and
// DeviceAdapterTimerImplementation of the GB300 device-adapter tag
// (include/dax_gb300_tag.h) are written on these calls, so that host code
// needs no CUDA headers and the process holds one CUDA runtime.
#include <atomic>
#include <cstdint>
#include <string>

#include "../../include/dax_gb300.h"
#include "kernels.cuh"

namespace {

std::atomic<unsigned long long> g_alloc_limit{~0ull};

int mem_fail(int code, const std::string& msg) {
  daxgb::set_last_error(msg);
  return code;
}

struct Timer {
  cudaEvent_t start = nullptr, stop = nullptr;
};

}  // namespace

extern "C" {

int dax_gb300_set_alloc_limit(uint64_t bytes) {
  g_alloc_limit.store(bytes == 0 ? ~0ull : bytes);
  return DAX_GB300_SUCCESS;
}

int dax_gb300_device_alloc(void** d_ptr, uint64_t bytes) {
  if (!d_ptr) return mem_fail(DAX_GB300_ERROR_BAD_VALUE, "NULL output pointer");
  *d_ptr = nullptr;
  if (bytes == 0) return DAX_GB300_SUCCESS;
  if (bytes > g_alloc_limit.load())
    return mem_fail(DAX_GB300_ERROR_OUT_OF_MEMORY,
                    "allocation of " + std::to_string(bytes) + " bytes above the set limit");
  const cudaError_t e = cudaMalloc(d_ptr, (size_t)bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();  // an out-of-memory error is not sticky; clear it
    *d_ptr = nullptr;
    return mem_fail(e == cudaErrorMemoryAllocation ? DAX_GB300_ERROR_OUT_OF_MEMORY
                                                   : DAX_GB300_ERROR_CUDA,
                    "could not allocate " + std::to_string(bytes) + " bytes of device memory: " +
                        cudaGetErrorString(e));
  }
  return DAX_GB300_SUCCESS;
}

int dax_gb300_device_free(void* d_ptr) {
  if (!d_ptr) return DAX_GB300_SUCCESS;
  const cudaError_t e = cudaFree(d_ptr);
  return e == cudaSuccess ? DAX_GB300_SUCCESS
                          : mem_fail(DAX_GB300_ERROR_CUDA,
                                     std::string("cudaFree: ") + cudaGetErrorString(e));
}

int dax_gb300_memcpy(void* dst, const void* src, uint64_t bytes, int kind) {
  if (bytes == 0) return DAX_GB300_SUCCESS;
  if (!dst || !src) return mem_fail(DAX_GB300_ERROR_BAD_VALUE, "NULL copy pointer");
  cudaMemcpyKind k;
  switch (kind) {
    case DAX_GB300_HOST_TO_DEVICE: k = cudaMemcpyHostToDevice; break;
    case DAX_GB300_DEVICE_TO_HOST: k = cudaMemcpyDeviceToHost; break;
    case DAX_GB300_DEVICE_TO_DEVICE: k = cudaMemcpyDeviceToDevice; break;
    default: return mem_fail(DAX_GB300_ERROR_BAD_VALUE, "unknown copy kind");
  }
  const cudaError_t e = cudaMemcpy(dst, src, (size_t)bytes, k);
  return e == cudaSuccess ? DAX_GB300_SUCCESS
                          : mem_fail(DAX_GB300_ERROR_CUDA,
                                     std::string("cudaMemcpy: ") + cudaGetErrorString(e));
}

int dax_gb300_timer_create(void** timer) {
  if (!timer) return mem_fail(DAX_GB300_ERROR_BAD_VALUE, "NULL timer pointer");
  Timer* t = new Timer;
  cudaError_t e = cudaEventCreate(&t->start);
  if (e == cudaSuccess) e = cudaEventCreate(&t->stop);
  if (e != cudaSuccess) {
    if (t->start) cudaEventDestroy(t->start);
    delete t;
    return mem_fail(DAX_GB300_ERROR_CUDA, std::string("cudaEventCreate: ") + cudaGetErrorString(e));
  }
  *timer = t;
  return DAX_GB300_SUCCESS;
}

int dax_gb300_timer_start(void* timer, void* stream) {
  Timer* t = static_cast<Timer*>(timer);
  if (!t) return mem_fail(DAX_GB300_ERROR_BAD_VALUE, "NULL timer");
  const cudaError_t e = cudaEventRecord(t->start, static_cast<cudaStream_t>(stream));
  return e == cudaSuccess ? DAX_GB300_SUCCESS
                          : mem_fail(DAX_GB300_ERROR_CUDA,
                                     std::string("cudaEventRecord: ") + cudaGetErrorString(e));
}

int dax_gb300_timer_elapsed(void* timer, void* stream, double* seconds) {
  Timer* t = static_cast<Timer*>(timer);
  if (!t || !seconds) return mem_fail(DAX_GB300_ERROR_BAD_VALUE, "NULL timer or output");
  cudaError_t e = cudaEventRecord(t->stop, static_cast<cudaStream_t>(stream));
  if (e == cudaSuccess) e = cudaEventSynchronize(t->stop);
  float ms = 0.0f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, t->start, t->stop);
  if (e != cudaSuccess)
    return mem_fail(DAX_GB300_ERROR_CUDA, std::string("timer: ") + cudaGetErrorString(e));
  *seconds = ms / 1000.0;
  return DAX_GB300_SUCCESS;
}

int dax_gb300_timer_destroy(void* timer) {
  Timer* t = static_cast<Timer*>(timer);
  if (!t) return DAX_GB300_SUCCESS;
  cudaEventDestroy(t->start);
  cudaEventDestroy(t->stop);
  delete t;
  return DAX_GB300_SUCCESS;
}

}  // extern "C"

// Marching cubes for callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc at the point where they need an
// isosurface: code running inside a fixed memory budget that was reserved up
// front (for example a renderer or simulation that hands the whole device to
// its own pool allocator), code that must not take the allocator's locks or
// risk an out-of-memory failure on a latency-critical path, and plugin hosts
// that give a plugin only the buffers they pass in.  dax_gb300_mc_noalloc
// serves them: it runs the same count + generate pipeline as
// dax_gb300_mc_count / dax_gb300_mc_generate, but its scratch is a fixed-size
// array compiled into this library instead of caller-provided memory, and it
// calls no allocating routine (no cudaMalloc, cudaFree or library allocator).
//
// The array is file-scope device memory: every GPU that loads the library
// holds it until the process exits, and every call on a device shares it.
#include <mutex>
#include <string>

#include "../../include/dax_gb300.h"
#include "common.cuh"
#include "kernels.cuh"

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;  // 32 MiB per device

// The scratch itself.  In host code this name is only a stand-in for the
// symbol, never a device address: the address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
void* g_scratch_ptr[kMaxDevices] = {nullptr};

// Device address of the scratch on the current device, looked up once per
// device with that device current (the first call on each device does this
// set-up, which is why that first call belongs outside any stream capture).
// The address is kept for the life of the process, so a cudaDeviceReset
// after the first call on a device is not supported: the reset unloads the
// module that holds the array.
int scratch_address(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    daxgb::set_last_error(std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    return DAX_GB300_ERROR_CUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    daxgb::set_last_error("device index out of range for the no-allocation scratch table");
    return DAX_GB300_ERROR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      daxgb::set_last_error(std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      return DAX_GB300_ERROR_CUDA;
    }
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return DAX_GB300_SUCCESS;
}

// d_totals must be memory the device can write 8-byte words to: device or
// managed memory, or page-locked host memory with a device mapping (then its
// device address is used).  Pageable host memory and pointers off an 8-byte
// boundary are refused before anything is queued.
int totals_view(int64_t** p) {
  if (reinterpret_cast<uintptr_t>(*p) & 7) {
    daxgb::set_last_error("d_totals must be 8-byte aligned");
    return DAX_GB300_ERROR_BAD_VALUE;
  }
  cudaPointerAttributes a;
  const cudaError_t e = cudaPointerGetAttributes(&a, *p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    daxgb::set_last_error("d_totals is not memory known to CUDA");
    return DAX_GB300_ERROR_BAD_VALUE;
  }
  if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return DAX_GB300_SUCCESS;
  if (a.type == cudaMemoryTypeHost && a.devicePointer) {
    *p = static_cast<int64_t*>(a.devicePointer);
    return DAX_GB300_SUCCESS;
  }
  daxgb::set_last_error("d_totals is pageable host memory: pass device memory or page-locked "
                        "host memory");
  return DAX_GB300_ERROR_BAD_VALUE;
}

// Copies the pipeline's totals and device error bits out of the scratch.
__global__ void k_noalloc_totals(const daxgb::Info* __restrict__ info, int64_t* __restrict__ out) {
  out[0] = info->total_a;
  out[1] = info->total_b;
  out[2] = info->error;
}

}  // namespace

extern "C" {

int dax_gb300_mc_noalloc(const dax_gb300_uniform_grid* grid, const float* d_field, float isovalue,
                         int merge, float* d_verts, int64_t vert_capacity, int32_t* d_conn,
                         int64_t tri_capacity, int64_t* d_totals, void* stream) {
  if (!d_totals) {
    daxgb::set_last_error("d_totals is NULL");
    return DAX_GB300_ERROR_BAD_VALUE;
  }
  const size_t need = dax_gb300_mc_scratch_bytes(grid);
  if (need == 0) {
    daxgb::set_last_error("invalid grid");
    return DAX_GB300_ERROR_BAD_VALUE;
  }
  if (need > kNoAllocScratchBytes) {
    daxgb::set_last_error("grid needs " + std::to_string(need) +
                          " bytes of scratch; dax_gb300_mc_noalloc holds " +
                          std::to_string(kNoAllocScratchBytes) + " bytes (32 MiB)");
    return DAX_GB300_ERROR_UNSUPPORTED;
  }
  int st = totals_view(&d_totals);
  if (st) return st;
  void* scratch = nullptr;
  st = scratch_address(&scratch);
  if (st) return st;
  // the count pass writes every scratch byte the generate pass reads
  st = dax_gb300_mc_count(grid, d_field, isovalue, scratch, kNoAllocScratchBytes, stream);
  if (st) return st;
  st = dax_gb300_mc_generate(grid, d_field, isovalue, merge, scratch, kNoAllocScratchBytes, d_verts,
                             vert_capacity, d_conn, tri_capacity, nullptr, nullptr, nullptr,
                             stream);
  if (st) return st;
  k_noalloc_totals<<<1, 1, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const daxgb::Info*>(scratch), d_totals);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    daxgb::set_last_error(std::string("totals kernel: ") + cudaGetErrorString(e));
    return DAX_GB300_ERROR_CUDA;
  }
  return DAX_GB300_SUCCESS;
}

}  // extern "C"

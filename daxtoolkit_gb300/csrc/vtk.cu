// Legacy-VTK POLYDATA writer (Benchmarks/MarchingCubes/Pipeline.h:51-98,
// PrintContentsToStream): the same bytes the reference's std::ostream writer
// produces -- four header lines, "POINTS n float", each point's three
// coordinates followed by a space with a newline after every third point
// (and one after the last if n is not a multiple of 3), "POLYGONS c c*(V+1)",
// one "V id id id" line per cell, then an empty line.  std::ostream prints a
// float as printf's %g of its double value with precision 6, which is what
// snprintf("%.6g") writes here.
//
// Host code: the points and connectivity may be in device memory (copied to
// the host first) or in host memory.  The text is formatted by several host
// threads over disjoint point and cell ranges and written in order.
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/dax_gb300.h"
#include "kernels.cuh"

namespace {

int vtk_fail(int code, const std::string& msg) {
  daxgb::set_last_error(msg);
  return code;
}

bool is_device(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();  // no device, or unknown host memory
    return false;
  }
  return a.type == cudaMemoryTypeDevice;
}

// Host copy of n elements of p when p is device memory, else p itself.
template <typename T>
const T* host_view(const T* p, long long n, std::vector<T>& keep, int* st) {
  *st = DAX_GB300_SUCCESS;
  if (n == 0 || !is_device(p)) return p;
  keep.resize((size_t)n);
  const cudaError_t e = cudaMemcpy(keep.data(), p, sizeof(T) * (size_t)n, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) {
    *st = vtk_fail(DAX_GB300_ERROR_CUDA, std::string("copying to the host: ") + cudaGetErrorString(e));
    return nullptr;
  }
  return keep.data();
}

void append_g(std::string& s, float v) {
  char buf[32];
  const int n = snprintf(buf, sizeof(buf), "%.6g", (double)v);
  s.append(buf, (size_t)n);
}

void append_i(std::string& s, long long v) {
  char buf[24];
  const int n = snprintf(buf, sizeof(buf), "%lld", v);
  s.append(buf, (size_t)n);
}

// Formats items [b, e) of `fmt` on `threads` threads into `parts`, in order.
template <typename F>
void format_parallel(long long n, int threads, std::vector<std::string>& parts, F fmt) {
  parts.assign((size_t)threads, std::string());
  std::vector<std::thread> pool;
  const long long per = (n + threads - 1) / threads;
  for (int t = 0; t < threads; ++t) {
    const long long b = t * per, e = b + per < n ? b + per : n;
    if (b >= e) break;
    pool.emplace_back([&, t, b, e] { fmt(parts[(size_t)t], b, e); });
  }
  for (auto& th : pool) th.join();
}

}  // namespace

extern "C" int dax_gb300_write_vtk_polydata(const char* path, const float* points,
                                            int64_t num_points, const int32_t* conn,
                                            int64_t num_cells, int verts_per_cell) {
  if (!path) return vtk_fail(DAX_GB300_ERROR_BAD_VALUE, "NULL path");
  if (num_points < 0 || num_cells < 0 || verts_per_cell < 1)
    return vtk_fail(DAX_GB300_ERROR_BAD_VALUE, "negative size or no vertices per cell");
  if ((num_points > 0 && !points) || (num_cells > 0 && !conn))
    return vtk_fail(DAX_GB300_ERROR_BAD_VALUE, "NULL points or connectivity");
  int st;
  std::vector<float> hp;
  std::vector<int32_t> hc;
  const float* P = host_view(points, 3 * num_points, hp, &st);
  if (st) return st;
  const int32_t* K = host_view(conn, num_cells * verts_per_cell, hc, &st);
  if (st) return st;
  unsigned hw = std::thread::hardware_concurrency();
  const int threads = (int)(hw < 1 ? 1 : (hw > 64 ? 64 : hw));
  std::vector<std::string> pts, cells;
  format_parallel(num_points, threads, pts, [&](std::string& s, long long b, long long e) {
    s.reserve((size_t)(e - b) * 40);
    for (long long i = b; i < e; ++i) {
      for (int a = 0; a < 3; ++a) {
        append_g(s, P[3 * i + a]);
        s.push_back(' ');
      }
      if (i % 3 == 2) s.push_back('\n');
    }
  });
  const int V = verts_per_cell;
  format_parallel(num_cells, threads, cells, [&](std::string& s, long long b, long long e) {
    s.reserve((size_t)(e - b) * (4 + 11 * V));
    for (long long c = b; c < e; ++c) {
      append_i(s, V);
      for (int v = 0; v < V; ++v) {
        s.push_back(' ');
        append_i(s, K[c * V + v]);
      }
      s.push_back('\n');
    }
  });
  FILE* fp = fopen(path, "wb");
  if (!fp) return vtk_fail(DAX_GB300_ERROR_BAD_VALUE, std::string("cannot open ") + path);
  std::string head = "# vtk DataFile Version 3.0\nvtk output\nASCII\nDATASET POLYDATA\nPOINTS ";
  append_i(head, num_points);
  head += " float\n";
  bool ok = fwrite(head.data(), 1, head.size(), fp) == head.size();
  for (const auto& s : pts) ok = ok && fwrite(s.data(), 1, s.size(), fp) == s.size();
  std::string mid = num_points % 3 ? "\n" : "";
  mid += "POLYGONS ";
  append_i(mid, num_cells);
  mid.push_back(' ');
  append_i(mid, num_cells * (V + 1));
  mid.push_back('\n');
  ok = ok && fwrite(mid.data(), 1, mid.size(), fp) == mid.size();
  for (const auto& s : cells) ok = ok && fwrite(s.data(), 1, s.size(), fp) == s.size();
  ok = ok && fputc('\n', fp) != EOF;
  ok = (fclose(fp) == 0) && ok;
  return ok ? DAX_GB300_SUCCESS : vtk_fail(DAX_GB300_ERROR_EXECUTION, std::string("writing ") + path);
}

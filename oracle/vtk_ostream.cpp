// The legacy-VTK POLYDATA file written through std::ostream, as the
// reference benchmark's PrintContentsToStream does
// (Benchmarks/MarchingCubes/Pipeline.h:51-98): header lines, "POINTS n float",
// every coordinate inserted with operator<<(float) followed by a space, a
// std::endl after every third point (and one after the last when n is not a
// multiple of 3), "POLYGONS c c*(V+1)", per cell V and its ids with
// operator<<(int), and a closing std::endl.  TEST INFRASTRUCTURE ONLY: the
// checker that pins the byte format of the library's writer and of
// oracle/vtk_writer.py to the C++ standard library's own float formatting.
//
//   vtk_ostream <points.f32> <n_points> <conn.i32> <n_cells> <verts_per_cell> <out.vtk>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <vector>

template <typename T>
static std::vector<T> read(const char* path, long long n) {
  std::vector<T> v((size_t)n);
  if (n > 0) {
    std::FILE* f = std::fopen(path, "rb");
    if (!f || std::fread(v.data(), sizeof(T), (size_t)n, f) != (size_t)n) std::exit(2);
    std::fclose(f);
  }
  return v;
}

int main(int argc, char** argv) {
  if (argc != 7) return 1;
  const long long np = std::atoll(argv[2]), nc = std::atoll(argv[4]);
  const int V = std::atoi(argv[5]);
  const std::vector<float> pts = read<float>(argv[1], 3 * np);
  const std::vector<int32_t> conn = read<int32_t>(argv[3], nc * V);
  std::ofstream stream(argv[6]);
  stream << "# vtk DataFile Version 3.0" << std::endl;
  stream << "vtk output" << std::endl;
  stream << "ASCII" << std::endl;
  stream << "DATASET POLYDATA" << std::endl;
  stream << "POINTS " << np << " float" << std::endl;
  for (long long i = 0; i < np; ++i) {
    stream << pts[3 * i] << " " << pts[3 * i + 1] << " " << pts[3 * i + 2] << " ";
    if (i % 3 == 2) stream << std::endl;
  }
  if (np % 3 != 0) stream << std::endl;
  stream << "POLYGONS " << nc << " " << nc * (V + 1) << std::endl;
  for (long long c = 0; c < nc; ++c) {
    stream << V << " ";
    for (int k = 0; k < V; ++k) {
      stream << conn[c * V + k];
      if (k + 1 < V) stream << " ";
    }
    stream << std::endl;
  }
  stream << std::endl;
  return stream.good() ? 0 : 3;
}

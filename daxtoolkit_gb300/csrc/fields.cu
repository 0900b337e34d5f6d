// Point-field worklets that feed the isosurface path.
//
// Magnitude (dax/worklet/Magnitude.h:27-38): |coord(p)| for every grid point,
// the field of the reference's own marching-cubes benchmark
// (Benchmarks/MarchingCubes/Pipeline.h:100-106).  dax::math::Magnitude is
// Sqrt(dot(x, x)) with the dot in component order (VectorAnalysis.h:125-130);
// sqrt is correctly rounded here and in the host C library, so the values
// match the reference's float arithmetic bit for bit.
#include "common.cuh"
#include "kernels.cuh"

namespace daxgb {

__global__ void __launch_bounds__(256) k_point_magnitude(Grid g, float* __restrict__ out) {
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < g.P;
       p += (long long)gridDim.x * blockDim.x) {
    const unsigned row = (unsigned)(p / g.nx);
    const int i = (int)(p - (long long)row * g.nx);
    int j, k;
    split_row(g, row, j, k);
    const float x = coord(g.ox, g.sx, i, g.mx), y = coord(g.oy, g.sy, j, g.my),
                z = coord(g.oz, g.sz, k, g.mz);
    out[p] = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z)));
  }
}

void launch_point_magnitude(const Grid& g, float* out, int num_sms, cudaStream_t s) {
  const int b = resident_blocks(k_point_magnitude, 256, 0, num_sms, (g.P + 255) / 256);
  k_point_magnitude<<<b, 256, 0, s>>>(g, out);
}

}  // namespace daxgb

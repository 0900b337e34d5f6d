// CellGradient on voxels (dax/worklet/CellGradient.h:35-47 ->
// dax/exec/Derivative.h:37-75): per cell
//     g = (sum_{v=0..7} f_v * dW_v) / (x6 - x0)       component-wise,
// with dW_v the derivative weights at the parametric centre (every entry
// +-0.25, dax/exec/internal/DerivativeWeights.h:30-69), summed in vertex
// order without fused multiply-add, and x6 - x0 the difference of the two
// implicit corner coordinates (not the spacing: both are rounded floats).
//
// One thread per cell in cell-id order.  Reads 4 B/point from HBM (the 8
// corner loads of neighbouring cells hit L1/L2), writes 12 B/cell: the write
// dominates, so the kernel is HBM-write bound.
#include "common.cuh"
#include "kernels.cuh"

namespace daxgb {

// Signs of dW_v for components x, y, z, bit v of each mask = negative.
constexpr unsigned kNegX = 0x99;  // v = 0, 3, 4, 7
constexpr unsigned kNegY = 0x33;  // v = 0, 1, 4, 5
constexpr unsigned kNegZ = 0x0F;  // v = 0, 1, 2, 3

__device__ __forceinline__ float dw(unsigned neg_mask, int v) {
  return ((neg_mask >> v) & 1u) ? -0.25f : 0.25f;
}

__global__ void __launch_bounds__(256) k_cell_gradient(Grid g, const float* __restrict__ f,
                                                       float* __restrict__ out) {
  const int cx = g.nx - 1, cy = g.ny - 1;
  const long long C = (long long)cx * cy * (g.nz - 1);
  const long long dy = g.nx, dz = (long long)g.nx * g.ny;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < C;
       c += (long long)gridDim.x * blockDim.x) {
    const long long row = c / cx;
    const int i = (int)(c - row * cx);
    const int j = (int)(row % cy);
    const int k = (int)(row / cy);
    const long long p0 = i + (long long)g.nx * (j + (long long)g.ny * k);
    float v[8];
    v[0] = __ldg(f + p0);
    v[1] = __ldg(f + p0 + 1);
    v[2] = __ldg(f + p0 + dy + 1);
    v[3] = __ldg(f + p0 + dy);
    v[4] = __ldg(f + p0 + dz);
    v[5] = __ldg(f + p0 + dz + 1);
    v[6] = __ldg(f + p0 + dz + dy + 1);
    v[7] = __ldg(f + p0 + dz + dy);
    float sx = 0.0f, sy = 0.0f, sz = 0.0f;
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      sx = __fadd_rn(sx, __fmul_rn(v[n], dw(kNegX, n)));
      sy = __fadd_rn(sy, __fmul_rn(v[n], dw(kNegY, n)));
      sz = __fadd_rn(sz, __fmul_rn(v[n], dw(kNegZ, n)));
    }
    const float wx = __fsub_rn(coord(g.ox, g.sx, i + 1, g.mx), coord(g.ox, g.sx, i, g.mx));
    const float wy = __fsub_rn(coord(g.oy, g.sy, j + 1, g.my), coord(g.oy, g.sy, j, g.my));
    const float wz = __fsub_rn(coord(g.oz, g.sz, k + 1, g.mz), coord(g.oz, g.sz, k, g.mz));
    out[3 * c + 0] = __fdiv_rn(sx, wx);
    out[3 * c + 1] = __fdiv_rn(sy, wy);
    out[3 * c + 2] = __fdiv_rn(sz, wz);
  }
}

void launch_cell_gradient(const Grid& g, const float* f, float* out, int num_sms, cudaStream_t s) {
  const long long C = (long long)(g.nx - 1) * (g.ny - 1) * (g.nz - 1);
  const long long want = (C + 255) / 256;
  const long long cap = (long long)num_sms * 16;
  const int blocks = (int)(want < 1 ? 1 : (want < cap ? want : cap));
  k_cell_gradient<<<blocks, 256, 0, s>>>(g, f, out);
}

}  // namespace daxgb

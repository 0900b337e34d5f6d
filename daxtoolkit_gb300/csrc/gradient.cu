// CellGradient on voxels (dax/worklet/CellGradient.h:35-47 ->
// dax/exec/Derivative.h:37-75): per cell
//     g = (sum_{v=0..7} f_v * dW_v) / (x6 - x0)       component-wise,
// with dW_v the derivative weights at the parametric centre (every entry
// +-0.25, dax/exec/internal/DerivativeWeights.h:30-69), summed in vertex
// order without fused multiply-add, and x6 - x0 the difference of the two
// implicit corner coordinates (not the spacing: both are rounded floats).
//
// A warp marches along z over a tile of 31 cells in x by kGradBand cell
// rows in y and kSeg cell planes.  Each step loads one point plane of the
// tile (kGradBand + 1 rows of 32 points, coalesced; lane 31's points are the
// +x corners of lane 30's cells, and every +x neighbour comes from the next
// lane) and keeps the previous plane in registers, so every field value is
// read from HBM once (plus the band's halo row and the segment's halo
// plane).  While every value in the two planes is 0 or at least 2^-124 in
// magnitude (products by +-0.25 exact), the weighted sums use fused
// multiply-adds, which then round exactly like the reference's separate
// multiply and add; otherwise the separate operations run.  The three
// divisions by the cell widths use the widths' correctly rounded
// reciprocals, one per column, row and plane, with a correction step that
// keeps each quotient the correctly rounded one (div_by_recip).  Each lane
// writes its cell's 12 bytes as one 8-byte store on the 8-byte-aligned half
// plus one 4-byte store.  (Staging a row through shared memory into fully
// coalesced stores measured slower on GB300, 0.63 against 0.57 ms at 512^3.)
// Algorithmic traffic: 4 B/point + 12 B/cell.
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

// One point plane of a warp's tile: rows j0 .. j0 + kGradBand of point column i
// (zero outside the grid).
__device__ __forceinline__ void load_point_plane(const Grid& g, const float* __restrict__ f, int i,
                                                 int j0, int k, float (&F)[kGradBand + 1]) {
#pragma unroll
  for (int t = 0; t <= kGradBand; ++t) {
    const int j = j0 + t;
    const long long p = (long long)i + (long long)g.nx * (j + (long long)g.ny * k);
    F[t] = (j < g.ny && i < g.nx) ? __ldg(f + p) : 0.0f;
  }
}

// True when every value v of the plane is 0 or has |v| >= 2^-124: then
// v * (+-0.25) is exact, and a fused multiply-add of it rounds exactly like
// the reference's multiply-then-add.
__device__ __forceinline__ bool plane_exact_quarter(const float (&F)[kGradBand + 1]) {
  bool ok = true;
#pragma unroll
  for (int t = 0; t <= kGradBand; ++t) {
    const float a = fabsf(F[t]);
    ok = ok && (a == 0.0f || a >= 0x1p-124f);
  }
  return ok;
}

__global__ void __launch_bounds__(kMarchWarps * 32, kGradMinBlocks)
    k_cell_gradient(Grid g, const float* __restrict__ f, float* __restrict__ out, MarchTiles mt) {
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const long long task = (long long)blockIdx.x * kMarchWarps + wib;
  if (task >= mt.tasks) return;  // the whole warp leaves; no block barrier follows
  const int xw = (int)(task % mt.nxw);
  const long long t2 = task / mt.nxw;
  const int band = (int)(t2 % mt.nband), seg = (int)(t2 / mt.nband);
  const int cx = g.nx - 1, cy = g.ny - 1, cz = g.nz - 1;
  // lanes 0..30 own cell columns i; lane 31 only supplies point column i
  const int i = kMarchCols * xw + lane;
  const bool own = lane < kMarchCols && i < cx;
  const int j0 = band * kGradBand;
  const int k0 = seg * kSeg, k1 = min(k0 + kSeg, cz);
  // the cell widths and their reciprocals: one per column, per row of the
  // band, per plane
  const float wx =
      own ? __fsub_rn(coord(g.ox, g.sx, i + 1, g.mx), coord(g.ox, g.sx, i, g.mx)) : 1.0f;
  const float rx = recip_or_zero(wx);
  float wy[kGradBand], ry[kGradBand];
#pragma unroll
  for (int t = 0; t < kGradBand; ++t) {
    wy[t] = __fsub_rn(coord(g.oy, g.sy, j0 + t + 1, g.my), coord(g.oy, g.sy, j0 + t, g.my));
    ry[t] = recip_or_zero(wy[t]);
  }

  float F0[kGradBand + 1], F1[kGradBand + 1];
  load_point_plane(g, f, i, j0, k0, F0);
  bool ok0 = plane_exact_quarter(F0);
  for (int kc = k0; kc < k1; ++kc) {
    load_point_plane(g, f, i, j0, kc + 1, F1);
    const bool ok1 = plane_exact_quarter(F1);
    // warp-uniform: the weighted sums may use fused multiply-adds
    const bool fused = __all_sync(kFull, ok0 && ok1);
    const float wz = __fsub_rn(coord(g.oz, g.sz, kc + 1, g.mz), coord(g.oz, g.sz, kc, g.mz));
    const float rz = recip_or_zero(wz);
    // row t of both planes at columns i and i + 1, carried from row to row
    float a0 = F0[0], b0 = F1[0];
    float a0n = __shfl_down_sync(kFull, a0, 1), b0n = __shfl_down_sync(kFull, b0, 1);
    float* o = out + 3 * ((long long)i + (long long)cx * (j0 + (long long)cy * kc));
    bool even = ((i + (long long)cx * (j0 + (long long)cy * kc)) & 1) == 0;
#pragma unroll
    for (int t = 0; t < kGradBand; ++t) {
      const int jc = j0 + t;
      if (jc >= cy) break;  // uniform across the warp
      const float a1 = F0[t + 1], b1 = F1[t + 1];
      const float a1n = __shfl_down_sync(kFull, a1, 1), b1n = __shfl_down_sync(kFull, b1, 1);
      if (own) {
        const float v[8] = {a0, a0n, a1n, a1, b0, b0n, b1n, b1};
        float sx = 0.0f, sy = 0.0f, sz = 0.0f;
        if (fused) {
#pragma unroll
          for (int n = 0; n < 8; ++n) {
            sx = __fmaf_rn(v[n], dw(kNegX, n), sx);
            sy = __fmaf_rn(v[n], dw(kNegY, n), sy);
            sz = __fmaf_rn(v[n], dw(kNegZ, n), sz);
          }
        } else {
#pragma unroll
          for (int n = 0; n < 8; ++n) {
            sx = __fadd_rn(sx, __fmul_rn(v[n], dw(kNegX, n)));
            sy = __fadd_rn(sy, __fmul_rn(v[n], dw(kNegY, n)));
            sz = __fadd_rn(sz, __fmul_rn(v[n], dw(kNegZ, n)));
          }
        }
        // the correctly rounded quotients (div_by_recip is exact: common.cuh)
        const float gx = div_by_recip(sx, wx, rx), gy = div_by_recip(sy, wy[t], ry[t]),
                    gz = div_by_recip(sz, wz, rz);
        if (even) {  // byte offset 12 c is 8-byte aligned
          *reinterpret_cast<float2*>(o) = make_float2(gx, gy);
          o[2] = gz;
        } else {     // byte offset 12 c + 4 is 8-byte aligned
          o[0] = gx;
          *reinterpret_cast<float2*>(o + 1) = make_float2(gy, gz);
        }
      }
      o += 3 * (long long)cx;
      even = even == ((cx & 1) == 0);
      a0 = a1;
      a0n = a1n;
      b0 = b1;
      b0n = b1n;
    }
#pragma unroll
    for (int t = 0; t <= kGradBand; ++t) F0[t] = F1[t];
    ok0 = ok1;
  }
}

MarchTiles march_tiles(int nx, int ny, int nz, int band) {
  MarchTiles mt;
  mt.nxw = (nx + kMarchCols - 1) / kMarchCols;
  mt.nband = (ny + band - 1) / band;
  mt.nseg = (nz + kSeg - 1) / kSeg;
  mt.tasks = (long long)mt.nxw * mt.nband * mt.nseg;
  return mt;
}

void launch_cell_gradient(const Grid& g, const float* f, float* out, int num_sms, cudaStream_t s) {
  (void)num_sms;
  const MarchTiles mt = march_tiles(g.nx - 1, g.ny - 1, g.nz - 1, kGradBand);  // cell tiles
  if (mt.tasks < 1) return;
  const long long blocks = (mt.tasks + kMarchWarps - 1) / kMarchWarps;
  k_cell_gradient<<<(unsigned)blocks, kMarchWarps * 32, 0, s>>>(g, f, out, mt);
}

}  // namespace daxgb

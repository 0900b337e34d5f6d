// CellGradient on voxels (dax/worklet/CellGradient.h:35-47 ->
// dax/exec/Derivative.h:37-75): per cell
//     g = (sum_{v=0..7} f_v * dW_v) / (x6 - x0)       component-wise,
// with dW_v the derivative weights at the parametric centre (every entry
// +-0.25, dax/exec/internal/DerivativeWeights.h:30-69), summed in vertex
// order without fused multiply-add, and x6 - x0 the difference of the two
// implicit corner coordinates (not the spacing: both are rounded floats).
//
// A warp marches along z over a tile of kGradCols = 62 cells in x (two per
// lane on lanes 0..30; lane 31 loads the tile's last two point columns and
// owns no cell), kGradBand cell rows in y and kGradSeg cell planes.  Each
// lane copies its two point columns of every point plane of the tile
// (kGradBand + 1 rows; one 8-byte copy per row where the rows allow it)
// into the warp's ring in shared memory with cp.async, kGradDepth planes
// ahead of the plane it computes, so the loads in flight hold no registers
// and need no warp synchronisation.  A lane's +x neighbour column comes from
// the next lane by one shuffle per row, and the previous plane stays in
// registers: every field value is read from HBM once (plus the band's halo
// row and the segment's halo plane).
//
// Two exact paths, chosen per plane pair and warp:
// * fast -- every value of the two planes is 0 or 2^-60 <= |v| < 2^86 and
//   every cell width is within 2^-30 <= |w| < 2^30.  Products by +-0.25 are
//   then exact, so fused multiply-adds round exactly like the reference's
//   multiply-then-add; a weighted sum x is 0 or 2^-85 <= |x| < 2^87 (the
//   values are multiples of 2^-83, and so is every rounded partial sum), so
//   div_fast gives the correctly rounded x / w.  The y and z sums share
//   their first two terms (same weights on v0 and v1).
// * exact -- otherwise: separate multiply and add as in the reference and
//   div_by_recip with its range checks (falling back to IEEE division).
// A lane's two cells are 24 contiguous bytes whose 8-byte alignment is the
// same for every lane of a row (the row's first cell index parity): three
// 8-byte stores, or 4 + 8 + 8 + 4 bytes (six 4-byte stores when the output
// itself is not 8-byte aligned).  (Staging the rows through shared memory
// into fully coalesced stores measured slower.)
// Algorithmic traffic: 4 B/point + 12 B/cell.
#include "common.cuh"
#include "kernels.cuh"

namespace daxgb {

// Signs of dW_v for components x, y, z, bit v of each mask = negative.
constexpr unsigned kNegX = 0x99;  // v = 0, 3, 4, 7
constexpr unsigned kNegY = 0x33;  // v = 0, 1, 4, 5
constexpr unsigned kNegZ = 0x0F;  // v = 0, 1, 2, 3

// Magnitude bit patterns (sign cleared) bounding the fast path's values.
constexpr unsigned kValLo = 0x21800000u;  // 2^-60
constexpr unsigned kValHi = 0x6a800000u;  // 2^86

constexpr int kGradCols = 2 * 31;     // cells per warp tile in x
constexpr int kGradRows = kGradBand + 1;  // point rows per plane of a tile

__device__ __forceinline__ float dw(unsigned neg_mask, int v) {
  return ((neg_mask >> v) & 1u) ? -0.25f : 0.25f;
}

// One point plane of a warp's tile, rows j0 .. j0 + kGradBand: a and b are
// the lane's point columns 2 lane and 2 lane + 1, n is column 2 lane + 2
// (the next lane's a); zero outside the grid.  ok: every value of a and b
// is 0 or 2^-60 <= |v| < 2^86 (no NaN or infinity).
struct TilePlane {
  float a[kGradRows], b[kGradRows], n[kGradRows];
  bool ok;
};

// Planes in flight per warp: each lane copies its own two point columns of
// a plane into the warp's ring in shared memory with cp.async (no registers
// held while the copy is in flight, no warp synchronisation: a lane reads
// back only what it copied) kGradDepth planes ahead of the plane it computes.
constexpr int kGradDepth = 3;

__device__ __forceinline__ void cp_async(void* dst, const void* src, int bytes, int src_bytes) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  if (bytes == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(d), "l"(src), "r"(src_bytes)
                 : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(d), "l"(src), "r"(src_bytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_ring() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(kGradDepth - 1) : "memory");
}

// Starts the copy of the lane's columns of one point plane (p: the point
// (first column, j0, k)) into `slot`, always closing a copy group; `live`
// false (a plane past the segment) copies nothing.  Columns outside the
// grid and point rows past `rows` are zero-filled (source size 0, from a
// valid address).
template <bool LOADV>
__device__ __forceinline__ void issue_tile_plane(const float* __restrict__ p, const float* f, int nx,
                                                 int rows, bool c0, bool c1, bool live,
                                                 float2* slot) {
  if (live) {
#pragma unroll
    for (int t = 0; t < kGradRows; ++t) {
      const float* q = p + (long long)t * nx;
      const bool row = t <= rows;
      if (LOADV) {  // nx even: c0 == c1, and q is 8-byte aligned
        const bool v = row && c0;
        cp_async(slot + 32 * t, v ? q : f, 8, v ? 8 : 0);
      } else {
        const bool v0 = row && c0, v1 = row && c1;
        cp_async(reinterpret_cast<float*>(slot + 32 * t), v0 ? q : f, 4, v0 ? 4 : 0);
        cp_async(reinterpret_cast<float*>(slot + 32 * t) + 1, v1 ? q + 1 : f, 4, v1 ? 4 : 0);
      }
    }
  }
  cp_async_commit();
}

// a and b of a plane whose copy group has completed.
__device__ __forceinline__ void read_tile_plane(const float2* slot, TilePlane& P) {
#pragma unroll
  for (int t = 0; t < kGradRows; ++t) {
    const float2 v = slot[32 * t];
    P.a[t] = v.x;
    P.b[t] = v.y;
  }
}

// The +x neighbour column and the band check, once the plane has arrived.
__device__ __forceinline__ void finish_tile_plane(TilePlane& P) {
  unsigned hi = 0u, lo = 0xffffffffu;
#pragma unroll
  for (int t = 0; t < kGradRows; ++t) {
    P.n[t] = __shfl_down_sync(kFull, P.a[t], 1);
    const unsigned ua = mag_bits(P.a[t]), ub = mag_bits(P.b[t]);
    hi = max(hi, max(ua, ub));
    lo = min(lo, min(ua - 1u, ub - 1u));  // a zero wraps to the maximum and drops out
  }
  P.ok = hi < kValHi && lo >= kValLo - 1u;
}

// One cell's gradient from its eight point values in vertex order.
template <bool FAST>
__device__ __forceinline__ float3 cell_gradient(const float (&v)[8], float wx, float rx, float wy,
                                                float ry, float wz, float rz) {
  float3 gr;
  if (FAST) {
    float sx = __fmaf_rn(v[0], -0.25f, 0.0f);  // 0 + v0 dW0: a -0 product gives +0
    float sy = __fmaf_rn(v[1], -0.25f, sx);
    float sz = sy;
    sx = __fmaf_rn(v[1], 0.25f, sx);
#pragma unroll
    for (int n = 2; n < 8; ++n) {
      sx = __fmaf_rn(v[n], dw(kNegX, n), sx);
      sy = __fmaf_rn(v[n], dw(kNegY, n), sy);
      sz = __fmaf_rn(v[n], dw(kNegZ, n), sz);
    }
    gr.x = div_fast(sx, wx, rx);
    gr.y = div_fast(sy, wy, ry);
    gr.z = div_fast(sz, wz, rz);
  } else {
    float sx = 0.0f, sy = 0.0f, sz = 0.0f;
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      sx = __fadd_rn(sx, __fmul_rn(v[n], dw(kNegX, n)));
      sy = __fadd_rn(sy, __fmul_rn(v[n], dw(kNegY, n)));
      sz = __fadd_rn(sz, __fmul_rn(v[n], dw(kNegZ, n)));
    }
    // the correctly rounded quotients (div_by_recip is exact: common.cuh)
    gr.x = div_by_recip(sx, wx, rx);
    gr.y = div_by_recip(sy, wy, ry);
    gr.z = div_by_recip(sz, wz, rz);
  }
  return gr;
}

__device__ __forceinline__ void store2(float* o, float x, float y) {
  *reinterpret_cast<float2*>(o) = make_float2(x, y);
}

// Per-warp constants of a tile.
struct GradTile {
  int rows;        // cell rows of the band
  int own;         // cells of this lane: 2, 1 (at the grid's x end) or 0
  float wx0, rx0, wx1, rx1;
  float wy[kGradBand], ry[kGradBand];
  long long row_floats;  // 3 cx
  bool flip;       // row start parity flips from row to row (cx odd)
};

// The gradients of the band's cell rows between planes P and Q; o is the
// lane's first cell in the plane's first row, `even` that cell's parity.
template <bool FAST, bool VEC>
__device__ __forceinline__ void tile_rows(const TilePlane& P, const TilePlane& Q, const GradTile& T,
                                          float wz, float rz, float* o, bool even) {
#pragma unroll
  for (int t = 0; t < kGradBand; ++t) {
    if (t >= T.rows) break;  // uniform across the warp
    const float u0[8] = {P.a[t], P.b[t], P.b[t + 1], P.a[t + 1],
                         Q.a[t], Q.b[t], Q.b[t + 1], Q.a[t + 1]};
    const float u1[8] = {P.b[t], P.n[t], P.n[t + 1], P.b[t + 1],
                         Q.b[t], Q.n[t], Q.n[t + 1], Q.b[t + 1]};
    const float3 g0 = cell_gradient<FAST>(u0, T.wx0, T.rx0, T.wy[t], T.ry[t], wz, rz);
    const float3 g1 = cell_gradient<FAST>(u1, T.wx1, T.rx1, T.wy[t], T.ry[t], wz, rz);
    if (T.own == 2) {
      if (VEC && even) {
        store2(o, g0.x, g0.y);
        store2(o + 2, g0.z, g1.x);
        store2(o + 4, g1.y, g1.z);
      } else if (VEC) {
        o[0] = g0.x;
        store2(o + 1, g0.y, g0.z);
        store2(o + 3, g1.x, g1.y);
        o[5] = g1.z;
      } else {
        o[0] = g0.x;
        o[1] = g0.y;
        o[2] = g0.z;
        o[3] = g1.x;
        o[4] = g1.y;
        o[5] = g1.z;
      }
    } else if (T.own == 1) {
      o[0] = g0.x;
      o[1] = g0.y;
      o[2] = g0.z;
    }
    o += T.row_floats;
    even = even != T.flip;
  }
}

// One warp tile (task) of one grid; the kernels below map blocks to tasks.
template <bool VEC, bool LOADV>
__device__ __forceinline__ void cell_gradient_task(const Grid& g, const float* __restrict__ f,
                                                   float* __restrict__ out, const MarchTiles& mt,
                                                   long long task) {
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  if (task >= mt.tasks) return;  // the whole warp leaves; no block barrier follows
  const int xw = (int)(task % mt.nxw);
  const long long t2 = task / mt.nxw;
  const int band = (int)(t2 % mt.nband), seg = (int)(t2 / mt.nband);
  const int cx = g.nx - 1, cy = g.ny - 1, cz = g.nz - 1;
  const int i = kGradCols * xw + 2 * lane;  // the lane's first point (and cell) column
  const bool c0 = i < g.nx, c1 = i + 1 < g.nx;
  const int j0 = band * kGradBand;
  const int k0 = seg * kGradSeg, k1 = min(k0 + kGradSeg, cz);

  GradTile T;
  T.rows = min(kGradBand, cy - j0);
  T.own = lane == 31 ? 0 : (i + 1 < cx ? 2 : (i < cx ? 1 : 0));
  // the cell widths and their reciprocals: per column, per row of the band,
  // per plane
  T.wx0 = T.own >= 1 ? __fsub_rn(coord(g.ox, g.sx, i + 1, g.mx), coord(g.ox, g.sx, i, g.mx)) : 1.0f;
  T.wx1 = T.own == 2 ? __fsub_rn(coord(g.ox, g.sx, i + 2, g.mx), coord(g.ox, g.sx, i + 1, g.mx)) : 1.0f;
  T.rx0 = recip_or_zero(T.wx0);
  T.rx1 = recip_or_zero(T.wx1);
  bool widths_ok = width_in_band(T.wx0) && width_in_band(T.wx1);
#pragma unroll
  for (int t = 0; t < kGradBand; ++t) {
    T.wy[t] = __fsub_rn(coord(g.oy, g.sy, j0 + t + 1, g.my), coord(g.oy, g.sy, j0 + t, g.my));
    T.ry[t] = recip_or_zero(T.wy[t]);
    widths_ok = widths_ok && (t >= T.rows || width_in_band(T.wy[t]));
  }
  widths_ok = __all_sync(kFull, widths_ok);
  T.row_floats = 3 * (long long)cx;
  T.flip = (cx & 1) != 0;

  const long long plane = (long long)g.nx * g.ny;
  const float* p = f + i + (long long)g.nx * j0 + plane * k0;  // point (i, j0, k0)
  float* const o0 = out + 3 * ((long long)i + (long long)cx * j0);  // cell (i, j0, 0)
  const long long row0 = (long long)kGradCols * xw + (long long)cx * j0;  // first cell of (j0, 0)
  const long long cplane = (long long)cx * cy;

  // the warp's ring: kGradDepth plane slots of kGradRows rows x 32 lanes
  __shared__ float2 ring[kGradWarps][kGradDepth][kGradRows * 32];
  float2* const lane_ring = &ring[wib][0][lane];
  auto slot_of = [&](int k) { return lane_ring + (k - k0) % kGradDepth * (kGradRows * 32); };
  auto issue = [&](int k) {
    issue_tile_plane<LOADV>(p + plane * (k - k0), f, g.nx, T.rows, c0, c1, k <= k1, slot_of(k));
  };

  // plane kc of P, Q = kc + 1 read from the ring, kc + kGradDepth started
  auto step = [&](TilePlane& P, TilePlane& Q, int kc) {
    issue(kc + kGradDepth);
    cp_async_wait_ring();  // the groups after plane kc + 1's may still be in flight
    read_tile_plane(slot_of(kc + 1), Q);
    finish_tile_plane(Q);
    const float wz = __fsub_rn(coord(g.oz, g.sz, kc + 1, g.mz), coord(g.oz, g.sz, kc, g.mz));
    const float rz = recip_or_zero(wz);
    const bool fast = __all_sync(kFull, P.ok && Q.ok) && widths_ok && width_in_band(wz);
    float* o = o0 + 3 * cplane * kc;
    const bool even = ((row0 + cplane * kc) & 1) == 0;
    if (fast)
      tile_rows<true, VEC>(P, Q, T, wz, rz, o, even);
    else
      tile_rows<false, VEC>(P, Q, T, wz, rz, o, even);
  };

  TilePlane A, B;
#pragma unroll
  for (int d = 0; d < kGradDepth; ++d) issue(k0 + d);
  asm volatile("cp.async.wait_group %0;\n" ::"n"(kGradDepth - 1) : "memory");
  read_tile_plane(slot_of(k0), A);
  finish_tile_plane(A);
  for (int kc = k0; kc < k1; kc += 2) {
    step(A, B, kc);
    if (kc + 1 >= k1) break;
    step(B, A, kc + 1);
  }
}

template <bool VEC, bool LOADV>
__global__ void __launch_bounds__(kGradWarps * 32, kGradMinBlocks)
    k_cell_gradient(Grid g, const float* __restrict__ f, float* __restrict__ out, MarchTiles mt) {
  cell_gradient_task<VEC, LOADV>(g, f, out, mt,
                                 (long long)blockIdx.x * kGradWarps + (threadIdx.x >> 5));
}

// Cell tiles of one grid's CellGradient.
__host__ __device__ inline MarchTiles grad_tiles(const Grid& g) {
  MarchTiles mt;
  mt.nxw = (g.nx - 1 + kGradCols - 1) / kGradCols;
  mt.nband = (g.ny - 1 + kGradBand - 1) / kGradBand;
  mt.nseg = (g.nz - 1 + kGradSeg - 1) / kGradSeg;
  mt.tasks = (long long)mt.nxw * mt.nband * mt.nseg;
  return mt;
}

// A grid set: block b works for the grid whose first block (block0) is the
// last at or before b; the grid's gradients start at its first cell.
template <bool VEC, bool LOADV>
__global__ void __launch_bounds__(kGradWarps * 32, kGradMinBlocks)
    k_cell_gradient_set(GridSet S, const long long* __restrict__ block0,
                        float* __restrict__ out) {
  const int si = block_slot(block0, S.count, blockIdx.x);
  const Grid g = S.slots[si].g;
  cell_gradient_task<VEC, LOADV>(g, S.slots[si].field, out + 3 * S.slots[si].cell0, grad_tiles(g),
                                 ((long long)blockIdx.x - __ldg(block0 + si)) * kGradWarps +
                                     (threadIdx.x >> 5));
}

long long grad_blocks(const Grid& g) {
  if (g.nx < 2 || g.ny < 2 || g.nz < 2) return 0;
  return (grad_tiles(g).tasks + kGradWarps - 1) / kGradWarps;
}

void launch_cell_gradient_set(const GridSet& S, const long long* block0, long long blocks,
                              bool vec, bool loadv, float* out, cudaStream_t s) {
  if (blocks <= 0) return;
  const dim3 block(kGradWarps * 32);
  const unsigned nb = (unsigned)blocks;
  if (vec && loadv)
    k_cell_gradient_set<true, true><<<nb, block, 0, s>>>(S, block0, out);
  else if (vec)
    k_cell_gradient_set<true, false><<<nb, block, 0, s>>>(S, block0, out);
  else if (loadv)
    k_cell_gradient_set<false, true><<<nb, block, 0, s>>>(S, block0, out);
  else
    k_cell_gradient_set<false, false><<<nb, block, 0, s>>>(S, block0, out);
}

void launch_cell_gradient(const Grid& g, const float* f, float* out, int num_sms, cudaStream_t s) {
  (void)num_sms;
  const int cx = g.nx - 1, cy = g.ny - 1, cz = g.nz - 1;
  if (cx < 1 || cy < 1 || cz < 1) return;
  MarchTiles mt;  // cell tiles
  mt.nxw = (cx + kGradCols - 1) / kGradCols;
  mt.nband = (cy + kGradBand - 1) / kGradBand;
  mt.nseg = (cz + kGradSeg - 1) / kGradSeg;
  mt.tasks = (long long)mt.nxw * mt.nband * mt.nseg;
  const unsigned blocks = (unsigned)((mt.tasks + kGradWarps - 1) / kGradWarps);
  const dim3 block(kGradWarps * 32);
  const bool vec = (reinterpret_cast<uintptr_t>(out) & 7) == 0;
  const bool loadv = (g.nx & 1) == 0 && (reinterpret_cast<uintptr_t>(f) & 7) == 0;
  if (vec && loadv)
    k_cell_gradient<true, true><<<blocks, block, 0, s>>>(g, f, out, mt);
  else if (vec)
    k_cell_gradient<true, false><<<blocks, block, 0, s>>>(g, f, out, mt);
  else if (loadv)
    k_cell_gradient<false, true><<<blocks, block, 0, s>>>(g, f, out, mt);
  else
    k_cell_gradient<false, false><<<blocks, block, 0, s>>>(g, f, out, mt);
}

}  // namespace daxgb

// Adjoints of the isosurface vertices and of CellGradient with respect to the
// point field, as deterministic gathers (no atomics): every dL/df_p is
// summed by one thread in a fixed order.
//
// CellGradient: g_c[a] = sum_v f_v dW_v[a] / width_c[a] with dW = +-0.25
// (dax/exec/Derivative.h:37-58), so
//     dL/df_p = sum over the <= 8 cells c containing p, a in {x,y,z}:
//               s_a * 0.25 * dL/dg_c[a] / width_c[a]
// with s_a = +1 when p is on the cell's upper face along a, else -1.
// k_grad_adjoint marches along z over a warp tile (31 point columns x kAdjBand
// point rows x kSeg planes).  Per cell plane and cell row jc it forms, at
// point column i, the x-pair sums
//     Hx = ax(i-1) - ax(i),   Hy = ay(i-1) + ay(i),   Hz = az(i-1) + az(i)
// (a = 0.25 dL/dg / width, zero outside the cells), so that a point row j
// gets from cell plane kc
//     P = Hx[j-1] + Hx[j] + Hy[j-1] - Hy[j],   Z = Hz[j-1] + Hz[j]
// and dL/df(i, j, k) = (P + Z)[plane k-1] + (P - Z)[plane k].  Each cell
// gradient is read from HBM once (plus a band's halo row and a segment's
// halo plane) and each point written once: 12 B/cell + 4 B/point.
//
// Isosurface (merged): vertex v on edge (A, B) along `axis` is
//     x_v = c_A + w (c_B - c_A),   w = (iso - f_A) / (f_B - f_A)
// (dax/worklet/MarchingCubes.h:160-161, dax/math/VectorAnalysis.h:35-50).
// Only the axis component of c_B - c_A is non-zero (h = its float value), so
//     dL/df_A += g (iso - f_B) / d^2,   dL/df_B -= g (iso - f_A) / d^2,
// with g = dL/dx_v[axis] * h and d = f_B - f_A.  k_edge_adjoint visits every
// point row word; the few words with a crossing edge at one of their points
// gather each such point's <= 6 edges in a fixed order (forward x, y, z,
// then backward x, y, z) and add them to the point's value.  An edge's
// vertex id is its owner word's offset plus its rank in that word, exactly
// as the forward pass numbered it.
#include "common.cuh"
#include "kernels.cuh"

namespace daxgb {

namespace {

__device__ __forceinline__ float width_x(const Grid& g, int i) {
  return __fsub_rn(coord(g.ox, g.sx, i + 1, g.mx), coord(g.ox, g.sx, i, g.mx));
}
__device__ __forceinline__ float width_y(const Grid& g, int j) {
  return __fsub_rn(coord(g.oy, g.sy, j + 1, g.my), coord(g.oy, g.sy, j, g.my));
}
__device__ __forceinline__ float width_z(const Grid& g, int k) {
  return __fsub_rn(coord(g.oz, g.sz, k + 1, g.mz), coord(g.oz, g.sz, k, g.mz));
}

}  // namespace

// Lane L of a warp tile holds cell column ic = 31 xw - 1 + L and outputs
// point column ic + 1 (lanes 0..30), whose -x cell is its own column and
// whose +x cell is lane L + 1's.  Per cell plane the tile's kAdjBand + 1 cell
// rows (jc = j0 - 1 + t) are loaded together (three 4-byte loads per cell,
// 384 contiguous bytes per warp load), then reduced row by row into the
// point rows t = 0..kAdjBand-1 they bracket.
__global__ void __launch_bounds__(kMarchWarps * 32, kAdjMinBlocks)
    k_grad_adjoint(Grid g, const float* __restrict__ dg, float* __restrict__ out, MarchTiles mt) {
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const long long task = (long long)blockIdx.x * kMarchWarps + wib;
  if (task >= mt.tasks) return;  // the whole warp leaves; no block barrier follows
  const int xw = (int)(task % mt.nxw);
  const long long t2 = task / mt.nxw;
  const int band = (int)(t2 % mt.nband), seg = (int)(t2 / mt.nband);
  const int cx = g.nx - 1, cy = g.ny - 1, cz = g.nz - 1;
  const int ic = kMarchCols * xw - 1 + lane;  // this lane's cell column
  const bool col = ic >= 0 && ic < cx;
  const int i = ic + 1;                       // this lane's point column
  const bool pcol = lane < kMarchCols && i < g.nx;
  const int j0 = band * kAdjBand;
  const int k0 = seg * kSeg, k1 = min(k0 + kSeg, g.nz);

  // 0.25 / width of this lane's cell column and of the tile's cell rows
  const float rx = col ? __fdiv_rn(0.25f, width_x(g, ic)) : 0.0f;
  float ry[kAdjBand + 1];
#pragma unroll
  for (int t = 0; t <= kAdjBand; ++t) {
    const int jc = j0 - 1 + t;
    ry[t] = (jc >= 0 && jc < cy) ? __fdiv_rn(0.25f, width_y(g, jc)) : 0.0f;
  }

  float U[kAdjBand];  // (P + Z) of the previous cell plane, per point row
#pragma unroll
  for (int t = 0; t < kAdjBand; ++t) U[t] = 0.0f;
  for (int kc = k0 > 0 ? k0 - 1 : k0; kc < k1; ++kc) {
    float gx[kAdjBand + 1], gy[kAdjBand + 1], gz[kAdjBand + 1];
    float rz = 0.0f;
    if (kc < cz) {
      rz = __fdiv_rn(0.25f, width_z(g, kc));
#pragma unroll
      for (int t = 0; t <= kAdjBand; ++t) {
        const int jc = j0 - 1 + t;
        const bool ok = col && jc >= 0 && jc < cy;
        const float* c = dg + 3 * ((long long)ic + (long long)cx * (jc + (long long)cy * kc));
        gx[t] = ok ? __ldg(c) : 0.0f;
        gy[t] = ok ? __ldg(c + 1) : 0.0f;
        gz[t] = ok ? __ldg(c + 2) : 0.0f;
      }
    } else {
#pragma unroll
      for (int t = 0; t <= kAdjBand; ++t) gx[t] = gy[t] = gz[t] = 0.0f;
    }
    const bool emit = kc >= k0;
    // x-pair sums of cell row t at this lane's point column
    float hx0, hy0, hz0;
    {
      const float ax = __fmul_rn(gx[0], rx);
      hx0 = __fsub_rn(ax, __shfl_down_sync(kFull, ax, 1));
      hy0 = __fmul_rn(__fadd_rn(gy[0], __shfl_down_sync(kFull, gy[0], 1)), ry[0]);
      hz0 = __fmul_rn(__fadd_rn(gz[0], __shfl_down_sync(kFull, gz[0], 1)), rz);
    }
#pragma unroll
    for (int t = 0; t < kAdjBand; ++t) {
      const float ax = __fmul_rn(gx[t + 1], rx);
      const float hx1 = __fsub_rn(ax, __shfl_down_sync(kFull, ax, 1));
      const float hy1 =
          __fmul_rn(__fadd_rn(gy[t + 1], __shfl_down_sync(kFull, gy[t + 1], 1)), ry[t + 1]);
      const float hz1 = __fmul_rn(__fadd_rn(gz[t + 1], __shfl_down_sync(kFull, gz[t + 1], 1)), rz);
      const float P = __fadd_rn(__fadd_rn(hx0, hx1), __fsub_rn(hy0, hy1));
      const float Z = __fadd_rn(hz0, hz1);
      const int j = j0 + t;
      if (emit && pcol && j < g.ny)
        out[(long long)i + (long long)g.nx * (j + (long long)g.ny * kc)] =
            __fadd_rn(U[t], __fsub_rn(P, Z));
      U[t] = __fadd_rn(P, Z);
      hx0 = hx1;
      hy0 = hy1;
      hz0 = hz1;
    }
  }
}

namespace {

// Crossing masks of owner word (row (j, k), word m) and its first vertex id.
struct EdgeOwner {
  uint32_t X, Y, Z;
  long long base;
};

__device__ __forceinline__ EdgeOwner edge_owner(const Grid& g, const uint32_t* __restrict__ bits,
                                                const uint32_t* __restrict__ wv, int j, int k,
                                                int m) {
  const long long r = (long long)k * g.ny + j;
  const long long pos = r * g.nx + 32ll * m;
  const uint32_t pm = low_mask(g.nx - 32 * m);
  uint32_t a, a1;
  bits_at2(bits, pos, a, a1);
  EdgeOwner o;
  o.X = (a ^ a1) & low_mask(g.nx - 1 - 32 * m);
  o.Y = j < g.ny - 1 ? (a ^ bits_at(bits, pos + g.nx)) & pm : 0u;
  o.Z = k < g.nz - 1 ? (a ^ bits_at(bits, pos + (long long)g.nx * g.ny)) & pm : 0u;
  o.base = (long long)__ldg(wv + r * g.wr + m);
  return o;
}

// Vertex id of the edge along `axis` owned by bit b of an owner word: the
// forward pass numbers a word's edges in (point, axis) order.
__device__ __forceinline__ long long edge_id(const EdgeOwner& o, int b, int axis) {
  const uint32_t lm = (1u << b) - 1u;
  long long id = o.base + __popc(o.X & lm) + __popc(o.Y & lm) + __popc(o.Z & lm);
  if (axis >= 1) id += (o.X >> b) & 1u;
  if (axis >= 2) id += (o.Y >> b) & 1u;
  return id;
}

// Contribution of the edge (pa -> pb) along `axis`, vertex vid, to dL/df at
// its end `at_a ? pa : pb`; idx_a = pa's index along the axis.
__device__ __forceinline__ float edge_term(const Grid& g, const float* __restrict__ f, float iso,
                                           const float* __restrict__ dverts, long long vid,
                                           int axis, long long pa, long long pb, int idx_a,
                                           bool at_a) {
  const float fa = __ldg(f + pa), fb = __ldg(f + pb);
  const float d = __fsub_rn(fb, fa);
  const float h = axis == 0 ? width_x(g, idx_a) : (axis == 1 ? width_y(g, idx_a) : width_z(g, idx_a));
  const float gv = __fmul_rn(__ldg(dverts + 3 * vid + axis), h);
  const float num = at_a ? __fsub_rn(iso, fb) : -__fsub_rn(iso, fa);
  return __fdiv_rn(__fmul_rn(gv, num), __fmul_rn(d, d));
}

}  // namespace

__global__ void __launch_bounds__(256) k_edge_adjoint(Grid g, const float* __restrict__ f,
                                                      float iso,
                                                      const uint32_t* __restrict__ bits,
                                                      const uint32_t* __restrict__ wv,
                                                      const float* __restrict__ dverts,
                                                      float* __restrict__ out) {
  const long long W = g.R * g.wr;  // < 2^27 for grids below 2^31 points
  const long long dy = g.nx, dz = (long long)g.nx * g.ny;
  for (long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x; w < W;
       w += (long long)gridDim.x * blockDim.x) {
    int m, j, k;
    const unsigned r = split_word(g, (unsigned)w, m);
    split_row(g, r, j, k);
    const long long pos = (long long)r * g.nx + 32ll * m;
    const uint32_t pm = low_mask(g.nx - 32 * m);
    uint32_t a, a1;
    bits_at2(bits, pos, a, a1);
    // points of this word with an incident crossing edge, per direction
    const uint32_t xf = (a ^ a1) & low_mask(g.nx - 1 - 32 * m);
    const uint32_t yf = j < g.ny - 1 ? (a ^ bits_at(bits, pos + dy)) & pm : 0u;
    const uint32_t zf = k < g.nz - 1 ? (a ^ bits_at(bits, pos + dz)) & pm : 0u;
    const uint32_t xb = pos > 0 ? (a ^ bits_at(bits, pos - 1)) & pm & (m == 0 ? ~1u : kFull) : 0u;
    const uint32_t yb = j > 0 ? (a ^ bits_at(bits, pos - dy)) & pm : 0u;
    const uint32_t zb = k > 0 ? (a ^ bits_at(bits, pos - dz)) & pm : 0u;
    uint32_t inc = xf | yf | zf | xb | yb | zb;
    if (inc == 0u) continue;
    EdgeOwner own;
    own.X = xf;
    own.Y = yf;
    own.Z = zf;
    own.base = (long long)__ldg(wv + w);
    EdgeOwner oy{}, oz{};
    if (yb) oy = edge_owner(g, bits, wv, j - 1, k, m);
    if (zb) oz = edge_owner(g, bits, wv, j, k - 1, m);
    while (inc) {
      const int b = __ffs(inc) - 1;
      inc &= inc - 1u;
      const uint32_t bit = 1u << b;
      const int i = 32 * m + b;
      const long long p = pos + b;
      float acc = 0.0f;
      if (xf & bit) acc = __fadd_rn(acc, edge_term(g, f, iso, dverts, edge_id(own, b, 0), 0, p, p + 1, i, true));
      if (yf & bit) acc = __fadd_rn(acc, edge_term(g, f, iso, dverts, edge_id(own, b, 1), 1, p, p + dy, j, true));
      if (zf & bit) acc = __fadd_rn(acc, edge_term(g, f, iso, dverts, edge_id(own, b, 2), 2, p, p + dz, k, true));
      if (xb & bit) {
        long long vid;
        if (b > 0) {
          vid = edge_id(own, b - 1, 0);
        } else {  // the owner is the last point of the previous word
          const EdgeOwner ox = edge_owner(g, bits, wv, j, k, m - 1);
          vid = edge_id(ox, 31, 0);
        }
        acc = __fadd_rn(acc, edge_term(g, f, iso, dverts, vid, 0, p - 1, p, i - 1, false));
      }
      if (yb & bit)
        acc = __fadd_rn(acc, edge_term(g, f, iso, dverts, edge_id(oy, b, 1), 1, p - dy, p, j - 1, false));
      if (zb & bit)
        acc = __fadd_rn(acc, edge_term(g, f, iso, dverts, edge_id(oz, b, 2), 2, p - dz, p, k - 1, false));
      out[p] = __fadd_rn(out[p], acc);
    }
  }
}

void launch_field_adjoint(const Grid& g, const float* f, float iso, const uint32_t* bits,
                          const WordOffsets* o, const float* dverts, const float* dgrad,
                          float* out, int num_sms, cudaStream_t s) {
  if (dgrad) {
    const MarchTiles mt = march_tiles(g.nx, g.ny, g.nz, kAdjBand);  // tiles of points
    const long long blocks = (mt.tasks + kMarchWarps - 1) / kMarchWarps;
    k_grad_adjoint<<<(unsigned)blocks, kMarchWarps * 32, 0, s>>>(g, dgrad, out, mt);
  } else {
    cudaMemsetAsync(out, 0, (size_t)g.P * sizeof(float), s);
  }
  if (dverts) {
    const long long want = (g.R * g.wr + 255) / 256;
    const int blocks = resident_blocks(k_edge_adjoint, 256, 0, num_sms, want);
    k_edge_adjoint<<<blocks, 256, 0, s>>>(g, f, iso, bits, o->wv, dverts, out);
  }
}

}  // namespace daxgb

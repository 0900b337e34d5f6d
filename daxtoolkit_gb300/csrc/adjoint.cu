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
__device__ __forceinline__ void grad_adjoint_task(const Grid& g, const float* __restrict__ dg,
                                                  float* __restrict__ out, const MarchTiles& mt,
                                                  long long task) {
  const int lane = threadIdx.x & 31;
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

__global__ void __launch_bounds__(kMarchWarps * 32, kAdjMinBlocks)
    k_grad_adjoint(Grid g, const float* __restrict__ dg, float* __restrict__ out, MarchTiles mt) {
  grad_adjoint_task(g, dg, out, mt, (long long)blockIdx.x * kMarchWarps + (threadIdx.x >> 5));
}

// A grid set: the block's grid (block0 as in k_cell_gradient_set); cell
// gradients and the output field are concatenated over the set.
__global__ void __launch_bounds__(kMarchWarps * 32, kAdjMinBlocks)
    k_grad_adjoint_set(GridSet S, const long long* __restrict__ block0,
                       const float* __restrict__ dg, float* __restrict__ out) {
  const int si = block_slot(block0, S.count, blockIdx.x);
  const Grid g = S.slots[si].g;
  grad_adjoint_task(g, dg + 3 * S.slots[si].cell0, out + S.slots[si].point0,
                    march_tiles(g.nx, g.ny, g.nz, kAdjBand),
                    ((long long)blockIdx.x - __ldg(block0 + si)) * kMarchWarps +
                        (threadIdx.x >> 5));
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

// Contribution to dL/df at one end of an edge along `axis` with end values
// fa (at the lower end A) and fb, upstream dL/dx_v[axis] dv and axis width
// h; at_a: the end is A.
__device__ __forceinline__ float edge_term(float iso, float fa, float fb, float dv, float h,
                                           bool at_a) {
  const float d = __fsub_rn(fb, fa);
  const float gv = __fmul_rn(dv, h);
  const float num = at_a ? __fsub_rn(iso, fb) : -__fsub_rn(iso, fa);
  return __fdiv_rn(__fmul_rn(gv, num), __fmul_rn(d, d));
}

__device__ __forceinline__ uint32_t rank_below(uint32_t X, uint32_t Y, uint32_t Z, uint32_t lm) {
  return (uint32_t)(__popc(X & lm) + __popc(Y & lm) + __popc(Z & lm));
}

// Position of the n-th (0-based) set bit of u; n < popc(u).
__device__ __forceinline__ int nth_set_bit(uint32_t u, int n) {
  int p = 0;
#pragma unroll
  for (int step = 16; step > 0; step >>= 1)
    if (__popc(u & ((1u << (p + step)) - 1u)) <= n) p += step;
  return p;
}

}  // namespace

// A warp takes 32 consecutive point row words (lane = word) and finds the
// points with an incident crossing edge and the owner words of their
// backward edges; those points are then dealt to the lanes (lane = point),
// which load all of a point's end values and vertex gradients before
// summing its terms in the fixed order.
__device__ __forceinline__ void edge_adjoint_words(const Grid& g, const float* __restrict__ f,
                                                   float iso, const uint32_t* __restrict__ bits,
                                                   const uint32_t* __restrict__ wv,
                                                   const float* __restrict__ dverts,
                                                   float* __restrict__ out, long long w0) {
  const long long W = g.R * g.wr;  // < 2^27 for grids below 2^31 points
  const long long dy = g.nx, dz = (long long)g.nx * g.ny;
  const int lane = threadIdx.x & 31;
  {
    // ---- lane = word ------------------------------------------------------
    const long long w = w0 + lane;
    uint32_t inc = 0u, xf = 0u, yf = 0u, zf = 0u, xb = 0u, yb = 0u, zb = 0u, base = 0u;
    uint32_t r = 0u;
    int m = 0, j = 0, k = 0;
    if (w < W) {
      r = split_word(g, (unsigned)w, m);
      split_row(g, r, j, k);
      const long long pos = (long long)r * g.nx + 32ll * m;
      const uint32_t pm = low_mask(g.nx - 32 * m);
      uint32_t a, a1;
      bits_at2(bits, pos, a, a1);
      // points of this word with an incident crossing edge, per direction
      xf = (a ^ a1) & low_mask(g.nx - 1 - 32 * m);
      yf = j < g.ny - 1 ? (a ^ bits_at(bits, pos + dy)) & pm : 0u;
      zf = k < g.nz - 1 ? (a ^ bits_at(bits, pos + dz)) & pm : 0u;
      xb = pos > 0 ? (a ^ bits_at(bits, pos - 1)) & pm & (m == 0 ? ~1u : kFull) : 0u;
      yb = j > 0 ? (a ^ bits_at(bits, pos - dy)) & pm : 0u;
      zb = k > 0 ? (a ^ bits_at(bits, pos - dz)) & pm : 0u;
      inc = xf | yf | zf | xb | yb | zb;
    }
    if (__ballot_sync(kFull, inc != 0u) == 0u) return;
    // owner words of the backward edges: (j - 1, k), (j, k - 1), and the
    // x edge of bit 0, owned by the previous word's point 31
    uint32_t oyX = 0u, oyY = 0u, oyZ = 0u, oyB = 0u, ozX = 0u, ozY = 0u, ozZ = 0u, ozB = 0u;
    uint32_t ox31 = 0u;
    if (inc) {
      base = __ldg(wv + w);
      if (yb) {
        const EdgeOwner o = edge_owner(g, bits, wv, j - 1, k, m);
        oyX = o.X;
        oyY = o.Y;
        oyZ = o.Z;
        oyB = (uint32_t)o.base;
      }
      if (zb) {
        const EdgeOwner o = edge_owner(g, bits, wv, j, k - 1, m);
        ozX = o.X;
        ozY = o.Y;
        ozZ = o.Z;
        ozB = (uint32_t)o.base;
      }
      if (xb & 1u) ox31 = (uint32_t)edge_id(edge_owner(g, bits, wv, j, k, m - 1), 31, 0);
    }
    int total;
    int pre = __popc(inc);
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int y = __shfl_up_sync(kFull, pre, d);
      if (lane >= d) pre += y;
    }
    total = __shfl_sync(kFull, pre, 31);
    pre -= __popc(inc);  // exclusive: incident points of the words before this lane's
    // ---- lane = incident point ------------------------------------------
    for (int t0 = 0; t0 < total; t0 += 32) {
      const int t = t0 + lane;
      int s = 0;  // the word holding point t: the last s with pre[s] <= t
#pragma unroll
      for (int step = 16; step > 0; step >>= 1) {
        const int ps = __shfl_sync(kFull, pre, s + step);
        if (ps <= t) s += step;
      }
      const int rank = t - __shfl_sync(kFull, pre, s);
      const uint32_t sinc = __shfl_sync(kFull, inc, s);
      const uint32_t sxf = __shfl_sync(kFull, xf, s), syf = __shfl_sync(kFull, yf, s),
                     szf = __shfl_sync(kFull, zf, s);
      const uint32_t sxb = __shfl_sync(kFull, xb, s), syb = __shfl_sync(kFull, yb, s),
                     szb = __shfl_sync(kFull, zb, s);
      const uint32_t sbase = __shfl_sync(kFull, base, s);
      const uint32_t syX = __shfl_sync(kFull, oyX, s), syY = __shfl_sync(kFull, oyY, s),
                     syZ = __shfl_sync(kFull, oyZ, s), syB = __shfl_sync(kFull, oyB, s);
      const uint32_t szX = __shfl_sync(kFull, ozX, s), szY = __shfl_sync(kFull, ozY, s),
                     szZ = __shfl_sync(kFull, ozZ, s), szB = __shfl_sync(kFull, ozB, s);
      const uint32_t sox = __shfl_sync(kFull, ox31, s), sr = __shfl_sync(kFull, r, s);
      const int sm = __shfl_sync(kFull, m, s), sj = __shfl_sync(kFull, j, s),
                sk = __shfl_sync(kFull, k, s);
      if (t >= total) continue;
      const int b = nth_set_bit(sinc, rank);
      const int i = 32 * sm + b;
      const long long p = (long long)sr * g.nx + i;
      const bool fx = (sxf >> b) & 1u, fy = (syf >> b) & 1u, fz = (szf >> b) & 1u;
      const bool bx = (sxb >> b) & 1u, by = (syb >> b) & 1u, bz = (szb >> b) & 1u;
      // vertex ids, as the forward pass numbered them (owner word offset +
      // rank of the edge in (point, axis) order)
      const uint32_t lm = (1u << b) - 1u;
      const uint32_t own = sbase + rank_below(sxf, syf, szf, lm);
      const uint32_t vfx = own, vfy = own + (fx ? 1u : 0u), vfz = vfy + (fy ? 1u : 0u);
      const uint32_t vbx = b > 0 ? sbase + rank_below(sxf, syf, szf, lm >> 1) : sox;
      const uint32_t vby = syB + rank_below(syX, syY, syZ, lm) + ((syX >> b) & 1u);
      const uint32_t vbz = szB + rank_below(szX, szY, szZ, lm) + ((szX >> b) & 1u) + ((szY >> b) & 1u);
      // every load of the point first
      const float fp = __ldg(f + p);
      const float fxn = fx ? __ldg(f + p + 1) : 0.0f, fyn = fy ? __ldg(f + p + dy) : 0.0f,
                  fzn = fz ? __ldg(f + p + dz) : 0.0f;
      const float fxp = bx ? __ldg(f + p - 1) : 0.0f, fyp = by ? __ldg(f + p - dy) : 0.0f,
                  fzp = bz ? __ldg(f + p - dz) : 0.0f;
      const float gfx = fx ? __ldg(dverts + 3ll * vfx + 0) : 0.0f;
      const float gfy = fy ? __ldg(dverts + 3ll * vfy + 1) : 0.0f;
      const float gfz = fz ? __ldg(dverts + 3ll * vfz + 2) : 0.0f;
      const float gbx = bx ? __ldg(dverts + 3ll * vbx + 0) : 0.0f;
      const float gby = by ? __ldg(dverts + 3ll * vby + 1) : 0.0f;
      const float gbz = bz ? __ldg(dverts + 3ll * vbz + 2) : 0.0f;
      const float prev = out[p];
      // forward x, y, z (the point is the edge's A end), then backward x, y, z
      float acc = 0.0f;
      if (fx) acc = __fadd_rn(acc, edge_term(iso, fp, fxn, gfx, width_x(g, i), true));
      if (fy) acc = __fadd_rn(acc, edge_term(iso, fp, fyn, gfy, width_y(g, sj), true));
      if (fz) acc = __fadd_rn(acc, edge_term(iso, fp, fzn, gfz, width_z(g, sk), true));
      if (bx) acc = __fadd_rn(acc, edge_term(iso, fxp, fp, gbx, width_x(g, i - 1), false));
      if (by) acc = __fadd_rn(acc, edge_term(iso, fyp, fp, gby, width_y(g, sj - 1), false));
      if (bz) acc = __fadd_rn(acc, edge_term(iso, fzp, fp, gbz, width_z(g, sk - 1), false));
      out[p] = __fadd_rn(prev, acc);
    }
  }
}

__global__ void __launch_bounds__(256) k_edge_adjoint(Grid g, const float* __restrict__ f,
                                                      float iso,
                                                      const uint32_t* __restrict__ bits,
                                                      const uint32_t* __restrict__ wv,
                                                      const float* __restrict__ dverts,
                                                      float* __restrict__ out) {
  const long long W = g.R * g.wr;
  const long long warp0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long w0 = warp0 * 32; w0 < W; w0 += nwarps * 32)
    edge_adjoint_words(g, f, iso, bits, wv, dverts, out, w0);
}

// A grid set: each block takes 256 consecutive row words of its grid
// (block0 per grid); bits, word offsets and vertex gradients are the set's,
// the output field is concatenated over the set.
__global__ void __launch_bounds__(256) k_edge_adjoint_set(GridSet S,
                                                          const long long* __restrict__ block0,
                                                          const uint32_t* __restrict__ bits,
                                                          const uint32_t* __restrict__ wv,
                                                          const float* __restrict__ dverts,
                                                          float* __restrict__ out) {
  const int si = block_slot(block0, S.count, blockIdx.x);
  const GridSlot& sl = S.slots[si];
  const Grid g = sl.g;
  const long long w0 = ((long long)blockIdx.x - __ldg(block0 + si)) * 256 + (threadIdx.x & ~31);
  if (w0 < g.R * g.wr)
    edge_adjoint_words(g, sl.field, sl.iso, bits + sl.word0, wv + sl.rw0, dverts,
                       out + sl.point0, w0);
}

long long adjoint_grad_blocks(const Grid& g) {
  return (march_tiles(g.nx, g.ny, g.nz, kAdjBand).tasks + kMarchWarps - 1) / kMarchWarps;
}
long long adjoint_edge_blocks(const Grid& g) { return (g.R * g.wr + 255) / 256; }

void launch_field_adjoint_set(const GridSet& S, const long long* grad_block0,
                              long long grad_blocks, const long long* edge_block0,
                              long long edge_blocks, long long points, const uint32_t* bits,
                              const uint32_t* wv, const float* dverts, const float* dgrad,
                              float* out, cudaStream_t s) {
  if (dgrad && grad_blocks > 0)
    k_grad_adjoint_set<<<(unsigned)grad_blocks, kMarchWarps * 32, 0, s>>>(S, grad_block0, dgrad,
                                                                          out);
  else
    cudaMemsetAsync(out, 0, (size_t)points * sizeof(float), s);
  if (dverts && edge_blocks > 0)
    k_edge_adjoint_set<<<(unsigned)edge_blocks, 256, 0, s>>>(S, edge_block0, bits, wv, dverts,
                                                             out);
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

// Marching cubes on the classification bit stream.
//
// K2 (k_mc_rows): for every point row r = (j, k)
//     T[r] = triangles of cell row r      = sum NumFaces[case(i)]
//     V[r] = crossing edges owned by row r = edges (p, p + e_axis) whose end
//            points classify differently, axis x < y < z
//   then a single-pass decoupled look-back scan over tiles of 256 rows turns
//   them into exclusive row offsets.  V counts exactly the vertices of the
//   merged output: a cell's triangle-table row references exactly its
//   sign-change edges, every grid edge belongs to a cell, and the reference's
//   merged order, ascending (first id, second id), is ascending (owner point,
//   axis) on a uniform grid -- i.e. row order, then x, then axis.  So the
//   reference's Sort/Unique/LowerBounds
//   (dax/cont/DispatcherGenerateInterpolatedCells.h:276-291) becomes a rank.
//
// K3 (k_mc_emit): for every row with output, recompute cases from the bits,
//   write vertices at V-offset + rank and triangles at T-offset + rank; a
//   triangle corner's vertex id is the row offset of the edge's owner row
//   plus the edge's rank inside that row.  Field values are read only at
//   crossing-edge end points.
#include "common.cuh"
#include "kernels.cuh"
#include "mc_case.cuh"

namespace daxgb {

// Edge e of the hexahedron (cellVertEdges, dax/worklet/MarchingCubes.h:131-135)
// as (owner offset di, dj, dk, axis) of its lower-id end point:
// bits 0..2 = di, dj, dk; bits 3..4 = axis (0 x, 1 y, 2 z).
__constant__ unsigned char kEdgeOwner[12] = {
    0 | (0 << 3), 1 | (1 << 3), 2 | (0 << 3), 0 | (1 << 3), 4 | (0 << 3), 5 | (1 << 3),
    6 | (0 << 3), 4 | (1 << 3), 0 | (2 << 3), 1 | (2 << 3), 3 | (2 << 3), 2 | (2 << 3)};

struct CornerWords {
  uint32_t a, a1, b, b1, c, c1, d, d1;
};

// The eight corner-bit words of cells 32m..32m+31 of cell row (j, k):
// a = (i, j, k), a1 = (i+1, j, k), b = (i, j+1, k), c = (i, j, k+1), d = (i, j+1, k+1).
__device__ __forceinline__ CornerWords corner_words(const Grid& g, const uint32_t* bits,
                                                   long long pos) {
  const long long dy = g.nx, dz = (long long)g.nx * g.ny;
  CornerWords w;
  w.a = bits_at(bits, pos);
  w.a1 = bits_at(bits, pos + 1);
  w.b = bits_at(bits, pos + dy);
  w.b1 = bits_at(bits, pos + dy + 1);
  w.c = bits_at(bits, pos + dz);
  w.c1 = bits_at(bits, pos + dz + 1);
  w.d = bits_at(bits, pos + dy + dz);
  w.d1 = bits_at(bits, pos + dy + dz + 1);
  return w;
}

// Case index of cell q of the word; vertex order v0..v7 =
// (i,j,k) (i+1,j,k) (i+1,j+1,k) (i,j+1,k) and the same at k+1
// (dax/exec/internal/TopologyUniform.h:150-157); bit n = value[n] > iso.
__device__ __forceinline__ int case_of(const CornerWords& w, int q) {
  return (int)(((w.a >> q) & 1u) | (((w.a1 >> q) & 1u) << 1) | (((w.b1 >> q) & 1u) << 2) |
               (((w.b >> q) & 1u) << 3) | (((w.c >> q) & 1u) << 4) | (((w.c1 >> q) & 1u) << 5) |
               (((w.d1 >> q) & 1u) << 6) | (((w.d >> q) & 1u) << 7));
}

// Cells of the word that are neither all-inside nor all-outside.
__device__ __forceinline__ uint32_t active_cells(const CornerWords& w, uint32_t cell_mask) {
  const uint32_t all1 = w.a & w.a1 & w.b & w.b1 & w.c & w.c1 & w.d & w.d1;
  const uint32_t any1 = w.a | w.a1 | w.b | w.b1 | w.c | w.c1 | w.d | w.d1;
  return any1 & ~all1 & cell_mask;
}

// Crossing-edge masks of point row (j, k), word m: bit q of X/Y/Z set when the
// x/y/z edge owned by point i = 32m + q is a sign-change edge.
__device__ __forceinline__ void crossing_masks(const Grid& g, const uint32_t* bits, int j, int k,
                                               int m, uint32_t& X, uint32_t& Y, uint32_t& Z) {
  const long long pos = ((long long)k * g.ny + j) * g.nx + 32ll * m;
  const int i0 = 32 * m;
  const uint32_t pmask = low_mask(g.nx - i0);
  const uint32_t xmask = low_mask(g.nx - 1 - i0);
  const uint32_t a = bits_at(bits, pos);
  X = (a ^ bits_at(bits, pos + 1)) & xmask;
  Y = (j < g.ny - 1) ? ((a ^ bits_at(bits, pos + g.nx)) & pmask) : 0u;
  Z = (k < g.nz - 1) ? ((a ^ bits_at(bits, pos + (long long)g.nx * g.ny)) & pmask) : 0u;
}

// ---------------------------------------------------------------------------
// K2: per-row counts + look-back scan.  256 rows per tile, G lanes per row.
template <int G>
__global__ void __launch_bounds__(256) k_mc_rows(Grid g, const uint32_t* __restrict__ bits,
                                                 long long* __restrict__ row_t,
                                                 long long* __restrict__ row_v,
                                                 unsigned long long* __restrict__ status,
                                                 Info* __restrict__ info, int tiles) {
  constexpr int RT = kRowsPerTile;
  constexpr int GPB = 256 / G;
  __shared__ int s_tile;
  __shared__ int s_t[RT], s_v[RT];
  __shared__ long long s_wt[8], s_wv[8];
  __shared__ long long s_ex[2];
  if (threadIdx.x == 0) s_tile = (int)atomicAdd(&info->ticket, 1u);
  __syncthreads();
  const int tile = s_tile;
  const long long r0 = (long long)tile * RT;
  const int gl = threadIdx.x & (G - 1);
  const int grp = threadIdx.x / G;
  for (int lr = grp; lr < RT; lr += GPB) {
    const long long r = r0 + lr;
    int t = 0, v = 0;
    if (r < g.R) {
      const int j = (int)(r % g.ny), k = (int)(r / g.ny);
      const bool cells = (j < g.ny - 1) && (k < g.nz - 1);
      for (int m = gl; m < g.wr; m += G) {
        uint32_t X, Y, Z;
        crossing_masks(g, bits, j, k, m, X, Y, Z);
        v += __popc(X) + __popc(Y) + __popc(Z);
        if (cells) {
          const long long pos = r * g.nx + 32ll * m;
          const CornerWords w = corner_words(g, bits, pos);
          uint32_t act = active_cells(w, low_mask(g.nx - 1 - 32 * m));
          while (act) {
            const int q = __ffs(act) - 1;
            act &= act - 1;
            t += mc_num_tris(case_of(w, q));
          }
        }
      }
    }
    t = group_sum(t, G);
    v = group_sum(v, G);
    if (gl == 0) {
      s_t[lr] = t;
      s_v[lr] = v;
    }
  }
  __syncthreads();
  // block-wide exclusive scan, thread tid <-> row r0 + tid
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const long long t0 = s_t[tid], v0 = s_v[tid];
  long long ti = t0, vi = v0;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const long long ut = __shfl_up_sync(kFull, ti, o), uv = __shfl_up_sync(kFull, vi, o);
    if (lane >= o) { ti += ut; vi += uv; }
  }
  if (lane == 31) { s_wt[warp] = ti; s_wv[warp] = vi; }
  __syncthreads();
  long long wt = 0, wv = 0, aggt = 0, aggv = 0;
#pragma unroll
  for (int w = 0; w < 8; ++w) {
    if (w < warp) { wt += s_wt[w]; wv += s_wv[w]; }
    aggt += s_wt[w];
    aggv += s_wv[w];
  }
  if (warp == 0) s_ex[0] = warp_lookback(status, tile, aggt, &info->error);
  if (warp == 1) s_ex[1] = warp_lookback(status + tiles, tile, aggv, &info->error);
  __syncthreads();
  const long long r = r0 + tid;
  if (r < g.R) {
    row_t[r] = s_ex[0] + wt + ti - t0;
    row_v[r] = s_ex[1] + wv + vi - v0;
  }
  if (tile == tiles - 1 && tid == 0) {
    row_t[g.R] = s_ex[0] + aggt;
    row_v[g.R] = s_ex[1] + aggv;
    info->total_a = s_ex[0] + aggt;
    info->total_b = s_ex[1] + aggv;
  }
}

void launch_mc_rows(const Grid& g, const uint32_t* bits, long long* row_t, long long* row_v,
                    unsigned long long* status, Info* info, int tiles, cudaStream_t s) {
  switch (lanes_per_row(g.wr)) {
    case 1: k_mc_rows<1><<<tiles, 256, 0, s>>>(g, bits, row_t, row_v, status, info, tiles); break;
    case 2: k_mc_rows<2><<<tiles, 256, 0, s>>>(g, bits, row_t, row_v, status, info, tiles); break;
    case 4: k_mc_rows<4><<<tiles, 256, 0, s>>>(g, bits, row_t, row_v, status, info, tiles); break;
    case 8: k_mc_rows<8><<<tiles, 256, 0, s>>>(g, bits, row_t, row_v, status, info, tiles); break;
    case 16: k_mc_rows<16><<<tiles, 256, 0, s>>>(g, bits, row_t, row_v, status, info, tiles); break;
    default: k_mc_rows<32><<<tiles, 256, 0, s>>>(g, bits, row_t, row_v, status, info, tiles); break;
  }
}

// ---------------------------------------------------------------------------
// K3: emit.  One group of G lanes per row, rows in a grid-stride loop.

// Vertex on the edge owned by point (i, j, k) along `axis`:
// weight = (iso - f[A]) / (f[B] - f[A]) (dax/worklet/MarchingCubes.h:160-161),
// position = Lerp(coord A, coord B, weight) per component
// (dax/exec/internal/kernel/GenerateWorklets.h:79-92).
__device__ __forceinline__ void emit_vertex(const Grid& g, const float* __restrict__ f, float iso,
                                            int i, int j, int k, int axis, long long vid,
                                            float* __restrict__ verts, int32_t* __restrict__ ra,
                                            int32_t* __restrict__ rb, float* __restrict__ rw) {
  const long long pa = ((long long)k * g.ny + j) * g.nx + i;
  const long long pb = pa + (axis == 0 ? 1ll : (axis == 1 ? (long long)g.nx : (long long)g.nx * g.ny));
  const float fa = __ldg(f + pa), fb = __ldg(f + pb);
  const float w = __fdiv_rn(__fsub_rn(iso, fa), __fsub_rn(fb, fa));
  const float xa = coord(g.ox, g.sx, i, g.mx), ya = coord(g.oy, g.sy, j, g.my),
              za = coord(g.oz, g.sz, k, g.mz);
  const float xb = axis == 0 ? coord(g.ox, g.sx, i + 1, g.mx) : xa;
  const float yb = axis == 1 ? coord(g.oy, g.sy, j + 1, g.my) : ya;
  const float zb = axis == 2 ? coord(g.oz, g.sz, k + 1, g.mz) : za;
  verts[3 * vid + 0] = lerp_rn(xa, xb, w);
  verts[3 * vid + 1] = lerp_rn(ya, yb, w);
  verts[3 * vid + 2] = lerp_rn(za, zb, w);
  if (ra) ra[vid] = (int32_t)pa;
  if (rb) rb[vid] = (int32_t)pb;
  if (rw) rw[vid] = w;
}

template <int G, bool MERGE>
__global__ void __launch_bounds__(256) k_mc_emit(Grid g, const float* __restrict__ f, float iso,
                                                 const uint32_t* __restrict__ bits,
                                                 const long long* __restrict__ row_t,
                                                 const long long* __restrict__ row_v,
                                                 Info* __restrict__ info,
                                                 float* __restrict__ verts, long long vcap,
                                                 int32_t* __restrict__ conn, long long tcap,
                                                 int32_t* __restrict__ ra, int32_t* __restrict__ rb,
                                                 float* __restrict__ rw) {
  constexpr int GPB = 256 / G;
  extern __shared__ uint32_t s_rows[];  // [GPB][4 rows][X, Y, Z, prefix][wr]
  {
    const long long T = info->total_a;
    const long long V = MERGE ? info->total_b : 3 * T;
    if (T > tcap || V > vcap) {
      if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&info->error, kErrCapacity);
      return;
    }
  }
  const int gl = threadIdx.x & (G - 1);
  const int grp = threadIdx.x / G;
  const int wr = g.wr;
  uint32_t* sm = s_rows + (size_t)grp * 16 * wr;
  const long long ngroups = (long long)gridDim.x * GPB;
  for (long long r = (long long)blockIdx.x * GPB + grp; r < g.R; r += ngroups) {
    const long long vb = row_v[r], ve = row_v[r + 1];
    const long long tb = row_t[r], te = row_t[r + 1];
    if (vb == ve && tb == te) continue;
    const int j = (int)(r % g.ny), k = (int)(r / g.ny);
    long long qbase[4] = {vb, 0, 0, 0};
    if (MERGE) {
      // crossing masks + in-row prefix for the owner rows (j..j+1, k..k+1)
      const int nq = (te > tb) ? 4 : 1;
      for (int qi = 0; qi < nq; ++qi) {
        const int jq = j + (qi & 1), kq = k + (qi >> 1);
        if (qi) qbase[qi] = row_v[(long long)kq * g.ny + jq];
        int carry = 0;
        for (int m0 = 0; m0 < wr; m0 += G) {
          const int m = m0 + gl;
          uint32_t X = 0, Y = 0, Z = 0;
          if (m < wr) crossing_masks(g, bits, jq, kq, m, X, Y, Z);
          const int cnt = __popc(X) + __popc(Y) + __popc(Z);
          const int incl = group_inclusive_scan(cnt, G);
          if (m < wr) {
            uint32_t* q = sm + qi * 4 * wr;
            q[m] = X;
            q[wr + m] = Y;
            q[2 * wr + m] = Z;
            q[3 * wr + m] = (uint32_t)(carry + incl - cnt);
          }
          carry += group_last(incl, G);
        }
      }
      __syncwarp(group_mask(G));
      // vertices owned by row r
      if (ve > vb) {
        for (int m = gl; m < wr; m += G) {
          const uint32_t X = sm[m], Y = sm[wr + m], Z = sm[2 * wr + m];
          long long vid = vb + sm[3 * wr + m];
          uint32_t u = X | Y | Z;
          while (u) {
            const int q = __ffs(u) - 1;
            u &= u - 1;
            const int i = 32 * m + q;
            if ((X >> q) & 1u) emit_vertex(g, f, iso, i, j, k, 0, vid++, verts, ra, rb, rw);
            if ((Y >> q) & 1u) emit_vertex(g, f, iso, i, j, k, 1, vid++, verts, ra, rb, rw);
            if ((Z >> q) & 1u) emit_vertex(g, f, iso, i, j, k, 2, vid++, verts, ra, rb, rw);
          }
        }
      }
    }
    if (te > tb) {
      long long carry = 0;
      const long long pos0 = r * g.nx;
      for (int m0 = 0; m0 < wr; m0 += G) {
        const int m = m0 + gl;
        CornerWords w{};
        uint32_t act = 0;
        int cnt = 0;
        if (m < wr) {
          w = corner_words(g, bits, pos0 + 32ll * m);
          act = active_cells(w, low_mask(g.nx - 1 - 32 * m));
          for (uint32_t u = act; u; u &= u - 1) cnt += mc_num_tris(case_of(w, __ffs(u) - 1));
        }
        const int incl = group_inclusive_scan(cnt, G);
        long long tid = tb + carry + incl - cnt;
        for (uint32_t u = act; u; u &= u - 1) {
          const int q = __ffs(u) - 1;
          const int i = 32 * m + q;
          const uint64_t cw = kMcCase[case_of(w, q)];
          const int nt = (int)(cw >> 60);
          for (int tt = 0; tt < nt; ++tt, ++tid) {
#pragma unroll
            for (int corner = 0; corner < 3; ++corner) {
              const int e = mc_edge(cw, 3 * tt + corner);
              const int info_e = kEdgeOwner[e];
              const int di = info_e & 1, dj = (info_e >> 1) & 1, dk = (info_e >> 2) & 1;
              const int axis = info_e >> 3;
              if (MERGE) {
                const int qi = dj + 2 * dk;
                const int ii = i + di;
                const int wq = ii >> 5, bq = ii & 31;
                const uint32_t* qs = sm + qi * 4 * wr;
                const uint32_t lm = (1u << bq) - 1u;
                const uint32_t X = qs[wq], Y = qs[wr + wq], Z = qs[2 * wr + wq];
                int rank = (int)qs[3 * wr + wq] + __popc(X & lm) + __popc(Y & lm) + __popc(Z & lm);
                if (axis >= 1) rank += (X >> bq) & 1u;
                if (axis >= 2) rank += (Y >> bq) & 1u;
                conn[3 * tid + corner] = (int32_t)(qbase[qi] + rank);
              } else {
                const long long vid = 3 * tid + corner;
                conn[vid] = (int32_t)vid;
                emit_vertex(g, f, iso, i + di, j + dj, k + dk, axis, vid, verts, ra, rb, rw);
              }
            }
          }
        }
        carry += group_last(incl, G);
      }
    }
    __syncwarp(group_mask(G));
  }
}

template <int G>
static void launch_emit_g(const Grid& g, const float* f, float iso, bool merge,
                          const uint32_t* bits, const long long* row_t, const long long* row_v,
                          Info* info, float* verts, long long vcap, int32_t* conn, long long tcap,
                          int32_t* ra, int32_t* rb, float* rw, int num_sms, cudaStream_t s) {
  constexpr int GPB = 256 / G;
  const size_t smem = merge ? (size_t)GPB * 16 * g.wr * sizeof(uint32_t) : 0;
  const long long want = (g.R + GPB - 1) / GPB;
  const long long cap = (long long)num_sms * 8;
  const int blocks = (int)(want < 1 ? 1 : (want < cap ? want : cap));
  if (merge) {
    if (smem > 48 * 1024)
      cudaFuncSetAttribute(k_mc_emit<G, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem);
    k_mc_emit<G, true><<<blocks, 256, smem, s>>>(g, f, iso, bits, row_t, row_v, info, verts, vcap,
                                                 conn, tcap, ra, rb, rw);
  } else {
    k_mc_emit<G, false><<<blocks, 256, 0, s>>>(g, f, iso, bits, row_t, row_v, info, verts, vcap,
                                               conn, tcap, ra, rb, rw);
  }
}

void launch_mc_emit(const Grid& g, const float* f, float iso, bool merge, const uint32_t* bits,
                    const long long* row_t, const long long* row_v, Info* info, float* verts,
                    long long vcap, int32_t* conn, long long tcap, int32_t* ra, int32_t* rb,
                    float* rw, int num_sms, cudaStream_t s) {
#define DAXGB_EMIT(G)                                                                           \
  launch_emit_g<G>(g, f, iso, merge, bits, row_t, row_v, info, verts, vcap, conn, tcap, ra, rb, \
                   rw, num_sms, s)
  switch (lanes_per_row(g.wr)) {
    case 1: DAXGB_EMIT(1); break;
    case 2: DAXGB_EMIT(2); break;
    case 4: DAXGB_EMIT(4); break;
    case 8: DAXGB_EMIT(8); break;
    case 16: DAXGB_EMIT(16); break;
    default: DAXGB_EMIT(32); break;
  }
#undef DAXGB_EMIT
}

// CompactPointField: out[v] = Lerp(in[first], in[second], weight).
__global__ void k_interpolate(const int32_t* __restrict__ ra, const int32_t* __restrict__ rb,
                              const float* __restrict__ rw, long long n,
                              const float* __restrict__ in, float* __restrict__ out) {
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (long long)gridDim.x * blockDim.x)
    out[v] = lerp_rn(__ldg(in + ra[v]), __ldg(in + rb[v]), rw[v]);
}

void launch_interpolate(const int32_t* ra, const int32_t* rb, const float* rw, long long n,
                        const float* in, float* out, int num_sms, cudaStream_t s) {
  const long long want = (n + 255) / 256;
  const long long cap = (long long)num_sms * 16;
  const int blocks = (int)(want < 1 ? 1 : (want < cap ? want : cap));
  k_interpolate<<<blocks, 256, 0, s>>>(ra, rb, rw, n, in, out);
}

}  // namespace daxgb

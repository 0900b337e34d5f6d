// Marching cubes on the classification bit stream.
//
// Work is indexed by "row words": word m of point row r covers points
// i = 32m .. 32m+31 of that row (and the cells whose first point they are);
// row words are numbered r * wr + m, which is point order.
//
// K2 (k_mc_scan): for every row word
//     T = triangles of its cells            = sum NumFaces[case(i)]
//     V = crossing edges its points own      = edges (p, p + e_axis) whose end
//         points classify differently, axis x < y < z
//     A = 1 if T or V is non-zero
//   and a single-pass decoupled look-back scan (three chains) over tiles of
//   1024 words turns them into exclusive offsets per word plus a compacted
//   list of the active words.  V counts exactly the vertices of the merged
//   output: a cell's triangle-table row references exactly its sign-change
//   edges, every grid edge belongs to a cell, and the reference's merged
//   order, ascending (first id, second id), is ascending (owner point, axis)
//   on a uniform grid -- point order, then axis.  So the reference's
//   Sort/Unique/LowerBounds (dax/cont/DispatcherGenerateInterpolatedCells.h:
//   276-291) becomes a rank: offset of the owner word + popcount.
//
// K3 (k_mc_emit): one thread per ACTIVE word (from the compacted list):
//   recompute cases from the bits, write the word's vertices at its V offset
//   and its cells' triangles at its T offset; a triangle corner's vertex id
//   is the V offset of the edge's owner word plus the edge's rank inside it.
//   Field values are read only at crossing-edge end points.
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
// K2: counts per row word + three-chain look-back scan.

// Triangle and crossing-edge counts of word m of row r.  Eight word fetches
// per 32 points: (a, a+x) of the four rows (j..j+1, k..k+1).
__device__ __forceinline__ void mc_word_counts(const Grid& g, const uint32_t* bits, long long r,
                                               int m, int& t, int& v) {
  const int j = (int)(r % g.ny), k = (int)(r / g.ny);
  const bool hy = j < g.ny - 1, hz = k < g.nz - 1;
  const long long dy = g.nx, dz = (long long)g.nx * g.ny;
  const long long pos = r * g.nx + 32ll * m;
  const uint32_t pmask = low_mask(g.nx - 32 * m);
  const uint32_t xmask = low_mask(g.nx - 1 - 32 * m);
  CornerWords w{};
  bits_at2(bits, pos, w.a, w.a1);
  if (hy) bits_at2(bits, pos + dy, w.b, w.b1);
  if (hz) bits_at2(bits, pos + dz, w.c, w.c1);
  if (hy && hz) bits_at2(bits, pos + dy + dz, w.d, w.d1);
  v = __popc((w.a ^ w.a1) & xmask);
  if (hy) v += __popc((w.a ^ w.b) & pmask);
  if (hz) v += __popc((w.a ^ w.c) & pmask);
  t = 0;
  if (hy && hz) {
    uint32_t act = active_cells(w, xmask);
    while (act) {
      const int q = __ffs(act) - 1;
      act &= act - 1;
      t += mc_num_tris(case_of(w, q));
    }
  }
}

constexpr int kWordsPerThread = 4;
constexpr int kWordsPerTile = 256 * kWordsPerThread;

__device__ __forceinline__ void locate_word(const GridSet& S, long long gw, int& si, long long& r,
                                            int& m) {
  si = S.count == 1 ? 0 : slot_of_rowword(S, gw);
  const GridSlot& sl = S.count == 1 ? S.one : S.slots[si];
  const long long lw = gw - sl.rw0;
  r = lw / sl.g.wr;
  m = (int)(lw - r * sl.g.wr);
}

__global__ void __launch_bounds__(256) k_mc_scan(GridSet S, const uint32_t* __restrict__ bits,
                                                 uint32_t* __restrict__ wt,
                                                 uint32_t* __restrict__ wv,
                                                 uint32_t* __restrict__ act,
                                                 unsigned long long* __restrict__ status,
                                                 Info* __restrict__ info, int tiles) {
  __shared__ int s_tile;
  const int tid = threadIdx.x;
  while (true) {
    if (tid == 0) s_tile = (int)atomicAdd(&info->ticket, 1u);
    __syncthreads();
    const int tile = s_tile;
    __syncthreads();
    if (tile >= tiles) break;
    const long long w0 = (long long)tile * kWordsPerTile + (long long)tid * kWordsPerThread;
    int tc[kWordsPerThread], vc[kWordsPerThread];
#pragma unroll
    for (int e = 0; e < kWordsPerThread; ++e) {
      tc[e] = vc[e] = 0;
      const long long gw = w0 + e;
      if (gw < S.rowwords) {
        int si, m;
        long long r;
        locate_word(S, gw, si, r, m);
        const GridSlot& sl = S.count == 1 ? S.one : S.slots[si];
        if (sl.g.nx >= 2 && sl.g.ny >= 2 && sl.g.nz >= 2)
          mc_word_counts(sl.g, bits + sl.word0, r, m, tc[e], vc[e]);
      }
    }
    long long mine[3] = {0, 0, 0};
#pragma unroll
    for (int e = 0; e < kWordsPerThread; ++e) {
      mine[0] += tc[e];
      mine[1] += vc[e];
      mine[2] += (tc[e] | vc[e]) ? 1 : 0;
    }
    long long ex[3], agg[3], base[3];
    block_exclusive_scan<3>(mine, ex, agg);
    block_lookback<3>(status, tiles, tile, agg, &info->error, base);
    long long ot = base[0] + ex[0], ov = base[1] + ex[1], oa = base[2] + ex[2];
#pragma unroll
    for (int e = 0; e < kWordsPerThread; ++e) {
      const long long gw = w0 + e;
      if (gw < S.rowwords) {
        wt[gw] = (uint32_t)ot;
        wv[gw] = (uint32_t)ov;
        if (tc[e] | vc[e]) act[oa++] = (uint32_t)gw;
      }
      ot += tc[e];
      ov += vc[e];
    }
    if (tile == tiles - 1 && tid == 0) {
      const long long T = base[0] + agg[0], V = base[1] + agg[1], A = base[2] + agg[2];
      wt[S.rowwords] = (uint32_t)T;
      wv[S.rowwords] = (uint32_t)V;
      info->total_a = T;
      info->total_b = V;
      info->total_c = A;
      if (T > 2147483647ll || V > 2147483647ll) atomicOr(&info->error, kErrOverflow);
    }
  }
}

void launch_mc_scan(const GridSet& S, const uint32_t* bits, uint32_t* wt, uint32_t* wv,
                    uint32_t* act, unsigned long long* status, Info* info, int tiles, int num_sms,
                    cudaStream_t s) {
  const int blocks = resident_blocks(k_mc_scan, 256, 0, num_sms, tiles);
  k_mc_scan<<<blocks, 256, 0, s>>>(S, bits, wt, wv, act, status, info, tiles);
}

int mc_scan_tiles(long long rowwords) {
  return (int)((rowwords + kWordsPerTile - 1) / kWordsPerTile);
}

// ---------------------------------------------------------------------------
// K3: emit, one thread per active row word.

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

// Crossing masks of one owner word plus its global vertex offset.
struct OwnerWord {
  uint32_t X, Y, Z;
  long long base;
};

__device__ __forceinline__ OwnerWord owner_word(const Grid& g, const uint32_t* bits,
                                                const uint32_t* wv_grid, int jq, int kq, int wq) {
  const long long rq = (long long)kq * g.ny + jq;
  const long long pos = rq * g.nx + 32ll * wq;
  uint32_t a, a1;
  bits_at2(bits, pos, a, a1);
  const uint32_t pm = low_mask(g.nx - 32 * wq);
  OwnerWord o;
  o.X = (a ^ a1) & low_mask(g.nx - 1 - 32 * wq);
  o.Y = jq < g.ny - 1 ? (a ^ bits_at(bits, pos + g.nx)) & pm : 0u;
  o.Z = kq < g.nz - 1 ? (a ^ bits_at(bits, pos + (long long)g.nx * g.ny)) & pm : 0u;
  o.base = __ldg(wv_grid + rq * g.wr + wq);
  return o;
}

__device__ __forceinline__ long long owner_rank_id(const OwnerWord& o, int b, int axis) {
  const uint32_t lm = (1u << b) - 1u;
  long long id = o.base + __popc(o.X & lm) + __popc(o.Y & lm) + __popc(o.Z & lm);
  if (axis >= 1) id += (o.X >> b) & 1u;
  if (axis >= 2) id += (o.Y >> b) & 1u;
  return id;
}

template <bool MERGE>
__global__ void __launch_bounds__(256) k_mc_emit(GridSet S, const uint32_t* __restrict__ bits,
                                                 const uint32_t* __restrict__ wt,
                                                 const uint32_t* __restrict__ wv,
                                                 const uint32_t* __restrict__ act,
                                                 Info* __restrict__ info,
                                                 float* __restrict__ verts, long long vcap,
                                                 int32_t* __restrict__ conn, long long tcap,
                                                 int32_t* __restrict__ ra, int32_t* __restrict__ rb,
                                                 float* __restrict__ rw) {
  const long long T = info->total_a;
  const long long V = MERGE ? info->total_b : 3 * T;
  const long long A = info->total_c;
  if (T > tcap || V > vcap || (info->error & (kErrOverflow | kErrTimeout))) {
    if (blockIdx.x == 0 && threadIdx.x == 0 && (T > tcap || V > vcap))
      atomicOr(&info->error, kErrCapacity);
    return;
  }
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long ai = (long long)blockIdx.x * blockDim.x + threadIdx.x; ai < A; ai += stride) {
    const long long gw = __ldg(act + ai);
    int si, m;
    long long r;
    locate_word(S, gw, si, r, m);
    const GridSlot& sl = S.count == 1 ? S.one : S.slots[si];
    const Grid& g = sl.g;
    const uint32_t* gb = bits + sl.word0;
    const uint32_t* wvg = wv + sl.rw0;
    const float* f = sl.field;
    const float iso = sl.iso;
    const long long t0 = __ldg(wt + gw), t1 = __ldg(wt + gw + 1);
    const long long v0 = __ldg(wv + gw), v1 = __ldg(wv + gw + 1);
    const int j = (int)(r % g.ny), k = (int)(r / g.ny);
    const long long dy = g.nx, dz = (long long)g.nx * g.ny;
    const long long pos = r * g.nx + 32ll * m;
    const uint32_t pmask = low_mask(g.nx - 32 * m);
    const uint32_t xmask = low_mask(g.nx - 1 - 32 * m);
    const bool hy = j < g.ny - 1, hz = k < g.nz - 1;
    CornerWords w{};
    bits_at2(gb, pos, w.a, w.a1);
    if (hy) bits_at2(gb, pos + dy, w.b, w.b1);
    if (hz) bits_at2(gb, pos + dz, w.c, w.c1);
    if (hy && hz) bits_at2(gb, pos + dy + dz, w.d, w.d1);
    if (MERGE && v1 > v0) {
      const uint32_t X = (w.a ^ w.a1) & xmask;
      const uint32_t Y = hy ? (w.a ^ w.b) & pmask : 0u;
      const uint32_t Z = hz ? (w.a ^ w.c) & pmask : 0u;
      long long vid = v0;
      for (uint32_t u = X | Y | Z; u; u &= u - 1) {
        const int q = __ffs(u) - 1;
        const int i = 32 * m + q;
        if ((X >> q) & 1u) emit_vertex(g, f, iso, i, j, k, 0, vid++, verts, ra, rb, rw);
        if ((Y >> q) & 1u) emit_vertex(g, f, iso, i, j, k, 1, vid++, verts, ra, rb, rw);
        if ((Z >> q) & 1u) emit_vertex(g, f, iso, i, j, k, 2, vid++, verts, ra, rb, rw);
      }
    }
    if (t1 == t0) continue;
    // first vertex of this grid in the concatenated output (0 for one grid)
    const long long vbase0 = S.count == 1 ? 0 : (MERGE ? (long long)__ldg(wv + sl.rw0)
                                                       : 3ll * __ldg(wt + sl.rw0));
    OwnerWord ow[4];
    if (MERGE) {
#pragma unroll
      for (int qi = 0; qi < 4; ++qi)
        ow[qi] = owner_word(g, gb, wvg, j + (qi & 1), k + (qi >> 1), m);
    }
    long long tri = t0;
    for (uint32_t u = active_cells(w, xmask); u; u &= u - 1) {
      const int q = __ffs(u) - 1;
      const int i = 32 * m + q;
      const uint64_t cw = kMcCase[case_of(w, q)];
      const int nt = (int)(cw >> 60);
      for (int tt = 0; tt < nt; ++tt, ++tri) {
#pragma unroll
        for (int corner = 0; corner < 3; ++corner) {
          const int e = mc_edge(cw, 3 * tt + corner);
          const int info_e = kEdgeOwner[e];
          const int di = info_e & 1, dj = (info_e >> 1) & 1, dk = (info_e >> 2) & 1;
          const int axis = info_e >> 3;
          if (MERGE) {
            const int ii = i + di;
            long long vid;
            if ((ii >> 5) == m) {
              vid = owner_rank_id(ow[dj + 2 * dk], ii & 31, axis);
            } else {  // the owner point is the first point of the next word
              const OwnerWord o = owner_word(g, gb, wvg, j + dj, k + dk, m + 1);
              vid = owner_rank_id(o, 0, axis);
            }
            conn[3 * tri + corner] = (int32_t)(vid - vbase0);
          } else {
            const long long vid = 3 * tri + corner;
            conn[vid] = (int32_t)(vid - vbase0);
            emit_vertex(g, f, iso, i + di, j + dj, k + dk, axis, vid, verts, ra, rb, rw);
          }
        }
      }
    }
  }
}

void launch_mc_emit(const GridSet& S, bool merge, const uint32_t* bits, const uint32_t* wt,
                    const uint32_t* wv, const uint32_t* act, Info* info, float* verts,
                    long long vcap, int32_t* conn, long long tcap, int32_t* ra, int32_t* rb,
                    float* rw, int num_sms, cudaStream_t s) {
  // the active count lives on the device: launch one resident wave, grid-stride
  const long long want = (S.rowwords + 255) / 256;
  if (merge) {
    const int blocks = resident_blocks(k_mc_emit<true>, 256, 0, num_sms, want);
    k_mc_emit<true><<<blocks, 256, 0, s>>>(S, bits, wt, wv, act, info, verts, vcap, conn, tcap,
                                           ra, rb, rw);
  } else {
    const int blocks = resident_blocks(k_mc_emit<false>, 256, 0, num_sms, want);
    k_mc_emit<false><<<blocks, 256, 0, s>>>(S, bits, wt, wv, act, info, verts, vcap, conn, tcap,
                                            ra, rb, rw);
  }
}

// Per-grid offsets: goff[2g], goff[2g+1] = first triangle / merged vertex of
// grid g; goff[2G], goff[2G+1] = totals.
__global__ void k_grid_offsets(GridSet S, const uint32_t* __restrict__ wt,
                               const uint32_t* __restrict__ wv, long long* __restrict__ goff) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= S.count; i += gridDim.x * blockDim.x) {
    const long long w = i < S.count ? load_slot(S, i).rw0 : S.rowwords;
    goff[2 * i] = wt[w];
    goff[2 * i + 1] = wv[w];
  }
}

void launch_grid_offsets(const GridSet& S, const uint32_t* wt, const uint32_t* wv,
                         long long* goff, cudaStream_t s) {
  k_grid_offsets<<<(S.count + 256) / 256, 256, 0, s>>>(S, wt, wv, goff);
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

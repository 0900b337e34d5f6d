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
// K2: counts per row word, then a single-pass scan.
//   K2a (k_mc_count): one thread per word; writes the packed counts
//       wc[w] = (triangles << 16) | crossing edges (both < 2^16: a word has
//       32 points and 32 cells).  No synchronisation.
//   K2b (k_mc_scan): single-pass decoupled look-back scan of wc (tiles of
//       4096 words, 16 per thread), writing per-word exclusive triangle and
//       vertex offsets wt / wv (uint32[rowwords + 1]) and the compacted list
//       act of active words (uint32[A]).

// The eight corner words of word m of row r (a, a+x of rows (j..j+1,
// k..k+1)) and the masks that decide which of them are meaningful.
struct WordBits {
  CornerWords w;
  uint32_t pmask, xmask;
  bool hy, hz;
};

__device__ __forceinline__ WordBits load_word_bits(const Grid& g, const uint32_t* bits, unsigned r,
                                                   int m) {
  WordBits wb;
  const int j = (int)(r % (unsigned)g.ny), k = (int)(r / (unsigned)g.ny);
  wb.hy = j < g.ny - 1;
  wb.hz = k < g.nz - 1;
  const long long dy = g.nx, dz = (long long)g.nx * g.ny;
  const long long pos = (long long)r * g.nx + 32ll * m;
  wb.pmask = low_mask(g.nx - 32 * m);
  wb.xmask = low_mask(g.nx - 1 - 32 * m);
  wb.w = CornerWords{};
  bits_at2(bits, pos, wb.w.a, wb.w.a1);
  if (wb.hy) bits_at2(bits, pos + dy, wb.w.b, wb.w.b1);
  if (wb.hz) bits_at2(bits, pos + dz, wb.w.c, wb.w.c1);
  if (wb.hy && wb.hz) bits_at2(bits, pos + dy + dz, wb.w.d, wb.w.d1);
  return wb;
}

__device__ __forceinline__ void locate_word(const GridSet& S, long long gw, int& si, unsigned& r,
                                            int& m) {
  si = S.count == 1 ? 0 : slot_of_rowword(S, gw);
  const GridSlot& sl = S.count == 1 ? S.one : S.slots[si];
  const unsigned lw = (unsigned)(gw - sl.rw0);
  r = lw / (unsigned)sl.g.wr;
  m = (int)(lw - r * (unsigned)sl.g.wr);
}

// Counts of one word from its eight corner words.
__device__ __forceinline__ uint32_t packed_counts(const CornerWords& w, bool hy, bool hz,
                                                  uint32_t pmask, uint32_t xmask,
                                                  const unsigned char* nf) {
  int v = __popc((w.a ^ w.a1) & xmask);
  if (hy) v += __popc((w.a ^ w.b) & pmask);
  if (hz) v += __popc((w.a ^ w.c) & pmask);
  int t = 0;
  if (hy && hz)
    for (uint32_t u = active_cells(w, xmask); u; u &= u - 1) t += nf[case_of(w, __ffs(u) - 1)];
  return ((uint32_t)t << 16) | (uint32_t)v;
}

// Four consecutive 32-bit windows of a row (x = 32m .. 32m+127) and their +x
// neighbours, from five word fetches.
__device__ __forceinline__ void row_windows4(const uint32_t* __restrict__ bits, long long pos,
                                             uint32_t (&a)[4], uint32_t (&a1)[4]) {
  const long long w = pos >> 5;
  const unsigned sh = (unsigned)(pos & 31);
  uint32_t x[5];
#pragma unroll
  for (int e = 0; e < 5; ++e) x[e] = __ldg(bits + w + e);
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    a[e] = __funnelshift_r(x[e], x[e + 1], sh);
    a1[e] = (a[e] >> 1) | (((x[e + 1] >> sh) & 1u) << 31);
  }
}

constexpr int kCountWords = 4;  // consecutive row words per thread in K2a

__global__ void __launch_bounds__(256) k_mc_count(GridSet S, const uint32_t* __restrict__ bits,
                                                  uint32_t* __restrict__ wc) {
  __shared__ unsigned char s_nf[256];  // NumFaces, indexed by divergent case ids
  s_nf[threadIdx.x] = (unsigned char)mc_num_tris(threadIdx.x);
  __syncthreads();
  const long long stride = (long long)gridDim.x * blockDim.x * kCountWords;
  for (long long g0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * kCountWords;
       g0 < S.rowwords; g0 += stride) {
    int si, m;
    unsigned r;
    locate_word(S, g0, si, r, m);
    const GridSlot& sl = S.count == 1 ? S.one : S.slots[si];
    const Grid& g = sl.g;
    uint32_t out[kCountWords] = {0, 0, 0, 0};
    const bool cells = g.nx >= 2 && g.ny >= 2 && g.nz >= 2;
    if (cells && m + kCountWords <= g.wr && g0 + kCountWords <= S.rowwords &&
        (S.count == 1 || g0 + kCountWords <= sl.rw0 + (long long)g.R * g.wr)) {
      // fast path: the four words lie in one row
      const uint32_t* gb = bits + sl.word0;
      const int j = (int)(r % (unsigned)g.ny), k = (int)(r / (unsigned)g.ny);
      const bool hy = j < g.ny - 1, hz = k < g.nz - 1;
      const long long dy = g.nx, dz = (long long)g.nx * g.ny;
      const long long pos = (long long)r * g.nx + 32ll * m;
      uint32_t a[4], a1[4], b[4] = {0, 0, 0, 0}, b1[4] = {0, 0, 0, 0}, c[4] = {0, 0, 0, 0},
               c1[4] = {0, 0, 0, 0}, d[4] = {0, 0, 0, 0}, d1[4] = {0, 0, 0, 0};
      row_windows4(gb, pos, a, a1);
      if (hy) row_windows4(gb, pos + dy, b, b1);
      if (hz) row_windows4(gb, pos + dz, c, c1);
      if (hy && hz) row_windows4(gb, pos + dy + dz, d, d1);
#pragma unroll
      for (int e = 0; e < kCountWords; ++e) {
        const CornerWords w{a[e], a1[e], b[e], b1[e], c[e], c1[e], d[e], d1[e]};
        out[e] = packed_counts(w, hy, hz, low_mask(g.nx - 32 * (m + e)),
                               low_mask(g.nx - 1 - 32 * (m + e)), s_nf);
      }
    } else {
      // words that straddle a row or grid end: one at a time
#pragma unroll
      for (int e = 0; e < kCountWords; ++e) {
        const long long gw = g0 + e;
        if (gw >= S.rowwords) break;
        int se, me;
        unsigned re;
        locate_word(S, gw, se, re, me);
        const GridSlot& sle = S.count == 1 ? S.one : S.slots[se];
        if (sle.g.nx >= 2 && sle.g.ny >= 2 && sle.g.nz >= 2) {
          const WordBits wb = load_word_bits(sle.g, bits + sle.word0, re, me);
          out[e] = packed_counts(wb.w, wb.hy, wb.hz, wb.pmask, wb.xmask, s_nf);
        }
      }
    }
    if (g0 + kCountWords <= S.rowwords) {
      *reinterpret_cast<uint4*>(wc + g0) = make_uint4(out[0], out[1], out[2], out[3]);
    } else {
#pragma unroll
      for (int e = 0; e < kCountWords; ++e)
        if (g0 + e < S.rowwords) wc[g0 + e] = out[e];
    }
  }
}

// Look-back by one warp over N independent status chains (status + c *
// stride + tile), same flag protocol and bounded waiting as warp_lookback.
template <int N>
__device__ __forceinline__ void warp_lookback_n(unsigned long long* st, int stride, int tile,
                                                const long long (&agg)[N], int* err,
                                                long long (&ex)[N]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int c = 0; c < N; ++c) ex[c] = 0;
  if (lane == 0) {
    const unsigned long long f = tile == 0 ? kFlagInc : kFlagAgg;
#pragma unroll
    for (int c = 0; c < N; ++c) st_release(st + c * stride + tile, f | (unsigned long long)agg[c]);
  }
  if (tile == 0) return;
  bool done[N];
#pragma unroll
  for (int c = 0; c < N; ++c) done[c] = false;
  int p = tile - 1, spins = 0;
  while (true) {
    bool all = true;
#pragma unroll
    for (int c = 0; c < N; ++c) all = all && done[c];
    if (all) break;
    const int idx = p - lane;
    unsigned long long w[N];
    int first[N];
    bool missing = false;
#pragma unroll
    for (int c = 0; c < N; ++c) {
      w[c] = (!done[c] && idx >= 0) ? ld_acquire(st + c * stride + idx) : kFlagInc;
      const unsigned inc = __ballot_sync(kFull, (w[c] >> 62) == 2u);
      const unsigned none = __ballot_sync(kFull, (w[c] >> 62) == 0u);
      first[c] = inc ? __ffs(inc) - 1 : 32;
      const unsigned need = first[c] >= 31 ? kFull : ((2u << first[c]) - 1u);
      missing = missing || (none & need);
    }
    if (missing) {
      if (++spins > kSpinLimit) {
        if (lane == 0) atomicOr(err, kErrTimeout);
        break;
      }
      if (spins > 16) __nanosleep(32);
      continue;
    }
#pragma unroll
    for (int c = 0; c < N; ++c) {
      long long v = (lane <= first[c] && idx >= 0) ? (long long)(w[c] & kValMask) : 0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
      if (!done[c]) ex[c] += v;
      done[c] = done[c] || first[c] < 32;
    }
    p -= 32;
  }
  if (lane == 0) {
#pragma unroll
    for (int c = 0; c < N; ++c)
      st_release(st + c * stride + tile, kFlagInc | (unsigned long long)(ex[c] + agg[c]));
  }
}

constexpr int kScanItems = 16;                 // words per thread
constexpr int kScanTile = 256 * kScanItems;    // words per tile

__global__ void __launch_bounds__(256) k_mc_scan(long long rowwords,
                                                 const uint32_t* __restrict__ wc,
                                                 uint32_t* __restrict__ wt,
                                                 uint32_t* __restrict__ wv,
                                                 uint32_t* __restrict__ act,
                                                 unsigned long long* __restrict__ status,
                                                 Info* __restrict__ info, int tiles) {
  __shared__ int s_tile;
  __shared__ uint32_t s_wt[8], s_wv[8], s_wa[8];
  __shared__ long long s_ex[3];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) s_tile = (int)atomicAdd(&info->ticket, 1u);
  __syncthreads();
  const int tile = s_tile;
  const long long w0 = (long long)tile * kScanTile + (long long)tid * kScanItems;
  uint32_t c[kScanItems];
  const bool full = w0 + kScanItems <= rowwords;
  if (full) {
#pragma unroll
    for (int q = 0; q < kScanItems / 4; ++q) {
      const uint4 u = __ldcs(reinterpret_cast<const uint4*>(wc + w0) + q);
      c[4 * q] = u.x;
      c[4 * q + 1] = u.y;
      c[4 * q + 2] = u.z;
      c[4 * q + 3] = u.w;
    }
  } else {
#pragma unroll
    for (int e = 0; e < kScanItems; ++e) c[e] = w0 + e < rowwords ? wc[w0 + e] : 0u;
  }
  uint32_t st = 0, sv = 0, sa = 0;
#pragma unroll
  for (int e = 0; e < kScanItems; ++e) {
    st += c[e] >> 16;
    sv += c[e] & 0xffffu;
    sa += c[e] ? 1u : 0u;
  }
  // block exclusive scan of (st, sv, sa), 32-bit (a tile holds < 2^20 of each)
  uint32_t it = st, iv = sv, ia = sa;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t ut = __shfl_up_sync(kFull, it, o), uv = __shfl_up_sync(kFull, iv, o),
                   ua = __shfl_up_sync(kFull, ia, o);
    if (lane >= o) { it += ut; iv += uv; ia += ua; }
  }
  if (lane == 31) { s_wt[warp] = it; s_wv[warp] = iv; s_wa[warp] = ia; }
  __syncthreads();
  uint32_t bt = 0, bv = 0, ba = 0, tt = 0, tv = 0, ta = 0;
#pragma unroll
  for (int w = 0; w < 8; ++w) {
    if (w < warp) { bt += s_wt[w]; bv += s_wv[w]; ba += s_wa[w]; }
    tt += s_wt[w];
    tv += s_wv[w];
    ta += s_wa[w];
  }
  if (warp == 0) {
    const long long agg[3] = {(long long)tt, (long long)tv, (long long)ta};
    long long ex[3];
    warp_lookback_n<3>(status, tiles, tile, agg, &info->error, ex);
    if (lane == 0) {
      s_ex[0] = ex[0];
      s_ex[1] = ex[1];
      s_ex[2] = ex[2];
    }
  }
  __syncthreads();
  // offsets are stored as uint32; a total above 2^31 - 1 is reported below
  uint32_t ot = (uint32_t)s_ex[0] + bt + it - st;
  uint32_t ov = (uint32_t)s_ex[1] + bv + iv - sv;
  long long oa = s_ex[2] + ba + ia - sa;
#pragma unroll
  for (int q = 0; q < kScanItems / 4; ++q) {
    uint32_t t4[4], v4[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const uint32_t ce = c[4 * q + e];
      t4[e] = ot;
      v4[e] = ov;
      ot += ce >> 16;
      ov += ce & 0xffffu;
      if (ce) act[oa++] = (uint32_t)(w0 + 4 * q + e);
    }
    if (full) {
      reinterpret_cast<uint4*>(wt + w0)[q] = make_uint4(t4[0], t4[1], t4[2], t4[3]);
      reinterpret_cast<uint4*>(wv + w0)[q] = make_uint4(v4[0], v4[1], v4[2], v4[3]);
    } else {
#pragma unroll
      for (int e = 0; e < 4; ++e)
        if (w0 + 4 * q + e < rowwords) {
          wt[w0 + 4 * q + e] = t4[e];
          wv[w0 + 4 * q + e] = v4[e];
        }
    }
  }
  if (tile == tiles - 1 && tid == 0) {
    const long long T = s_ex[0] + tt, V = s_ex[1] + tv;
    wt[rowwords] = (uint32_t)T;
    wv[rowwords] = (uint32_t)V;
    info->total_a = T;
    info->total_b = V;
    info->total_c = s_ex[2] + ta;
    if (T > 2147483647ll || V > 2147483647ll) atomicOr(&info->error, kErrOverflow);
  }
}

int mc_scan_tiles(long long rowwords) { return (int)((rowwords + kScanTile - 1) / kScanTile); }

void launch_mc_scan(const GridSet& S, const uint32_t* bits, uint32_t* wc, uint32_t* wt,
                    uint32_t* wv, uint32_t* act, unsigned long long* status, Info* info,
                    int num_sms, cudaStream_t s) {
  const long long want = (S.rowwords + 256 * kCountWords - 1) / (256 * kCountWords);
  const int b1 = resident_blocks(k_mc_count, 256, 0, num_sms, want);
  k_mc_count<<<b1, 256, 0, s>>>(S, bits, wc);
  launch_word_scan(S.rowwords, wc, wt, wv, act, status, info, s);
}

void launch_word_scan(long long rowwords, const uint32_t* wc, uint32_t* wt, uint32_t* wv,
                      uint32_t* act, unsigned long long* status, Info* info, cudaStream_t s) {
  const int tiles = mc_scan_tiles(rowwords);
  k_mc_scan<<<tiles, 256, 0, s>>>(rowwords, wc, wt, wv, act, status, info, tiles);
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

// Global offsets of word gw (gw may equal rowwords: then the totals).
__device__ __forceinline__ long long word_t(const WordOffsets& o, long long gw) {
  return (long long)__ldg(o.wt + gw);
}
__device__ __forceinline__ long long word_v(const WordOffsets& o, long long gw) {
  return (long long)__ldg(o.wv + gw);
}

// Crossing masks of one owner word plus its global vertex offset.
struct OwnerWord {
  uint32_t X, Y, Z;
  long long base;
};

__device__ __forceinline__ OwnerWord owner_word(const Grid& g, const uint32_t* bits,
                                                const WordOffsets& o, long long rw0, int jq,
                                                int kq, int wq) {
  const long long rq = (long long)kq * g.ny + jq;
  const long long pos = rq * g.nx + 32ll * wq;
  uint32_t a, a1;
  bits_at2(bits, pos, a, a1);
  const uint32_t pm = low_mask(g.nx - 32 * wq);
  OwnerWord ow;
  ow.X = (a ^ a1) & low_mask(g.nx - 1 - 32 * wq);
  ow.Y = jq < g.ny - 1 ? (a ^ bits_at(bits, pos + g.nx)) & pm : 0u;
  ow.Z = kq < g.nz - 1 ? (a ^ bits_at(bits, pos + (long long)g.nx * g.ny)) & pm : 0u;
  ow.base = word_v(o, rw0 + rq * g.wr + wq);
  return ow;
}

__device__ __forceinline__ long long owner_rank_id(const OwnerWord& o, int b, int axis) {
  const uint32_t lm = (1u << b) - 1u;
  long long id = o.base + __popc(o.X & lm) + __popc(o.Y & lm) + __popc(o.Z & lm);
  if (axis >= 1) id += (o.X >> b) & 1u;
  if (axis >= 2) id += (o.Y >> b) & 1u;
  return id;
}

// K3: two kernels over the A active words (A on the device, the words in
// the compacted list act).  k_mc_emit_vertices writes the merged
// vertices a word's points own; k_mc_emit_triangles writes its cells'
// triangles (and, unmerged, their corner vertices).  Splitting the roles
// keeps each thread's chain of dependent memory round trips short and each
// kernel's register count low.
__device__ __forceinline__ bool emit_guard(Info* info, long long tcap, long long vcap, bool merge,
                                           long long& A) {
  const long long T = info->total_a;
  const long long V = merge ? info->total_b : 3 * T;
  A = info->total_c;
  if (T > tcap || V > vcap || (info->error & (kErrOverflow | kErrTimeout))) {
    if (blockIdx.x == 0 && threadIdx.x == 0 && (T > tcap || V > vcap))
      atomicOr(&info->error, kErrCapacity);
    return false;
  }
  return true;
}

constexpr int kVertexBatch = 4;

__global__ void __launch_bounds__(256) k_mc_emit_vertices(GridSet S,
                                                          const uint32_t* __restrict__ bits,
                                                          WordOffsets o,
                                                          Info* __restrict__ info,
                                                          float* __restrict__ verts, long long vcap,
                                                          long long tcap,
                                                          int32_t* __restrict__ ra,
                                                          int32_t* __restrict__ rb,
                                                          float* __restrict__ rw) {
  long long A;
  if (!emit_guard(info, tcap, vcap, true, A)) return;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long it = (long long)blockIdx.x * blockDim.x + threadIdx.x; it < A; it += stride) {
    const long long gw = __ldg(o.act + it);
    const long long v0 = word_v(o, gw), v1 = word_v(o, gw + 1);
    if (v1 == v0) continue;
    int si, m;
    unsigned r;
    locate_word(S, gw, si, r, m);
    const GridSlot& sl = S.count == 1 ? S.one : S.slots[si];
    const Grid& g = sl.g;
    const uint32_t* gb = bits + sl.word0;
    const float* f = sl.field;
    const float iso = sl.iso;
    const int j = (int)(r % (unsigned)g.ny), k = (int)(r / (unsigned)g.ny);
    const long long dy = g.nx, dz = (long long)g.nx * g.ny;
    const long long pos = (long long)r * g.nx + 32ll * m;
    const bool hy = j < g.ny - 1, hz = k < g.nz - 1;
    const uint32_t pmask = low_mask(g.nx - 32 * m);
    uint32_t a, a1, b = 0, c = 0;
    bits_at2(gb, pos, a, a1);
    if (hy) b = bits_at(gb, pos + dy);
    if (hz) c = bits_at(gb, pos + dz);
    uint32_t ux = (a ^ a1) & low_mask(g.nx - 1 - 32 * m);
    uint32_t uy = hy ? (a ^ b) & pmask : 0u;
    uint32_t uz = hz ? (a ^ c) & pmask : 0u;
    // edges in (point, axis) order, in batches whose field loads are all
    // issued before any arithmetic
    long long vid = v0;
    while (ux | uy | uz) {
      int ei[kVertexBatch], ea[kVertexBatch];
      int nb = 0;
#pragma unroll
      for (int s2 = 0; s2 < kVertexBatch; ++s2) {
        const uint32_t u = ux | uy | uz;
        if (u == 0) break;
        const int q = __ffs(u) - 1;
        const uint32_t bit = 1u << q;
        int ax;
        if (ux & bit) { ax = 0; ux &= ~bit; }
        else if (uy & bit) { ax = 1; uy &= ~bit; }
        else { ax = 2; uz &= ~bit; }
        ei[nb] = 32 * m + q;
        ea[nb] = ax;
        ++nb;
      }
      float fa[kVertexBatch], fb[kVertexBatch];
#pragma unroll
      for (int s2 = 0; s2 < kVertexBatch; ++s2) {
        if (s2 < nb) {
          const long long pa = (long long)r * g.nx + ei[s2];
          fa[s2] = __ldg(f + pa);
          fb[s2] = __ldg(f + pa + (ea[s2] == 0 ? 1ll : (ea[s2] == 1 ? dy : dz)));
        }
      }
#pragma unroll
      for (int s2 = 0; s2 < kVertexBatch; ++s2) {
        if (s2 < nb) {
          const int i = ei[s2], ax = ea[s2];
          const float w = __fdiv_rn(__fsub_rn(iso, fa[s2]), __fsub_rn(fb[s2], fa[s2]));
          const float xa = coord(g.ox, g.sx, i, g.mx), ya = coord(g.oy, g.sy, j, g.my),
                      za = coord(g.oz, g.sz, k, g.mz);
          const float xb = ax == 0 ? coord(g.ox, g.sx, i + 1, g.mx) : xa;
          const float yb = ax == 1 ? coord(g.oy, g.sy, j + 1, g.my) : ya;
          const float zb = ax == 2 ? coord(g.oz, g.sz, k + 1, g.mz) : za;
          verts[3 * vid + 0] = lerp_rn(xa, xb, w);
          verts[3 * vid + 1] = lerp_rn(ya, yb, w);
          verts[3 * vid + 2] = lerp_rn(za, zb, w);
          const long long pa = (long long)r * g.nx + i;
          if (ra) ra[vid] = (int32_t)pa;
          if (rb) rb[vid] = (int32_t)(pa + (ax == 0 ? 1ll : (ax == 1 ? dy : dz)));
          if (rw) rw[vid] = w;
          ++vid;
        }
      }
    }
  }
}

template <bool MERGE>
__global__ void __launch_bounds__(256) k_mc_emit_triangles(GridSet S,
                                                           const uint32_t* __restrict__ bits,
                                                           WordOffsets o,
                                                           Info* __restrict__ info,
                                                           float* __restrict__ verts,
                                                           long long vcap,
                                                           int32_t* __restrict__ conn,
                                                           long long tcap,
                                                           int32_t* __restrict__ ra,
                                                           int32_t* __restrict__ rb,
                                                           float* __restrict__ rw) {
  // case and edge tables in shared memory: lanes index them divergently
  __shared__ uint64_t s_case[256];
  __shared__ unsigned char s_edge[12];
  s_case[threadIdx.x] = kMcCase[threadIdx.x];
  if (threadIdx.x < 12) s_edge[threadIdx.x] = kEdgeOwner[threadIdx.x];
  __syncthreads();
  long long A;
  if (!emit_guard(info, tcap, vcap, MERGE, A)) return;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long it = (long long)blockIdx.x * blockDim.x + threadIdx.x; it < A; it += stride) {
    const long long gw = __ldg(o.act + it);
    const long long t0 = word_t(o, gw), t1 = word_t(o, gw + 1);
    if (t1 == t0) continue;
    int si, m;
    unsigned r;
    locate_word(S, gw, si, r, m);
    const GridSlot& sl = S.count == 1 ? S.one : S.slots[si];
    const Grid& g = sl.g;
    const uint32_t* gb = bits + sl.word0;
    const int j = (int)(r % (unsigned)g.ny), k = (int)(r / (unsigned)g.ny);
    const long long dy = g.nx, dz = (long long)g.nx * g.ny;
    const long long pos = (long long)r * g.nx + 32ll * m;
    CornerWords w{};
    bits_at2(gb, pos, w.a, w.a1);
    bits_at2(gb, pos + dy, w.b, w.b1);
    bits_at2(gb, pos + dz, w.c, w.c1);
    bits_at2(gb, pos + dy + dz, w.d, w.d1);
    // first vertex of this grid in the concatenated output (0 for one grid)
    const long long vbase0 =
        S.count == 1 ? 0 : (MERGE ? word_v(o, sl.rw0) : 3 * word_t(o, sl.rw0));
    OwnerWord ow[4];
    if (MERGE) {
#pragma unroll
      for (int qi = 0; qi < 4; ++qi)
        ow[qi] = owner_word(g, gb, o, sl.rw0, j + (qi & 1), k + (qi >> 1), m);
    }
    long long tri = t0;
    for (uint32_t u = active_cells(w, low_mask(g.nx - 1 - 32 * m)); u; u &= u - 1) {
      const int q = __ffs(u) - 1;
      const int i = 32 * m + q;
      const uint64_t cw = s_case[case_of(w, q)];
      const int nt = (int)(cw >> 60);
      for (int tt = 0; tt < nt; ++tt, ++tri) {
#pragma unroll
        for (int corner = 0; corner < 3; ++corner) {
          const int e = mc_edge(cw, 3 * tt + corner);
          const int info_e = s_edge[e];
          const int di = info_e & 1, dj = (info_e >> 1) & 1, dk = (info_e >> 2) & 1;
          const int axis = info_e >> 3;
          if (MERGE) {
            const int ii = i + di;
            long long vid;
            if ((ii >> 5) == m) {
              vid = owner_rank_id(ow[dj + 2 * dk], ii & 31, axis);
            } else {  // the owner point is the first point of the next word
              const OwnerWord ox = owner_word(g, gb, o, sl.rw0, j + dj, k + dk, m + 1);
              vid = owner_rank_id(ox, 0, axis);
            }
            conn[3 * tri + corner] = (int32_t)(vid - vbase0);
          } else {
            const long long vid = 3 * tri + corner;
            conn[vid] = (int32_t)(vid - vbase0);
            emit_vertex(g, sl.field, sl.iso, i + di, j + dj, k + dk, axis, vid, verts, ra, rb, rw);
          }
        }
      }
    }
  }
}

void launch_mc_emit(const GridSet& S, bool merge, const uint32_t* bits, const WordOffsets& o,
                    Info* info, float* verts, long long vcap, int32_t* conn, long long tcap,
                    int32_t* ra, int32_t* rb, float* rw, int num_sms, cudaStream_t s) {
  // the active count lives on the device: one resident wave, grid-stride
  const long long want = (S.rowwords + 255) / 256;
  if (merge) {
    const int bv = resident_blocks(k_mc_emit_vertices, 256, 0, num_sms, want);
    k_mc_emit_vertices<<<bv, 256, 0, s>>>(S, bits, o, info, verts, vcap, tcap, ra, rb, rw);
    const int bt = resident_blocks(k_mc_emit_triangles<true>, 256, 0, num_sms, want);
    k_mc_emit_triangles<true><<<bt, 256, 0, s>>>(S, bits, o, info, verts, vcap, conn, tcap,
                                                 ra, rb, rw);
  } else {
    const int bt = resident_blocks(k_mc_emit_triangles<false>, 256, 0, num_sms, want);
    k_mc_emit_triangles<false><<<bt, 256, 0, s>>>(S, bits, o, info, verts, vcap, conn, tcap,
                                                  ra, rb, rw);
  }
}

// Per-grid offsets: goff[2g], goff[2g+1] = first triangle / merged vertex of
// grid g; goff[2G], goff[2G+1] = totals.
__global__ void k_grid_offsets(GridSet S, WordOffsets o, long long* __restrict__ goff) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= S.count; i += gridDim.x * blockDim.x) {
    const long long w = i < S.count ? load_slot(S, i).rw0 : S.rowwords;
    goff[2 * i] = word_t(o, w);
    goff[2 * i + 1] = word_v(o, w);
  }
}

void launch_grid_offsets(const GridSet& S, const WordOffsets& o, long long* goff,
                         cudaStream_t s) {
  k_grid_offsets<<<(S.count + 256) / 256, 256, 0, s>>>(S, o, goff);
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

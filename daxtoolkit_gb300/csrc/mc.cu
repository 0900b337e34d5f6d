// Marching cubes on the classification bit stream.
//
// Work is indexed by "row words": word m of point row r covers points
// i = 32m .. 32m+31 of that row (and the cells whose first point they are);
// row words are numbered r * wr + m, which is point order.
//
// K2a (k_mc_count): for every row word
//     T = triangles of its cells            = sum NumFaces[case(i)]
//     V = crossing edges its points own      = edges (p, p + e_axis) whose end
//         points classify differently, axis x < y < z
//     A = 1 if T or V is non-zero
//   plus per-tile totals; K2b (k_word_scan) turns them into exclusive
//   offsets per word and a compacted list of the active words
//   (reduce-then-scan: no block waits on another).  V counts exactly the
//   vertices of the merged output: a cell's triangle-table row references
//   exactly its sign-change edges, every grid edge belongs to a cell, and
//   the reference's merged order, ascending (first id, second id), is
//   ascending (owner point, axis) on a uniform grid -- point order, then
//   axis.  So the reference's Sort/Unique/LowerBounds
//   (dax/cont/DispatcherGenerateInterpolatedCells.h:276-291) becomes a rank:
//   offset of the owner word + popcount.
//
// K3 (k_mc_emit): warps take 32 active words at a time and deal their active
//   cells to the lanes; a cell writes its triangles at its word's T offset
//   plus the counts of the word's earlier active cells, a triangle corner's
//   vertex id is the V offset of the edge's owner word plus the edge's rank
//   inside it, and each merged vertex is written by the one cell that is its
//   owner point's own.  Field values are read only at crossing-edge end
//   points.
#include "common.cuh"
#include "kernels.cuh"
#include "mc_case.cuh"
#include "mc_words.cuh"

namespace daxgb {

// Edge e of the hexahedron (cellVertEdges, dax/worklet/MarchingCubes.h:131-135)
// as (owner offset di, dj, dk, axis) of its lower-id end point:
// bits 0..2 = di, dj, dk; bits 3..4 = axis (0 x, 1 y, 2 z).
__constant__ unsigned char kEdgeOwner[12] = {
    0 | (0 << 3), 1 | (1 << 3), 2 | (0 << 3), 0 | (1 << 3), 4 | (0 << 3), 5 | (1 << 3),
    6 | (0 << 3), 4 | (1 << 3), 0 | (2 << 3), 1 | (2 << 3), 3 | (2 << 3), 2 | (2 << 3)};

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
// K2: counts per row word, then the scan.

// Slot, point row and word index of global row word gw; keys: the slots'
// first row words staged in shared memory, or null; from >= 0: a slot that
// starts at or before gw (the search steps forward from it).
__device__ __forceinline__ void locate_word(const GridSet& S, long long gw, int& si, unsigned& r,
                                            int& m, const long long* keys = nullptr,
                                            int from = -1) {
  si = S.count == 1 ? 0
       : from >= 0  ? slot_after(S, keys, from, gw)
                    : (keys ? slot_search(keys, S.count, gw) : slot_of_rowword(S, gw));
  const GridSlot& sl = S.count == 1 ? S.one : S.slots[si];
  const unsigned lw = (unsigned)(gw - sl.rw0);
  r = split_word(sl.g, lw, m);
}

// Position of the n-th (0-based) set bit of u; n < popc(u).
__device__ __forceinline__ int nth_bit(uint32_t u, int n) {
  int p = 0;
#pragma unroll
  for (int step = 16; step > 0; step >>= 1)
    if (__popc(u & ((1u << (p + step)) - 1u)) <= n) p += step;
  return p;
}

constexpr int kCountWords = 4;  // consecutive row words per count group

// K2a: one 256-thread block per tile of kScanTile row words (grid-stride
// over tiles).  Thread t counts the 4-word groups t + 256 e (e = 0..3) of
// the tile, so a warp's groups are consecutive; the block then writes the
// tile's totals (triangles, crossing edges, active words) to
// tile_tot[0 / 1 / 2][tile] for the scan.
__global__ void __launch_bounds__(256) k_mc_count(GridSet S, const uint32_t* __restrict__ bits,
                                                  uint32_t* __restrict__ wc,
                                                  uint32_t* __restrict__ tile_tot, int tiles,
                                                  int tile_begin, int tile_end) {
  __shared__ unsigned char s_nf[256];  // NumFaces, indexed by divergent case ids
  __shared__ uint32_t s_red[24];
  __shared__ long long s_keys[kStagedSlots];
  s_nf[threadIdx.x] = (unsigned char)mc_num_tris(threadIdx.x);
  const long long* keys =
      stage_slot_keys(S, s_keys, [](const GridSlot& sl) { return sl.rw0; }) ? s_keys : nullptr;
  pdl_trigger();
  pdl_wait();  // the classification's bits
  for (int tile = tile_begin + blockIdx.x; tile < tile_end; tile += gridDim.x) {
    uint32_t st = 0, sv = 0, sa = 0;
#pragma unroll 1
    for (int e = 0; e < kScanItems / kCountWords; ++e) {
      const long long g0 = (long long)tile * kScanTile + (long long)(threadIdx.x + 256 * e) * kCountWords;
      // the slot of the warp's first group, searched once (the warp's
      // groups are consecutive); every lane steps forward from it
      const long long gw0 = g0 - (long long)(threadIdx.x & 31) * kCountWords;
      const int s0 = S.count == 1 || gw0 >= S.rowwords
                         ? 0
                         : (keys ? slot_search(keys, S.count, gw0) : slot_of_rowword(S, gw0));
      if (g0 >= S.rowwords) break;
      int si, m;
      unsigned r;
      locate_word(S, g0, si, r, m, keys, s0);
      const GridSlot& sl = S.count == 1 ? S.one : S.slots[si];
      const Grid& g = sl.g;
      uint32_t out[kCountWords] = {0, 0, 0, 0};
      const bool cells = g.nx >= 2 && g.ny >= 2 && g.nz >= 2;
      if (cells && m + kCountWords <= g.wr && g0 + kCountWords <= S.rowwords &&
          (S.count == 1 || g0 + kCountWords <= sl.rw0 + (long long)g.R * g.wr)) {
        // fast path: the four words lie in one row
        const uint32_t* gb = bits + sl.word0;
        int j, k;
  split_row(g, r, j, k);
        const bool hy = j < g.ny - 1, hz = k < g.nz - 1;
        const long long dy = g.nx, dz = (long long)g.nx * g.ny;
        const long long pos = (long long)r * g.nx + 32ll * m;
        uint32_t a[4], a1[4], b[4] = {0, 0, 0, 0}, b1[4] = {0, 0, 0, 0}, c[4] = {0, 0, 0, 0},
                 c1[4] = {0, 0, 0, 0}, d[4] = {0, 0, 0, 0}, d1[4] = {0, 0, 0, 0};
        row_windows4(gb, pos, a, a1);
        if (hy) row_windows4(gb, pos + dy, b, b1);
        if (hz) row_windows4(gb, pos + dz, c, c1);
        if (hy && hz) row_windows4(gb, pos + dy + dz, d, d1);
        // most groups lie wholly inside or outside: every corner window of
        // every word equal means no crossing edge and no active cell
        uint32_t diff = 0;
#pragma unroll
        for (int q = 0; q < kCountWords; ++q) {
          diff |= a[q] ^ a1[q];
          if (hy) diff |= (a[q] ^ b[q]) | (a[q] ^ b1[q]);
          if (hz) diff |= (a[q] ^ c[q]) | (a[q] ^ c1[q]);
          if (hy && hz) diff |= (a[q] ^ d[q]) | (a[q] ^ d1[q]);
        }
        if (diff) {
#pragma unroll
          for (int q = 0; q < kCountWords; ++q) {
            const CornerWords w{a[q], a1[q], b[q], b1[q], c[q], c1[q], d[q], d1[q]};
            out[q] = packed_counts(w, hy, hz, low_mask(g.nx - 32 * (m + q)),
                                   low_mask(g.nx - 1 - 32 * (m + q)), s_nf);
          }
        }
      } else {
        // words that straddle a row or grid end: one at a time
#pragma unroll
        for (int q = 0; q < kCountWords; ++q) {
          const long long gw = g0 + q;
          if (gw >= S.rowwords) break;
          int sq, mq;
          unsigned rq;
          locate_word(S, gw, sq, rq, mq, keys, si);
          const GridSlot& slq = S.count == 1 ? S.one : S.slots[sq];
          if (slq.g.nx >= 2 && slq.g.ny >= 2 && slq.g.nz >= 2) {
            const WordBits wb = load_word_bits(slq.g, bits + slq.word0, rq, mq);
            out[q] = packed_counts(wb.w, wb.hy, wb.hz, wb.pmask, wb.xmask, s_nf);
          }
        }
      }
      if (g0 + kCountWords <= S.rowwords) {
        *reinterpret_cast<uint4*>(wc + g0) = make_uint4(out[0], out[1], out[2], out[3]);
      } else {
#pragma unroll
        for (int q = 0; q < kCountWords; ++q)
          if (g0 + q < S.rowwords) wc[g0 + q] = out[q];
      }
#pragma unroll
      for (int q = 0; q < kCountWords; ++q) {
        st += out[q] >> 16;
        sv += out[q] & 0xffffu;
        sa += out[q] ? 1u : 0u;
      }
    }
    block_sum3(st, sv, sa, s_red);
    if (threadIdx.x == 0) {
      tile_tot[tile] = st;
      tile_tot[tiles + tile] = sv;
      tile_tot[2 * tiles + tile] = sa;
    }
  }
}

// K2b: scan of the packed per-word counts wc = (a << 16) | b with the tile
// totals tile_tot[0 / 1 / 2][tiles] (sums of a, of b and of non-zero words)
// written by the count pass: reduce-then-scan, so no block waits on
// another.  Block `tile` sums the totals of the tiles before it, scans its
// own kScanTile words and writes the exclusive offsets wt (a) and wv (b),
// the compacted list act of its non-zero words, and -- the last tile -- the
// totals, the end entries wt[rowwords] / wv[rowwords] and the error word.
//
// PIPE (the pipelined marching cubes): blocks cover tiles tile_begin + b of
// one slab, later slabs run later; each block flags an offset above 2^31 - 1
// itself (emits of earlier slabs run before the last tile), the error word
// and emit counters were cleared by the first slab's classification, and
// for every boundary word B.e[i] in its words a thread records the number
// of active words before it in slab_act[i] (the last tile: slab_act[B.n] =
// all active words).
template <bool PIPE>
__global__ void __launch_bounds__(256) k_word_scan(long long rowwords,
                                                   const uint32_t* __restrict__ wc,
                                                   const uint32_t* __restrict__ tile_tot,
                                                   int tiles, uint32_t* __restrict__ wt,
                                                   uint32_t* __restrict__ wv,
                                                   uint32_t* __restrict__ act,
                                                   Info* __restrict__ info, int tile_begin,
                                                   SlabBounds B, uint32_t* __restrict__ slab_act,
                                                   const uint32_t* __restrict__ abort) {
  __shared__ uint32_t s_red[24];
  __shared__ unsigned long long s_pre[3 * 8];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int tile = tile_begin + blockIdx.x;
  pdl_trigger();
  pdl_wait();  // the count pass's per-word counts and tile totals
  // the tile's counts first: their loads are in flight while the prefix over
  // the earlier tiles is summed
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
  // exclusive prefix over the tiles before this one (64-bit: totals may pass
  // 2^32); unrolled so that a thread's loads are issued together
  unsigned long long pt = 0, pv = 0, pa = 0;
#pragma unroll 4
  for (int x = tid; x < tile; x += 256) {
    pt += __ldg(tile_tot + x);
    pv += __ldg(tile_tot + tiles + x);
    pa += __ldg(tile_tot + 2 * tiles + x);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    pt += __shfl_xor_sync(kFull, pt, o);
    pv += __shfl_xor_sync(kFull, pv, o);
    pa += __shfl_xor_sync(kFull, pa, o);
  }
  if (lane == 0) {
    s_pre[warp] = pt;
    s_pre[8 + warp] = pv;
    s_pre[16 + warp] = pa;
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
  if (lane == 31) { s_red[warp] = it; s_red[8 + warp] = iv; s_red[16 + warp] = ia; }
  __syncthreads();
  uint32_t bt = 0, bv = 0, ba = 0, tt = 0, tv = 0, ta = 0;
  unsigned long long et = 0, ev = 0, ea = 0;
#pragma unroll
  for (int w = 0; w < 8; ++w) {
    if (w < warp) { bt += s_red[w]; bv += s_red[8 + w]; ba += s_red[16 + w]; }
    tt += s_red[w];
    tv += s_red[8 + w];
    ta += s_red[16 + w];
    et += s_pre[w];
    ev += s_pre[8 + w];
    ea += s_pre[16 + w];
  }
  // offsets are stored as uint32; a total above 2^31 - 1 is reported below
  uint32_t ot = (uint32_t)et + bt + it - st;
  uint32_t ov = (uint32_t)ev + bv + iv - sv;
  long long oa = (long long)ea + ba + ia - sa;
  if (PIPE) {
    if (tid == 0 && (et + tt > 2147483647ull || ev + tv > 2147483647ull))
      atomicOr(&info->error, kErrOverflow);
    for (int i = 0; i < B.n; ++i) {
      const long long d = B.e[i] - w0;
      if (d >= 0 && d < kScanItems) {
        long long p = oa;
#pragma unroll
        for (int e = 0; e < kScanItems; ++e)
          if (e < d && c[e]) ++p;
        slab_act[i] = (uint32_t)p;
      }
    }
  }
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
    const long long T = (long long)(et + tt), V = (long long)(ev + tv);
    wt[rowwords] = (uint32_t)T;
    wv[rowwords] = (uint32_t)V;
    info->total_a = T;
    info->total_b = V;
    info->total_c = (long long)(ea + ta);
    if (PIPE) {
      slab_act[B.n] = (uint32_t)(ea + ta);
    } else {
      info->error = ((T > 2147483647ll || V > 2147483647ll) ? kErrOverflow : 0) |
                    ((abort && *(volatile const uint32_t*)abort) ? kErrTimeout : 0) |
                    (*(volatile int*)&info->aborted ? kErrTimeout : 0);
      info->ticket = 0;
      info->done = 0;
    }
  }
}

int word_scan_tiles(long long rowwords) {
  return (int)((rowwords + kScanTile - 1) / kScanTile);
}

void launch_word_scan(long long rowwords, const uint32_t* wc, const uint32_t* tile_tot,
                      uint32_t* wt, uint32_t* wv, uint32_t* act, Info* info, cudaStream_t s,
                      const uint32_t* abort) {
  const int tiles = word_scan_tiles(rowwords);
  launch_pdl(k_word_scan<false>, (unsigned)tiles, 256u, 0, s, rowwords, wc, tile_tot, tiles, wt, wv,
             act, info, 0, SlabBounds{}, (uint32_t*)nullptr, abort);
}

// K2a for grid sets: the same counts, with the triangles of the active
// cells dealt across the warp.  Batches of small grids have short rows (the
// 4-word groups straddle rows) and, with noisy fields, many active cells,
// so a lane looping over its own words' active cells would hold its warp
// for the busiest lane.  Here a lane gathers its 4 words' corner bits and
// counts their crossing edges; the warp then deals the active cells of its
// 128 words to the lanes, a cell per lane per round: each reads its word's
// corner bits from the warp's staging area and adds NumFaces of its case to
// the word's total there.  (For one large grid the per-lane loop is faster:
// its surface is sparse, and this kernel's staging costs occupancy.)
__global__ void __launch_bounds__(256) k_mc_count_dealt(GridSet S, const uint32_t* __restrict__ bits,
                                                        uint32_t* __restrict__ wc,
                                                        uint32_t* __restrict__ tile_tot, int tiles) {
  constexpr int kSlots = 32 * kCountWords;  // words per warp step
  __shared__ unsigned char s_nf[256];        // NumFaces
  __shared__ uint32_t s_red[24];
  __shared__ long long s_keys[kStagedSlots];
  __shared__ uint32_t s_win[8][8 * kSlots];  // corner word f of slot (4 lane + q) at f * kSlots + slot
  __shared__ uint32_t s_tri[8][kSlots];      // triangles of slot
  s_nf[threadIdx.x] = (unsigned char)mc_num_tris(threadIdx.x);
  const long long* keys =
      stage_slot_keys(S, s_keys, [](const GridSlot& sl) { return sl.rw0; }) ? s_keys : nullptr;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  uint32_t* const win = s_win[wib];
  uint32_t* const tri = s_tri[wib];
  for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    uint32_t st = 0, sv = 0, sa = 0;
#pragma unroll 1
    for (int e = 0; e < kScanItems / kCountWords; ++e) {
      const long long gw0 = (long long)tile * kScanTile + (long long)(256 * e + 32 * wib) * kCountWords;
      if (gw0 >= S.rowwords) break;  // uniform across the warp
      const long long g0 = gw0 + (long long)lane * kCountWords;
      const int s0 = keys ? slot_search(keys, S.count, gw0) : slot_of_rowword(S, gw0);
      // ---- lane = 4 words: corner bits, crossing edges, active cells ------
      CornerWords w[kCountWords];
      uint32_t v[kCountWords], am[kCountWords], t[kCountWords] = {0, 0, 0, 0};
#pragma unroll
      for (int q = 0; q < kCountWords; ++q) {
        w[q] = CornerWords{};
        v[q] = am[q] = 0u;
        const long long gw = g0 + q;
        if (gw < S.rowwords) {
          int sq, mq;
          unsigned rq;
          locate_word(S, gw, sq, rq, mq, keys, s0);
          const GridSlot& slq = S.slots[sq];
          if (slq.g.nx >= 2 && slq.g.ny >= 2 && slq.g.nz >= 2) {
            const WordBits wb = load_word_bits(slq.g, bits + slq.word0, rq, mq);
            w[q] = wb.w;
            int vv = __popc((wb.w.a ^ wb.w.a1) & wb.xmask);
            if (wb.hy) vv += __popc((wb.w.a ^ wb.w.b) & wb.pmask);
            if (wb.hz) vv += __popc((wb.w.a ^ wb.w.c) & wb.pmask);
            v[q] = (uint32_t)vv;
            am[q] = (wb.hy && wb.hz) ? active_cells(wb.w, wb.xmask) : 0u;
          }
        }
      }
      // ---- lane = active cell -------------------------------------------
      const int cnt = __popc(am[0]) + __popc(am[1]) + __popc(am[2]) + __popc(am[3]);
      int pre = cnt;  // inclusive scan of the lanes' active cells
#pragma unroll
      for (int dd = 1; dd < 32; dd <<= 1) {
        const int y = __shfl_up_sync(kFull, pre, dd);
        if (lane >= dd) pre += y;
      }
      const int total = __shfl_sync(kFull, pre, 31);
      pre -= cnt;
      if (total > 0) {
#pragma unroll
        for (int q = 0; q < kCountWords; ++q) {
          const int slot = kCountWords * lane + q;
          tri[slot] = 0u;
          if (am[q]) {
            win[0 * kSlots + slot] = w[q].a;
            win[1 * kSlots + slot] = w[q].a1;
            win[2 * kSlots + slot] = w[q].b;
            win[3 * kSlots + slot] = w[q].b1;
            win[4 * kSlots + slot] = w[q].c;
            win[5 * kSlots + slot] = w[q].c1;
            win[6 * kSlots + slot] = w[q].d;
            win[7 * kSlots + slot] = w[q].d1;
          }
        }
        __syncwarp();
        for (int t0 = 0; t0 < total; t0 += 32) {
          const int tt = t0 + lane;
          int s = 0;  // the lane holding cell tt: the last s with pre[s] <= tt
#pragma unroll
          for (int step = 16; step > 0; step >>= 1) {
            const int ps = __shfl_sync(kFull, pre, s + step);
            if (ps <= tt) s += step;
          }
          int rnk = tt - __shfl_sync(kFull, pre, s);
          const uint32_t m0 = __shfl_sync(kFull, am[0], s), m1 = __shfl_sync(kFull, am[1], s),
                         m2 = __shfl_sync(kFull, am[2], s), m3 = __shfl_sync(kFull, am[3], s);
          if (tt < total) {
            // the word q of lane s holding the cell, and the cell's rank in it
            int q = 0;
            uint32_t mq = m0;
            const int c0 = __popc(m0), c01 = c0 + __popc(m1), c012 = c01 + __popc(m2);
            if (rnk >= c012) {
              q = 3;
              mq = m3;
              rnk -= c012;
            } else if (rnk >= c01) {
              q = 2;
              mq = m2;
              rnk -= c01;
            } else if (rnk >= c0) {
              q = 1;
              mq = m1;
              rnk -= c0;
            }
            const int slot = kCountWords * s + q;
            const CornerWords cw{win[0 * kSlots + slot], win[1 * kSlots + slot],
                                 win[2 * kSlots + slot], win[3 * kSlots + slot],
                                 win[4 * kSlots + slot], win[5 * kSlots + slot],
                                 win[6 * kSlots + slot], win[7 * kSlots + slot]};
            atomicAdd(&tri[slot], (uint32_t)s_nf[case_of(cw, nth_bit(mq, rnk))]);
          }
        }
        __syncwarp();
#pragma unroll
        for (int q = 0; q < kCountWords; ++q) t[q] = tri[kCountWords * lane + q];
        __syncwarp();
      }
#pragma unroll
      for (int q = 0; q < kCountWords; ++q) {
        const uint32_t out = (t[q] << 16) | v[q];
        if (g0 + q < S.rowwords) wc[g0 + q] = out;
        st += t[q];
        sv += v[q];
        sa += out ? 1u : 0u;
      }
    }
    block_sum3(st, sv, sa, s_red);
    if (threadIdx.x == 0) {
      tile_tot[tile] = st;
      tile_tot[tiles + tile] = sv;
      tile_tot[2 * tiles + tile] = sa;
    }
  }
}

void launch_mc_scan(const GridSet& S, const uint32_t* bits, const WordOffsets& o, Info* info,
                    int num_sms, cudaStream_t s, int dealt) {
  const int tiles = word_scan_tiles(S.rowwords);
  // the dealt pass reads the device slot table, which only grid sets have
  if (S.count == 1 && launch_mc_count_staged(S.one.g, bits, bit_words(S.one.g.P), o, info, num_sms, s)) {
    // one grid: each tile's bits staged in shared memory
  } else if (S.count > 1 && dealt != 0) {
    const int b1 = resident_blocks(k_mc_count_dealt, 256, 0, num_sms, tiles, kPassCount);
    k_mc_count_dealt<<<b1, 256, 0, s>>>(S, bits, o.wc, o.tile, tiles);
  } else {
    const int b1 = resident_blocks(k_mc_count, 256, 0, num_sms, tiles, kPassCount);
    k_mc_count<<<b1, 256, 0, s>>>(S, bits, o.wc, o.tile, tiles, 0, tiles);
  }
  launch_word_scan(S.rowwords, o.wc, o.tile, o.wt, o.wv, o.act, info, s);
}

// One slab of the pipelined marching cubes (one grid): the counts of tiles
// [tile_begin, tile_end), then their scan.
void launch_mc_scan_slab(const GridSet& S, const uint32_t* bits, const WordOffsets& o, Info* info,
                         int tile_begin, int tile_end, const SlabBounds& B, uint32_t* slab_act,
                         int pass, int num_sms, cudaStream_t s, cudaEvent_t after_count) {
  const int tiles = word_scan_tiles(S.rowwords);
  const int n = tile_end - tile_begin;
  const int b1 = resident_blocks(k_mc_count, 256, 0, num_sms, n, pass);
  k_mc_count<<<b1, 256, 0, s>>>(S, bits, o.wc, o.tile, tiles, tile_begin, tile_end);
  if (after_count) cudaEventRecord(after_count, s);
  k_word_scan<true><<<n, 256, 0, s>>>(S.rowwords, o.wc, o.tile, tiles, o.wt, o.wv, o.act, info,
                                      tile_begin, B, slab_act, nullptr);
}

// ---------------------------------------------------------------------------
// K3: emit.

// Vertex on the edge owned by point (i, j, k) along `axis`:
// weight = (iso - f[A]) / (f[B] - f[A]) (dax/worklet/MarchingCubes.h:160-161),
// position = Lerp(coord A, coord B, weight) per component
// (dax/exec/internal/kernel/GenerateWorklets.h:79-92).  A slot without a
// field is a slice: the end values are dot(N, coord - O), the same values
// Slice.h:137 computes per cell vertex.
__device__ __forceinline__ void emit_vertex(const GridSlot& sl, int i, int j, int k, int axis,
                                            long long vid, float* __restrict__ verts,
                                            int32_t* __restrict__ ra, int32_t* __restrict__ rb,
                                            float* __restrict__ rw) {
  const Grid& g = sl.g;
  const long long pa = ((long long)k * g.ny + j) * g.nx + i;
  const long long pb = pa + (axis == 0 ? 1ll : (axis == 1 ? (long long)g.nx : (long long)g.nx * g.ny));
  const float fa = slot_value(sl, pa, i, j, k);
  const float fb = slot_value(sl, pb, i + (axis == 0), j + (axis == 1), k + (axis == 2));
  const float w = __fdiv_rn(__fsub_rn(sl.iso, fa), __fsub_rn(fb, fa));
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

// Capacity and error check before any output is written; A = active words.
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

// The crossing edges owned by point (i, j, k) (own: bit 0 = x, 1 = y, 2 = z),
// written as vertices vid0, vid0 + 1, ... in axis order -- the merged
// order.  The point's value is loaded once and all end values are loaded
// before any is used; each vertex is the one emit_vertex would write.
__device__ __forceinline__ void emit_point_vertices(const GridSlot& sl, int i, int j, int k,
                                                    uint32_t own, long long vid0,
                                                    float* __restrict__ verts,
                                                    int32_t* __restrict__ ra,
                                                    int32_t* __restrict__ rb,
                                                    float* __restrict__ rw) {
  const Grid& g = sl.g;
  const long long pa = ((long long)k * g.ny + j) * g.nx + i;
  const long long dy = g.nx, dz = (long long)g.nx * g.ny;
  const float fa = slot_value(sl, pa, i, j, k);
  float fb[3];
  fb[0] = (own & 1u) ? slot_value(sl, pa + 1, i + 1, j, k) : 0.0f;
  fb[1] = (own & 2u) ? slot_value(sl, pa + dy, i, j + 1, k) : 0.0f;
  fb[2] = (own & 4u) ? slot_value(sl, pa + dz, i, j, k + 1) : 0.0f;
  const float xa = coord(g.ox, g.sx, i, g.mx), ya = coord(g.oy, g.sy, j, g.my),
              za = coord(g.oz, g.sz, k, g.mz);
  long long vid = vid0;
#pragma unroll
  for (int axis = 0; axis < 3; ++axis) {
    if (!((own >> axis) & 1u)) continue;
    const float w = __fdiv_rn(__fsub_rn(sl.iso, fa), __fsub_rn(fb[axis], fa));
    const float xb = axis == 0 ? coord(g.ox, g.sx, i + 1, g.mx) : xa;
    const float yb = axis == 1 ? coord(g.oy, g.sy, j + 1, g.my) : ya;
    const float zb = axis == 2 ? coord(g.oz, g.sz, k + 1, g.mz) : za;
    verts[3 * vid + 0] = lerp_rn(xa, xb, w);
    verts[3 * vid + 1] = lerp_rn(ya, yb, w);
    verts[3 * vid + 2] = lerp_rn(za, zb, w);
    if (ra) ra[vid] = (int32_t)pa;
    if (rb) rb[vid] = (int32_t)(pa + (axis == 0 ? 1ll : (axis == 1 ? dy : dz)));
    if (rw) rw[vid] = w;
    ++vid;
  }
}

// Bit of the flat bit stream at position p.
__device__ __forceinline__ uint32_t bit_at(const uint32_t* __restrict__ bits, long long p) {
  return (__ldg(bits + (p >> 5)) >> (unsigned)(p & 31)) & 1u;
}

// x (bit 0) and y (bit 1) crossing bits of point i of row (jq, kq).
__device__ __forceinline__ uint32_t point_xy_bits(const Grid& g, const uint32_t* bits, int jq,
                                                  int kq, int i) {
  const long long pos = ((long long)kq * g.ny + jq) * g.nx + i;
  const uint32_t a = bit_at(bits, pos);
  uint32_t r = (i + 1 < g.nx) ? (a ^ bit_at(bits, pos + 1)) : 0u;
  if (jq < g.ny - 1) r |= (a ^ bit_at(bits, pos + g.nx)) << 1;
  return r;
}

// One warp's staging of up to 32 active words, structure-of-arrays so that
// lane L writes column L without bank conflicts: per word the corner bit
// words, the crossing masks and first vertex ids of the four owner rows
// q = dj + 2 dk (rows (j + dj, k + dk) at word m), the active-cell mask, the
// global row word, the grid slot, the word's first point (i0 = 32 m, j, k),
// and -- when the word's last cell is active -- the x and y crossing bits of
// point 32m + 32 of owner rows 0..2, which that cell's +x corners need.
enum EmitField {
  kFWin = 0,     // 8: a, a1, b, b1, c, c1, d, d1
  kFOx = 8,      // 4
  kFOy = 12,     // 4
  kFOz = 16,     // 4
  kFOv = 20,     // 4
  kFAm = 24,
  kFWord = 25,
  kFSlot = 26,
  kFI0 = 27,
  kFJ = 28,
  kFK = 29,
  kFNx = 30,     // point 32m + 32 of owner row q <= 2: x bit at 2q, y bit at 2q + 1
  kFields = 31
};
constexpr int kEmitWarps = 8;

__device__ __forceinline__ uint32_t window(const uint32_t* st, int f, int s) { return st[f * 32 + s]; }

// Largest s in [0, 31] with pre[s] <= x, for a non-decreasing pre[0..31].
__device__ __forceinline__ int search32(const int* pre, int x) {
  int s = 0;
#pragma unroll
  for (int step = 16; step > 0; step >>= 1)
    if (pre[s + step] <= x) s += step;
  return s;
}

// Exclusive warp scan of v; *total receives the warp's sum.
__device__ __forceinline__ int warp_exclusive(int v, int lane, int* total) {
  int x = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int y = __shfl_up_sync(kFull, x, d);
    if (lane >= d) x += y;
  }
  *total = __shfl_sync(kFull, x, 31);
  return x - v;
}

// Merged vertex ids of the 12 edges of cell q of staged word s, into
// ids[e * 32 + lane] (meaningful for the cell's crossing edges only).  Edge
// e belongs to owner point (q + di) of owner row dj + 2 dk (kEdgeOwner); its
// id is the row word's first id, plus the edges its earlier points own,
// plus its own x (and y) edge before a y (z) edge.  Point q + 1 = 32 is the
// next word's first point: its first id is this word's first id plus all the
// word's edges, since ids are dense in point order.
__device__ __forceinline__ void cell_edge_ids(const uint32_t* st, int s, int q, uint32_t* ids,
                                              int lane) {
  const uint32_t lm = (1u << q) - 1u;
  uint32_t R[4], x[4], y[4], z[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const uint32_t X = window(st, kFOx + r, s), Y = window(st, kFOy + r, s),
                   Z = window(st, kFOz + r, s);
    R[r] = window(st, kFOv + r, s) + __popc(X & lm) + __popc(Y & lm) + __popc(Z & lm);
    x[r] = (X >> q) & 1u;
    y[r] = (Y >> q) & 1u;
    z[r] = (Z >> q) & 1u;
  }
  uint32_t x1[3], y1[3];
  if (q < 31) {
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      x1[r] = (window(st, kFOx + r, s) >> (q + 1)) & 1u;
      y1[r] = (window(st, kFOy + r, s) >> (q + 1)) & 1u;
    }
  } else {
    const uint32_t nb = window(st, kFNx, s);
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      x1[r] = (nb >> (2 * r)) & 1u;
      y1[r] = (nb >> (2 * r + 1)) & 1u;
    }
  }
  const uint32_t R1_0 = R[0] + x[0] + y[0] + z[0], R1_1 = R[1] + x[1] + y[1] + z[1],
                 R1_2 = R[2] + x[2] + y[2] + z[2];
  ids[0 * 32 + lane] = R[0];                          // row 0, q,     x
  ids[1 * 32 + lane] = R1_0 + x1[0];                  // row 0, q + 1, y
  ids[2 * 32 + lane] = R[1];                          // row 1, q,     x
  ids[3 * 32 + lane] = R[0] + x[0];                   // row 0, q,     y
  ids[4 * 32 + lane] = R[2];                          // row 2, q,     x
  ids[5 * 32 + lane] = R1_2 + x1[2];                  // row 2, q + 1, y
  ids[6 * 32 + lane] = R[3];                          // row 3, q,     x
  ids[7 * 32 + lane] = R[2] + x[2];                   // row 2, q,     y
  ids[8 * 32 + lane] = R[0] + x[0] + y[0];            // row 0, q,     z
  ids[9 * 32 + lane] = R1_0 + x1[0] + y1[0];          // row 0, q + 1, z
  ids[10 * 32 + lane] = R1_1 + x1[1] + y1[1];         // row 1, q + 1, z
  ids[11 * 32 + lane] = R[1] + x[1] + y[1];           // row 1, q,     z
}

// A warp takes `batch` (1..32) active words at a time from the counter
// *ticket; the last block to finish resets *ticket and *done.  Smaller
// batches shorten each warp's chain of dependent steps (the kernel's
// duration when its words are few), larger ones share each step over more
// words.
// range_end < 0: every active word, after a complete count pass.
// range_end >= 0 (one slab of the pipelined marching cubes, one grid): the
// active words act[slab_act[0] .. slab_act[1]), which lie below row word
// range_end; the capacity check uses the offsets at range_end, so a slab
// writes nothing unless everything up to its end fits.
template <bool MERGE>
__global__ void __launch_bounds__(kEmitWarps * 32, 4) k_mc_emit(GridSet S,
                                                            const uint32_t* __restrict__ bits,
                                                            WordOffsets o,
                                                            Info* __restrict__ info,
                                                            float* __restrict__ verts,
                                                            long long vcap,
                                                            int32_t* __restrict__ conn,
                                                            long long tcap,
                                                            int32_t* __restrict__ ra,
                                                            int32_t* __restrict__ rb,
                                                            float* __restrict__ rw,
                                                            long long range_end,
                                                            const uint32_t* __restrict__ slab_act,
                                                            unsigned* __restrict__ ticket,
                                                            unsigned* __restrict__ done,
                                                            int batch) {
  // case and edge tables in shared memory: lanes index them divergently
  __shared__ uint64_t s_case[256];
  __shared__ unsigned char s_edge[12];
  __shared__ uint32_t s_stage[kEmitWarps][kFields * 32];
  __shared__ int s_pre[kEmitWarps][33];    // active cells before word s
  __shared__ int s_ppre[kEmitWarps][33];   // owner points (points with owned edges) before word s
  __shared__ uint32_t s_ids[kEmitWarps][MERGE ? 12 * 32 : 1];  // a cell's 12 edge ids per lane
  __shared__ long long s_keys[kStagedSlots];
  s_case[threadIdx.x] = kMcCase[threadIdx.x];
  if (threadIdx.x < 12) s_edge[threadIdx.x] = kEdgeOwner[threadIdx.x];
  const long long* keys =
      stage_slot_keys(S, s_keys, [](const GridSlot& sl) { return sl.rw0; }) ? s_keys : nullptr;
  pdl_wait();  // the scan's offsets and totals
  long long A0 = 0, A;
  if (range_end < 0) {
    if (!emit_guard(info, tcap, vcap, MERGE, A)) return;
  } else {
    const long long T = word_t(o, range_end);
    const long long V = MERGE ? word_v(o, range_end) : 3 * T;
    if (T > tcap || V > vcap || (info->error & (kErrOverflow | kErrTimeout))) {
      if (blockIdx.x == 0 && threadIdx.x == 0 && (T > tcap || V > vcap))
        atomicOr(&info->error, kErrCapacity);
      return;
    }
    A0 = __ldg(slab_act);
    A = __ldg(slab_act + 1);
  }
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  uint32_t* st = s_stage[wib];
  int* pre = s_pre[wib];
  int* ppre = s_ppre[wib];
  uint32_t* ids = s_ids[wib];
  while (true) {
    // the next batch of active words, taken dynamically (batches differ
    // widely in cost)
    long long a0 = 0;
    if (lane == 0) a0 = A0 + (long long)batch * atomicAdd(ticket, 1u);
    a0 = __shfl_sync(kFull, a0, 0);
    if (a0 >= A) break;
    // ---- lane = word: gather the word's bits, masks and offsets ----------
    uint32_t am = 0, t0 = 0;
    int np = 0;
    if (lane < batch && a0 + lane < A) {
      const uint32_t gw = __ldg(o.act + a0 + lane);
      t0 = __ldg(o.wt + gw);
      int si, m;
      unsigned r;
      locate_word(S, gw, si, r, m, keys);
      const GridSlot& sl = S.count == 1 ? S.one : S.slots[si];
      const Grid& g = sl.g;
      int j, k;
      split_row(g, r, j, k);
      const bool hy = j < g.ny - 1, hz = k < g.nz - 1;
      const uint32_t* gb = bits + sl.word0;
      const long long dy = g.nx, dz = (long long)g.nx * g.ny;
      const long long pos = (long long)r * g.nx + 32ll * m;
      const uint32_t xmask = low_mask(g.nx - 1 - 32 * m), pmask = low_mask(g.nx - 32 * m);
      CornerWords w{};
      bits_at2(gb, pos, w.a, w.a1);
      if (hy) bits_at2(gb, pos + dy, w.b, w.b1);
      if (hz) bits_at2(gb, pos + dz, w.c, w.c1);
      st[kFWord * 32 + lane] = gw;
      st[kFSlot * 32 + lane] = (uint32_t)si;
      st[kFI0 * 32 + lane] = (uint32_t)(32 * m);
      st[kFJ * 32 + lane] = (uint32_t)j;
      st[kFK * 32 + lane] = (uint32_t)k;
      if (MERGE) {  // the crossing edges the word's own points own
        const uint32_t X = (w.a ^ w.a1) & xmask;
        const uint32_t Y = hy ? (w.a ^ w.b) & pmask : 0u;
        const uint32_t Z = hz ? (w.a ^ w.c) & pmask : 0u;
        st[(kFOx + 0) * 32 + lane] = X;
        st[(kFOy + 0) * 32 + lane] = Y;
        st[(kFOz + 0) * 32 + lane] = Z;
        st[(kFOv + 0) * 32 + lane] = __ldg(o.wv + gw);
        np = __popc(X | Y | Z);
      }
      if (hy && hz) {  // the row has cells
        bits_at2(gb, pos + dy + dz, w.d, w.d1);
        am = active_cells(w, xmask);
        st[(kFWin + 0) * 32 + lane] = w.a;
        st[(kFWin + 1) * 32 + lane] = w.a1;
        st[(kFWin + 2) * 32 + lane] = w.b;
        st[(kFWin + 3) * 32 + lane] = w.b1;
        st[(kFWin + 4) * 32 + lane] = w.c;
        st[(kFWin + 5) * 32 + lane] = w.c1;
        st[(kFWin + 6) * 32 + lane] = w.d;
        st[(kFWin + 7) * 32 + lane] = w.d1;
        if (MERGE && am) {
          // owner rows (j+1, k), (j, k+1), (j+1, k+1) of the cells' far corners
          const bool y2 = j + 1 < g.ny - 1, z2 = k + 1 < g.nz - 1;
          const uint32_t b2 = y2 ? bits_at(gb, pos + 2 * dy) : 0u;
          const uint32_t c2 = z2 ? bits_at(gb, pos + 2 * dz) : 0u;
          const uint32_t d2y = y2 ? bits_at(gb, pos + 2 * dy + dz) : 0u;
          const uint32_t d2z = z2 ? bits_at(gb, pos + dy + 2 * dz) : 0u;
          st[(kFOx + 1) * 32 + lane] = (w.b ^ w.b1) & xmask;
          st[(kFOy + 1) * 32 + lane] = y2 ? (w.b ^ b2) & pmask : 0u;
          st[(kFOz + 1) * 32 + lane] = (w.b ^ w.d) & pmask;
          st[(kFOx + 2) * 32 + lane] = (w.c ^ w.c1) & xmask;
          st[(kFOy + 2) * 32 + lane] = (w.c ^ w.d) & pmask;
          st[(kFOz + 2) * 32 + lane] = z2 ? (w.c ^ c2) & pmask : 0u;
          st[(kFOx + 3) * 32 + lane] = (w.d ^ w.d1) & xmask;
          st[(kFOy + 3) * 32 + lane] = y2 ? (w.d ^ d2y) & pmask : 0u;
          st[(kFOz + 3) * 32 + lane] = z2 ? (w.d ^ d2z) & pmask : 0u;
          const uint32_t rwy = (uint32_t)g.wr, rwz = (uint32_t)g.wr * (uint32_t)g.ny;
          st[(kFOv + 1) * 32 + lane] = __ldg(o.wv + gw + rwy);
          st[(kFOv + 2) * 32 + lane] = __ldg(o.wv + gw + rwz);
          st[(kFOv + 3) * 32 + lane] = __ldg(o.wv + gw + rwy + rwz);
          if (am >> 31) {  // the last cell's +x corners lie in word m + 1
            const int i1 = 32 * m + 32;
            st[kFNx * 32 + lane] = point_xy_bits(g, gb, j, k, i1) |
                                   (point_xy_bits(g, gb, j + 1, k, i1) << 2) |
                                   (point_xy_bits(g, gb, j, k + 1, i1) << 4);
          }
        }
      }
    }
    st[kFAm * 32 + lane] = am;
    int total_c, total_p;
    pre[lane + 1] = warp_exclusive(__popc(am), lane, &total_c) + __popc(am);
    ppre[lane + 1] = warp_exclusive(np, lane, &total_p) + np;
    if (lane == 0) pre[0] = ppre[0] = 0;
    // the batch's triangles are contiguous from its first word's offset
    long long tri_base = __shfl_sync(kFull, t0, 0);
    __syncwarp();
    if (MERGE) {
      // ---- lane = owner point: the points of the words that own crossing
      // edges, in point order; each writes its edges' vertices ---------------
      for (int t = lane; t < total_p; t += 32) {
        const int s = search32(ppre, t);
        const uint32_t X = window(st, kFOx, s), Y = window(st, kFOy, s), Z = window(st, kFOz, s);
        const int b = nth_bit(X | Y | Z, t - ppre[s]);
        const uint32_t lm = (1u << b) - 1u;
        const long long vid0 =
            (long long)window(st, kFOv, s) + __popc(X & lm) + __popc(Y & lm) + __popc(Z & lm);
        const uint32_t own = ((X >> b) & 1u) | (((Y >> b) & 1u) << 1) | (((Z >> b) & 1u) << 2);
        const GridSlot& sl = S.count == 1 ? S.one : S.slots[window(st, kFSlot, s)];
        emit_point_vertices(sl, (int)window(st, kFI0, s) + b, (int)window(st, kFJ, s),
                            (int)window(st, kFK, s), own, vid0, verts, ra, rb, rw);
      }
    }
    // ---- lane = active cell: its case, then all its triangles -------------
    for (int c0 = 0; c0 < total_c; c0 += 32) {
      const int c = c0 + lane;
      int nt = 0, s = 0, q = 0;
      uint64_t cw = 0;
      if (c < total_c) {
        s = search32(pre, c);
        q = nth_bit(window(st, kFAm, s), c - pre[s]);
        CornerWords w;
        w.a = window(st, kFWin + 0, s);
        w.a1 = window(st, kFWin + 1, s);
        w.b = window(st, kFWin + 2, s);
        w.b1 = window(st, kFWin + 3, s);
        w.c = window(st, kFWin + 4, s);
        w.c1 = window(st, kFWin + 5, s);
        w.d = window(st, kFWin + 6, s);
        w.d1 = window(st, kFWin + 7, s);
        cw = s_case[case_of(w, q)];
        nt = (int)(cw >> 60);
      }
      int chunk_tri;
      const int ex = warp_exclusive(nt, lane, &chunk_tri);
      if (nt > 0) {
        const long long tri0 = tri_base + ex;
        const GridSlot& sl = S.count == 1 ? S.one : S.slots[window(st, kFSlot, s)];
        // first vertex of this grid in the concatenated output (0 for one grid)
        const long long vbase0 =
            S.count == 1 ? 0 : (MERGE ? word_v(o, sl.rw0) : 3 * word_t(o, sl.rw0));
        if (MERGE) {
          cell_edge_ids(st, s, q, ids, lane);
          for (int t = 0; t < nt; ++t) {
            int32_t* out = conn + 3 * (tri0 + t);
#pragma unroll
            for (int corner = 0; corner < 3; ++corner)
              out[corner] = (int32_t)((long long)ids[mc_edge(cw, 3 * t + corner) * 32 + lane] - vbase0);
          }
        } else {
          const int i = (int)window(st, kFI0, s) + q, j = (int)window(st, kFJ, s),
                    k = (int)window(st, kFK, s);
          for (int t = 0; t < nt; ++t) {
#pragma unroll
            for (int corner = 0; corner < 3; ++corner) {
              const int info_e = s_edge[mc_edge(cw, 3 * t + corner)];
              const int di = info_e & 1, dj = (info_e >> 1) & 1, dk = (info_e >> 2) & 1;
              const long long vid = 3 * (tri0 + t) + corner;
              conn[vid] = (int32_t)(vid - vbase0);
              emit_vertex(sl, i + di, j + dj, k + dk, info_e >> 3, vid, verts, ra, rb, rw);
            }
          }
        }
      }
      tri_base += chunk_tri;
    }
    __syncwarp();
  }
  // the last block to finish resets the batch counter for the next launch
  // on this scratch
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(done, 1u) == gridDim.x - 1) {
      *ticket = 0;
      *done = 0;
      __threadfence();
    }
  }
}

void launch_mc_emit(const GridSet& S, bool merge, const uint32_t* bits, const WordOffsets& o,
                    Info* info, float* verts, long long vcap, int32_t* conn, long long tcap,
                    int32_t* ra, int32_t* rb, float* rw, int num_sms, cudaStream_t s) {
  launch_mc_emit_range(S, merge, bits, o, info, verts, vcap, conn, tcap, ra, rb, rw, 0,
                       S.rowwords, -1, nullptr, &info->ticket, &info->done, kEmitBatch,
                       kPassEmit, num_sms, s, true);
}

void launch_mc_emit_range(const GridSet& S, bool merge, const uint32_t* bits, const WordOffsets& o,
                          Info* info, float* verts, long long vcap, int32_t* conn, long long tcap,
                          int32_t* ra, int32_t* rb, float* rw, long long word_begin,
                          long long word_end, long long range_end, const uint32_t* slab_act,
                          unsigned* ticket, unsigned* done, int batch, int pass, int num_sms,
                          cudaStream_t s, bool pdl) {
  // the active count lives on the device: one resident wave, warp-stride
  const long long words = word_end - word_begin;
  const long long want = (words + 32 * kEmitWarps - 1) / (32 * kEmitWarps);
  auto go = [&](auto kernel) {
    const int b = resident_blocks(kernel, kEmitWarps * 32, 0, num_sms, want, pass);
    if (pdl)
      launch_pdl(kernel, (unsigned)b, (unsigned)(kEmitWarps * 32), 0, s, S, bits, o, info, verts,
                 vcap, conn, tcap, ra, rb, rw, range_end, slab_act, ticket, done, batch);
    else
      kernel<<<b, kEmitWarps * 32, 0, s>>>(S, bits, o, info, verts, vcap, conn, tcap, ra, rb, rw,
                                           range_end, slab_act, ticket, done, batch);
  };
  if (merge)
    go(k_mc_emit<true>);
  else
    go(k_mc_emit<false>);
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

// k components per point: out[v][c] = Lerp(in[first[v]][c], in[second[v]][c],
// weight[v]) for a Vector3 (or any float tuple) point field, the templated
// CompactPointField (DispatcherGenerateInterpolatedCells.h:107-141,
// GenerateWorklets.h:65-100).  Ids outside [0, P) give NaN, nothing is read.
__global__ void k_interpolate_n(const int32_t* __restrict__ ra, const int32_t* __restrict__ rb,
                                const float* __restrict__ rw, long long n, long long P, int k,
                                const float* __restrict__ in, float* __restrict__ out) {
  const long long total = n * k;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long v = e / k;
    const int c = (int)(e - v * k);
    const int a = __ldg(ra + v), b = __ldg(rb + v);
    float r = __int_as_float(0x7fc00000);
    if (a >= 0 && a < P && b >= 0 && b < P)
      r = lerp_rn(__ldg(in + (long long)a * k + c), __ldg(in + (long long)b * k + c), __ldg(rw + v));
    out[e] = r;
  }
}

void launch_interpolate_n(const int32_t* ra, const int32_t* rb, const float* rw, long long n,
                          long long P, int k, const float* in, float* out, int num_sms,
                          cudaStream_t s) {
  const long long want = (n * k + 255) / 256;
  const long long cap = (long long)num_sms * 16;
  const int blocks = (int)(want < 1 ? 1 : (want < cap ? want : cap));
  k_interpolate_n<<<blocks, 256, 0, s>>>(ra, rb, rw, n, P, k, in, out);
}

void launch_interpolate(const int32_t* ra, const int32_t* rb, const float* rw, long long n,
                        const float* in, float* out, int num_sms, cudaStream_t s) {
  const long long want = (n + 255) / 256;
  const long long cap = (long long)num_sms * 16;
  const int blocks = (int)(want < 1 ? 1 : (want < cap ? want : cap));
  k_interpolate<<<blocks, 256, 0, s>>>(ra, rb, rw, n, in, out);
}

}  // namespace daxgb

// Cell threshold on the in-range bit stream (bit = lo <= f <= hi), on the
// row-word pipeline marching cubes uses.
//
// K2a (k_thr_kept, k_thr_used): per row word w = (point row r = (j, k), word m)
//     kept[w] = cells 32m .. 32m+31 of cell row r whose 8 corners are all in
//               range (ThresholdFunction, dax/worklet/Threshold.h:30-66)
//     used[w] = points 32m .. 32m+31 of point row r that are a corner of a
//               kept cell (FillPointMask,
//               dax/cont/DispatcherGenerateTopology.h:206-227): the OR of the
//               kept masks of cell rows (j-1..j, k-1..k), each with its +x
//               neighbour cell
//     wc[w]   = popc(kept) << 16 | popc(used), and per-tile totals
// K2b (k_word_scan, shared with marching cubes): per-word exclusive offsets
//     wt (kept cells) and wv (used points), the compacted list act of the
//     words with either, and the totals.
// K3 (k_thr_emit): a warp loads 32 active words at once (lane = word),
//     starts the copies of the field values of all their used points into
//     shared memory (cp.async, one wait per batch), then walks the words
//     with lane = bit: the word's used points (coordinates and field:
//     StreamCompact with the point mask, :237-239 and :98-113) and
//     its kept cells, whose 8 corner ids are each corner's rank among the
//     used points.  That equals the reference's Copy/Sort/Unique/LowerBounds
//     of the connectivity (:229-258), because the used ids sorted ascending
//     are exactly the used points in point order.
#include "common.cuh"
#include "kernels.cuh"

namespace daxgb {

// Bit positions fit in 32 bits: grids hold fewer than 2^31 points, and the
// largest position read, a point plus two planes, stays below 2^32.
__device__ __forceinline__ uint32_t bits_at_u32(const uint32_t* __restrict__ bits, uint32_t pos) {
  return __funnelshift_r(__ldg(bits + (pos >> 5)), __ldg(bits + (pos >> 5) + 1), pos & 31u);
}

// Kept mask of cell-row word w (0 on rows without cells).
__device__ __forceinline__ uint32_t kept_word(const Grid& g, const uint32_t* __restrict__ bits,
                                              uint32_t w) {
  const uint32_t nx = (uint32_t)g.nx, dy = nx, dz = nx * (uint32_t)g.ny;
  int mi, ji, ki;
  const uint32_t r = split_word(g, w, mi);
  split_row(g, r, ji, ki);
  const uint32_t m = (uint32_t)mi, j = (uint32_t)ji, k = (uint32_t)ki;
  if (j + 1 >= (uint32_t)g.ny || k + 1 >= (uint32_t)g.nz) return 0u;
  const uint32_t pos = r * nx + 32u * m;
  const uint32_t p0 = pos, p1 = pos + dy, p2 = pos + dz, p3 = pos + dy + dz;
  return bits_at_u32(bits, p0) & bits_at_u32(bits, p0 + 1) & bits_at_u32(bits, p1) &
         bits_at_u32(bits, p1 + 1) & bits_at_u32(bits, p2) & bits_at_u32(bits, p2 + 1) &
         bits_at_u32(bits, p3) & bits_at_u32(bits, p3 + 1) & low_mask(g.nx - 1 - 32 * (int)m);
}

// K2a, first pass: kept masks of every cell-row word, four consecutive words
// per thread; four words of one row come from five bit-word fetches per
// corner row.
__global__ void __launch_bounds__(256) k_thr_kept(Grid g, const uint32_t* __restrict__ bits,
                                                  uint32_t* __restrict__ kept) {
  pdl_trigger();
  pdl_wait();  // the classification's bits
  const long long W = g.R * g.wr;  // < 2^27 for grids below 2^31 points
  const long long groups = (W + 3) / 4;
  const long long dy = g.nx, dz = (long long)g.nx * g.ny;
  for (long long q4 = (long long)blockIdx.x * blockDim.x + threadIdx.x; q4 < groups;
       q4 += (long long)gridDim.x * blockDim.x) {
    const long long w0 = 4 * q4;
    int m, j, k;
    const unsigned r = split_word(g, (unsigned)w0, m);
    split_row(g, r, j, k);
    uint32_t K[4] = {0u, 0u, 0u, 0u};
    if (m + 4 <= g.wr) {  // four words of one row
      if (j + 1 < g.ny && k + 1 < g.nz) {
        const long long pos = (long long)r * g.nx + 32ll * m;
        uint32_t a[4], a1[4], b[4], b1[4], c[4], c1[4], d[4], d1[4];
        row_windows4(bits, pos, a, a1);
        row_windows4(bits, pos + dy, b, b1);
        row_windows4(bits, pos + dz, c, c1);
        row_windows4(bits, pos + dy + dz, d, d1);
#pragma unroll
        for (int q = 0; q < 4; ++q)
          K[q] = a[q] & a1[q] & b[q] & b1[q] & c[q] & c1[q] & d[q] & d1[q] &
                 low_mask(g.nx - 1 - 32 * (m + q));
      }
    } else {
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (w0 + q < W) K[q] = kept_word(g, bits, (uint32_t)(w0 + q));
    }
    if (w0 + 4 <= W) {
      *reinterpret_cast<uint4*>(kept + w0) = make_uint4(K[0], K[1], K[2], K[3]);
    } else {
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (w0 + q < W) kept[w0 + q] = K[q];
    }
  }
}

// Used mask of point-row word w = (row r = (j, k), word m): the OR of the
// kept masks of cell rows (j - 1 .. j, k - 1 .. k), each with its +x
// neighbour cell.
__device__ __forceinline__ uint32_t used_word(const Grid& g, const uint32_t* __restrict__ kept,
                                              uint32_t w, uint32_t m, uint32_t j, uint32_t k) {
  const uint32_t wy = (uint32_t)g.wr, wz = (uint32_t)g.wr * (uint32_t)g.ny;
  uint32_t u = 0u;
#pragma unroll
  for (int c = 0; c < 4; ++c) {  // cell rows (j - (c & 1), k - (c >> 1))
    const uint32_t cj = c & 1, ck = c >> 1;
    if (j < cj || k < ck) continue;
    const uint32_t wq = w - cj * wy - ck * wz;
    const uint32_t K = __ldg(kept + wq);
    const uint32_t Kp = m > 0 ? __ldg(kept + wq - 1) : 0u;
    u |= K | (K << 1) | (Kp >> 31);
  }
  return u & low_mask(g.nx - 32 * (int)m);
}

// K2a, second pass: one 256-thread block per tile of kScanTile words
// (grid-stride over tiles), thread t taking the 4-word groups t + 256 e:
// used masks, packed counts and tile totals.
__global__ void __launch_bounds__(256) k_thr_used(Grid g, const uint32_t* __restrict__ kept,
                                                  uint32_t* __restrict__ used,
                                                  uint32_t* __restrict__ wc,
                                                  uint32_t* __restrict__ tile_tot, int tiles) {
  __shared__ uint32_t s_red[24];
  pdl_trigger();
  pdl_wait();  // the kept masks
  const long long W = g.R * g.wr;
  const uint32_t wy = (uint32_t)g.wr, wz = (uint32_t)g.wr * (uint32_t)g.ny;
  for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    uint32_t sk = 0, su = 0, sa = 0;
#pragma unroll 1
    for (int e = 0; e < kScanItems / 4; ++e) {
      const long long w0 = (long long)tile * kScanTile + 4ll * (threadIdx.x + 256 * e);
      if (w0 >= W) break;
      int mi, ji, ki;
      const uint32_t r = split_word(g, (uint32_t)w0, mi);
      split_row(g, r, ji, ki);
      const uint32_t m = (uint32_t)mi, j = (uint32_t)ji, k = (uint32_t)ki;
      uint32_t own[4] = {0u, 0u, 0u, 0u}, U[4] = {0u, 0u, 0u, 0u};
      if (m + 4 <= wy) {  // four words of one row: 5 kept words per cell row
#pragma unroll
        for (int c = 0; c < 4; ++c) {  // cell rows (j - (c & 1), k - (c >> 1))
          const uint32_t cj = c & 1, ck = c >> 1;
          if (j < cj || k < ck) continue;
          const uint32_t wq = (uint32_t)w0 - cj * wy - ck * wz;
          uint32_t K[5];
          K[0] = m > 0 ? __ldg(kept + wq - 1) : 0u;
#pragma unroll
          for (int q = 0; q < 4; ++q) K[q + 1] = __ldg(kept + wq + q);
#pragma unroll
          for (int q = 0; q < 4; ++q) U[q] |= K[q + 1] | (K[q + 1] << 1) | (K[q] >> 31);
          if (c == 0) {
#pragma unroll
            for (int q = 0; q < 4; ++q) own[q] = K[q + 1];
          }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) U[q] &= low_mask(g.nx - 32 * (int)(m + q));
      } else {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const long long w = w0 + q;
          if (w >= W) break;
          int mq, jq, kq;
          const uint32_t rq = split_word(g, (uint32_t)w, mq);
          split_row(g, rq, jq, kq);
          own[q] = __ldg(kept + w);
          U[q] = used_word(g, kept, (uint32_t)w, (uint32_t)mq, (uint32_t)jq, (uint32_t)kq);
        }
      }
      uint32_t pk[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        pk[q] = (uint32_t)__popc(own[q]) << 16 | (uint32_t)__popc(U[q]);
        sk += pk[q] >> 16;
        su += pk[q] & 0xffffu;
        sa += pk[q] ? 1u : 0u;
      }
      if (w0 + 4 <= W) {
        *reinterpret_cast<uint4*>(used + w0) = make_uint4(U[0], U[1], U[2], U[3]);
        *reinterpret_cast<uint4*>(wc + w0) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
      } else {
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (w0 + q < W) {
            used[w0 + q] = U[q];
            wc[w0 + q] = pk[q];
          }
      }
    }
    block_sum3(sk, su, sa, s_red);
    if (threadIdx.x == 0) {
      tile_tot[tile] = sk;
      tile_tot[tiles + tile] = su;
      tile_tot[2 * tiles + tile] = sa;
    }
  }
}

void launch_thr_count(const Grid& g, const uint32_t* bits, uint32_t* kept, uint32_t* used,
                      uint32_t* wc, uint32_t* tile_tot, int num_sms, cudaStream_t s) {
  const long long W = g.R * g.wr;
  const int b1 = resident_blocks(k_thr_kept, 256, 0, num_sms, (W + 1023) / 1024);
  launch_pdl(k_thr_kept, (unsigned)b1, 256u, 0, s, g, bits, kept);
  const int tiles = word_scan_tiles(W);
  const int b2 = resident_blocks(k_thr_used, 256, 0, num_sms, tiles);
  launch_pdl(k_thr_used, (unsigned)b2, 256u, 0, s, g, kept, used, wc, tile_tot, tiles);
}

// Per active word, what the emit loop needs: its masks and offsets, and for
// kept cells the used masks and offsets of corner rows q = dj + 2 dk
// (q = 1..3) at word m, and the first used-point offsets of rows q = 0..3 at
// word m + 1 (the +x corner of a cell at bit 31 is that word's first point,
// always used).
struct ThrWord {
  uint32_t w, u, kw, v0, t0;
  uint32_t r, m, j, k;  // the word's point row (j, k) and word index in the row
  uint32_t cu[3], cv[7];
};

__global__ void __launch_bounds__(256) k_thr_emit(Grid g, const float* __restrict__ f,
                                                  const uint32_t* __restrict__ kept,
                                                  const uint32_t* __restrict__ used,
                                                  const uint32_t* __restrict__ wt,
                                                  const uint32_t* __restrict__ wv,
                                                  const uint32_t* __restrict__ act,
                                                  Info* __restrict__ info,
                                                  int32_t* __restrict__ conn, long long kcap,
                                                  float* __restrict__ coords,
                                                  float* __restrict__ fout, long long ucap) {
  const long long K = info->total_a, U = info->total_b, A = info->total_c;
  if (K > kcap || U > ucap || (info->error & (kErrOverflow | kErrTimeout))) {
    if (blockIdx.x == 0 && threadIdx.x == 0 && (K > kcap || U > ucap))
      atomicOr(&info->error, kErrCapacity);
    return;
  }
  const int lane = threadIdx.x & 31;
  const uint32_t below = (1u << lane) - 1u;
  const bool conn16 = (reinterpret_cast<uintptr_t>(conn) & 15) == 0;
  const long long warp0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  const unsigned wr = (unsigned)g.wr;
  __shared__ float s_field[8][32][32];  // per warp: field value of bit `lane` of batch word s
  float (*const sf)[32] = s_field[threadIdx.x >> 5];
  for (long long a0 = warp0 * 32; a0 < A; a0 += nwarps * 32) {
    // lane L gathers active word a0 + L
    ThrWord d{};
    const int cnt = (int)min(32ll, A - a0);
    if (lane < cnt) {
      d.w = __ldg(act + a0 + lane);
      d.u = __ldg(used + d.w);
      d.kw = __ldg(kept + d.w);
      d.v0 = __ldg(wv + d.w);
      d.t0 = __ldg(wt + d.w);
      int mi, ji, ki;
      d.r = split_word(g, d.w, mi);
      split_row(g, d.r, ji, ki);
      d.m = (uint32_t)mi;
      d.j = (uint32_t)ji;
      d.k = (uint32_t)ki;
      if (d.kw) {  // a kept cell implies rows j + 1 and k + 1 exist
        const unsigned m = d.m;
        const uint32_t rows[4] = {d.w, d.w + wr, d.w + (unsigned)g.ny * wr,
                                  d.w + (unsigned)(g.ny + 1) * wr};
#pragma unroll
        for (int q = 1; q < 4; ++q) {
          d.cu[q - 1] = __ldg(used + rows[q]);
          d.cv[q - 1] = __ldg(wv + rows[q]);
        }
        if (m + 1 < wr) {
#pragma unroll
          for (int q = 0; q < 4; ++q) d.cv[3 + q] = __ldg(wv + rows[q] + 1);
        }
      }
    }
    if (fout) {
      // the field values of the batch's used points, all copies in flight at
      // once (a field read is a DRAM round trip: K1 streamed it evict-first)
      for (int s = 0; s < cnt; ++s) {
        const uint32_t u = __shfl_sync(kFull, d.u, s);
        const uint32_t r = __shfl_sync(kFull, d.r, s), m = __shfl_sync(kFull, d.m, s);
        const bool on = (u >> lane) & 1u;
        const float* src = on ? f + ((long long)r * g.nx + 32 * m + lane) : f;
        const unsigned dst = (unsigned)__cvta_generic_to_shared(&sf[s][lane]);
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(dst), "l"(src),
                     "r"(on ? 4 : 0)
                     : "memory");
      }
      asm volatile("cp.async.commit_group;\n" ::: "memory");
      asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    }
    for (int s = 0; s < cnt; ++s) {
      const uint32_t u = __shfl_sync(kFull, d.u, s);
      const uint32_t kw = __shfl_sync(kFull, d.kw, s);
      const uint32_t m = __shfl_sync(kFull, d.m, s);
      const int j = (int)__shfl_sync(kFull, d.j, s), k = (int)__shfl_sync(kFull, d.k, s);
      const int i = 32 * (int)m + lane;
      const uint32_t v0 = __shfl_sync(kFull, d.v0, s);
      if ((u >> lane) & 1u) {
        const long long id = (long long)v0 + __popc(u & below);
        float* c = coords + 3 * id;
        c[0] = coord(g.ox, g.sx, i, g.mx);
        c[1] = coord(g.oy, g.sy, j, g.my);
        c[2] = coord(g.oz, g.sz, k, g.mz);
        if (fout) fout[id] = sf[s][lane];
      }
      if (kw == 0u) continue;  // uniform across the warp
      const uint32_t t0 = __shfl_sync(kFull, d.t0, s);
      uint32_t cu[4], cv[8];  // corner rows q at word m (0..3); cv[4 + q]: at word m + 1
      cu[0] = u;
      cv[0] = v0;
#pragma unroll
      for (int e = 0; e < 3; ++e) cu[e + 1] = __shfl_sync(kFull, d.cu[e], s);
#pragma unroll
      for (int e = 0; e < 7; ++e) cv[e + 1] = __shfl_sync(kFull, d.cv[e], s);
      if ((kw >> lane) & 1u) {
        const long long cid = (long long)t0 + __popc(kw & below);
        // used-point ranks of the corners at i (lo) and i + 1 (hi) of corner
        // rows q = dj + 2 dk: hi = lo + the bit of point i, except on lane
        // 31, whose i + 1 is bit 0 of word m + 1
        int32_t lo[4], hi[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const uint32_t b = cv[q] + (uint32_t)__popc(cu[q] & below);
          lo[q] = (int32_t)b;
          hi[q] = (int32_t)(lane == 31 ? cv[4 + q] : b + ((cu[q] >> lane) & 1u));
        }
        // v0..v7: (i,j,k) (i+1,j,k) (i+1,j+1,k) (i,j+1,k), then the same at k+1
        const int32_t ids[8] = {lo[0], hi[0], hi[1], lo[1], lo[2], hi[2], hi[3], lo[3]};
        if (conn16) {
          int4* dst = reinterpret_cast<int4*>(conn + 8 * cid);
          dst[0] = make_int4(ids[0], ids[1], ids[2], ids[3]);
          dst[1] = make_int4(ids[4], ids[5], ids[6], ids[7]);
        } else {
#pragma unroll
          for (int v = 0; v < 8; ++v) conn[8 * cid + v] = ids[v];
        }
      }
    }
  }
}

// CompactPointField of DispatcherGenerateTopology (:98-113): any point
// field of `comps` floats per point, compacted to the used points in point
// order -- the order of the threshold's output coordinates.  A warp per row
// word, lane = bit: a used point's output index is its word's used-point
// offset plus its rank in the word.  Needs the count pass (used masks, word
// offsets, totals) on the same scratch; writes nothing when the used points
// exceed `cap`.
__global__ void __launch_bounds__(256) k_thr_compact_field(Grid g, const uint32_t* __restrict__ used,
                                                           const uint32_t* __restrict__ wv,
                                                           Info* __restrict__ info,
                                                           const float* __restrict__ in, int comps,
                                                           float* __restrict__ out, long long cap) {
  const long long U = info->total_b;
  if (U > cap || (info->error & (kErrOverflow | kErrTimeout))) {
    if (blockIdx.x == 0 && threadIdx.x == 0 && U > cap) atomicOr(&info->error, kErrCapacity);
    return;
  }
  const int lane = threadIdx.x & 31;
  const long long W = g.R * g.wr;
  const long long warp0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long w = warp0; w < W; w += nwarps) {
    const uint32_t u = __ldg(used + w);
    if (!((u >> lane) & 1u)) continue;
    int m;
    const unsigned r = split_word(g, (unsigned)w, m);
    const long long p = (long long)r * g.nx + 32ll * m + lane;
    const long long id = (long long)__ldg(wv + w) + __popc(u & ((1u << lane) - 1u));
    for (int c = 0; c < comps; ++c) out[id * comps + c] = __ldg(in + p * comps + c);
  }
}

void launch_thr_compact_field(const Grid& g, const uint32_t* used, const uint32_t* wv, Info* info,
                              const float* in, int comps, float* out, long long cap, int num_sms,
                              cudaStream_t s) {
  const long long want = (g.R * g.wr + 7) / 8;  // a warp per word, 8 warps a block
  const int blocks = resident_blocks(k_thr_compact_field, 256, 0, num_sms, want);
  k_thr_compact_field<<<blocks, 256, 0, s>>>(g, used, wv, info, in, comps, out, cap);
}

void launch_thr_emit(const Grid& g, const float* f, const WordOffsets& o, const uint32_t* kept,
                     const uint32_t* used, Info* info, int32_t* conn, long long kcap,
                     float* coords, float* fout, long long ucap, int num_sms, cudaStream_t s) {
  // the active count lives on the device: one resident wave, grid-stride
  const long long want = (g.R * g.wr + 255) / 256;
  const int blocks = resident_blocks(k_thr_emit, 256, 0, num_sms, want);
  // an ordinary launch: the warps split the active words statically, so all
  // blocks should start together on an idle device (launched early into the
  // SMs the scan frees, they measured 20 us slower at 512^3)
  k_thr_emit<<<blocks, 256, 0, s>>>(g, f, kept, used, o.wt, o.wv, o.act, info, conn, kcap, coords,
                                    fout, ucap);
}

}  // namespace daxgb
